// Batched PNCG: many independent meshes, one set of launches per iteration.
//
// The meshes' vertices and tiles are concatenated (tiles never span meshes,
// vertex chunks never span meshes).  An iteration is five kernels, captured
// once in a CUDA graph; every mesh carries its own SolverState, so each one
// runs the reference's PNCG iteration (benches/bench_pncg_branching_backends.py
// :254-456, 606-679) with its own beta, step and termination:
//   direction pass   one CTA per tile: p of the tile's mesh, p^T H p and the
//                    energy polynomial; one partial per tile
//   direction tail   one CTA per mesh: the mesh's tile partials in tile order,
//                    then the Armijo decision (dir_decide)
//   gradient pass    one CTA per tile at x + t_mesh p (grad_tile)
//   vertex pass      one CTA per vertex chunk: x, g, d and the 12 sums
//   vertex tail      one CTA per mesh: chunk partials in order, then beta and
//                    termination (vertex_decide); the last CTA to finish
//                    counts the meshes still running and sets the graph's
//                    while-condition
// Tiles and chunks of a finished mesh return at once.
#include "kernels.h"
#include "solver.h"
#include "solver_common.cuh"

namespace agb {

namespace {

constexpr int kTailThreads = 256;

template <class R, int MAT>
__global__ void __launch_bounds__(kElemThreads) batch_dir_kernel(BatchArgs b) {
  constexpr int N = 6;
  // float-float warp tree for c2 (terms of both signs); ARAP sums p^T H p only
  constexpr unsigned FF = snh_family(MAT) ? 0x2u : 0x0u;
  __shared__ V4<R> sx[kTileVerts];
  __shared__ V4<R> sp[kTileVerts];
  __shared__ Acc<R> red[kWarps * N];
  const SolveArgs& a = b.a;
  const int tile = blockIdx.x;
  if (b.cond && tile == 0 && threadIdx.x == 0)
    cudaGraphSetConditional((cudaGraphConditionalHandle)b.cond, 0u);  // the vertex tail re-arms
  pdl_trigger();
  SolverState* st = b.st + b.tile_mesh[tile];
  if (st->done) return;
  const R beta = (R)st->beta, inv_mean = (R)st->inv_mean;
  const int pb = st->pbuf;
  stage_dir<R>(a, tile_vertex(a.fv, tile, threadIdx.x), beta, inv_mean, p_prev<R>(a, pb), p_cur<R>(a, pb), sx,
               sp);
  __syncthreads();
  Acc<R> sums[N] = {};
  const int es = a.fv.tile_estart[tile], ee = a.fv.tile_estart[tile + 1];
  const V4<R>* csvd = MAT == AGB_ARAP ? svd_cache<R>(a, st->sbuf) : nullptr;
  for (int e = es + threadIdx.x; e < ee; e += blockDim.x) {
    ElemGeo<R> geo;
    uint32_t ids;
    load_elem_m<R, MAT>(a.fv, e, geo, ids);
    const int l[4] = {corner(ids, 0), corner(ids, 1), corner(ids, 2), corner(ids, 3)};
    R dF[3][3];
    vec_gradient(sp, l, geo.D, dF);
    if constexpr (snh_family(MAT)) {
      R G[3][3];
      vec_gradient(sx, l, geo.D, G);
      add_act<MAT>(geo, G);
      SnhPoint<R> s;
      snh_prepare(G, s);
      SnhDir<R> d;
      snh_dir(s, dF, d);
      sums[0].add(fmax(snh_hess_quad(s, d, geo.mu, geo.lam), R(0)));
      R c[5];
      snh_poly(s, d, geo.mu, geo.lam, c);
#pragma unroll
      for (int m = 0; m < 5; ++m) sums[1 + m].add(c[m]);
    } else {
      // the SVD at x, kept by the gradient pass that evaluated x
      Svd<R> sv;
      svd_get(csvd, (size_t)a.fv.n_cells, e, sv);
      R lk[3];
      arap_lambdas(sv, lk);
      sums[0].add(fmax(arap_hess_quad(sv, lk, dF, geo.mu), R(0)));
    }
  }
  block_reduce<N, FF, R>(sums, red);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) ((AccStore<R>*)b.part_dir)[(size_t)tile * N + k] = acc_store(sums[k]);
  }
}

template <class R, int MAT>
__global__ void __launch_bounds__(kTailThreads) batch_dir_tail_kernel(BatchArgs b) {
  constexpr int N = 6;
  __shared__ Acc<R> red[(kTailThreads / 32) * N];
  pdl_trigger();
  pdl_wait();
  SolverState* st = b.st + blockIdx.x;
  if (st->done) return;
  if (threadIdx.x == 0) st->refresh = 0;  // the refresh passes, if any, ran after the last vertex tail
  const int t0 = b.mesh_tile0[blockIdx.x], t1 = b.mesh_tile0[blockIdx.x + 1];
  Acc<R> s[N] = {};
  for (int t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
#pragma unroll
    for (int k = 0; k < N; ++k) s[k].add(acc_load<R>((const AccStore<R>*)b.part_dir + (size_t)t * N + k));
  }
  block_reduce<N, 0xffffffffu, R>(s, red);
  if (threadIdx.x == 0) {
    double tot[N];
#pragma unroll
    for (int k = 0; k < N; ++k) tot[k] = s[k].value();
    dir_decide<MAT>(st, tot);
  }
}

// ARAP: the gradient pass at the first trial step x + alpha_0 p of each
// tile's mesh (grad_tile's speculative form), its energy remainders summed
// per tile
template <class R>
__global__ void __launch_bounds__(kGradThreads, 4) batch_grad_spec_kernel(BatchArgs b) {
  __shared__ Acc<R> red[kGradWarps];
  Acc<R> rem[1] = {};
  const int tile = blockIdx.x;
  if (!grad_tile<R, AGB_ARAP, false, true>(b.a, tile, b.st + b.tile_mesh[tile], &rem[0])) return;
  block_reduce<1, 0x1u, R>(rem, red);
  if (threadIdx.x == 0) ((AccStore<R>*)b.part_grad)[tile] = acc_store(rem[0]);
}

// ARAP: per mesh, the Armijo test of alpha_0 from its tiles' remainders
template <class R>
__global__ void __launch_bounds__(kTailThreads) batch_spec_tail_kernel(BatchArgs b) {
  __shared__ Acc<R> red[kTailThreads / 32];
  pdl_trigger();
  pdl_wait();
  SolverState* st = b.st + blockIdx.x;
  if (st->done) return;
  const int t0 = b.mesh_tile0[blockIdx.x], t1 = b.mesh_tile0[blockIdx.x + 1];
  const double rem = block_sum_partials<R>((const AccStore<R>*)b.part_grad + t0, t1 - t0, 1, red);
  if (threadIdx.x == 0) spec_decide(st, rem);
}

// ARAP: trial remainders at alpha_0 2^-j, j = j0 .. j0+nt-1, per tile of a
// mesh whose step is not decided yet (three per tile into part_dir)
template <class R>
__global__ void __launch_bounds__(kElemThreads) batch_trial_kernel(BatchArgs b, int j0, int nt) {
  __shared__ Acc<R> red[kWarps * 3];
  const int tile = blockIdx.x;
  const SolverState* st = b.st + b.tile_mesh[tile];
  if (st->done || st->decided) return;
  Acc<R> sums[3] = {};
  trial_tile<R>(b.a, tile, st, j0, nt, sums);
  block_reduce<3, 0x7u, R>(sums, red);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < 3; ++j) ((AccStore<R>*)b.part_dir)[(size_t)tile * 6 + j] = acc_store(sums[j]);
  }
}

template <class R>
__global__ void __launch_bounds__(kTailThreads) batch_trial_tail_kernel(BatchArgs b, int j0, int nt) {
  __shared__ Acc<R> red[(kTailThreads / 32) * 3];
  SolverState* st = b.st + blockIdx.x;
  if (st->done || st->decided) return;
  const int t0 = b.mesh_tile0[blockIdx.x], t1 = b.mesh_tile0[blockIdx.x + 1];
  Acc<R> s[3] = {};
  for (int t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
#pragma unroll
    for (int j = 0; j < 3; ++j) s[j].add(acc_load<R>((const AccStore<R>*)b.part_dir + (size_t)t * 6 + j));
  }
  block_reduce<3, 0xffffffffu, R>(s, red);
  if (threadIdx.x == 0) {
    double tot[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) tot[j] = s[j].value();
    trial_decide(st, st->alpha0, j0, nt, tot);
  }
}

// fallback (ARAP): the pass after the trial passes, for the meshes whose
// speculative step was rejected
template <class R, int MAT, bool DELTA>
__global__ void __launch_bounds__(kGradThreads, 6) batch_grad_kernel(BatchArgs b, int fallback) {
  grad_tile<R, MAT, DELTA>(b.a, blockIdx.x, b.st + b.tile_mesh[blockIdx.x], nullptr, fallback != 0);
}

// phase (ARAP): 1 after the speculative gradient pass, for the meshes whose
// alpha_0 was accepted; 2 after the fallback passes, for the others; 0: all
template <class R, bool DELTA>
__global__ void __launch_bounds__(kVThreads) batch_vertex_kernel(BatchArgs b, int phase) {
  constexpr int N = 12;
  constexpr unsigned FF = (1u << 1) | (1u << 6) | (1u << 8) | (1u << 9);
  __shared__ Acc<R> red[(kVThreads / 32) * N];
  const SolveArgs& a = b.a;
  const int c = blockIdx.x;
  const int v0 = b.chunk_v0[c], v1 = b.chunk_v0[c + 1];
  const SolverState* st = b.st + b.chunk_mesh[c];
  pdl_trigger();
  pdl_wait();
  if (st->done) return;
  if ((phase == 1 && !st->spec_ok) || (phase == 2 && st->spec_ok)) return;
  const R t = (R)st->t;
  const V4<R>* P = p_cur<R>(a, st->pbuf);
  R s[N] = {};
  for (int i = v0 + threadIdx.x; i < v1; i += blockDim.x) vertex_update<R, DELTA>(a, i, a.off[i], a.off[i + 1], t, P, s);
  Acc<R> acc[N];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    acc[k] = Acc<R>{};
    acc[k].add(s[k]);
  }
  block_reduce<N, FF, R>(acc, red);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) ((AccStore<R>*)b.part_vert)[(size_t)c * N + k] = acc_store(acc[k]);
  }
}

// phase as in batch_vertex_kernel; the pass of phase 1 decides its meshes
// only, the others also count the meshes still running
template <class R>
__global__ void __launch_bounds__(kTailThreads) batch_vertex_tail_kernel(BatchArgs b, int phase) {
  constexpr int N = 12;
  __shared__ Acc<R> red[(kTailThreads / 32) * N];
  __shared__ bool s_last;
  pdl_wait();
  SolverState* st = b.st + blockIdx.x;
  // read by every thread before thread 0 writes the state
  const bool was_done = st->done != 0;
  const bool mine = phase == 0 || (phase == 1) == (st->spec_ok != 0);
  __syncthreads();
  if (phase == 1 && !mine) return;
  if (!was_done && mine) {
    const int c0 = b.mesh_chunk0[blockIdx.x], c1 = b.mesh_chunk0[blockIdx.x + 1];
    Acc<R> s[N] = {};
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
#pragma unroll
      for (int k = 0; k < N; ++k) s[k].add(acc_load<R>((const AccStore<R>*)b.part_vert + (size_t)c * N + k));
    }
    block_reduce<N, 0xffffffffu, R>(s, red);
    if (threadIdx.x == 0) {
      double tot[N];
#pragma unroll
      for (int k = 0; k < N; ++k) tot[k] = s[k].value();
      vertex_decide(st, tot);
      if (b.a.svd) st->sbuf ^= 1;  // the gradient pass's SVDs are those at the new x
    }
  }
  if (phase == 1) return;
  if (threadIdx.x == 0) {
    if (!st->done) atomicAdd(&b.bs->n_active, 1u);
    __threadfence();
    s_last = atomicAdd(&b.bs->arrived, 1u) == (unsigned)b.n_meshes - 1u;
  }
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return;
  __threadfence();
  BatchState* bs = b.bs;
  const unsigned active = atomicAdd(&bs->n_active, 0u);
  bs->iter += 1;
  bs->n_active = 0u;
  bs->arrived = 0u;
  if (b.cond)
    cudaGraphSetConditional((cudaGraphConditionalHandle)b.cond,
                            (active > 0u && bs->iter < bs->iter_limit) ? 1u : 0u);
}

// reference-state refresh of the models that asked for one (FP32)
// (grid-stride over tiles / chunks with a resident-sized grid)
template <int MAT>
__global__ void __launch_bounds__(kGradThreads) batch_ref_elem_kernel(BatchArgs b) {
  pdl_trigger();
  pdl_wait();
  for (int tile = blockIdx.x; tile < b.a.fv.n_tiles; tile += gridDim.x) {
    if (!b.st[b.tile_mesh[tile]].refresh) continue;  // uniform across the CTA
    ref_tile<MAT>(b.a, tile);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kVThreads) batch_ref_vertex_kernel(BatchArgs b) {
  pdl_trigger();
  pdl_wait();
  for (int c = blockIdx.x; c < b.n_chunks; c += gridDim.x) {
    if (!b.st[b.chunk_mesh[c]].refresh) continue;
    for (int i = b.chunk_v0[c] + threadIdx.x; i < b.chunk_v0[c + 1]; i += blockDim.x) ref_vertex(b.a, i);
  }
}

__global__ void batch_force_refresh_kernel(BatchArgs b) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < b.n_meshes; m += gridDim.x * blockDim.x) b.st[m].refresh = 1;
}

template <class R, int MAT>
__global__ void __launch_bounds__(kElemThreads) batch_energy_pass_kernel(BatchArgs b) {
  energy_tile<R, MAT>(b.a, blockIdx.x, (AccStore<R>*)b.part_grad + blockIdx.x);
}

template <class R>
__global__ void __launch_bounds__(kTailThreads) batch_energy_kernel(BatchArgs b) {
  __shared__ Acc<R> red[kTailThreads / 32];
  const int t0 = b.mesh_tile0[blockIdx.x], t1 = b.mesh_tile0[blockIdx.x + 1];
  const double e = block_sum_partials<R>((const AccStore<R>*)b.part_grad + t0, t1 - t0, 1, red);
  if (threadIdx.x == 0) b.st[blockIdx.x].energy = e + b.st[blockIdx.x].ext_energy;
}

template <class R>
__global__ void batch_init_vertex_kernel(BatchArgs b, const R* __restrict__ u, const V4<R>* __restrict__ fixed,
                                         const int32_t* __restrict__ uoi) {
  const SolveArgs& a = b.a;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n_points; i += gridDim.x * blockDim.x) {
    const size_t k = 3 * (size_t)uoi[i];
    const V4<R> fx = fixed[i];
    const int mask = (int)fx.w;
    V4<R> x{u[k], u[k + 1], u[k + 2], fx.w};
    if (mask & 1) x.x = fx.x;
    if (mask & 2) x.y = fx.y;
    if (mask & 4) x.z = fx.z;
    const V4<R> z{R(0), R(0), R(0), R(0)};
    ((V4<R>*)a.xa)[2 * i] = x;
    ((V4<R>*)a.xa)[2 * i + 1] = z;
    ((V4<R>*)a.gd)[2 * i] = z;
    ((V4<R>*)a.gd)[2 * i + 1] = z;
    ((V4<R>*)a.p0)[i] = z;
    ((V4<R>*)a.p1)[i] = z;
    if (a.delta) {
      ((V4<R>*)a.xref)[i] = z;
      ((V4<R>*)a.gref)[i] = z;
    }
  }
}

__global__ void batch_init_state_kernel(BatchArgs b, SolverState proto) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < b.n_meshes; m += gridDim.x * blockDim.x) {
    SolverState st = proto;
    st.beta = 0.0;
    st.inv_mean = 1.0;
    st.gd = st.t = st.alpha0 = st.hq = st.gnorm = st.gnorm0 = st.energy = st.ext_energy = st.delta_e = 0.0;
    st.iter = 0;
    st.iter_limit = 0;
    st.done = 0;
    st.result = AGB_RUNNING;
    st.init = 1;
    st.reset_beta = st.ls_fail = st.ls_steps = st.ls_ok = 0;
    st.decided = 1;
    st.error = 0;
    st.pbuf = 0;
    st.refresh = 0;
    st.gnorm_ref = 0.0;
    st.sbuf = 0;
    st.spec_ok = 0;
    b.st[m] = st;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *b.bs = BatchState{0, 0, 0u, 0u};
}

__global__ void batch_set_limit_kernel(BatchState* bs, int n) { bs->iter_limit = bs->iter + n; }

template <class... P, class... A>
cudaError_t launch_pdl_b(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

cudaError_t batch_refresh(const BatchArgs& b, cudaStream_t s) {
  cudaError_t e = b.a.fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE
                      ? launch_pdl_b(batch_ref_elem_kernel<AGB_STABLE_NEO_HOOKEAN_MUSCLE>,
                                     dim3(ref_blocks(b.a.fv.n_tiles)), dim3(kGradThreads), ref_smem_bytes(), s, b)
                      : launch_pdl_b(batch_ref_elem_kernel<AGB_STABLE_NEO_HOOKEAN>, dim3(ref_blocks(b.a.fv.n_tiles)),
                                     dim3(kGradThreads), ref_smem_bytes(), s, b);
  const int vb = b.n_chunks < kSMs * 8 ? b.n_chunks : kSMs * 8;
  if (e == cudaSuccess) e = launch_pdl_b(batch_ref_vertex_kernel, dim3(vb > 0 ? vb : 1), dim3(kVThreads), 0, s, b);
  return e;
}

template <class R, int MAT, bool DELTA>
cudaError_t batch_grad_and_vertex_d(const BatchArgs& b, cudaStream_t s, int fallback = 0) {
  const int phase = fallback ? 2 : 0;
  cudaError_t e = launch_pdl_b(batch_grad_kernel<R, MAT, DELTA>, dim3(b.a.fv.n_tiles), dim3(kGradThreads),
                               grad_smem_bytes<R>(), s, b, fallback);
  if (e == cudaSuccess)
    e = launch_pdl_b(batch_vertex_kernel<R, DELTA>, dim3(b.n_chunks), dim3(kVThreads), 0, s, b, phase);
  if (e == cudaSuccess)
    e = launch_pdl_b(batch_vertex_tail_kernel<R>, dim3(b.n_meshes), dim3(kTailThreads), 0, s, b, phase);
  if (e == cudaSuccess && DELTA) e = batch_refresh(b, s);
  return e;
}

template <class R, int MAT>
cudaError_t batch_grad_and_vertex_m(const BatchArgs& b, cudaStream_t s) {
  if (b.a.delta) {
    if (!kRefDelta<R, MAT> || !b.a.xref || !b.a.gref) return cudaErrorInvalidValue;
    return batch_grad_and_vertex_d<R, MAT, kRefDelta<R, MAT>>(b, s);
  }
  return batch_grad_and_vertex_d<R, MAT, false>(b, s);
}

template <class R>
cudaError_t batch_grad_and_vertex(const BatchArgs& b, cudaStream_t s) {
  if (b.a.fv.material == AGB_ARAP) return batch_grad_and_vertex_d<R, AGB_ARAP, false>(b, s);
  return b.a.fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE
             ? batch_grad_and_vertex_m<R, AGB_STABLE_NEO_HOOKEAN_MUSCLE>(b, s)
             : batch_grad_and_vertex_m<R, AGB_STABLE_NEO_HOOKEAN>(b, s);
}

template <class R, int MAT>
cudaError_t batch_iteration_m(const BatchArgs& b, cudaStream_t s) {
  batch_dir_kernel<R, MAT><<<b.a.fv.n_tiles, kElemThreads, 0, s>>>(b);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = launch_pdl_b(batch_dir_tail_kernel<R, MAT>, dim3(b.n_meshes), dim3(kTailThreads), 0, s, b);
  if (e == cudaSuccess) e = batch_grad_and_vertex_m<R, MAT>(b, s);
  return e;
}

// ARAP: the speculative gradient pass at alpha_0 and its vertex pass for the
// meshes that accept it; for the others the trial passes (three halvings
// each), then the gradient and vertex passes at the step they decide.  Every
// pass returns at once for a mesh it does not concern.
template <class R>
cudaError_t batch_iteration_arap(const BatchArgs& b, cudaStream_t s) {
  constexpr int A = AGB_ARAP;
  const int nt = b.a.fv.n_tiles, max_bt = b.a.max_bt;
  batch_dir_kernel<R, A><<<nt, kElemThreads, 0, s>>>(b);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = launch_pdl_b(batch_dir_tail_kernel<R, A>, dim3(b.n_meshes), dim3(kTailThreads), 0, s, b);
  if (e == cudaSuccess)
    e = launch_pdl_b(batch_grad_spec_kernel<R>, dim3(nt), dim3(kGradThreads), grad_spec_smem_bytes<R>(), s, b);
  if (e == cudaSuccess) e = launch_pdl_b(batch_spec_tail_kernel<R>, dim3(b.n_meshes), dim3(kTailThreads), 0, s, b);
  if (e == cudaSuccess)
    e = launch_pdl_b(batch_vertex_kernel<R, false>, dim3(b.n_chunks), dim3(kVThreads), 0, s, b, 1);
  if (e == cudaSuccess)
    e = launch_pdl_b(batch_vertex_tail_kernel<R>, dim3(b.n_meshes), dim3(kTailThreads), 0, s, b, 1);
  for (int j0 = 1; e == cudaSuccess && j0 <= max_bt; j0 += 3) {
    const int k = max_bt - j0 + 1 < 3 ? max_bt - j0 + 1 : 3;
    batch_trial_kernel<R><<<nt, kElemThreads, 0, s>>>(b, j0, k);
    batch_trial_tail_kernel<R><<<b.n_meshes, kTailThreads, 0, s>>>(b, j0, k);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = batch_grad_and_vertex_d<R, A, false>(b, s, 1);
  return e;
}

template <class R>
cudaError_t batch_iteration_t(const BatchArgs& b, cudaStream_t s) {
  if (b.a.fv.material == AGB_ARAP) return batch_iteration_arap<R>(b, s);
  return b.a.fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE ? batch_iteration_m<R, AGB_STABLE_NEO_HOOKEAN_MUSCLE>(b, s)
                                                          : batch_iteration_m<R, AGB_STABLE_NEO_HOOKEAN>(b, s);
}

template <class R>
cudaError_t batch_prepare_t() {
  const cudaFuncAttribute m = cudaFuncAttributeMaxDynamicSharedMemorySize;
  const int g = (int)grad_smem_bytes<R>();
  constexpr int SNH = AGB_STABLE_NEO_HOOKEAN, MU = AGB_STABLE_NEO_HOOKEAN_MUSCLE;
  cudaError_t e = cudaFuncSetAttribute(batch_grad_kernel<R, SNH, false>, m, g);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_grad_kernel<R, AGB_ARAP, false>, m, g);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_grad_spec_kernel<R>, m, (int)grad_spec_smem_bytes<R>());
  if (e == cudaSuccess && kRefDelta<R, SNH>) e = cudaFuncSetAttribute(batch_grad_kernel<R, SNH, kRefDelta<R, SNH>>, m, g);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(batch_grad_kernel<R, MU, false>, m, g);
  if (e == cudaSuccess && kRefDelta<R, MU>) e = cudaFuncSetAttribute(batch_grad_kernel<R, MU, kRefDelta<R, MU>>, m, g);
  return e;
}

}  // namespace

cudaError_t batch_prepare_kernels(int precision) {
  return precision == AGB_F64 ? batch_prepare_t<double>() : batch_prepare_t<float>();
}

cudaError_t launch_batch_init(const BatchArgs& b, const void* u_user, const void* fixed,
                              const int32_t* uoi, const SolverState& proto, cudaStream_t s) {
  const int blocks = b.a.n_points > 0 ? std::min((b.a.n_points + 255) / 256, 4096) : 1;
  if (b.a.precision == AGB_F64)
    batch_init_vertex_kernel<double><<<blocks, 256, 0, s>>>(b, (const double*)u_user, (const V4<double>*)fixed, uoi);
  else
    batch_init_vertex_kernel<float><<<blocks, 256, 0, s>>>(b, (const float*)u_user, (const V4<float>*)fixed, uoi);
  batch_init_state_kernel<<<(b.n_meshes + 255) / 256, 256, 0, s>>>(b, proto);
  return cudaGetLastError();
}

cudaError_t launch_batch_iteration(const BatchArgs& b, cudaStream_t s) {
  if (b.a.fv.n_tiles == 0 || b.n_meshes == 0) return cudaErrorInvalidValue;
  const cudaError_t e =
      b.a.precision == AGB_F64 ? batch_iteration_t<double>(b, s) : batch_iteration_t<float>(b, s);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_batch_first(const BatchArgs& b, cudaStream_t s) {
  if (b.a.fv.n_tiles == 0 || b.n_meshes == 0) return cudaErrorInvalidValue;
  if (b.a.delta) {  // x_ref = x_0 and g(x_0) in FP64 for every model
    batch_force_refresh_kernel<<<(b.n_meshes + 255) / 256, 256, 0, s>>>(b);
    const cudaError_t e = batch_refresh(b, s);
    if (e != cudaSuccess) return e;
  }
  const cudaError_t e =
      b.a.precision == AGB_F64 ? batch_grad_and_vertex<double>(b, s) : batch_grad_and_vertex<float>(b, s);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_batch_set_limit(const BatchArgs& b, int n, cudaStream_t s) {
  batch_set_limit_kernel<<<1, 1, 0, s>>>(b.bs, n);
  return cudaGetLastError();
}

cudaError_t launch_batch_energy(const BatchArgs& b, cudaStream_t s) {
  if (b.n_meshes == 0) return cudaSuccess;
  const bool mu = b.a.fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE;
  const bool arap = b.a.fv.material == AGB_ARAP;
  if (b.a.precision == AGB_F64) {
    if (arap)
      batch_energy_pass_kernel<double, AGB_ARAP><<<b.a.fv.n_tiles, kElemThreads, 0, s>>>(b);
    else if (mu)
      batch_energy_pass_kernel<double, AGB_STABLE_NEO_HOOKEAN_MUSCLE><<<b.a.fv.n_tiles, kElemThreads, 0, s>>>(b);
    else
      batch_energy_pass_kernel<double, AGB_STABLE_NEO_HOOKEAN><<<b.a.fv.n_tiles, kElemThreads, 0, s>>>(b);
    batch_energy_kernel<double><<<b.n_meshes, kTailThreads, 0, s>>>(b);
  } else {
    if (arap)
      batch_energy_pass_kernel<float, AGB_ARAP><<<b.a.fv.n_tiles, kElemThreads, 0, s>>>(b);
    else if (mu)
      batch_energy_pass_kernel<float, AGB_STABLE_NEO_HOOKEAN_MUSCLE><<<b.a.fv.n_tiles, kElemThreads, 0, s>>>(b);
    else
      batch_energy_pass_kernel<float, AGB_STABLE_NEO_HOOKEAN><<<b.a.fv.n_tiles, kElemThreads, 0, s>>>(b);
    batch_energy_kernel<float><<<b.n_meshes, kTailThreads, 0, s>>>(b);
  }
  return cudaGetLastError();
}

}  // namespace agb
