// PNCG on the device (benches/bench_pncg_branching_backends.py:254-456,
// 606-679, with the first trial step alpha_0 = overstep * (-g.p / p.Hp)).
//
// One iteration k is three kernels, all driven by SolverState in device
// memory (no host round trip):
//   direction pass  p_k = -P_k g_k + beta_k p_{k-1} formed per tile vertex;
//                   per element: clamped p^T H_e p (alpha_0) and, for stable
//                   Neo-Hookean, the coefficients c_2..c_6 of
//                   Psi_e(F + t dF) - Psi_e(F) - t P:dF, which is an exact
//                   polynomial in t; the last block runs the Armijo
//                   backtracking of the reference on
//                   dE(t) = t g.p + sum_m C_m t^m -- the same trial points
//                   and decisions as evaluating fun(x + t p) per trial,
//                   without the O(1) cancellation of f(x+tp) - f(x)
//   gradient pass   at x_{k+1} = x_k + t p_k: energy, gradient, clamped
//                   Hessian diagonal -> tile slots, accumulated per warp in
//                   private shared-memory copies (no atomics, fixed order)
//   [ARAP]          (not polynomial in t) the gradient pass evaluates the
//                   first trial step alpha_0 speculatively, sums the
//                   elements' energy remainders there and takes the Armijo
//                   decision; only when it rejects do trial passes (three
//                   halvings each) and a second gradient pass run.  Each
//                   element's SVD at x is kept between passes (U and V as
//                   quaternions, sigma - 1), so the direction pass needs none
//                   and the trial SVDs start from it.
//   vertex pass     x_{k+1}, g_{k+1}, d_{k+1}, p_k written; dot products of
//                   the Dai-Kou beta, the descent check and the convergence
//                   norm reduced; the last block decides beta_{k+1}, the
//                   preconditioner mean and termination, and sets the CUDA
//                   graph's while-condition.
// The gradient and vertex passes are launched as programmatic dependents of
// the pass before them: they read their constant inputs (element records,
// slot offsets) before griddepcontrol.wait and everything the previous pass
// writes after it.
#include <math.h>

#include "bulk.cuh"
#include "kernels.h"
#include "solver.h"
#include "solver_common.cuh"

namespace agb {


// Persistent grids: the vertex pass and the direction pass launch as many
// CTAs as are resident at once (152 SMs x CTAs per SM) and stride over
// vertices / tiles, so each CTA's block reduction covers several vertices
// or tiles and the completion sums a few hundred partials in one level.
constexpr int kVertexCtasPerSM = 2;
constexpr int kDirCtasPerSM = 3;

// SolverState as 32-bit words, for the last blocks' shared copy
constexpr int kStateWords = (int)(sizeof(SolverState) / 4);
static_assert(sizeof(SolverState) % 4 == 0 && kStateWords <= kVThreads && kStateWords <= kElemThreads,
              "the state is copied one word per thread");

int solver_vertex_blocks(int n_points) {
  int b = (n_points + kVThreads - 1) / kVThreads;
  const int cap = kSMs * kVertexCtasPerSM;
  return b < 1 ? 1 : (b > cap ? cap : b);
}

static int dir_blocks(int n_tiles) { return n_tiles < kSMs * kDirCtasPerSM ? n_tiles : kSMs * kDirCtasPerSM; }

template <class R, int MAT>
__global__ void __launch_bounds__(kElemThreads, kDirCtasPerSM) solver_dir_kernel(SolveArgs a, int use_cond) {
  constexpr int N = snh_family(MAT) ? 6 : 1;
  // float-float warp trees only for c2 (terms of both signs); p^T H p is a
  // sum of clamped non-negative terms, c3..c6 are higher-order corrections
  constexpr unsigned FF = snh_family(MAT) ? 0x2u : 0x0u;
  __shared__ V4<R> sxp[kTileVerts];  // (x, p.x)
  __shared__ V2<R> sq[kTileVerts];   // (p.y, p.z)
  __shared__ Acc<R> red[kWarps * N];
  __shared__ SolverState sst;
  SolverState* st = a.st;
  pdl_trigger();
  static_assert(kTileVerts == kElemThreads, "one staged vertex per thread");
  int tile = blockIdx.x;
  // constant inputs first: the thread's first element record and vertex id
  int es = a.fv.tile_estart[tile], ee = a.fv.tile_estart[tile + 1];
  int e = es + threadIdx.x;
  ElemGeo<R> geo;
  uint32_t ids = 0;
  if (e < ee) load_elem_m<R, MAT>(a.fv, e, geo, ids);
  int vid = tile_vertex(a.fv, tile, threadIdx.x);
  pdl_wait();  // launched as a dependent of the vertex pass in an unrolled loop body
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (use_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond, 0u);  // vertex pass re-arms
    // the refresh passes, if any, ran after the last vertex pass (a guarded
    // pass that goes on finds no refresh pending)
    if (!a.guard) st->refresh = 0;
  }
  if (st->done || guard_skip(a, st)) return;
  const R beta = (R)st->beta, inv_mean = (R)st->inv_mean;
  const int pb = st->pbuf;
  const V4<R>* pprev = p_prev<R>(a, pb);
  V4<R>* pcur = p_cur<R>(a, pb);
  const V4<R>* csvd = MAT == AGB_ARAP ? svd_cache<R>(a, st->sbuf) : nullptr;

  // pHp and c3..c6 in plain R, c2 (terms of both signs) in float-float
  R plain[N] = {};
  Acc<R> c2acc = {};
  for (; tile < a.fv.n_tiles; tile += gridDim.x) {
    stage_dir_packed<R>(a, vid, beta, inv_mean, pprev, pcur, sxp, sq);
    // the next tile's vertex id, in flight while this tile computes
    vid = tile_vertex(a.fv, tile + gridDim.x, threadIdx.x);
    __syncthreads();
    // next tile of this CTA, for the record prefetch at the end of this one
    const int tn = tile + gridDim.x;
    const int esn = tn < a.fv.n_tiles ? a.fv.tile_estart[tn] : 0;
    const int een = tn < a.fv.n_tiles ? a.fv.tile_estart[tn + 1] : 0;
    // e walks the thread's elements of this tile (stride blockDim.x); the
    // record of the following element -- in this tile or the CTA's next
    // tile -- is loaded while the current one computes
    const bool had = e < ee;
    while (e < ee) {
      int en = e + blockDim.x;
      const bool last = en >= ee;
      if (last) en = esn + threadIdx.x;
      ElemGeo<R> geon;
      uint32_t idsn = 0;
      if (last ? en < een : true) load_elem_m<R, MAT>(a.fv, en, geon, idsn);
      const int l[4] = {corner(ids, 0), corner(ids, 1), corner(ids, 2), corner(ids, 3)};
      R G[3][3], dF[3][3];
      dir_gradients(sxp, sq, l, geo.D, G, dF);
      add_act<MAT>(geo, G);
      if constexpr (snh_family(MAT)) {
        SnhPoint<R> s;
        snh_prepare(G, s);
        SnhDir<R> d;
        snh_dir(s, dF, d);
        plain[0] += fmax(snh_hess_quad(s, d, geo.mu, geo.lam), R(0));
        R c[5];
        snh_poly(s, d, geo.mu, geo.lam, c);
        c2acc.add(c[0]);
#pragma unroll
        for (int m = 1; m < 5; ++m) plain[1 + m] += c[m];
      } else {
        // the SVD at x, kept by the gradient pass that evaluated x
        Svd<R> sv;
        svd_get(csvd, (size_t)a.fv.n_cells, e, sv);
        R lk[3];
        arap_lambdas(sv, lk);
        plain[0] += fmax(arap_hess_quad(sv, lk, dF, geo.mu), R(0));
      }
      geo = geon;
      ids = idsn;
      e = en;
      if (last) break;
    }
    if (!had) {  // no element of this tile for this thread: start on the next tile
      e = esn + threadIdx.x;
      if (e < een) load_elem_m<R, MAT>(a.fv, e, geo, ids);
    }
    es = esn;
    ee = een;
    __syncthreads();
  }
  double tot[N];
  Acc<R> sums[N];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    sums[k] = Acc<R>{};
    sums[k].add(plain[k]);
  }
  if constexpr (N > 1) sums[1] = c2acc;
  // the last block decides on a shared copy of the state (see the vertex pass)
  if (!grid_reduce_masked_state<N, FF, R>(sums, (AccStore<R>*)a.part_a, a.cnt_a, gridDim.x, red, tot,
                                          (const uint32_t*)st, (uint32_t*)&sst, kStateWords))
    return;
  if (threadIdx.x == 0) dir_decide<MAT>(&sst, tot);
  __syncthreads();
  if ((int)threadIdx.x < kStateWords) ((uint32_t*)st)[threadIdx.x] = ((const uint32_t*)&sst)[threadIdx.x];
}

// ---------------------------------------------------------------------------
// ARAP trial pass: remainders at trial steps alpha_0 2^-j, j = j0 .. j0+nt-1
// (nt <= 3), each trial SVD warm-started from the cached one at x.  The
// speculative gradient pass tests alpha_0 itself; these passes run only when
// it was rejected (they return at once once a step is decided) and try three
// halvings each.
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(kElemThreads) solver_trial_kernel(SolveArgs a, int j0, int nt) {
  __shared__ Acc<R> red[kWarps * 3];
  SolverState* st = a.st;
  if (st->done || st->decided) return;
  const double a0 = st->alpha0;
  Acc<R> sums[3] = {};
  trial_tile<R>(a, blockIdx.x, st, j0, nt, sums);
  double tot[3];
  if (!grid_reduce2<3, 0x7u, R>(sums, (AccStore<R>*)a.part_t, (AccStore<R>*)a.gpart_t, a.cnt_t,
                                gridDim.x, red, tot))
    return;
  if (threadIdx.x != 0) return;
  trial_decide(st, a0, j0, nt, tot);
}

// ---------------------------------------------------------------------------
// gradient pass at x + t p
//
// Elements of a tile come in warp groups (<= 32) whose corner k is a distinct
// vertex for every lane (host-side edge colouring), so warp w adds its
// lanes' corner-k contributions into its private copy acc[w] with plain
// shared-memory loads and stores.  The copies are summed in warp order.
// ---------------------------------------------------------------------------
size_t solver_grad_smem(int precision) {
  return precision == AGB_F64 ? grad_smem_bytes<double>() : grad_smem_bytes<float>();
}

// The tiles run in reverse order: the direction pass before this one walks
// them forward, so its last tiles' element records are the ones most likely
// still in L2 when this pass starts (the result does not depend on the
// order: each tile writes its own slots).
template <class R, int MAT, bool DELTA>
__global__ void __launch_bounds__(kGradThreads, 5) solver_grad_kernel(SolveArgs a, int fallback) {
  grad_tile<R, MAT, DELTA>(a, gridDim.x - 1 - blockIdx.x, a.st, nullptr, fallback != 0);
}

// ARAP: the gradient pass at the first trial step x + alpha_0 p, with the
// Armijo test of that step (grad_tile's SPEC form; the remainders reduce
// through the trial partials)
template <class R>
__global__ void __launch_bounds__(kGradThreads, 4) solver_grad_spec_kernel(SolveArgs a) {
  __shared__ Acc<R> red[kGradWarps];
  Acc<R> rem[1] = {};
  if (!grad_tile<R, AGB_ARAP, false, true>(a, blockIdx.x, a.st, &rem[0])) return;
  double tot[1];
  if (!grid_reduce2<1, 0x1u, R>(rem, (AccStore<R>*)a.part_t, (AccStore<R>*)a.gpart_t, a.cnt_t, gridDim.x, red,
                                tot))
    return;
  if (threadIdx.x == 0) spec_decide(a.st, tot[0]);
}

// ---------------------------------------------------------------------------
// vertex pass
// ---------------------------------------------------------------------------
// phase (ARAP): 1 after the speculative gradient pass, running only if its
// step was accepted; 2 after the fallback passes, running only if it was not;
// 0 otherwise (always runs)
template <class R, bool DELTA>
__global__ void __launch_bounds__(kVThreads, kVertexCtasPerSM) solver_vertex_kernel(SolveArgs a, int use_cond,
                                                                                   int phase) {
  constexpr int N = 12;
  __shared__ Acc<R> red[(kVThreads / 32) * N];
  const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
  // constant inputs before the dependency wait
  int s0 = 0, s1 = 0;
  if (i0 < a.n_points) {
    s0 = a.off[i0];
    s1 = a.off[i0 + 1];
  }
  pdl_wait();
  SolverState* st = a.st;
  if (st->done) {
    if (use_cond && blockIdx.x == 0 && threadIdx.x == 0)
      cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond, 0u);
    return;
  }
  if (guard_skip(a, st)) return;  // the loop condition stays as the direction pass left it: 0
  // ARAP: the pass after the speculative gradient pass, or the one after the
  // fallback passes, whichever applies (the other leaves the condition alone)
  if ((phase == 1 && !st->spec_ok) || (phase == 2 && st->spec_ok)) return;
  const R t = (R)st->t;
  const V4<R>* P = p_cur<R>(a, st->pbuf);
  // 0 gPg 1 gPy 2 yPy 3 sum|d| 4 count 5 zgg 6 zgy 7 zyy 8 y.p 9 p.g 10 g.g 11 ext energy
  // a thread sums its few vertices in R; float-float starts at the warp trees
  R s[N] = {};
  for (int i = i0; i < a.n_points; i += gridDim.x * blockDim.x) {
    if (i != i0) {
      s0 = a.off[i];
      s1 = a.off[i + 1];
    }
    vertex_update<R, DELTA>(a, i, s0, s1, t, P, s);
  }
  double tot[N];
  // float-float block sums for the quantities whose terms change sign
  constexpr unsigned FF = (1u << 1) | (1u << 6) | (1u << 8) | (1u << 9);
  Acc<R> acc[N];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    acc[k] = Acc<R>{};
    acc[k].add(s[k]);
  }
  if (!grid_reduce_masked<N, FF, R>(acc, (AccStore<R>*)a.part_v, a.cnt_v, gridDim.x, red, tot)) return;
  if (threadIdx.x != 0) return;
  vertex_decide(st, tot);
  if (a.svd) st->sbuf ^= 1;  // the gradient pass's SVDs are those at the new x
  const bool go = !st->done && st->iter < st->iter_limit;
  if (use_cond)
    cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond,
                            (go && !(a.refresh_exits && st->refresh)) ? 1u : 0u);
}

// The FP32 vertex pass with its inputs streamed by bulk copies.  Each CTA
// walks chunks of kVThreads consecutive vertices (chunk c = blockIdx.x + k *
// gridDim.x, one vertex per thread: the vertex of each thread is the one the
// grid-stride kernel above gives it, so the sums and results are the same
// bits).  Thread 0 copies a chunk's positions, gradient/diagonal, direction,
// reference gradient, force and its contiguous range of slots into shared
// memory with cp.async.bulk, one chunk ahead (two stages, one mbarrier
// each), so the loads of a chunk are in flight while the one before it
// computes and no thread waits on a dependent global load.  Slots beyond the
// stage's capacity are read from global memory.
constexpr int kVSlotCap = 768;  // slots staged per chunk
constexpr size_t kVsXa = 0;
constexpr size_t kVsGd = kVsXa + (size_t)kVThreads * 32;
constexpr size_t kVsP = kVsGd + (size_t)kVThreads * 32;
constexpr size_t kVsR = kVsP + (size_t)kVThreads * 16;
constexpr size_t kVsF = kVsR + (size_t)kVThreads * 16;
constexpr size_t kVsS = kVsF + (size_t)kVThreads * 16;
constexpr size_t kVStage = kVsS + (size_t)kVSlotCap * 32;
constexpr size_t kVBulkSmem = 2 * kVStage;

template <bool DELTA>
__global__ void __launch_bounds__(kVThreads, kVertexCtasPerSM) solver_vertex_bulk_kernel(SolveArgs a, int use_cond,
                                                                                        int phase) {
  using R = float;
  constexpr int N = 12;
  extern __shared__ __align__(128) unsigned char vsm[];
  __shared__ Acc<R> red[(kVThreads / 32) * N];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ int s_base[2];  // first slot of the chunk in each stage
  __shared__ SolverState sst;
  const int n = a.n_points, tid = threadIdx.x;
  const int nchunks = (n + kVThreads - 1) / kVThreads;
  int c = blockIdx.x;
  // constant inputs before the dependency wait: this thread's slot range in
  // its first chunk, and thread 0's chunk bounds for the first two chunks
  int s0 = 0, s1 = 0;
  if (c * kVThreads + tid < n) {
    s0 = a.off[c * kVThreads + tid];
    s1 = a.off[c * kVThreads + tid + 1];
  }
  int blo[2] = {0, 0}, bhi[2] = {0, 0};
  if (tid == 0) {
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int cc = c + j * gridDim.x;
      if (cc < nchunks) {
        blo[j] = a.off[cc * kVThreads];
        bhi[j] = a.off[min(cc * kVThreads + kVThreads, n)];
      }
    }
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  pdl_wait();
  SolverState* st = a.st;
  if (st->done) {
    if (use_cond && blockIdx.x == 0 && tid == 0) cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond, 0u);
    return;
  }
  if (guard_skip(a, st)) return;
  if ((phase == 1 && !st->spec_ok) || (phase == 2 && st->spec_ok)) return;
  const R t = (R)st->t;
  const V4<R>* P = p_cur<R>(a, st->pbuf);
  const V4<R>* XA = (const V4<R>*)a.xa;
  const V4<R>* GD = (const V4<R>*)a.gd;
  const V4<R>* GR = (const V4<R>*)a.gref;
  const V4<R>* FO = (const V4<R>*)a.force;
  const V4<R>* SL = (const V4<R>*)a.slots;
  // thread 0: copy chunk cc (slot range [lo, hi)) into `stage`
  auto issue = [&](int cc, int stage, int lo, int hi) {
    const int v0 = cc * kVThreads, cnt = min(kVThreads, n - v0);
    const int ns = min(hi - lo, kVSlotCap);
    unsigned char* b = vsm + (size_t)stage * kVStage;
    const uint32_t vb = 16u * (uint32_t)cnt;
    // positions and gradient/diagonal 32 B per vertex, direction (and the
    // reference gradient, the force) 16 B, slots 32 B
    const uint32_t bytes = 5u * vb + (DELTA ? vb : 0u) + (FO ? vb : 0u) + 32u * (uint32_t)ns;
    s_base[stage] = lo;
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bar[stage], bytes);
    bulk_g2s(b + kVsXa, XA + 2 * (size_t)v0, 2 * vb, &bar[stage]);
    bulk_g2s(b + kVsGd, GD + 2 * (size_t)v0, 2 * vb, &bar[stage]);
    bulk_g2s(b + kVsP, P + v0, vb, &bar[stage]);
    if (DELTA) bulk_g2s(b + kVsR, GR + v0, vb, &bar[stage]);
    if (FO) bulk_g2s(b + kVsF, FO + v0, vb, &bar[stage]);
    if (ns > 0) bulk_g2s(b + kVsS, SL + 2 * (size_t)lo, 32u * (uint32_t)ns, &bar[stage]);
  };
  if (tid == 0 && c < nchunks) issue(c, 0, blo[0], bhi[0]);
  __syncthreads();
  // 0 gPg 1 gPy 2 yPy 3 sum|d| 4 count 5 zgg 6 zgy 7 zyy 8 y.p 9 p.g 10 g.g 11 ext energy
  R s[N] = {};
  bool bad = false;
  for (int k = 0; c < nchunks; c += gridDim.x, ++k) {
    const int stage = k & 1;
    const int cn = c + gridDim.x;
    if (tid == 0 && cn < nchunks) {
      issue(cn, stage ^ 1, blo[1], bhi[1]);
      // bounds of the chunk after it, for the next issue
      const int c2 = cn + gridDim.x;
      if (c2 < nchunks) {
        blo[1] = a.off[c2 * kVThreads];
        bhi[1] = a.off[min(c2 * kVThreads + kVThreads, n)];
      }
    }
    // this thread's slot range in the next chunk
    int s0n = 0, s1n = 0;
    const int in_next = cn * kVThreads + tid;
    if (cn < nchunks && in_next < n) {
      s0n = a.off[in_next];
      s1n = a.off[in_next + 1];
    }
    if (!mbar_wait(&bar[stage], (uint32_t)(k >> 1) & 1u)) bad = true;
    const int i = c * kVThreads + tid;
    if (i < n && !bad) {
      const unsigned char* b = vsm + (size_t)stage * kVStage;
      VertexIn<R> in;
      in.x = ((const V4<R>*)(b + kVsXa))[2 * tid];
      in.xl = ((const V4<R>*)(b + kVsXa))[2 * tid + 1];
      in.g = ((const V4<R>*)(b + kVsGd))[2 * tid];
      in.p = ((const V4<R>*)(b + kVsP))[tid];
      if (DELTA) in.r = ((const V4<R>*)(b + kVsR))[tid];
      if (FO) in.f = ((const V4<R>*)(b + kVsF))[tid];
      in.s0 = s0;
      in.s1 = s1;
      const V4<R>* ss = (const V4<R>*)(b + kVsS);
      const int base = s_base[stage];
      R gs[3] = {R(0), R(0), R(0)}, ds[3] = {R(0), R(0), R(0)};
      for (int q = s0; q < s1; ++q) {
        const int j = q - base;
        const V4<R> sg = j < kVSlotCap ? ss[2 * j] : SL[2 * (size_t)q];
        const V4<R> sd = j < kVSlotCap ? ss[2 * j + 1] : SL[2 * (size_t)q + 1];
        gs[0] += sg.x;
        gs[1] += sg.y;
        gs[2] += sg.z;
        ds[0] += sd.x;
        ds[1] += sd.y;
        ds[2] += sd.z;
      }
      vertex_apply<R, DELTA>(a, i, in, t, gs, ds, s);
    }
    s0 = s0n;
    s1 = s1n;
    __syncthreads();  // this stage is read before it is refilled
  }
  if (bad) atomicMax(&st->error, 2);  // a copy never completed: the solve stops with a device error
  double tot[N];
  constexpr unsigned FF = (1u << 1) | (1u << 6) | (1u << 8) | (1u << 9);
  Acc<R> acc[N];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    acc[k] = Acc<R>{};
    acc[k].add(s[k]);
  }
  // the last block decides on a shared copy of the state, loaded with the
  // block partials, and writes it back in one coalesced store
  if (!grid_reduce_masked_state<N, FF, R>(acc, (AccStore<R>*)a.part_v, a.cnt_v, gridDim.x, red, tot,
                                          (const uint32_t*)st, (uint32_t*)&sst, kStateWords))
    return;
  if (tid == 0) {
    if (sst.error) {
      sst.done = 1;
    } else {
      vertex_decide(&sst, tot);
      if (a.svd) sst.sbuf ^= 1;
    }
    const bool go = !sst.done && sst.iter < sst.iter_limit;
    if (use_cond)
      cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond,
                              (go && !(a.refresh_exits && sst.refresh)) ? 1u : 0u);
  }
  __syncthreads();
  if (tid < kStateWords) ((uint32_t*)st)[tid] = ((const uint32_t*)&sst)[tid];
}

// total energy at x, on demand: an element pass into per-tile partials, then
// their sum plus the external work of the last vertex pass
template <class R, int MAT>
__global__ void __launch_bounds__(kElemThreads) solver_energy_pass_kernel(SolveArgs a) {
  energy_tile<R, MAT>(a, blockIdx.x, (AccStore<R>*)a.part_b + blockIdx.x);
}

template <class R>
__global__ void __launch_bounds__(256) solver_energy_kernel(SolveArgs a) {
  __shared__ Acc<R> red[8];
  const double e = block_sum_partials<R>((const AccStore<R>*)a.part_b, a.fv.n_tiles, 1, red);
  if (threadIdx.x == 0) a.st->energy = e + a.st->ext_energy;
}

// refresh of the reference state (FP32 stable Neo-Hookean); in the iteration
// graph both follow the vertex pass as programmatic dependents and return at
// once unless it asked for a refresh
// (grid-stride over tiles with a resident-sized grid, so that the usual case
// -- no refresh due -- costs one short wave)
template <int MAT>
__global__ void __launch_bounds__(kGradThreads) solver_ref_elem_kernel(SolveArgs a) {
  pdl_trigger();
  pdl_wait();
  if (!a.st->refresh) return;
  for (int tile = blockIdx.x; tile < a.fv.n_tiles; tile += gridDim.x) {
    ref_tile<MAT>(a, tile);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kVThreads) solver_ref_vertex_kernel(SolveArgs a) {
  pdl_trigger();
  pdl_wait();
  if (a.cond_outer && blockIdx.x == 0 && threadIdx.x == 0) {
    // after the inner loop of agb_solver_iterate: go on (and re-arm the inner
    // loop) unless the solve ended or reached its iteration limit
    const SolverState* st = a.st;
    const bool go = !st->done && st->iter < st->iter_limit;
    cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond_outer, go ? 1u : 0u);
    cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond, go ? 1u : 0u);
  }
  if (!a.st->refresh) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n_points; i += gridDim.x * blockDim.x) ref_vertex(a, i);
}

// ---------------------------------------------------------------------------
// set-up and read-back
// ---------------------------------------------------------------------------
template <class R>
__global__ void solver_init_kernel(SolveArgs a, const R* __restrict__ u, const V4<R>* __restrict__ fixed,
                                   const int32_t* __restrict__ uoi) {
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
    if (a.delta) {  // x_ref = 0, g(x_ref) = -f (no element stress at u = 0)
      V4<R> f = z;
      if (a.force) f = ((const V4<R>*)a.force)[i];
      ((V4<R>*)a.xref)[i] = z;
      ((V4<R>*)a.gref)[i] = V4<R>{-f.x, -f.y, -f.z, R(0)};
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    SolverState* st = a.st;
    st->beta = 0.0;
    st->inv_mean = 1.0;
    st->gd = 0.0;
    st->t = 0.0;
    st->alpha0 = 0.0;
    st->hq = 0.0;
    st->gnorm = 0.0;
    st->gnorm0 = 0.0;
    st->energy = 0.0;
    st->ext_energy = 0.0;
    st->delta_e = 0.0;
    st->iter = 0;
    st->iter_limit = 0;
    st->done = 0;
    st->result = AGB_RUNNING;
    st->init = 1;
    st->reset_beta = 0;
    st->ls_fail = 0;
    st->ls_steps = 0;
    st->ls_ok = 0;
    st->decided = 1;
    st->error = 0;
    st->pbuf = 0;
    st->refresh = 0;
    st->gnorm_ref = 0.0;
    st->sbuf = 0;
    st->spec_ok = 0;
  }
}

__global__ void solver_set_limit_kernel(SolverState* st, int n) { st->iter_limit = st->iter + n; }

__global__ void solver_force_refresh_kernel(SolverState* st) { st->refresh = 1; }

template <class R>
__global__ void solver_unpack_kernel(int n, const V4<R>* __restrict__ xa, const int32_t* __restrict__ uoi,
                                     R* __restrict__ u) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const size_t k = 3 * (size_t)uoi[i];
    const V4<R> v = xa[2 * i], l = xa[2 * i + 1];
    u[k] = v.x + l.x;
    u[k + 1] = v.y + l.y;
    u[k + 2] = v.z + l.z;
  }
}

template <class R>
static cudaError_t prepare_t() {
  const int g = (int)grad_smem_bytes<R>();
  const cudaFuncAttribute m = cudaFuncAttributeMaxDynamicSharedMemorySize;
  cudaError_t e = cudaFuncSetAttribute(solver_grad_kernel<R, AGB_ARAP, false>, m, g);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(solver_grad_spec_kernel<R>, m, (int)grad_spec_smem_bytes<R>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(solver_grad_kernel<R, AGB_STABLE_NEO_HOOKEAN, false>, m, g);
  if (e == cudaSuccess && kRefDelta<R, AGB_STABLE_NEO_HOOKEAN>)
    e = cudaFuncSetAttribute(solver_grad_kernel<R, AGB_STABLE_NEO_HOOKEAN, kRefDelta<R, AGB_STABLE_NEO_HOOKEAN>>, m, g);
  constexpr int MU = AGB_STABLE_NEO_HOOKEAN_MUSCLE;
  if (e == cudaSuccess) e = cudaFuncSetAttribute(solver_grad_kernel<R, MU, false>, m, g);
  if (e == cudaSuccess && kRefDelta<R, MU>) e = cudaFuncSetAttribute(solver_grad_kernel<R, MU, kRefDelta<R, MU>>, m, g);
  if constexpr (sizeof(R) == 4) {
    if (e == cudaSuccess) e = cudaFuncSetAttribute(solver_vertex_bulk_kernel<false>, m, (int)kVBulkSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(solver_vertex_bulk_kernel<true>, m, (int)kVBulkSmem);
  }
  return e;
}

cudaError_t solver_prepare_kernels(int precision) {
  return precision == AGB_F64 ? prepare_t<double>() : prepare_t<float>();
}

cudaError_t launch_solver_init(const SolveArgs& a, const void* u_user, const void* fixed,
                               const int32_t* uoi, cudaStream_t s) {
  const int blocks = solver_vertex_blocks(a.n_points);
  if (a.precision == AGB_F64)
    solver_init_kernel<double><<<blocks, kVThreads, 0, s>>>(a, (const double*)u_user,
                                                           (const V4<double>*)fixed, uoi);
  else
    solver_init_kernel<float><<<blocks, kVThreads, 0, s>>>(a, (const float*)u_user,
                                                          (const V4<float>*)fixed, uoi);
  return cudaGetLastError();
}

cudaError_t launch_solver_set_limit(const SolveArgs& a, int n_steps, cudaStream_t s) {
  solver_set_limit_kernel<<<1, 1, 0, s>>>(a.st, n_steps);
  return cudaGetLastError();
}

cudaError_t launch_solver_energy(const SolveArgs& a, cudaStream_t s) {
  if (a.fv.n_tiles == 0) return cudaErrorInvalidValue;
  const int nt = a.fv.n_tiles;
  if (a.precision == AGB_F64) {
    if (a.fv.material == AGB_ARAP)
      solver_energy_pass_kernel<double, AGB_ARAP><<<nt, kElemThreads, 0, s>>>(a);
    else if (a.fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE)
      solver_energy_pass_kernel<double, AGB_STABLE_NEO_HOOKEAN_MUSCLE><<<nt, kElemThreads, 0, s>>>(a);
    else
      solver_energy_pass_kernel<double, AGB_STABLE_NEO_HOOKEAN><<<nt, kElemThreads, 0, s>>>(a);
    solver_energy_kernel<double><<<1, 256, 0, s>>>(a);
  } else {
    if (a.fv.material == AGB_ARAP)
      solver_energy_pass_kernel<float, AGB_ARAP><<<nt, kElemThreads, 0, s>>>(a);
    else if (a.fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE)
      solver_energy_pass_kernel<float, AGB_STABLE_NEO_HOOKEAN_MUSCLE><<<nt, kElemThreads, 0, s>>>(a);
    else
      solver_energy_pass_kernel<float, AGB_STABLE_NEO_HOOKEAN><<<nt, kElemThreads, 0, s>>>(a);
    solver_energy_kernel<float><<<1, 256, 0, s>>>(a);
  }
  return cudaGetLastError();
}

// launch with programmatic stream serialisation: the kernel may start while
// the previous kernel in the stream finishes and waits in griddepcontrol.wait
template <class... P, class... A>
static cudaError_t launch_pdl(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              A... args) {
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

// the direction pass (pdl: as a programmatic dependent)
template <class R, int MAT>
static cudaError_t launch_dir(const SolveArgs& a, int use_cond, bool pdl, cudaStream_t s) {
  const dim3 g(dir_blocks(a.fv.n_tiles)), b(kElemThreads);
  if (pdl) return launch_pdl(solver_dir_kernel<R, MAT>, g, b, 0, s, a, use_cond);
  solver_dir_kernel<R, MAT><<<g, b, 0, s>>>(a, use_cond);
  return cudaGetLastError();
}

// the vertex pass as a programmatic dependent: FP32 streams its inputs with
// bulk copies, FP64 uses the grid-stride kernel
template <class R, bool DELTA>
static cudaError_t launch_vertex(const SolveArgs& a, int use_cond, int phase, cudaStream_t s) {
  if constexpr (sizeof(R) == 4)
    return launch_pdl(solver_vertex_bulk_kernel<DELTA>, dim3(a.vblocks), dim3(kVThreads), kVBulkSmem, s, a,
                      use_cond, phase);
  else
    return launch_pdl(solver_vertex_kernel<R, DELTA>, dim3(a.vblocks), dim3(kVThreads), 0, s, a, use_cond, phase);
}

template <class R, int MAT, bool DELTA>
static cudaError_t launch_iteration_d(const SolveArgs& a, bool use_cond, bool first, int max_bt,
                                      cudaStream_t s) {
  const dim3 eg(a.fv.n_tiles), eb(kElemThreads);
  if (!first) {
    // a guarded iteration follows another one: its direction pass is a
    // programmatic dependent of that iteration's vertex pass
    cudaError_t e = launch_dir<R, MAT>(a, use_cond ? 1 : 0, a.guard != 0, s);
    if (e != cudaSuccess) return e;
    if constexpr (MAT == AGB_ARAP) {
      // speculative gradient pass at alpha_0 and its vertex pass; when the
      // step is rejected, trial passes from alpha_0 / 2, then the gradient
      // and vertex passes at the step they decide (each of these returns at
      // once when the speculative step was accepted)
      const dim3 gb(kGradThreads), vg(a.vblocks), vb(kVThreads);
      const int uc = use_cond ? 1 : 0;
      cudaError_t e = launch_pdl(solver_grad_spec_kernel<R>, eg, gb, grad_spec_smem_bytes<R>(), s, a);
      if (e == cudaSuccess) e = launch_vertex<R, DELTA>(a, uc, 1, s);
      if (e != cudaSuccess) return e;
      for (int j0 = 1; j0 <= max_bt; j0 += 3)
        solver_trial_kernel<R><<<eg, eb, 0, s>>>(a, j0, max_bt - j0 + 1 < 3 ? max_bt - j0 + 1 : 3);
      e = launch_pdl(solver_grad_kernel<R, MAT, DELTA>, eg, gb, grad_smem_bytes<R>(), s, a, 1);
      if (e != cudaSuccess) return e;
      return launch_vertex<R, DELTA>(a, uc, 2, s);
    }
  }
  cudaError_t e = launch_pdl(solver_grad_kernel<R, MAT, DELTA>, eg, dim3(kGradThreads), grad_smem_bytes<R>(), s, a, 0);
  if (e != cudaSuccess) return e;
  return launch_vertex<R, DELTA>(a, use_cond ? 1 : 0, 0, s);
}

template <class R, int MAT>
static cudaError_t launch_iteration_t(const SolveArgs& a, bool use_cond, bool first, int max_bt,
                                      cudaStream_t s) {
  if (a.delta) {  // the reference-state kernels read x_ref and g(x_ref)
    if (!kRefDelta<R, MAT> || !a.xref || !a.gref) return cudaErrorInvalidValue;
    return launch_iteration_d<R, MAT, kRefDelta<R, MAT>>(a, use_cond, first, max_bt, s);
  }
  return launch_iteration_d<R, MAT, false>(a, use_cond, first, max_bt, s);
}


static cudaError_t launch_iteration(const SolveArgs& a, bool use_cond, bool first, cudaStream_t s) {
  if (a.fv.n_tiles == 0) return cudaErrorInvalidValue;
  const int max_bt = a.max_bt;
  cudaError_t e;
  if (a.precision == AGB_F64) {
    if (a.fv.material == AGB_ARAP)
      e = launch_iteration_t<double, AGB_ARAP>(a, use_cond, first, max_bt, s);
    else if (a.fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE)
      e = launch_iteration_t<double, AGB_STABLE_NEO_HOOKEAN_MUSCLE>(a, use_cond, first, max_bt, s);
    else
      e = launch_iteration_t<double, AGB_STABLE_NEO_HOOKEAN>(a, use_cond, first, max_bt, s);
  } else {
    if (a.fv.material == AGB_ARAP)
      e = launch_iteration_t<float, AGB_ARAP>(a, use_cond, first, max_bt, s);
    else if (a.fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE)
      e = launch_iteration_t<float, AGB_STABLE_NEO_HOOKEAN_MUSCLE>(a, use_cond, first, max_bt, s);
    else
      e = launch_iteration_t<float, AGB_STABLE_NEO_HOOKEAN>(a, use_cond, first, max_bt, s);
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

template <class R, int MAT, bool DELTA>
static cudaError_t launch_pass_d(const SolveArgs& a, int which, cudaStream_t s) {
  const dim3 eg(a.fv.n_tiles);
  if (which == 0) launch_dir<R, MAT>(a, 0, false, s);
  if (which == 1) {
    if constexpr (MAT == AGB_ARAP)  // the iteration's gradient pass is the speculative one
      solver_grad_spec_kernel<R><<<eg, kGradThreads, grad_spec_smem_bytes<R>(), s>>>(a);
    else
      solver_grad_kernel<R, MAT, DELTA><<<eg, kGradThreads, grad_smem_bytes<R>(), s>>>(a, 0);
  }
  if (which == 2) {
    if constexpr (sizeof(R) == 4)
      solver_vertex_bulk_kernel<DELTA><<<a.vblocks, kVThreads, kVBulkSmem, s>>>(a, 0, 0);
    else
      solver_vertex_kernel<R, DELTA><<<a.vblocks, kVThreads, 0, s>>>(a, 0, 0);
  }
  return cudaGetLastError();
}

template <class R, int MAT>
static cudaError_t launch_pass_t(const SolveArgs& a, int which, cudaStream_t s) {
  if (a.delta && (!kRefDelta<R, MAT> || !a.xref || !a.gref)) return cudaErrorInvalidValue;
  if (a.delta) return launch_pass_d<R, MAT, kRefDelta<R, MAT>>(a, which, s);
  return launch_pass_d<R, MAT, false>(a, which, s);
}


cudaError_t launch_solver_pass(const SolveArgs& a, int which, cudaStream_t s) {
  if (a.precision == AGB_F64) {
    if (a.fv.material == AGB_ARAP) return launch_pass_t<double, AGB_ARAP>(a, which, s);
    if (a.fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE)
      return launch_pass_t<double, AGB_STABLE_NEO_HOOKEAN_MUSCLE>(a, which, s);
    return launch_pass_t<double, AGB_STABLE_NEO_HOOKEAN>(a, which, s);
  }
  if (a.fv.material == AGB_ARAP) return launch_pass_t<float, AGB_ARAP>(a, which, s);
  if (a.fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE)
    return launch_pass_t<float, AGB_STABLE_NEO_HOOKEAN_MUSCLE>(a, which, s);
  return launch_pass_t<float, AGB_STABLE_NEO_HOOKEAN>(a, which, s);
}

cudaError_t launch_solver_iteration(const SolveArgs& a, bool use_cond, cudaStream_t s) {
  return launch_iteration(a, use_cond, false, s);
}

cudaError_t launch_solver_first(const SolveArgs& a, cudaStream_t s) {
  return launch_iteration(a, false, true, s);
}

cudaError_t launch_solver_unpack_x(const SolveArgs& a, const void*, const int32_t* uoi, void* u,
                                   cudaStream_t s) {
  const int blocks = solver_vertex_blocks(a.n_points);
  if (a.precision == AGB_F64)
    solver_unpack_kernel<double><<<blocks, kVThreads, 0, s>>>(a.n_points, (const V4<double>*)a.xa, uoi,
                                                             (double*)u);
  else
    solver_unpack_kernel<float><<<blocks, kVThreads, 0, s>>>(a.n_points, (const V4<float>*)a.xa, uoi,
                                                            (float*)u);
  return cudaGetLastError();
}

cudaError_t launch_solver_refresh(const SolveArgs& a, cudaStream_t s, bool pdl) {
  if (!a.delta) return cudaSuccess;
  if (!a.xref || !a.gref || a.precision != AGB_F32 || !snh_family(a.fv.material)) return cudaErrorInvalidValue;
  const dim3 grid(ref_blocks(a.fv.n_tiles));
  auto ek = a.fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE ? solver_ref_elem_kernel<AGB_STABLE_NEO_HOOKEAN_MUSCLE>
                                                           : solver_ref_elem_kernel<AGB_STABLE_NEO_HOOKEAN>;
  cudaError_t e = cudaSuccess;
  if (pdl) {
    e = launch_pdl(ek, grid, dim3(kGradThreads), ref_smem_bytes(), s, a);
    if (e == cudaSuccess) e = launch_pdl(solver_ref_vertex_kernel, dim3(a.vblocks), dim3(kVThreads), 0, s, a);
  } else {
    ek<<<grid, kGradThreads, ref_smem_bytes(), s>>>(a);
    solver_ref_vertex_kernel<<<a.vblocks, kVThreads, 0, s>>>(a);
  }
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_solver_force_refresh(const SolveArgs& a, cudaStream_t s) {
  solver_force_refresh_kernel<<<1, 1, 0, s>>>(a.st);
  return cudaGetLastError();
}

}  // namespace agb
