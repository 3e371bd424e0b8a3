// Differentiation of the converged equilibrium.
//
// The reference differentiates its forward solve by hand (the inverse
// experiments, e.g. exp/2025/09/24/inverse-grin/src/32-inverse.py:223-300):
//   1. solve H(u*) lam = dL/du on the free DOFs with Jacobi-preconditioned CG
//      (jax.scipy.sparse.linalg.cg with M = 1/hess_diag, tol 1e-5), built on
//      the potentials' hess_prod;
//   2. pull lam back to the material parameters through the backward of the
//      grad kernel (Warp's tape over the arrays marked requires_grad,
//      warp/fem/_base.py:80-117, utils/_material.py:34-38), which gives
//      d(lam . g)/d theta per cell, and dL/d theta = -(that).
//
// Here step 1 is a device CG over the solver's tiled mesh: an element pass
// forms p = z + beta p_prev on the fly, applies H_e (the same hess_prod
// element math as the API) and accumulates H p per tile in shared memory
// (warp groups with distinct corner vertices, as in the gradient pass); two
// vertex passes update q = H p, alpha, lam, the residual and beta, with all
// scalars on the device and the loop in a CUDA graph WHILE node.  Step 2 is
// one element pass over the evaluation API's tiles.
#include "kernels.h"
#include "solver.h"
#include "tile.cuh"

namespace agb {

namespace {

constexpr int kCgThreads = 128;
constexpr int kCgWarps = kCgThreads / 32;
constexpr int kCgVerts = kTileVerts / kCgThreads;
constexpr int kVThreadsCg = 256;

__device__ __forceinline__ void pdl_wait_cg() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger_cg() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class R>
__device__ __forceinline__ V4<R>* cg_p_prev(const CgArgs& c, int pb) {
  return (V4<R>*)(pb ? c.p1 : c.p0);
}
template <class R>
__device__ __forceinline__ V4<R>* cg_p_cur(const CgArgs& c, int pb) {
  return (V4<R>*)(pb ? c.p0 : c.p1);
}

// z = M^-1 r per component (M^-1 = 0 on fixed components)
template <class R>
__device__ __forceinline__ V4<R> cg_precond(const V4<R>& m, const V4<R>& r) {
  return V4<R>{mul_rn(m.x, r.x), mul_rn(m.y, r.y), mul_rn(m.z, r.z), R(0)};
}

// p = z + beta p_prev, explicitly rounded so every pass forms the same p
template <class R>
__device__ __forceinline__ V4<R> cg_dir(const V4<R>& z, const V4<R>& po, R beta) {
  return V4<R>{fma_rn(beta, po.x, z.x), fma_rn(beta, po.y, z.y), fma_rn(beta, po.z, z.z), R(0)};
}

// ---------------------------------------------------------------------------
// set-up: lam = 0, r = masked rhs, M^-1 from the diagonal at u*, p buffers 0;
// sums r.M^-1 r and r.r
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(kVThreadsCg) cg_init_kernel(CgArgs c, const R* __restrict__ rhs,
                                                              const int32_t* __restrict__ uoi) {
  __shared__ Acc<R> red[(kVThreadsCg / 32) * 2];
  const SolveArgs& a = c.a;
  const V4<R>* XA = (const V4<R>*)a.xa;
  const V4<R>* GD = (const V4<R>*)a.gd;
  const R inv_mean = (R)a.st->inv_mean;
  Acc<R> s[2] = {};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n_points; i += gridDim.x * blockDim.x) {
    const int mask = (int)XA[2 * i].w;
    const V4<R> d = GD[2 * i + 1];
    const size_t k = 3 * (size_t)uoi[i];
    const R rv[3] = {rhs[k], rhs[k + 1], rhs[k + 2]};
    const R dv[3] = {d.x, d.y, d.z};
    R r[3], m[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const bool fixed = (mask >> q) & 1;
      r[q] = fixed ? R(0) : rv[q];
      m[q] = fixed ? R(0) : precond(dv[q], inv_mean);
      s[0].add(r[q] * m[q] * r[q]);
      s[1].add(r[q] * r[q]);
    }
    const V4<R> z{R(0), R(0), R(0), R(0)};
    ((V4<R>*)c.res)[i] = V4<R>{r[0], r[1], r[2], R(0)};
    ((V4<R>*)c.minv)[i] = V4<R>{m[0], m[1], m[2], R(0)};
    ((V4<R>*)c.lam)[i] = z;
    ((V4<R>*)c.q)[i] = z;
    ((V4<R>*)c.p0)[i] = z;
    ((V4<R>*)c.p1)[i] = z;
  }
  double tot[2];
  if (!grid_reduce_masked<2, 0x0u, R>(s, (AccStore<R>*)c.part, c.cnt, gridDim.x, red, tot)) return;
  if (threadIdx.x != 0) return;
  CgState* cs = c.cs;
  cs->rz = tot[0];
  cs->rr = tot[1];
  cs->rr0 = tot[1];
  cs->alpha = 0.0;
  cs->beta = 0.0;
  cs->iter = 0;
  cs->pbuf = 0;
  cs->result = AGB_RUNNING;
  const double rn = sqrt(tot[1]);
  cs->done = 0;
  if (!isfinite(rn)) {
    cs->done = 1;
    cs->result = AGB_NAN_ENCOUNTERED;
  } else if (rn <= cs->atol || tot[1] == 0.0) {
    cs->done = 1;
    cs->result = AGB_PRIMARY_SUCCESS;
  }
}

// ---------------------------------------------------------------------------
// element pass: p = z + beta p_prev (stored), q_e = H_e(u*) p_e -> slots
// ---------------------------------------------------------------------------
template <class R>
__host__ __device__ constexpr size_t cg_smem_bytes() {
  // u* hi (x y z lo.x), lo (lo.y lo.z), p, per-warp accumulators
  return (size_t)kTileVerts * (sizeof(V4<R>) + sizeof(V2<R>) + sizeof(V4<R>) + kCgWarps * sizeof(V4<R>));
}

template <class R, int MAT>
__global__ void __launch_bounds__(kCgThreads) cg_prod_kernel(CgArgs c) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V4<R>* sh = reinterpret_cast<V4<R>*>(smem_raw);
  V4<R>* sp = sh + kTileVerts;
  V4<R>* acc = sp + kTileVerts;  // [warp][vertex]
  V2<R>* sl = reinterpret_cast<V2<R>*>(acc + kCgWarps * kTileVerts);
  const SolveArgs& a = c.a;
  const int tile = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gs = a.fv.tile_gstart[tile], ge = a.fv.tile_gstart[tile + 1];
  int g = gs + warp, n = 0;
  ElemGeo<R> geo;
  uint32_t ids = 0;
  if (g < ge) {
    const int e0 = a.fv.group_estart[g];
    n = a.fv.group_estart[g + 1] - e0;
    if (lane < n) load_elem_m<R, MAT>(a.fv, e0 + lane, geo, ids);
  }
  const int vs = a.fv.tile_vstart[tile], nv = a.fv.tile_vstart[tile + 1] - vs;
  pdl_trigger_cg();
  pdl_wait_cg();
  CgState* cs = c.cs;
  if (c.cond && blockIdx.x == 0 && threadIdx.x == 0)
    cudaGraphSetConditional((cudaGraphConditionalHandle)c.cond, 0u);  // the second vertex pass re-arms
  if (cs->done) return;
  const R beta = (R)cs->beta;
  const int pb = cs->pbuf;
  const V4<R>* po = cg_p_prev<R>(c, pb);
  V4<R>* pc = cg_p_cur<R>(c, pb);
  const V4<R>* XA = (const V4<R>*)a.xa;
#pragma unroll
  for (int j = 0; j < kCgVerts; ++j) {
    const int i = threadIdx.x + j * kCgThreads;
    if (i >= nv) continue;
    const int v = a.fv.tv_vid[vs + i];
    const V4<R> x = ldg4(XA + 2 * v), xl = ldg4(XA + 2 * v + 1);
    const V4<R> z = cg_precond(ldg4((const V4<R>*)c.minv + v), ldg4((const V4<R>*)c.res + v));
    const V4<R> p = cg_dir(z, ldg4(po + v), beta);
    pc[v] = p;  // tiles sharing v store equal values
    sh[i] = V4<R>{x.x, x.y, x.z, xl.x};
    sl[i] = V2<R>{xl.y, xl.z};
    sp[i] = p;
  }
  for (int i = threadIdx.x; i < kCgWarps * kTileVerts; i += blockDim.x) acc[i] = V4<R>{R(0), R(0), R(0), R(0)};
  __syncthreads();

  V4<R>* my = acc + warp * kTileVerts;
  while (g < ge) {
    const int gn = g + kCgWarps;
    int nn = 0;
    ElemGeo<R> geon;
    uint32_t idsn = 0;
    if (gn < ge) {
      const int e0n = a.fv.group_estart[gn];
      nn = a.fv.group_estart[gn + 1] - e0n;
      if (lane < nn) load_elem_m<R, MAT>(a.fv, e0n + lane, geon, idsn);
    }
    const int l[4] = {corner(ids, 0), corner(ids, 1), corner(ids, 2), corner(ids, 3)};
    R f[4][3];
    if (lane < n) {
      R G[3][3], dF[3][3], M[3][3];
      {
        const V4<R> h0 = sh[l[0]];
        const V2<R> q0 = sl[l[0]];
        R e[3][3];
#pragma unroll
        for (int k = 1; k < 4; ++k) {
          const V4<R> h = sh[l[k]];
          const V2<R> q = sl[l[k]];
          e[0][k - 1] = pair_diff(h.x, h.w, h0.x, h0.w);
          e[1][k - 1] = pair_diff(h.y, q.x, h0.y, q0.x);
          e[2][k - 1] = pair_diff(h.z, q.y, h0.z, q0.y);
        }
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j)
            G[i][j] = e[i][0] * geo.D[0][j] + e[i][1] * geo.D[1][j] + e[i][2] * geo.D[2][j];
      }
      {
        const V4<R> w0 = sp[l[0]], w1 = sp[l[1]], w2 = sp[l[2]], w3 = sp[l[3]];
        const R e[3][3] = {{w1.x - w0.x, w2.x - w0.x, w3.x - w0.x},
                           {w1.y - w0.y, w2.y - w0.y, w3.y - w0.y},
                           {w1.z - w0.z, w2.z - w0.z, w3.z - w0.z}};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j)
            dF[i][j] = e[i][0] * geo.D[0][j] + e[i][1] * geo.D[1][j] + e[i][2] * geo.D[2][j];
      }
      add_act<MAT>(geo, G);
      if constexpr (snh_family(MAT)) {
        SnhPoint<R> s;
        snh_prepare(G, s);
        SnhDir<R> d;
        snh_dir(s, dF, d);
        snh_hess_prod(s, d, dF, geo.mu, geo.lam, M);
      } else {
        const R jm1 = (G[0][0] + G[1][1] + G[2][2]) + inv2(G) + det3(G);
        Svd<R> sv;
        svd_rv(G, jm1, sv);
        R lk[3];
        arap_lambdas(sv, lk);
        arap_hess_prod(sv, lk, dF, geo.mu, M);
      }
      corner_vjp(M, geo.D, f);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      __syncwarp();
      if (lane < n) {
        V4<R> q = my[l[k]];
        q.x += f[k][0];
        q.y += f[k][1];
        q.z += f[k][2];
        my[l[k]] = q;
      }
    }
    __syncwarp();
    g = gn;
    n = nn;
    geo = geon;
    ids = idsn;
  }
  __syncthreads();
  V4<R>* slots = (V4<R>*)a.slots;
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    V4<R> q = acc[i];
#pragma unroll
    for (int w = 1; w < kCgWarps; ++w) {
      const V4<R> r = acc[w * kTileVerts + i];
      q.x += r.x;
      q.y += r.y;
      q.z += r.z;
    }
    slots[2 * a.slot_of_tv[vs + i]] = V4<R>{q.x, q.y, q.z, R(0)};
  }
}

// ---------------------------------------------------------------------------
// vertex pass 1: q = sum of slots on free DOFs; alpha = r.z / p.q
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(kVThreadsCg) cg_vertex1_kernel(CgArgs c) {
  __shared__ Acc<R> red[(kVThreadsCg / 32) * 1];
  const SolveArgs& a = c.a;
  pdl_trigger_cg();
  pdl_wait_cg();
  CgState* cs = c.cs;
  if (cs->done) return;
  const V4<R>* XA = (const V4<R>*)a.xa;
  const V4<R>* slots = (const V4<R>*)a.slots;
  const V4<R>* pc = cg_p_cur<R>(c, cs->pbuf);
  Acc<R> s[1] = {};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n_points; i += gridDim.x * blockDim.x) {
    const int mask = (int)XA[2 * i].w;
    R q[3] = {R(0), R(0), R(0)};
    for (int k = a.off[i]; k < a.off[i + 1]; ++k) {
      const V4<R> v = slots[2 * k];
      q[0] += v.x;
      q[1] += v.y;
      q[2] += v.z;
    }
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if ((mask >> d) & 1) q[d] = R(0);
    const V4<R> p = pc[i];
    s[0].add(p.x * q[0] + p.y * q[1] + p.z * q[2]);
    ((V4<R>*)c.q)[i] = V4<R>{q[0], q[1], q[2], R(0)};
  }
  double tot[1];
  if (!grid_reduce_masked<1, 0x1u, R>(s, (AccStore<R>*)c.part, c.cnt, gridDim.x, red, tot)) return;
  if (threadIdx.x != 0) return;
  const double pq = tot[0];
  if (!(pq > 0.0) || !isfinite(pq)) {  // H not positive definite along p, or NaN
    cs->done = 1;
    cs->result = isfinite(pq) ? AGB_LINE_SEARCH_FAILED : AGB_NAN_ENCOUNTERED;
    cs->alpha = 0.0;
    return;
  }
  cs->alpha = cs->rz / pq;
}

// ---------------------------------------------------------------------------
// vertex pass 2: lam += alpha p, r -= alpha q, z = M^-1 r; beta, convergence
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(kVThreadsCg) cg_vertex2_kernel(CgArgs c) {
  __shared__ Acc<R> red[(kVThreadsCg / 32) * 2];
  const SolveArgs& a = c.a;
  pdl_trigger_cg();
  pdl_wait_cg();
  CgState* cs = c.cs;
  if (cs->done) return;
  const R alpha = (R)cs->alpha;
  const V4<R>* pc = cg_p_cur<R>(c, cs->pbuf);
  V4<R>* L = (V4<R>*)c.lam;
  V4<R>* Rs = (V4<R>*)c.res;
  const V4<R>* Q = (const V4<R>*)c.q;
  const V4<R>* M = (const V4<R>*)c.minv;
  Acc<R> s[2] = {};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n_points; i += gridDim.x * blockDim.x) {
    const V4<R> p = pc[i], q = Q[i], m = M[i];
    V4<R> l = L[i], r = Rs[i];
    l = V4<R>{fma_rn(alpha, p.x, l.x), fma_rn(alpha, p.y, l.y), fma_rn(alpha, p.z, l.z), R(0)};
    r = V4<R>{fma_rn(-alpha, q.x, r.x), fma_rn(-alpha, q.y, r.y), fma_rn(-alpha, q.z, r.z), R(0)};
    const V4<R> z = cg_precond(m, r);
    s[0].add(r.x * z.x + r.y * z.y + r.z * z.z);
    s[1].add(r.x * r.x + r.y * r.y + r.z * r.z);
    L[i] = l;
    Rs[i] = r;
  }
  double tot[2];
  if (!grid_reduce_masked<2, 0x0u, R>(s, (AccStore<R>*)c.part, c.cnt, gridDim.x, red, tot)) return;
  if (threadIdx.x != 0) return;
  const double rz = tot[0], rr = tot[1];
  cs->beta = cs->rz > 0.0 ? rz / cs->rz : 0.0;
  cs->rz = rz;
  cs->rr = rr;
  cs->iter += 1;
  cs->pbuf ^= 1;
  const double rn = sqrt(rr);
  if (!isfinite(rn)) {
    cs->done = 1;
    cs->result = AGB_NAN_ENCOUNTERED;
  } else if (rn <= fmax(cs->atol, cs->rtol * sqrt(cs->rr0))) {
    cs->done = 1;
    cs->result = AGB_PRIMARY_SUCCESS;
  } else if (cs->iter >= cs->max_iter) {
    cs->done = 1;
    cs->result = AGB_MAX_STEPS_REACHED;
  }
  if (c.cond)
    cudaGraphSetConditional((cudaGraphConditionalHandle)c.cond,
                            (!cs->done && cs->iter < cs->iter_limit) ? 1u : 0u);
}

template <class R>
__global__ void __launch_bounds__(256) cg_unpack_kernel(int n, const V4<R>* __restrict__ v,
                                                        const int32_t* __restrict__ uoi, R* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const size_t k = 3 * (size_t)uoi[i];
    const V4<R> x = v[i];
    out[k] = x.x;
    out[k + 1] = x.y;
    out[k + 2] = x.z;
  }
}

__global__ void cg_set_limit_kernel(CgState* cs, int n) { cs->iter_limit = cs->iter + n; }

template <class... P, class... A>
cudaError_t launch_pdl_cg(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A... args) {
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

template <class R, int MAT>
cudaError_t cg_iteration_t(const CgArgs& c, cudaStream_t s) {
  // the element pass opens the loop body: a plain launch
  cg_prod_kernel<R, MAT><<<c.a.fv.n_tiles, kCgThreads, cg_smem_bytes<R>(), s>>>(c);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = launch_pdl_cg(cg_vertex1_kernel<R>, dim3(c.vblocks), dim3(kVThreadsCg), 0, s, c);
  if (e == cudaSuccess) e = launch_pdl_cg(cg_vertex2_kernel<R>, dim3(c.vblocks), dim3(kVThreadsCg), 0, s, c);
  return e;
}

template <class R>
cudaError_t cg_prepare_t() {
  const int b = (int)cg_smem_bytes<R>();
  const cudaFuncAttribute m = cudaFuncAttributeMaxDynamicSharedMemorySize;
  cudaError_t e = cudaFuncSetAttribute(cg_prod_kernel<R, AGB_ARAP>, m, b);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(cg_prod_kernel<R, AGB_STABLE_NEO_HOOKEAN>, m, b);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(cg_prod_kernel<R, AGB_STABLE_NEO_HOOKEAN_MUSCLE>, m, b);
  return e;
}

// ---------------------------------------------------------------------------
// material VJP: out_mu[c] += d(w . g)/d mu_c, out_lambda[c] += d(w . g)/d lambda_c
// ---------------------------------------------------------------------------
template <class R, int MAT>
__global__ void __launch_bounds__(kElemThreads) param_vjp_kernel(FemView fv, const V4<R>* __restrict__ u,
                                                                 const V4<R>* __restrict__ w,
                                                                 const R* __restrict__ vol,
                                                                 const int32_t* __restrict__ elem_user,
                                                                 R* __restrict__ out_mu, R* __restrict__ out_lam) {
  __shared__ V4<R> su[kTileVerts];
  __shared__ V4<R> sw[kTileVerts];
  const int tile = blockIdx.x;
  const int vs = fv.tile_vstart[tile], nv = fv.tile_vstart[tile + 1] - vs;
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    const int v = fv.tv_vid[vs + i];
    su[i] = ldg4(u + v);
    sw[i] = ldg4(w + v);
  }
  __syncthreads();
  for (int e = fv.tile_estart[tile] + threadIdx.x; e < fv.tile_estart[tile + 1]; e += blockDim.x) {
    ElemGeo<R> geo;
    uint32_t ids;
    load_elem_m<R, MAT>(fv, e, geo, ids);
    const int l[4] = {corner(ids, 0), corner(ids, 1), corner(ids, 2), corner(ids, 3)};
    R cu[4][3], cw[4][3], G[3][3], W[3][3];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const V4<R> a = su[l[k]], b = sw[l[k]];
      cu[k][0] = a.x;
      cu[k][1] = a.y;
      cu[k][2] = a.z;
      cw[k][0] = b.x;
      cw[k][1] = b.y;
      cw[k][2] = b.z;
    }
    corner_gradient(cu, geo.D, G);
    add_act<MAT>(geo, G);
    corner_gradient(cw, geo.D, W);  // muscle: W A (the records hold D A)
    R dmu, dlam = R(0);
    if constexpr (snh_family(MAT)) {
      // P = mu' (F - cof F) + lambda' (J - 1) cof F  (mu' = mu dV, lambda' = lambda dV)
      SnhPoint<R> s;
      snh_prepare(G, s);
      R P1[3][3];
      snh_pk1(s, R(1), R(0), P1);
      dmu = ddot3(P1, W);
      dlam = s.jm1 * ddot3(s.cofF, W);
    } else {
      // P = mu' (F - R)
      const R jm1 = (G[0][0] + G[1][1] + G[2][2]) + inv2(G) + det3(G);
      Svd<R> sv;
      svd_rv(G, jm1, sv);
      R P1[3][3];
      arap_pk1(sv, R(1), P1);
      dmu = ddot3(P1, W);
    }
    const R dv = vol[e];
    const int c = elem_user[e];
    out_mu[c] += dv * dmu;
    if (out_lam) out_lam[c] += dv * dlam;
  }
}

// d(w . grad)/d a for the muscle activation a (six entries per cell, A = I + sym(a)).
// With F_m = F A = I + G_m, W' = sum_a w_a (D A)_a and P, dP premultiplied by dV:
//   d/dA [P(F A) : W_0 A] = A^-1 (F_m^T dP[W'] + W'^T P(F_m))   (A symmetric)
// and d/da = (Z00, Z11, Z22, Z01 + Z10, Z02 + Z20, Z12 + Z21)
// (warp/fem/_stable_neo_hookean_muscle.py:18-46, func/_misc.py:48-53).
template <class R>
__global__ void __launch_bounds__(kElemThreads) activation_vjp_kernel(FemView fv, const V4<R>* __restrict__ u,
                                                                      const V4<R>* __restrict__ w,
                                                                      const int32_t* __restrict__ elem_user,
                                                                      R* __restrict__ out_act) {
  __shared__ V4<R> su[kTileVerts];
  __shared__ V4<R> sw[kTileVerts];
  const int tile = blockIdx.x;
  const int vs = fv.tile_vstart[tile], nv = fv.tile_vstart[tile + 1] - vs;
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    const int v = fv.tv_vid[vs + i];
    su[i] = ldg4(u + v);
    sw[i] = ldg4(w + v);
  }
  __syncthreads();
  for (int e = fv.tile_estart[tile] + threadIdx.x; e < fv.tile_estart[tile + 1]; e += blockDim.x) {
    ElemGeo<R> geo;
    uint32_t ids;
    load_elem_m<R, AGB_STABLE_NEO_HOOKEAN_MUSCLE>(fv, e, geo, ids);
    const int l[4] = {corner(ids, 0), corner(ids, 1), corner(ids, 2), corner(ids, 3)};
    R cu[4][3], cw[4][3], G[3][3], W[3][3];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const V4<R> a = su[l[k]], b = sw[l[k]];
      cu[k][0] = a.x;
      cu[k][1] = a.y;
      cu[k][2] = a.z;
      cw[k][0] = b.x;
      cw[k][1] = b.y;
      cw[k][2] = b.z;
    }
    corner_gradient(cu, geo.D, G);
    add_act<AGB_STABLE_NEO_HOOKEAN_MUSCLE>(geo, G);
    corner_gradient(cw, geo.D, W);
    SnhPoint<R> s;
    snh_prepare(G, s);
    R P[3][3], H[3][3];
    snh_pk1(s, geo.mu, geo.lam, P);
    SnhDir<R> d;
    snh_dir(s, W, d);
    snh_hess_prod(s, d, W, geo.mu, geo.lam, H);
    R T[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        R t = R(0);
#pragma unroll
        for (int k = 0; k < 3; ++k) t += (G[k][i] + (k == i ? R(1) : R(0))) * H[k][j] + W[k][i] * P[k][j];
        T[i][j] = t;
      }
    R A[3][3] = {{R(1) + geo.S[0], geo.S[3], geo.S[4]},
                 {geo.S[3], R(1) + geo.S[1], geo.S[5]},
                 {geo.S[4], geo.S[5], R(1) + geo.S[2]}};
    R cA[3][3];
    cof3(A, cA);  // symmetric A: A^-1 = cof(A) / det(A)
    const R inv_det = R(1) / det3(A);
    R Z[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) Z[i][j] = inv_det * (cA[i][0] * T[0][j] + cA[i][1] * T[1][j] + cA[i][2] * T[2][j]);
    R* o = out_act + 6 * (size_t)elem_user[e];
    o[0] += Z[0][0];
    o[1] += Z[1][1];
    o[2] += Z[2][2];
    o[3] += Z[0][1] + Z[1][0];
    o[4] += Z[0][2] + Z[2][0];
    o[5] += Z[1][2] + Z[2][1];
  }
}

}  // namespace

size_t cg_smem(int precision) {
  return precision == AGB_F64 ? cg_smem_bytes<double>() : cg_smem_bytes<float>();
}

cudaError_t cg_prepare_kernels(int precision) {
  return precision == AGB_F64 ? cg_prepare_t<double>() : cg_prepare_t<float>();
}

cudaError_t launch_cg_init(const CgArgs& c, const void* rhs, const int32_t* uoi, cudaStream_t s) {
  if (c.a.precision == AGB_F64)
    cg_init_kernel<double><<<c.vblocks, kVThreadsCg, 0, s>>>(c, (const double*)rhs, uoi);
  else
    cg_init_kernel<float><<<c.vblocks, kVThreadsCg, 0, s>>>(c, (const float*)rhs, uoi);
  return cudaGetLastError();
}

cudaError_t launch_cg_iteration(const CgArgs& c, cudaStream_t s) {
  if (c.a.fv.n_tiles == 0) return cudaErrorInvalidValue;
  cudaError_t e;
  if (c.a.precision == AGB_F64)
    e = c.a.fv.material == AGB_ARAP ? cg_iteration_t<double, AGB_ARAP>(c, s)
        : c.a.fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE
            ? cg_iteration_t<double, AGB_STABLE_NEO_HOOKEAN_MUSCLE>(c, s)
            : cg_iteration_t<double, AGB_STABLE_NEO_HOOKEAN>(c, s);
  else
    e = c.a.fv.material == AGB_ARAP ? cg_iteration_t<float, AGB_ARAP>(c, s)
        : c.a.fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE
            ? cg_iteration_t<float, AGB_STABLE_NEO_HOOKEAN_MUSCLE>(c, s)
            : cg_iteration_t<float, AGB_STABLE_NEO_HOOKEAN>(c, s);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_cg_set_limit(const CgArgs& c, int n, cudaStream_t s) {
  cg_set_limit_kernel<<<1, 1, 0, s>>>(c.cs, n);
  return cudaGetLastError();
}

cudaError_t launch_cg_unpack(const CgArgs& c, const int32_t* uoi, void* out, cudaStream_t s) {
  const int blocks = (c.a.n_points + 255) / 256 < 1024 ? (c.a.n_points + 255) / 256 : 1024;
  if (blocks == 0) return cudaSuccess;
  if (c.a.precision == AGB_F64)
    cg_unpack_kernel<double><<<blocks, 256, 0, s>>>(c.a.n_points, (const V4<double>*)c.lam, uoi, (double*)out);
  else
    cg_unpack_kernel<float><<<blocks, 256, 0, s>>>(c.a.n_points, (const V4<float>*)c.lam, uoi, (float*)out);
  return cudaGetLastError();
}

cudaError_t launch_param_vjp(const FemView& fv, int precision, const void* u, const void* w, const void* vol,
                             const int32_t* elem_user, void* out_mu, void* out_lam, cudaStream_t s) {
  if (fv.n_tiles == 0) return cudaSuccess;
  const dim3 g(fv.n_tiles), b(kElemThreads);
  const bool muscle = fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE;
  if (precision == AGB_F64) {
    if (muscle)
      param_vjp_kernel<double, AGB_STABLE_NEO_HOOKEAN_MUSCLE><<<g, b, 0, s>>>(
          fv, (const V4<double>*)u, (const V4<double>*)w, (const double*)vol, elem_user, (double*)out_mu,
          (double*)out_lam);
    else if (fv.material == AGB_ARAP)
      param_vjp_kernel<double, AGB_ARAP><<<g, b, 0, s>>>(fv, (const V4<double>*)u, (const V4<double>*)w,
                                                          (const double*)vol, elem_user, (double*)out_mu,
                                                          (double*)out_lam);
    else
      param_vjp_kernel<double, AGB_STABLE_NEO_HOOKEAN><<<g, b, 0, s>>>(
          fv, (const V4<double>*)u, (const V4<double>*)w, (const double*)vol, elem_user, (double*)out_mu,
          (double*)out_lam);
  } else {
    if (muscle)
      param_vjp_kernel<float, AGB_STABLE_NEO_HOOKEAN_MUSCLE><<<g, b, 0, s>>>(
          fv, (const V4<float>*)u, (const V4<float>*)w, (const float*)vol, elem_user, (float*)out_mu,
          (float*)out_lam);
    else if (fv.material == AGB_ARAP)
      param_vjp_kernel<float, AGB_ARAP><<<g, b, 0, s>>>(fv, (const V4<float>*)u, (const V4<float>*)w,
                                                         (const float*)vol, elem_user, (float*)out_mu,
                                                         (float*)out_lam);
    else
      param_vjp_kernel<float, AGB_STABLE_NEO_HOOKEAN><<<g, b, 0, s>>>(
          fv, (const V4<float>*)u, (const V4<float>*)w, (const float*)vol, elem_user, (float*)out_mu,
          (float*)out_lam);
  }
  return cudaGetLastError();
}

cudaError_t launch_activation_vjp(const FemView& fv, int precision, const void* u, const void* w,
                                  const int32_t* elem_user, void* out_act, cudaStream_t s) {
  if (fv.n_tiles == 0) return cudaSuccess;
  if (fv.material != AGB_STABLE_NEO_HOOKEAN_MUSCLE || !fv.act) return cudaErrorInvalidValue;
  const dim3 g(fv.n_tiles), b(kElemThreads);
  if (precision == AGB_F64)
    activation_vjp_kernel<double><<<g, b, 0, s>>>(fv, (const V4<double>*)u, (const V4<double>*)w, elem_user,
                                                  (double*)out_act);
  else
    activation_vjp_kernel<float><<<g, b, 0, s>>>(fv, (const V4<float>*)u, (const V4<float>*)w, elem_user,
                                                 (float*)out_act);
  return cudaGetLastError();
}

}  // namespace agb
