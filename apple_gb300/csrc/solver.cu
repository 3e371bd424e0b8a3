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
//   [ARAP]          trial passes evaluate the remainder at up to three trial
//                   steps each (ARAP is not polynomial in t)
//   gradient pass   at x_{k+1} = x_k + t p_k: energy, gradient, clamped
//                   Hessian diagonal -> tile slots, accumulated per warp in
//                   private shared-memory copies (no atomics, fixed order)
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

#include "kernels.h"
#include "solver.h"
#include "tile.cuh"

namespace agb {

constexpr int kVThreads = 256;
constexpr int kWarps = kElemThreads / 32;
// gradient pass: 4 warps per tile, one private accumulator copy per warp
constexpr int kGradThreads = 128;
constexpr int kGradWarps = kGradThreads / 32;

// Persistent grids: the vertex pass and the direction pass launch as many
// CTAs as are resident at once (152 SMs x CTAs per SM) and stride over
// vertices / tiles, so each CTA's block reduction covers several vertices
// or tiles and the completion sums a few hundred partials in one level.
constexpr int kSMs = 152;
constexpr int kVertexCtasPerSM = 4;
constexpr int kDirCtasPerSM = 3;

int solver_vertex_blocks(int n_points) {
  int b = (n_points + kVThreads - 1) / kVThreads;
  const int cap = kSMs * kVertexCtasPerSM;
  return b < 1 ? 1 : (b > cap ? cap : b);
}

static int dir_blocks(int n_tiles) { return n_tiles < kSMs * kDirCtasPerSM ? n_tiles : kSMs * kDirCtasPerSM; }

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ double initial_alpha(double gd, double hq, double overstep) {
  double a = -gd / hq;
  if (isnan(a)) a = 0.0;
  if (isinf(a)) a = a > 0 ? 1.0 : 0.0;
  if (!(a > 0.0 && isfinite(a))) a = 1.0;
  return a * overstep;
}

// A rejected line search restarts with steepest descent; along steepest
// descent it ends the solve (LINE_SEARCH_FAILED).
__device__ __forceinline__ void reject_step(SolverState* st, int ls) {
  st->t = 0.0;
  st->delta_e = 0.0;
  st->ls_ok = 0;
  st->ls_steps = ls;
  st->reset_beta = 1;
  if (st->beta == 0.0) st->ls_fail = 1;
}

// search directions: p[pbuf] = p_prev, p[pbuf ^ 1] = p of this iteration
template <class R>
__device__ __forceinline__ V4<R>* p_prev(const SolveArgs& a, int pb) {
  return (V4<R>*)(pb ? a.p1 : a.p0);
}
template <class R>
__device__ __forceinline__ V4<R>* p_cur(const SolveArgs& a, int pb) {
  return (V4<R>*)(pb ? a.p0 : a.p1);
}

template <class R>
__device__ __forceinline__ void stage_direction(const SolveArgs& a, int vs, int nv, const V4<R>* P,
                                                R (*sh)[kTileVerts], R (*sl)[kTileVerts],
                                                R (*sp)[kTileVerts]) {
  const V4<R>* XA = (const V4<R>*)a.xa;
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    const int v = a.fv.tv_vid[vs + i];
    const V4<R> x = ldg4(XA + 2 * v), xl = ldg4(XA + 2 * v + 1), p = ldg4(P + v);
    sh[0][i] = x.x;
    sh[1][i] = x.y;
    sh[2][i] = x.z;
    sl[0][i] = xl.x;
    sl[1][i] = xl.y;
    sl[2][i] = xl.z;
    sp[0][i] = p.x;
    sp[1][i] = p.y;
    sp[2][i] = p.z;
  }
}

template <class R>
__device__ __forceinline__ void gather_corners(R (*s)[kTileVerts], const int (&l)[4], R (&w)[4][3]) {
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) w[a][c] = s[c][l[a]];
}

// G = sum_a (x_a - x_0) D_a^T with the differences taken on hi + lo pairs
template <class R>
__device__ __forceinline__ void position_gradient(R (*sh)[kTileVerts], R (*sl)[kTileVerts],
                                                  const int (&l)[4], const R (&D)[3][3],
                                                  R (&G)[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const R h0 = sh[i][l[0]], l0 = sl[i][l[0]];
    const R e1 = pair_diff(sh[i][l[1]], sl[i][l[1]], h0, l0);
    const R e2 = pair_diff(sh[i][l[2]], sl[i][l[2]], h0, l0);
    const R e3 = pair_diff(sh[i][l[3]], sl[i][l[3]], h0, l0);
#pragma unroll
    for (int j = 0; j < 3; ++j) G[i][j] = e1 * D[0][j] + e2 * D[1][j] + e3 * D[2][j];
  }
}

// ---------------------------------------------------------------------------
// direction pass
// ---------------------------------------------------------------------------
// positions for the line-search pass: the hi word only (the polynomial's
// coefficients need ~1e-3 relative accuracy, not the float-float pair);
// one 16-byte vector per vertex so a corner is one shared-memory load
// p = -P g + beta p_prev for the thread's tile vertex v (kTileVerts ==
// kElemThreads; v < 0: none): staged with x_hi for the tile's elements and
// stored as this iteration's direction (tiles sharing v store equal values)
template <class R>
__device__ __forceinline__ void stage_dir(const SolveArgs& a, int v, R beta, R inv_mean,
                                          const V4<R>* pprev, V4<R>* pcur, V4<R>* sx, V4<R>* sp) {
  if (v < 0) return;
  const V4<R> x = ldg4((const V4<R>*)a.xa + 2 * v), g = ldg4((const V4<R>*)a.gd + 2 * v),
              d = ldg4((const V4<R>*)a.gd + 2 * v + 1), po = ldg4(pprev + v);
  R p[3];
  pdir(g, d, po, beta, inv_mean, p);
  const V4<R> pv{p[0], p[1], p[2], R(0)};
  pcur[v] = pv;
  sx[threadIdx.x] = V4<R>{x.x, x.y, x.z, R(0)};
  sp[threadIdx.x] = pv;
}

// the thread's vertex of a tile, or -1
__device__ __forceinline__ int tile_vertex(const FemView& fv, int tile, int i) {
  if (tile >= fv.n_tiles) return -1;
  const int vs = fv.tile_vstart[tile];
  return i < fv.tile_vstart[tile + 1] - vs ? fv.tv_vid[vs + i] : -1;
}

// W = sum_a (w_a - w_0) D_a^T from 16-byte staged corners
template <class R>
__device__ __forceinline__ void vec_gradient(const V4<R>* s, const int (&l)[4], const R (&D)[3][3],
                                             R (&W)[3][3]) {
  const V4<R> w0 = s[l[0]], w1 = s[l[1]], w2 = s[l[2]], w3 = s[l[3]];
  const R e[3][3] = {{w1.x - w0.x, w2.x - w0.x, w3.x - w0.x},
                     {w1.y - w0.y, w2.y - w0.y, w3.y - w0.y},
                     {w1.z - w0.z, w2.z - w0.z, w3.z - w0.z}};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) W[i][j] = e[i][0] * D[0][j] + e[i][1] * D[1][j] + e[i][2] * D[2][j];
}

template <class R, int MAT>
__global__ void __launch_bounds__(kElemThreads, kDirCtasPerSM) solver_dir_kernel(SolveArgs a, int use_cond) {
  constexpr int N = (MAT == AGB_STABLE_NEO_HOOKEAN) ? 6 : 1;
  // float-float warp trees only for c2 (terms of both signs); p^T H p is a
  // sum of clamped non-negative terms, c3..c6 are higher-order corrections
  constexpr unsigned FF = (MAT == AGB_STABLE_NEO_HOOKEAN) ? 0x2u : 0x0u;
  __shared__ V4<R> sx[kTileVerts];
  __shared__ V4<R> sp[kTileVerts];
  __shared__ Acc<R> red[kWarps * N];
  SolverState* st = a.st;
  pdl_trigger();
  if (use_cond && blockIdx.x == 0 && threadIdx.x == 0)
    cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond, 0u);  // vertex pass re-arms
  static_assert(kTileVerts == kElemThreads, "one staged vertex per thread");
  int tile = blockIdx.x;
  // constant inputs first: the thread's first element record and vertex id
  int es = a.fv.tile_estart[tile], ee = a.fv.tile_estart[tile + 1];
  int e = es + threadIdx.x;
  ElemGeo<R> geo;
  uint32_t ids = 0;
  if (e < ee) load_elem<R>(a.fv, e, geo, ids);
  int vid = tile_vertex(a.fv, tile, threadIdx.x);
  if (st->done) return;
  const R beta = (R)st->beta, inv_mean = (R)st->inv_mean;
  const int pb = st->pbuf;
  const V4<R>* pprev = p_prev<R>(a, pb);
  V4<R>* pcur = p_cur<R>(a, pb);

  Acc<R> sums[N] = {};
  for (; tile < a.fv.n_tiles; tile += gridDim.x) {
    stage_dir<R>(a, vid, beta, inv_mean, pprev, pcur, sx, sp);
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
      if (last ? en < een : true) load_elem<R>(a.fv, en, geon, idsn);
      const int l[4] = {corner(ids, 0), corner(ids, 1), corner(ids, 2), corner(ids, 3)};
      R G[3][3], dF[3][3];
      vec_gradient(sx, l, geo.D, G);
      vec_gradient(sp, l, geo.D, dF);
      if constexpr (MAT == AGB_STABLE_NEO_HOOKEAN) {
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
        const R jm1 = (G[0][0] + G[1][1] + G[2][2]) + inv2(G) + det3(G);
        Svd<R> sv;
        svd_rv(G, jm1, sv);
        R lk[3];
        arap_lambdas(sv, lk);
        sums[0].add(fmax(arap_hess_quad(sv, lk, dF, geo.mu), R(0)));
      }
      geo = geon;
      ids = idsn;
      e = en;
      if (last) break;
    }
    if (!had) {  // no element of this tile for this thread: start on the next tile
      e = esn + threadIdx.x;
      if (e < een) load_elem<R>(a.fv, e, geo, ids);
    }
    es = esn;
    ee = een;
    __syncthreads();
  }
  double tot[N];
  if (!grid_reduce_masked<N, FF, R>(sums, (AccStore<R>*)a.part_a, a.cnt_a, gridDim.x, red, tot)) return;
  if (threadIdx.x != 0) return;
  const double hq = tot[0];
  st->hq = hq;
  const double gd = st->gd;
  const double a0 = initial_alpha(gd, hq, st->overstep);
  st->alpha0 = a0;
  if constexpr (MAT == AGB_STABLE_NEO_HOOKEAN) {
    double t = a0, de = 0.0;
    int ls = 0;
    bool ok = false;
    for (;;) {
      de = t * (gd + t * (tot[1] + t * (tot[2] + t * (tot[3] + t * (tot[4] + t * tot[5])))));
      ok = isfinite(de) && de <= st->armijo_c * t * gd;
      if (ok || ls >= st->max_bt || !(t > 0.0)) break;
      t *= 0.5;
      ++ls;
    }
    if (ok) {
      st->t = t;
      st->delta_e = de;
      st->ls_ok = 1;
      st->ls_steps = ls;
    } else {
      reject_step(st, ls);
    }
    st->decided = 1;
  } else {
    st->t = 0.0;
    st->decided = 0;
  }
}

// ---------------------------------------------------------------------------
// ARAP trial pass: remainders at trial steps alpha_0 2^-j, j = j0 .. j0+2
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(kElemThreads) solver_trial_kernel(SolveArgs a, int j0) {
  __shared__ R sh[3][kTileVerts];
  __shared__ R sl[3][kTileVerts];
  __shared__ R sp[3][kTileVerts];
  __shared__ Acc<R> red[kWarps * 3];
  SolverState* st = a.st;
  if (st->done || st->decided) return;
  const double a0 = st->alpha0;
  R tj[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) tj[j] = (R)ldexp(a0, -(j0 + j));
  const int tile = blockIdx.x;
  const int vs = a.fv.tile_vstart[tile], nv = a.fv.tile_vstart[tile + 1] - vs;
  const int es = a.fv.tile_estart[tile], ee = a.fv.tile_estart[tile + 1];
  stage_direction<R>(a, vs, nv, p_cur<R>(a, st->pbuf), sh, sl, sp);
  __syncthreads();
  Acc<R> sums[3] = {};
  for (int e = es + threadIdx.x; e < ee; e += blockDim.x) {
    ElemGeo<R> geo;
    uint32_t ids;
    load_elem<R>(a.fv, e, geo, ids);
    const int l[4] = {corner(ids, 0), corner(ids, 1), corner(ids, 2), corner(ids, 3)};
    R w[4][3], G[3][3], dF[3][3];
    position_gradient(sh, sl, l, geo.D, G);
    gather_corners(sp, l, w);
    corner_gradient(w, geo.D, dF);
    Svd<R> base;
    svd_rv(G, (G[0][0] + G[1][1] + G[2][2]) + inv2(G) + det3(G), base);
#pragma unroll 1
    for (int j = 0; j < 3; ++j) {
      R Gt[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) Gt[i][k] = fma_rn(tj[j], dF[i][k], G[i][k]);
      Svd<R> trial;
      svd_rv(Gt, (Gt[0][0] + Gt[1][1] + Gt[2][2]) + inv2(Gt) + det3(Gt), trial);
      sums[j].add(arap_remainder(base, trial, tj[j], dF, geo.mu));
    }
  }
  double tot[3];
  if (!grid_reduce2<3, 0x7u, R>(sums, (AccStore<R>*)a.part_t, (AccStore<R>*)a.gpart_t, a.cnt_t,
                                gridDim.x, red, tot))
    return;
  if (threadIdx.x != 0) return;
  const double gd = st->gd;
  for (int j = 0; j < 3; ++j) {
    const int J = j0 + j;
    if (J > st->max_bt) break;
    const double t = ldexp(a0, -J);
    const double de = gd * t + tot[j];
    if (isfinite(de) && de <= st->armijo_c * t * gd) {
      st->t = t;
      st->delta_e = de;
      st->ls_ok = 1;
      st->ls_steps = J;
      st->decided = 1;
      return;
    }
  }
  if (j0 + 2 >= st->max_bt) {
    reject_step(st, st->max_bt);
    st->decided = 1;
  }
}

// ---------------------------------------------------------------------------
// gradient pass at x + t p
//
// Elements of a tile come in warp groups (<= 32) whose corner k is a distinct
// vertex for every lane (host-side edge colouring), so warp w adds its
// lanes' corner-k contributions into its private copy acc[w] with plain
// shared-memory loads and stores.  The copies are summed in warp order.
// ---------------------------------------------------------------------------
template <class R>
__host__ __device__ constexpr size_t grad_smem_bytes() {
  // staged hi (V4: x y z lo.x) and lo (V2: lo.y lo.z) + per-warp accumulators (V4 + V2)
  return (size_t)kTileVerts * (size_t)(kGradWarps + 1) * (sizeof(V4<R>) + sizeof(V2<R>));
}

size_t solver_grad_smem(int precision) {
  return precision == AGB_F64 ? grad_smem_bytes<double>() : grad_smem_bytes<float>();
}

// x + t p as hi + lo pairs: (hi.x hi.y hi.z lo.x) and (lo.y lo.z) per vertex
constexpr int kGradVerts = kTileVerts / kGradThreads;  // staged vertices per thread

template <class R>
__device__ __forceinline__ void stage_point(const SolveArgs& a, const int (&vid)[kGradVerts], const V4<R>* P,
                                            R t, V4<R>* sh, V2<R>* sl) {
  const V4<R>* XA = (const V4<R>*)a.xa;
#pragma unroll
  for (int j = 0; j < kGradVerts; ++j) {
    const int v = vid[j], i = threadIdx.x + j * kGradThreads;
    if (v < 0) continue;
    const V4<R> x = ldg4(XA + 2 * v), xl = ldg4(XA + 2 * v + 1), p = ldg4(P + v);
    R hx = x.x, lx = xl.x, hy = x.y, ly = xl.y, hz = x.z, lz = xl.z;
    pair_add(hx, lx, mul_rn(t, p.x));
    pair_add(hy, ly, mul_rn(t, p.y));
    pair_add(hz, lz, mul_rn(t, p.z));
    sh[i] = V4<R>{hx, hy, hz, lx};
    sl[i] = V2<R>{ly, lz};
  }
}

// G = sum_a (x_a - x_0) D_a^T with the differences taken on hi + lo pairs
template <class R>
__device__ __forceinline__ void pair_gradient(const V4<R>* sh, const V2<R>* sl, const int (&l)[4],
                                              const R (&D)[3][3], R (&G)[3][3]) {
  const V4<R> h0 = sh[l[0]];
  const V2<R> q0 = sl[l[0]];
  R e[3][3];
#pragma unroll
  for (int a = 1; a < 4; ++a) {
    const V4<R> h = sh[l[a]];
    const V2<R> q = sl[l[a]];
    e[0][a - 1] = pair_diff(h.x, h.w, h0.x, h0.w);
    e[1][a - 1] = pair_diff(h.y, q.x, h0.y, q0.x);
    e[2][a - 1] = pair_diff(h.z, q.y, h0.z, q0.y);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) G[i][j] = e[i][0] * D[0][j] + e[i][1] * D[1][j] + e[i][2] * D[2][j];
}

template <class R, int MAT>
__global__ void __launch_bounds__(kGradThreads, MAT == AGB_STABLE_NEO_HOOKEAN ? 7 : 5) solver_grad_kernel(SolveArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V4<R>* sh = reinterpret_cast<V4<R>*>(smem_raw);
  V4<R>* acc4 = sh + kTileVerts;  // [warp][vertex]: gx gy gz dx
  V2<R>* sl = reinterpret_cast<V2<R>*>(acc4 + kGradWarps * kTileVerts);
  V2<R>* acc2 = sl + kTileVerts;  // [warp][vertex]: dy dz
  __shared__ Acc<R> red[kGradWarps];
  const int tile = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gs = a.fv.tile_gstart[tile], ge = a.fv.tile_gstart[tile + 1];
  // constant inputs: the first group's element record
  int g = gs + warp;
  int n = 0;
  ElemGeo<R> geo;
  uint32_t ids = 0;
  if (g < ge) {
    const int e0 = a.fv.group_estart[g];
    n = a.fv.group_estart[g + 1] - e0;
    if (lane < n) load_elem<R>(a.fv, e0 + lane, geo, ids);
  }
  const int vs = a.fv.tile_vstart[tile], nv = a.fv.tile_vstart[tile + 1] - vs;
  int vid[kGradVerts], sidx[kGradVerts];
#pragma unroll
  for (int j = 0; j < kGradVerts; ++j) {
    const int i = threadIdx.x + j * kGradThreads;
    vid[j] = i < nv ? a.fv.tv_vid[vs + i] : -1;
    sidx[j] = i < nv ? a.slot_of_tv[vs + i] : 0;
  }
  pdl_trigger();
  pdl_wait();
  SolverState* st = a.st;
  if (st->done) return;
  stage_point<R>(a, vid, p_cur<R>(a, st->pbuf), (R)st->t, sh, sl);
  for (int i = threadIdx.x; i < kGradWarps * kTileVerts; i += blockDim.x) {
    acc4[i] = V4<R>{R(0), R(0), R(0), R(0)};
    acc2[i] = V2<R>{R(0), R(0)};
  }
  __syncthreads();

  V4<R>* my4 = acc4 + warp * kTileVerts;
  V2<R>* my2 = acc2 + warp * kTileVerts;
  Acc<R> sums[1] = {};
  while (g < ge) {
    // prefetch the warp's next group while this one computes
    const int gn = g + kGradWarps;
    int nn = 0;
    ElemGeo<R> geon;
    uint32_t idsn = 0;
    if (gn < ge) {
      const int e0n = a.fv.group_estart[gn];
      nn = a.fv.group_estart[gn + 1] - e0n;
      if (lane < nn) load_elem<R>(a.fv, e0n + lane, geon, idsn);
    }
    const int l[4] = {corner(ids, 0), corner(ids, 1), corner(ids, 2), corner(ids, 3)};
    R f[4][3], hd[4][3];
    if (lane < n) {
      R G[3][3], P[3][3];
      pair_gradient(sh, sl, l, geo.D, G);
      if constexpr (MAT == AGB_STABLE_NEO_HOOKEAN) {
        SnhPoint<R> s;
        snh_prepare(G, s);
        sums[0].add(snh_energy(s, geo.mu, geo.lam));
        snh_pk1(s, geo.mu, geo.lam, P);
        corner_vjp(P, geo.D, f);
        snh_hess_diag(s, geo.D, geo.mu, geo.lam, hd);
      } else {
        const R jm1 = (G[0][0] + G[1][1] + G[2][2]) + inv2(G) + det3(G);
        Svd<R> sv;
        svd_rv(G, jm1, sv);
        sums[0].add(arap_energy(sv, geo.mu));
        arap_pk1(sv, geo.mu, P);
        corner_vjp(P, geo.D, f);
        R lk[3];
        arap_lambdas(sv, lk);
        arap_hess_diag(sv, lk, geo.D, geo.mu, hd);
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      __syncwarp();
      if (lane < n) {
        const int v = l[k];
        V4<R> q4 = my4[v];
        V2<R> q2 = my2[v];
        q4.x += f[k][0];
        q4.y += f[k][1];
        q4.z += f[k][2];
        q4.w += fmax(hd[k][0], R(0));
        q2.x += fmax(hd[k][1], R(0));
        q2.y += fmax(hd[k][2], R(0));
        my4[v] = q4;
        my2[v] = q2;
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
#pragma unroll
  for (int j = 0; j < kGradVerts; ++j) {
    const int i = threadIdx.x + j * kGradThreads;
    if (i >= nv) continue;
    V4<R> q4 = acc4[i];
    V2<R> q2 = acc2[i];
#pragma unroll
    for (int w = 1; w < kGradWarps; ++w) {
      const V4<R> r4 = acc4[w * kTileVerts + i];
      const V2<R> r2 = acc2[w * kTileVerts + i];
      q4.x += r4.x;
      q4.y += r4.y;
      q4.z += r4.z;
      q4.w += r4.w;
      q2.x += r2.x;
      q2.y += r2.y;
    }
    slots[2 * sidx[j]] = V4<R>{q4.x, q4.y, q4.z, R(0)};
    slots[2 * sidx[j] + 1] = V4<R>{q4.w, q2.x, q2.y, R(0)};
  }
  block_reduce<1, 0x0u, R>(sums, red);
  if (threadIdx.x == 0) ((AccStore<R>*)a.part_b)[blockIdx.x] = acc_store(sums[0]);
}

// ---------------------------------------------------------------------------
// vertex pass
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(kVThreads, kVertexCtasPerSM) solver_vertex_kernel(SolveArgs a, int use_cond) {
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
  const R t = (R)st->t;
  V4<R>* XA = (V4<R>*)a.xa;
  V4<R>* GD = (V4<R>*)a.gd;
  const V4<R>* P = p_cur<R>(a, st->pbuf);
  const V4<R>* F = (const V4<R>*)a.force;
  const V4<R>* slots = (const V4<R>*)a.slots;
  // 0 gPg 1 gPy 2 yPy 3 sum|d| 4 count 5 zgg 6 zgy 7 zyy 8 y.p 9 p.g 10 g.g 11 ext energy
  // a thread sums its few vertices in R; float-float starts at the warp trees
  R s[N] = {};
  for (int i = i0; i < a.n_points; i += gridDim.x * blockDim.x) {
    if (i != i0) {
      s0 = a.off[i];
      s1 = a.off[i + 1];
    }
    const V4<R> x = XA[2 * i], xl = XA[2 * i + 1], g = GD[2 * i], pv = ldg4(P + i);
    const int mask = (int)x.w;
    const R p[3] = {pv.x, pv.y, pv.z};
    R xh[3] = {x.x, x.y, x.z}, xlo[3] = {xl.x, xl.y, xl.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) pair_add(xh[c], xlo[c], mul_rn(t, p[c]));
    const R xn[3] = {xh[0] + xlo[0], xh[1] + xlo[1], xh[2] + xlo[2]};
    R gs[3] = {R(0), R(0), R(0)}, ds[3] = {R(0), R(0), R(0)};
    for (int k = s0; k < s1; ++k) {
      const V4<R> sg = slots[2 * k], sd = slots[2 * k + 1];
      gs[0] += sg.x;
      gs[1] += sg.y;
      gs[2] += sg.z;
      ds[0] += sd.x;
      ds[1] += sd.y;
      ds[2] += sd.z;
    }
    if (F) {
      const V4<R> f = ldg4(F + i);
      gs[0] -= f.x;
      gs[1] -= f.y;
      gs[2] -= f.z;
      s[11] += -(f.x * xn[0] + f.y * xn[1] + f.z * xn[2]);
    }
    const R go[3] = {g.x, g.y, g.z};
    R gn[3], dn[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const bool fixed = (mask >> c) & 1;
      gn[c] = fixed ? R(0) : gs[c];
      dn[c] = fixed ? R(0) : ds[c];
      if (fixed) continue;
      const R y = gn[c] - go[c];
      const R ad = fabs(dn[c]);
      if (ad > R(0)) {
        const R P = rcp_rn(ad);
        s[0] += gn[c] * gn[c] * P;
        s[1] += gn[c] * y * P;
        s[2] += y * y * P;
        s[3] += ad;
        s[4] += R(1);
      } else {
        s[5] += gn[c] * gn[c];
        s[6] += gn[c] * y;
        s[7] += y * y;
      }
      s[8] += y * p[c];
      s[9] += p[c] * gn[c];
      s[10] += gn[c] * gn[c];
    }
    XA[2 * i] = V4<R>{xh[0], xh[1], xh[2], x.w};
    XA[2 * i + 1] = V4<R>{xlo[0], xlo[1], xlo[2], R(0)};
    GD[2 * i] = V4<R>{gn[0], gn[1], gn[2], R(0)};
    GD[2 * i + 1] = V4<R>{dn[0], dn[1], dn[2], R(0)};
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
  const double cnt = tot[4], sad = tot[3];
  const double inv_m = (cnt > 0.0 && sad > 0.0) ? cnt / sad : 1.0;
  const double gPg = tot[0] + inv_m * tot[5];
  const double gPy = tot[1] + inv_m * tot[6];
  const double yPy = tot[2] + inv_m * tot[7];
  const double yp = tot[8], pg = tot[9], gg = tot[10];
  const double gnorm = sqrt(gg);
  const bool first = st->init != 0;
  double b = 0.0;
  if (!first) {
    b = fabs(yp) > 1.0e-12 ? gPy / yp - (yPy / yp) * (pg / yp) : INFINITY;
    if (st->reset_beta || !isfinite(b) || fabs(b) > st->beta_max) b = 0.0;
  }
  double gd = -gPg + b * pg;
  if (!(isfinite(gd) && gd < 0.0)) {
    b = 0.0;
    gd = -gPg;
  }
  st->beta = b;
  st->inv_mean = inv_m;
  st->pbuf ^= 1;  // this iteration's p becomes p_prev
  st->gd = gd;
  st->gnorm = gnorm;
  st->ext_energy = tot[11];
  st->reset_beta = 0;
  if (first) {
    st->gnorm0 = gnorm;
    st->init = 0;
  } else {
    st->iter += 1;
  }
  int result = AGB_RUNNING;
  if (!isfinite(gnorm) || !isfinite(gPg) || !isfinite(tot[11]))
    result = AGB_NAN_ENCOUNTERED;
  else if (!first && st->ls_fail)
    result = AGB_LINE_SEARCH_FAILED;
  else if (gnorm <= fmax(st->atol, st->rtol * st->gnorm0))
    result = AGB_PRIMARY_SUCCESS;
  else if (st->iter >= st->max_steps)
    result = AGB_MAX_STEPS_REACHED;
  if (result != AGB_RUNNING) {
    st->done = 1;
    st->result = result;
  }
  if (use_cond)
    cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond,
                            (!st->done && st->iter < st->iter_limit) ? 1u : 0u);
}

// total energy at x: gradient-pass partials + external work (on demand)
template <class R>
__global__ void __launch_bounds__(256) solver_energy_kernel(SolveArgs a) {
  __shared__ Acc<R> red[8];
  const double e = block_sum_partials<R>((const AccStore<R>*)a.part_b, a.fv.n_tiles, 1, red);
  if (threadIdx.x == 0) a.st->energy = e + a.st->ext_energy;
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
  }
}

__global__ void solver_set_limit_kernel(SolverState* st, int n) { st->iter_limit = st->iter + n; }

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
  cudaError_t e = cudaFuncSetAttribute(solver_grad_kernel<R, AGB_ARAP>, m, g);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(solver_grad_kernel<R, AGB_STABLE_NEO_HOOKEAN>, m, g);
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
  if (a.precision == AGB_F64)
    solver_energy_kernel<double><<<1, 256, 0, s>>>(a);
  else
    solver_energy_kernel<float><<<1, 256, 0, s>>>(a);
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

template <class R, int MAT>
static cudaError_t launch_iteration_t(const SolveArgs& a, bool use_cond, bool first, int max_bt,
                                      cudaStream_t s) {
  const dim3 eg(a.fv.n_tiles), eb(kElemThreads);
  if (!first) {
    solver_dir_kernel<R, MAT><<<dir_blocks(a.fv.n_tiles), eb, 0, s>>>(a, use_cond ? 1 : 0);
    if constexpr (MAT == AGB_ARAP) {
      for (int j0 = 0; j0 <= max_bt; j0 += 3) solver_trial_kernel<R><<<eg, eb, 0, s>>>(a, j0);
    }
  }
  cudaError_t e = launch_pdl(solver_grad_kernel<R, MAT>, eg, dim3(kGradThreads), grad_smem_bytes<R>(), s, a);
  if (e != cudaSuccess) return e;
  return launch_pdl(solver_vertex_kernel<R>, dim3(a.vblocks), dim3(kVThreads), 0, s, a, use_cond ? 1 : 0);
}

static cudaError_t launch_iteration(const SolveArgs& a, bool use_cond, bool first, cudaStream_t s) {
  if (a.fv.n_tiles == 0) return cudaErrorInvalidValue;
  const int max_bt = a.max_bt;
  cudaError_t e;
  if (a.precision == AGB_F64) {
    if (a.fv.material == AGB_ARAP)
      e = launch_iteration_t<double, AGB_ARAP>(a, use_cond, first, max_bt, s);
    else
      e = launch_iteration_t<double, AGB_STABLE_NEO_HOOKEAN>(a, use_cond, first, max_bt, s);
  } else {
    if (a.fv.material == AGB_ARAP)
      e = launch_iteration_t<float, AGB_ARAP>(a, use_cond, first, max_bt, s);
    else
      e = launch_iteration_t<float, AGB_STABLE_NEO_HOOKEAN>(a, use_cond, first, max_bt, s);
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

template <class R, int MAT>
static cudaError_t launch_pass_t(const SolveArgs& a, int which, cudaStream_t s) {
  const dim3 eg(a.fv.n_tiles), eb(kElemThreads);
  if (which == 0) solver_dir_kernel<R, MAT><<<dir_blocks(a.fv.n_tiles), eb, 0, s>>>(a, 0);
  if (which == 1) solver_grad_kernel<R, MAT><<<eg, kGradThreads, grad_smem_bytes<R>(), s>>>(a);
  if (which == 2) solver_vertex_kernel<R><<<a.vblocks, kVThreads, 0, s>>>(a, 0);
  return cudaGetLastError();
}

cudaError_t launch_solver_pass(const SolveArgs& a, int which, cudaStream_t s) {
  if (a.precision == AGB_F64) {
    if (a.fv.material == AGB_ARAP) return launch_pass_t<double, AGB_ARAP>(a, which, s);
    return launch_pass_t<double, AGB_STABLE_NEO_HOOKEAN>(a, which, s);
  }
  if (a.fv.material == AGB_ARAP) return launch_pass_t<float, AGB_ARAP>(a, which, s);
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

}  // namespace agb
