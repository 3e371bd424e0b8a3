// Device helpers shared by the single-mesh solver (solver.cu) and the
// batched solver (batch.cu): launch constants, dependent-launch controls,
// vertex staging of the element passes and the scalar decisions of the
// passes' last blocks.
#pragma once

#include <math.h>

#include "solver.h"
#include "tile.cuh"

namespace agb {

constexpr int kSMs = 152;
constexpr int kVThreads = 256;
constexpr int kWarps = kElemThreads / 32;
// gradient pass: 4 warps per tile, one private accumulator copy per warp
constexpr int kGradThreads = 128;
constexpr int kGradWarps = kGradThreads / 32;

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// the passes of a guarded iteration (SolveArgs::guard) skip it when the one
// before it ended the solve's run: limit reached or refresh due
__device__ __forceinline__ bool guard_skip(const SolveArgs& a, const SolverState* st) {
  return a.guard && (st->iter >= st->iter_limit || st->refresh);
}

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

// ARAP: the per-element SVD cache svd[b] (SolveArgs::svd)
template <class R>
__device__ __forceinline__ V4<R>* svd_cache(const SolveArgs& a, int b) {
  return (V4<R>*)a.svd + (size_t)b * 3 * (size_t)a.fv.n_cells;
}
template <class R>
__device__ __forceinline__ void svd_put(V4<R>* c, size_t n, int e, const Svd<R>& d) {
  R q[4];
  quat_of_rotation(d.U, q);
  c[e] = V4<R>{q[0], q[1], q[2], q[3]};
  quat_of_rotation(d.V, q);
  c[n + e] = V4<R>{q[0], q[1], q[2], q[3]};
  c[2 * n + e] = V4<R>{d.sm1[0], d.sm1[1], d.sm1[2], R(0)};
}
template <class R>
struct SvdPacked {
  V4<R> u, v, m;
};
template <class R>
__device__ __forceinline__ SvdPacked<R> svd_load(const V4<R>* c, size_t n, int e) {
  return SvdPacked<R>{ldg4(c + e), ldg4(c + n + e), ldg4(c + 2 * n + e)};
}
template <class R>
__device__ __forceinline__ void svd_unpack(const SvdPacked<R>& p, Svd<R>& d) {
  const V4<R>&u = p.u, &v = p.v, &m = p.m;
  const R qu[4] = {u.x, u.y, u.z, u.w}, qv[4] = {v.x, v.y, v.z, v.w};
  rotation_of_quat(qu, d.U);
  rotation_of_quat(qv, d.V);
  d.sm1[0] = m.x;
  d.sm1[1] = m.y;
  d.sm1[2] = m.z;
#pragma unroll
  for (int k = 0; k < 3; ++k) d.s[k] = R(1) + d.sm1[k];
}
template <class R>
__device__ __forceinline__ void svd_get(const V4<R>* c, size_t n, int e, Svd<R>& d) {
  svd_unpack(svd_load(c, n, e), d);
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

// the same, staged as 24 bytes per vertex: (x, p.x) and (p.y, p.z), so that
// a corner of both fields is one 16-byte and one 8-byte shared-memory load
template <class R>
__device__ __forceinline__ void stage_dir_packed(const SolveArgs& a, int v, R beta, R inv_mean,
                                                 const V4<R>* pprev, V4<R>* pcur, V4<R>* sxp, V2<R>* sq) {
  if (v < 0) return;
  const V4<R> x = ldg4((const V4<R>*)a.xa + 2 * v), g = ldg4((const V4<R>*)a.gd + 2 * v),
              d = ldg4((const V4<R>*)a.gd + 2 * v + 1), po = ldg4(pprev + v);
  R p[3];
  pdir(g, d, po, beta, inv_mean, p);
  pcur[v] = V4<R>{p[0], p[1], p[2], R(0)};
  sxp[threadIdx.x] = V4<R>{x.x, x.y, x.z, p[0]};
  sq[threadIdx.x] = V2<R>{p[1], p[2]};
}

// G = sum_a (x_a - x_0) D_a^T and dF = sum_a (p_a - p_0) D_a^T from the
// packed staging (the same arithmetic as vec_gradient on each field)
template <class R>
__device__ __forceinline__ void dir_gradients(const V4<R>* sxp, const V2<R>* sq, const int (&l)[4],
                                              const R (&D)[3][3], R (&G)[3][3], R (&dF)[3][3]) {
  const V4<R> w0 = sxp[l[0]], w1 = sxp[l[1]], w2 = sxp[l[2]], w3 = sxp[l[3]];
  const V2<R> q0 = sq[l[0]], q1 = sq[l[1]], q2 = sq[l[2]], q3 = sq[l[3]];
  const R e[3][3] = {{w1.x - w0.x, w2.x - w0.x, w3.x - w0.x},
                     {w1.y - w0.y, w2.y - w0.y, w3.y - w0.y},
                     {w1.z - w0.z, w2.z - w0.z, w3.z - w0.z}};
  const R f[3][3] = {{w1.w - w0.w, w2.w - w0.w, w3.w - w0.w},
                     {q1.x - q0.x, q2.x - q0.x, q3.x - q0.x},
                     {q1.y - q0.y, q2.y - q0.y, q3.y - q0.y}};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      G[i][j] = e[i][0] * D[0][j] + e[i][1] * D[1][j] + e[i][2] * D[2][j];
      dF[i][j] = f[i][0] * D[0][j] + f[i][1] * D[1][j] + f[i][2] * D[2][j];
    }
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

template <class R>
__host__ __device__ constexpr size_t grad_smem_bytes() {
  // staged hi (V4: x y z lo.x) and lo (V2: lo.y lo.z) + per-warp accumulators (V4 + V2)
  return (size_t)kTileVerts * (size_t)(kGradWarps + 1) * (sizeof(V4<R>) + sizeof(V2<R>));
}
// the speculative ARAP gradient pass also stages p
template <class R>
__host__ __device__ constexpr size_t grad_spec_smem_bytes() {
  return grad_smem_bytes<R>() + (size_t)kTileVerts * sizeof(V4<R>);
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

// x as hi + lo pairs (as stage_point with t = 0) and p, for the speculative
// ARAP gradient pass
template <class R>
__device__ __forceinline__ void stage_point_dir(const SolveArgs& a, const int (&vid)[kGradVerts], const V4<R>* P,
                                                V4<R>* sh, V2<R>* sl, V4<R>* sp) {
  const V4<R>* XA = (const V4<R>*)a.xa;
#pragma unroll
  for (int j = 0; j < kGradVerts; ++j) {
    const int v = vid[j], i = threadIdx.x + j * kGradThreads;
    if (v < 0) continue;
    const V4<R> x = ldg4(XA + 2 * v), xl = ldg4(XA + 2 * v + 1), p = ldg4(P + v);
    sh[i] = V4<R>{x.x, x.y, x.z, xl.x};
    sl[i] = V2<R>{xl.y, xl.z};
    sp[i] = V4<R>{p.x, p.y, p.z, R(0)};
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


// Last block of the direction pass (thread 0): alpha_0 from p^T H p and, for
// stable Neo-Hookean, the reference's Armijo backtracking on the closed-form
// energy change dE(t) = t g.p + sum_m C_m t^m; tot = {p^T H p, C_2..C_6}.
template <int MAT>
__device__ __forceinline__ void dir_decide(SolverState* st, const double* tot) {
  const double hq = tot[0];
  st->hq = hq;
  const double gd = st->gd;
  const double a0 = initial_alpha(gd, hq, st->overstep);
  st->alpha0 = a0;
  if constexpr (snh_family(MAT)) {
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
    // ARAP: the speculative gradient pass evaluates alpha_0
    st->t = 0.0;
    st->decided = 0;
    st->spec_ok = 0;
  }
}

// Last block of the speculative ARAP gradient pass (thread 0): the Armijo
// test of the first trial step t = alpha_0 on dE = t g.p + sum of the
// elements' remainders.  Accepted: the pass's gradient is the iteration's.
// Rejected: the trial passes go on from alpha_0 / 2, as the reference's
// backtracking does, and a fallback gradient pass evaluates the step they
// decide.
__device__ __forceinline__ void spec_decide(SolverState* st, double rem) {
  const double t = st->alpha0, gd = st->gd;
  const double de = gd * t + rem;
  if (isfinite(de) && de <= st->armijo_c * t * gd) {
    st->t = t;
    st->delta_e = de;
    st->ls_ok = 1;
    st->ls_steps = 0;
    st->decided = 1;
    st->spec_ok = 1;
  } else if (st->max_bt <= 0) {
    reject_step(st, 0);
    st->decided = 1;
  }
}

// ARAP trial pass over one tile (kElemThreads threads): each element's
// remainder at the trial steps alpha_0 2^-j, j = j0 .. j0+nt-1 (nt <= 3),
// into sums[j]; each trial SVD is warm-started from the cached one at x
template <class R>
__device__ __forceinline__ void trial_tile(const SolveArgs& a, int tile, const SolverState* st, int j0, int nt,
                                           Acc<R> (&sums)[3]) {
  __shared__ R sh[3][kTileVerts];
  __shared__ R sl[3][kTileVerts];
  __shared__ R sp[3][kTileVerts];
  const double a0 = st->alpha0;
  R tj[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) tj[j] = (R)ldexp(a0, -(j0 + j));
  const int vs = a.fv.tile_vstart[tile], nv = a.fv.tile_vstart[tile + 1] - vs;
  const int es = a.fv.tile_estart[tile], ee = a.fv.tile_estart[tile + 1];
  stage_direction<R>(a, vs, nv, p_cur<R>(a, st->pbuf), sh, sl, sp);
  const V4<R>* cbase = svd_cache<R>(a, st->sbuf);
  __syncthreads();
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
    svd_get(cbase, (size_t)a.fv.n_cells, e, base);
#pragma unroll 1
    for (int j = 0; j < nt; ++j) {
      R Gt[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) Gt[i][k] = fma_rn(tj[j], dF[i][k], G[i][k]);
      Svd<R> trial;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) trial.V[i][k] = base.V[i][k];
      svd_rv<R, true>(Gt, (Gt[0][0] + Gt[1][1] + Gt[2][2]) + inv2(Gt) + det3(Gt), trial);
      sums[j].add(arap_remainder(base, trial, tj[j], dF, geo.mu));
    }
  }
}

// thread 0 after the trial sums tot[j] of steps alpha_0 2^-(j0 + j): the
// reference's Armijo test, in order; after the last halving a rejection
__device__ __forceinline__ void trial_decide(SolverState* st, double a0, int j0, int nt, const double* tot) {
  const double gd = st->gd;
  for (int j = 0; j < nt; ++j) {
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
  if (j0 + nt - 1 >= st->max_bt) {
    reject_step(st, st->max_bt);
    st->decided = 1;
  }
}

// Last block of the vertex pass (thread 0): Dai-Kou beta, preconditioner
// mean, descent check and termination from the 12 sums
// 0 gPg 1 gPy 2 yPy 3 sum|d| 4 count 5 zgg 6 zgy 7 zyy 8 y.p 9 p.g 10 g.g 11 ext energy
__device__ __forceinline__ void vertex_decide(SolverState* st, const double* tot) {
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
  } else if (st->ref_ratio > 0.0) {
    if (first)
      st->gnorm_ref = gnorm;
    else if (gnorm <= st->ref_ratio * st->gnorm_ref) {
      st->refresh = 1;
      st->gnorm_ref = gnorm;
    }
  }
}

// One vertex of the vertex pass: x <- x + t p (float-float), g and d from the
// vertex's slots s0..s1 (fixed order), external force, DOF mask; the 12 sums
// of vertex_decide accumulate into s.  vertex_load issues the vertex's
// independent loads, vertex_finish reads its slots and does the rest.
// (Loading vertex i+1 before finishing vertex i was measured slower: the
// kernel then runs at its 128-register cap with spills.)
template <class R>
struct VertexIn {
  V4<R> x, xl, g, p, r, f;
  int s0, s1;
};

template <class R, bool DELTA>
__device__ __forceinline__ void vertex_load(const SolveArgs& a, int i, int s0, int s1, const V4<R>* P,
                                            VertexIn<R>& in) {
  const V4<R>* XA = (const V4<R>*)a.xa;
  const V4<R>* GD = (const V4<R>*)a.gd;
  const V4<R>* F = (const V4<R>*)a.force;
  in.x = XA[2 * i];
  in.xl = XA[2 * i + 1];
  in.g = GD[2 * i];
  in.p = ldg4(P + i);
  if constexpr (DELTA) in.r = ldg4((const V4<R>*)a.gref + i);
  if (F) in.f = ldg4(F + i);
  in.s0 = s0;
  in.s1 = s1;
}

// the rest of a vertex once its slots are summed (gs, ds in slot order)
template <class R, bool DELTA>
__device__ __forceinline__ void vertex_apply(const SolveArgs& a, int i, const VertexIn<R>& in, R t,
                                             R (&gs)[3], const R (&ds)[3], R (&s)[12]) {
  V4<R>* XA = (V4<R>*)a.xa;
  V4<R>* GD = (V4<R>*)a.gd;
  const bool ext = a.force != nullptr;
  const int mask = (int)in.x.w;
  const R p[3] = {in.p.x, in.p.y, in.p.z};
  R xh[3] = {in.x.x, in.x.y, in.x.z}, xlo[3] = {in.xl.x, in.xl.y, in.xl.z};
#pragma unroll
  for (int c = 0; c < 3; ++c) pair_add(xh[c], xlo[c], mul_rn(t, p[c]));
  const R xn[3] = {xh[0] + xlo[0], xh[1] + xlo[1], xh[2] + xlo[2]};
  if constexpr (DELTA) {
    // g = g(x_ref) + sum_e (f_e(x) - f_e(x_ref)); the force is folded into g(x_ref)
    gs[0] += in.r.x;
    gs[1] += in.r.y;
    gs[2] += in.r.z;
    if (ext) s[11] += -(in.f.x * xn[0] + in.f.y * xn[1] + in.f.z * xn[2]);
  } else if (ext) {
    gs[0] -= in.f.x;
    gs[1] -= in.f.y;
    gs[2] -= in.f.z;
    s[11] += -(in.f.x * xn[0] + in.f.y * xn[1] + in.f.z * xn[2]);
  }
  const R go[3] = {in.g.x, in.g.y, in.g.z};
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
  XA[2 * i] = V4<R>{xh[0], xh[1], xh[2], in.x.w};
  XA[2 * i + 1] = V4<R>{xlo[0], xlo[1], xlo[2], R(0)};
  GD[2 * i] = V4<R>{gn[0], gn[1], gn[2], R(0)};
  GD[2 * i + 1] = V4<R>{dn[0], dn[1], dn[2], R(0)};
}

template <class R, bool DELTA>
__device__ __forceinline__ void vertex_finish(const SolveArgs& a, int i, const VertexIn<R>& in, R t,
                                              R (&s)[12]) {
  const V4<R>* slots = (const V4<R>*)a.slots;
  R gs[3] = {R(0), R(0), R(0)}, ds[3] = {R(0), R(0), R(0)};
  for (int k = in.s0; k < in.s1; ++k) {
    const V4<R> sg = slots[2 * k], sd = slots[2 * k + 1];
    gs[0] += sg.x;
    gs[1] += sg.y;
    gs[2] += sg.z;
    ds[0] += sd.x;
    ds[1] += sd.y;
    ds[2] += sd.z;
  }
  vertex_apply<R, DELTA>(a, i, in, t, gs, ds, s);
}

template <class R, bool DELTA>
__device__ __forceinline__ void vertex_update(const SolveArgs& a, int i, int s0, int s1, R t, const V4<R>* P,
                                              R (&s)[12]) {
  VertexIn<R> in;
  vertex_load<R, DELTA>(a, i, s0, s1, P, in);
  vertex_finish<R, DELTA>(a, i, in, t, s);
}

// Whether a solver instantiation uses the reference-state correction: FP32
// stable Neo-Hookean (FP64 has the precision; ARAP is not polynomial).
template <class R, int MAT>
constexpr bool kRefDelta = snh_family(MAT) && sizeof(R) == 4;

// x + t p relative to the reference: (x_ref, d.x) and (d.y, d.z) per vertex,
// d = (x_hi + t p - x_ref) + x_lo with the hi/lo pair updated by two-sum
template <class R>
__device__ __forceinline__ void stage_point_delta(const SolveArgs& a, const int (&vid)[kGradVerts], const V4<R>* P,
                                                  R t, V4<R>* sh, V2<R>* sl) {
  const V4<R>* XA = (const V4<R>*)a.xa;
  const V4<R>* XR = (const V4<R>*)a.xref;
#pragma unroll
  for (int j = 0; j < kGradVerts; ++j) {
    const int v = vid[j], i = threadIdx.x + j * kGradThreads;
    if (v < 0) continue;
    const V4<R> x = ldg4(XA + 2 * v), xl = ldg4(XA + 2 * v + 1), p = ldg4(P + v), r = ldg4(XR + v);
    R hx = x.x, lx = xl.x, hy = x.y, ly = xl.y, hz = x.z, lz = xl.z;
    pair_add(hx, lx, mul_rn(t, p.x));
    pair_add(hy, ly, mul_rn(t, p.y));
    pair_add(hz, lz, mul_rn(t, p.z));
    sh[i] = V4<R>{r.x, r.y, r.z, add_rn(sub_rn(hx, r.x), lx)};
    sl[i] = V2<R>{add_rn(sub_rn(hy, r.y), ly), add_rn(sub_rn(hz, r.z), lz)};
  }
}

// A = grad of x_ref, dG = grad of d from the delta staging
template <class R>
__device__ __forceinline__ void delta_gradient(const V4<R>* sh, const V2<R>* sl, const int (&l)[4],
                                               const R (&D)[3][3], R (&A)[3][3], R (&dG)[3][3]) {
  const V4<R> h0 = sh[l[0]];
  const V2<R> q0 = sl[l[0]];
  R ea[3][3], ed[3][3];
#pragma unroll
  for (int k = 1; k < 4; ++k) {
    const V4<R> h = sh[l[k]];
    const V2<R> q = sl[l[k]];
    ea[0][k - 1] = h.x - h0.x;
    ea[1][k - 1] = h.y - h0.y;
    ea[2][k - 1] = h.z - h0.z;
    ed[0][k - 1] = h.w - h0.w;
    ed[1][k - 1] = q.x - q0.x;
    ed[2][k - 1] = q.y - q0.y;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      A[i][j] = ea[i][0] * D[0][j] + ea[i][1] * D[1][j] + ea[i][2] * D[2][j];
      dG[i][j] = ed[i][0] * D[0][j] + ed[i][1] * D[1][j] + ed[i][2] * D[2][j];
    }
}

// The gradient pass over one tile (one CTA of kGradThreads threads, dynamic
// shared memory grad_smem_bytes<R>(), plus kTileVerts V4<R> with SPEC): stage
// x + t p, per warp group forces and clamped diagonal into the warp's private
// accumulator, then one slot per tile vertex.  (The energy is not needed by
// the iteration; energy_tile evaluates it on demand.)  st is the state of the
// tile's mesh; the first group's record, the vertex ids and the slot indices
// are read before the dependency wait.
//
// ARAP keeps each element's SVD at x in svd[sbuf] and writes the SVD at the
// evaluated point into svd[sbuf ^ 1].  SPEC (ARAP, speculative): the pass
// evaluates at x + alpha_0 p, with the SVD warm-started from the cached one
// at x, and adds each element's line-search remainder
// Psi(F + t dF) - Psi(F) - t P(F):dF into *rem, so that the Armijo test of
// the first trial step needs no pass of its own.  FALLBACK: a pass launched
// after the speculative one that returns at once unless that one's step was
// rejected.  Returns false when the pass returned without work.
template <class R, int MAT, bool DELTA = kRefDelta<R, MAT>, bool SPEC = false>
__device__ __forceinline__ bool grad_tile(const SolveArgs& a, int tile, const SolverState* st,
                                          Acc<R>* rem = nullptr, bool fallback = false) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V4<R>* sh = reinterpret_cast<V4<R>*>(smem_raw);
  V4<R>* acc4 = sh + kTileVerts;  // [warp][vertex]: gx gy gz dx
  V2<R>* sl = reinterpret_cast<V2<R>*>(acc4 + kGradWarps * kTileVerts);
  V2<R>* acc2 = sl + kTileVerts;  // [warp][vertex]: dy dz
  V4<R>* sp = reinterpret_cast<V4<R>*>(acc2 + kGradWarps * kTileVerts);  // SPEC: p
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gs = a.fv.tile_gstart[tile], ge = a.fv.tile_gstart[tile + 1];
  // constant inputs: the first group's element record
  int g = gs + warp;
  int n = 0, e0 = 0;
  ElemGeo<R> geo;
  uint32_t ids = 0;
  if (g < ge) {
    e0 = a.fv.group_estart[g];
    n = a.fv.group_estart[g + 1] - e0;
    if (lane < n) load_elem_m<R, MAT>(a.fv, e0 + lane, geo, ids);
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
  if (st->done || guard_skip(a, st)) return false;
  if (fallback && st->spec_ok) return false;
  // ARAP: base SVDs (x) and the SVDs written by this pass
  const size_t ncell = (size_t)a.fv.n_cells;
  const V4<R>* cbase = nullptr;
  V4<R>* cnext = nullptr;
  if constexpr (MAT == AGB_ARAP) {
    if (a.svd) {
      cbase = svd_cache<R>(a, st->sbuf);
      cnext = svd_cache<R>(a, st->sbuf ^ 1);
    }
  }
  // SPEC: the cached SVDs of the warp's current group (the next group's are
  // loaded with its records, one group ahead)
  SvdPacked<R> cs{};
  if constexpr (SPEC) {
    if (g < ge && lane < n) cs = svd_load(cbase, ncell, e0 + lane);
  }
  R t;
  if constexpr (SPEC) {
    t = (R)st->alpha0;
    stage_point_dir<R>(a, vid, p_cur<R>(a, st->pbuf), sh, sl, sp);
  } else {
    t = (R)st->t;
    if constexpr (DELTA)
      stage_point_delta<R>(a, vid, p_cur<R>(a, st->pbuf), t, sh, sl);
    else
      stage_point<R>(a, vid, p_cur<R>(a, st->pbuf), t, sh, sl);
  }
  for (int i = threadIdx.x; i < kGradWarps * kTileVerts; i += blockDim.x) {
    acc4[i] = V4<R>{R(0), R(0), R(0), R(0)};
    acc2[i] = V2<R>{R(0), R(0)};
  }
  __syncthreads();

  V4<R>* my4 = acc4 + warp * kTileVerts;
  V2<R>* my2 = acc2 + warp * kTileVerts;
  while (g < ge) {
    // prefetch the warp's next group while this one computes
    const int gn = g + kGradWarps;
    int nn = 0, e0n = 0;
    ElemGeo<R> geon;
    uint32_t idsn = 0;
    SvdPacked<R> csn{};
    if (gn < ge) {
      e0n = a.fv.group_estart[gn];
      nn = a.fv.group_estart[gn + 1] - e0n;
      if (lane < nn) {
        load_elem_m<R, MAT>(a.fv, e0n + lane, geon, idsn);
        if constexpr (SPEC) csn = svd_load(cbase, ncell, e0n + lane);
      }
    }
    const int l[4] = {corner(ids, 0), corner(ids, 1), corner(ids, 2), corner(ids, 3)};
    R f[4][3], hd[4][3];
    if (lane < n) {
      R G[3][3], P[3][3];
      if constexpr (SPEC) {
        // trial point x + t p: G + t dF, its SVD warm-started from the one at x
        R dF[3][3];
        pair_gradient(sh, sl, l, geo.D, G);
        vec_gradient(sp, l, geo.D, dF);
        Svd<R> base, sv;
        svd_unpack(cs, base);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            G[i][k] = fma_rn(t, dF[i][k], G[i][k]);
            sv.V[i][k] = base.V[i][k];
          }
        svd_rv<R, true>(G, (G[0][0] + G[1][1] + G[2][2]) + inv2(G) + det3(G), sv);
        rem->add(arap_remainder(base, sv, t, dF, geo.mu));
        svd_put(cnext, ncell, e0 + lane, sv);
        arap_pk1(sv, geo.mu, P);
        corner_vjp(P, geo.D, f);
        R lk[3];
        arap_lambdas(sv, lk);
        arap_hess_diag(sv, lk, geo.D, geo.mu, hd);
      } else if constexpr (DELTA) {
        // f_e(x) - f_e(x_ref) from P(A + dG) - P(A); energy and diagonal at A + dG
        R dG[3][3];
        delta_gradient(sh, sl, l, geo.D, G, dG);
        add_act<MAT>(geo, G);
        SnhPoint<R> s, s2;
        snh_prepare(G, s);
        snh_pk1_delta(s, dG, geo.mu, geo.lam, P, s2);
        corner_vjp(P, geo.D, f);
        snh_hess_diag(s2, geo.D, geo.mu, geo.lam, hd);
      } else if constexpr (snh_family(MAT)) {
        pair_gradient(sh, sl, l, geo.D, G);
        add_act<MAT>(geo, G);
        SnhPoint<R> s;
        snh_prepare(G, s);
        snh_pk1(s, geo.mu, geo.lam, P);
        corner_vjp(P, geo.D, f);
        snh_hess_diag(s, geo.D, geo.mu, geo.lam, hd);
      } else {
        pair_gradient(sh, sl, l, geo.D, G);
        const R jm1 = (G[0][0] + G[1][1] + G[2][2]) + inv2(G) + det3(G);
        Svd<R> sv;
        svd_rv(G, jm1, sv);
        if (cnext) svd_put(cnext, ncell, e0 + lane, sv);
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
    e0 = e0n;
    geo = geon;
    ids = idsn;
    if constexpr (SPEC) cs = csn;
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
  return true;
}

// ---------------------------------------------------------------------------
// refresh of the reference state: x_ref = x_hi, and g(x_ref) = sum_e f_e(x_ref)
// - f_ext with the FP32 element data in FP64 arithmetic, stored as a float
// pair.  The element pass runs one CTA per tile (kGradThreads threads, warp
// groups, per-warp FP64 accumulators) and writes each tile vertex's sum as
// three doubles into its 32-byte slot; the vertex pass adds the slots.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr size_t ref_smem_bytes() {
  return (size_t)kTileVerts * (size_t)(kGradWarps + 1) * sizeof(V4<double>);
}
// grid of the refresh element pass: at most 4 CTAs per SM (40 KB of shared
// memory each), striding over the tiles
inline int ref_blocks(int n_tiles) { return n_tiles < kSMs * 4 ? (n_tiles > 0 ? n_tiles : 1) : kSMs * 4; }

template <int MAT>
__device__ __forceinline__ void ref_tile(const SolveArgs& a, int tile) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V4<double>* sx = reinterpret_cast<V4<double>*>(smem_raw);
  V4<double>* acc = sx + kTileVerts;  // [warp][vertex]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int vs = a.fv.tile_vstart[tile], nv = a.fv.tile_vstart[tile + 1] - vs;
  const V4<float>* XA = (const V4<float>*)a.xa;
  V4<float>* XR = (V4<float>*)a.xref;
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    const int v = a.fv.tv_vid[vs + i];
    const V4<float> x = XA[2 * v];
    XR[v] = V4<float>{x.x, x.y, x.z, 0.f};  // tiles sharing v store equal values
    sx[i] = V4<double>{(double)x.x, (double)x.y, (double)x.z, 0.0};
  }
  for (int i = threadIdx.x; i < kGradWarps * kTileVerts; i += blockDim.x) acc[i] = V4<double>{0.0, 0.0, 0.0, 0.0};
  __syncthreads();
  V4<double>* my = acc + warp * kTileVerts;
  for (int g = a.fv.tile_gstart[tile] + warp; g < a.fv.tile_gstart[tile + 1]; g += kGradWarps) {
    const int e0 = a.fv.group_estart[g], n = a.fv.group_estart[g + 1] - e0;
    double f[4][3] = {};
    int l[4] = {0, 0, 0, 0};
    if (lane < n) {
      ElemGeo<float> gf;
      uint32_t ids;
      load_elem_m<float, MAT>(a.fv, e0 + lane, gf, ids);
      ElemGeo<double> geo;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) geo.D[i][j] = (double)gf.D[i][j];
      geo.mu = (double)gf.mu;
      geo.lam = (double)gf.lam;
#pragma unroll
      for (int k = 0; k < 6; ++k) geo.S[k] = (double)gf.S[k];
#pragma unroll
      for (int k = 0; k < 4; ++k) l[k] = corner(ids, k);
      double G[3][3], P[3][3];
      vec_gradient(sx, l, geo.D, G);
      add_act<MAT>(geo, G);
      SnhPoint<double> s;
      snh_prepare(G, s);
      snh_pk1(s, geo.mu, geo.lam, P);
      corner_vjp(P, geo.D, f);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      __syncwarp();
      if (lane < n) {
        V4<double> q = my[l[k]];
        q.x += f[k][0];
        q.y += f[k][1];
        q.z += f[k][2];
        my[l[k]] = q;
      }
    }
    __syncwarp();
  }
  __syncthreads();
  double* slots = (double*)a.slots;  // 4 doubles per 32-byte slot
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    V4<double> q = acc[i];
#pragma unroll
    for (int w = 1; w < kGradWarps; ++w) {
      const V4<double> r = acc[w * kTileVerts + i];
      q.x += r.x;
      q.y += r.y;
      q.z += r.z;
    }
    const size_t k = 4 * (size_t)a.slot_of_tv[vs + i];
    slots[k] = q.x;
    slots[k + 1] = q.y;
    slots[k + 2] = q.z;
  }
}

__device__ __forceinline__ void ref_vertex(const SolveArgs& a, int i) {
  const double* slots = (const double*)a.slots;
  double g[3] = {0.0, 0.0, 0.0};
  for (int k = a.off[i]; k < a.off[i + 1]; ++k) {
    g[0] += slots[4 * (size_t)k];
    g[1] += slots[4 * (size_t)k + 1];
    g[2] += slots[4 * (size_t)k + 2];
  }
  if (a.force) {
    const V4<float> f = ((const V4<float>*)a.force)[i];
    g[0] -= (double)f.x;
    g[1] -= (double)f.y;
    g[2] -= (double)f.z;
  }
  // one float suffices: g(x_ref) is itself a residual (at most 1/ref_ratio
  // times the current one), so its rounding is far below the current ||g||
  const V4<float> gr{(float)g[0], (float)g[1], (float)g[2], 0.f};
  ((V4<float>*)a.gref)[i] = gr;
  // the stored g of this iterate becomes the new reference's value too
  // (x_ref = x_hi differs from x by x_lo only), so the next y = g - g_prev
  // of the Dai-Kou beta does not see the change of reference
  const int mask = (int)((const V4<float>*)a.xa)[2 * i].w;
  ((V4<float>*)a.gd)[2 * i] = V4<float>{(mask & 1) ? 0.f : gr.x, (mask & 2) ? 0.f : gr.y, (mask & 4) ? 0.f : gr.z, 0.f};
}

// Energy at x (no line-search offset), one CTA of kElemThreads threads per
// tile: sum of Psi_e dV_e over the tile's elements into `out` (the reporting
// energy of the solver; FP32 element math, float-float block sum).
template <class R, int MAT>
__device__ __forceinline__ void energy_tile(const SolveArgs& a, int tile, AccStore<R>* out) {
  __shared__ V4<R> sh[kTileVerts];
  __shared__ V2<R> sl[kTileVerts];
  __shared__ Acc<R> red[kElemThreads / 32];
  const int vs = a.fv.tile_vstart[tile], nv = a.fv.tile_vstart[tile + 1] - vs;
  const V4<R>* XA = (const V4<R>*)a.xa;
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    const int v = a.fv.tv_vid[vs + i];
    const V4<R> x = XA[2 * v], xl = XA[2 * v + 1];
    sh[i] = V4<R>{x.x, x.y, x.z, xl.x};
    sl[i] = V2<R>{xl.y, xl.z};
  }
  __syncthreads();
  Acc<R> sums[1] = {};
  for (int e = a.fv.tile_estart[tile] + threadIdx.x; e < a.fv.tile_estart[tile + 1]; e += blockDim.x) {
    ElemGeo<R> geo;
    uint32_t ids;
    load_elem_m<R, MAT>(a.fv, e, geo, ids);
    const int l[4] = {corner(ids, 0), corner(ids, 1), corner(ids, 2), corner(ids, 3)};
    R G[3][3];
    pair_gradient(sh, sl, l, geo.D, G);
    add_act<MAT>(geo, G);
    if constexpr (snh_family(MAT)) {
      SnhPoint<R> s;
      snh_prepare(G, s);
      sums[0].add(snh_energy(s, geo.mu, geo.lam));
    } else {
      const R jm1 = (G[0][0] + G[1][1] + G[2][2]) + inv2(G) + det3(G);
      Svd<R> sv;
      svd_rv(G, jm1, sv);
      sums[0].add(arap_energy(sv, geo.mu));
    }
  }
  block_reduce<1, 0xffffffffu, R>(sums, red);
  if (threadIdx.x == 0) *out = acc_store(sums[0]);
}

}  // namespace agb
