// Device-side layout helpers shared by the element and vertex passes.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "agb_internal.h"
#include "elem_math.cuh"
#include "reduce.cuh"

namespace agb {

// One vertex of a (n_points, 3) field in device order, padded to 4 lanes so
// that a vertex is one aligned vector load.  For the solver's position array
// the w lane holds the fixed-component mask (bits 0..2) as a small integer.
template <class R>
struct alignas(4 * sizeof(R)) V4 {
  R x, y, z, w;
};

template <class R>
struct alignas(2 * sizeof(R)) V2 {
  R x, y;
};

template <class R>
__device__ __forceinline__ V4<R> ldg4(const V4<R>* p);
template <>
__device__ __forceinline__ V4<float> ldg4<float>(const V4<float>* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  return V4<float>{v.x, v.y, v.z, v.w};
}
template <>
__device__ __forceinline__ V4<double> ldg4<double>(const V4<double>* p) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p));
  const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
  return V4<double>{a.x, a.y, b.x, b.y};
}

// Element record.  FP32: three float4 streams per element,
//   A = (D00 D01 D02 D10), B = (D11 D12 D20 D21), C = (D22 mu' lambda' ids)
// (D = rows 1..3 of dhdX, mu' = mu dV, lambda' = lambda dV, ids = four 8-bit
// local corner ids).  FP64: 11 component-major double streams + ids.
template <class R>
__device__ __forceinline__ void load_elem(const FemView& fv, int e, ElemGeo<R>& g, uint32_t& ids);

template <>
__device__ __forceinline__ void load_elem<float>(const FemView& fv, int e, ElemGeo<float>& g,
                                                 uint32_t& ids) {
  const float4* rec = static_cast<const float4*>(fv.rec);
  const size_t n = (size_t)fv.n_cells;
  const float4 A = __ldg(rec + e);
  const float4 B = __ldg(rec + n + e);
  const float4 C = __ldg(rec + 2 * n + e);
  g.D[0][0] = A.x; g.D[0][1] = A.y; g.D[0][2] = A.z;
  g.D[1][0] = A.w; g.D[1][1] = B.x; g.D[1][2] = B.y;
  g.D[2][0] = B.z; g.D[2][1] = B.w; g.D[2][2] = C.x;
  g.mu = C.y;
  g.lam = C.z;
  ids = __float_as_uint(C.w);
}

template <>
__device__ __forceinline__ void load_elem<double>(const FemView& fv, int e, ElemGeo<double>& g,
                                                  uint32_t& ids) {
  const double* rec = static_cast<const double*>(fv.rec);
  const size_t n = (size_t)fv.n_cells;
#pragma unroll
  for (int k = 0; k < 9; ++k) g.D[k / 3][k % 3] = __ldg(rec + k * n + e);
  g.mu = __ldg(rec + 9 * n + e);
  g.lam = __ldg(rec + 10 * n + e);
  ids = __ldg(fv.ids + e);
}

// the stable Neo-Hookean family (plain and muscle) shares the element math
constexpr bool snh_family(int mat) { return mat != AGB_ARAP; }

// Muscle (warp/fem/_stable_neo_hookean_muscle.py:18-114): G_m = F A with
// A = I + sym(a).  The records hold D A, so grad(u) A = sum_a (u_a - u_0) (D A)_a
// comes out of the usual corner gradient, and G_m - I = S + grad(u) A with
// S = A - I from the activation stream.
template <class R>
__device__ __forceinline__ void load_act(const FemView& fv, int e, ElemGeo<R>& g);
template <>
__device__ __forceinline__ void load_act<float>(const FemView& fv, int e, ElemGeo<float>& g) {
  const float4* a = static_cast<const float4*>(fv.act);
  const float4 s0 = __ldg(a + e), s1 = __ldg(a + (size_t)fv.n_cells + e);
  g.S[0] = s0.x;
  g.S[1] = s0.y;
  g.S[2] = s0.z;
  g.S[3] = s0.w;
  g.S[4] = s1.x;
  g.S[5] = s1.y;
}
template <>
__device__ __forceinline__ void load_act<double>(const FemView& fv, int e, ElemGeo<double>& g) {
  const double* a = static_cast<const double*>(fv.act);
#pragma unroll
  for (int k = 0; k < 6; ++k) g.S[k] = __ldg(a + (size_t)k * fv.n_cells + e);
}

template <class R, int MAT>
__device__ __forceinline__ void load_elem_m(const FemView& fv, int e, ElemGeo<R>& g, uint32_t& ids) {
  load_elem<R>(fv, e, g, ids);
  if constexpr (MAT == AGB_STABLE_NEO_HOOKEAN_MUSCLE) load_act<R>(fv, e, g);
}

// G += S for the muscle (no-op otherwise)
template <int MAT, class R>
__device__ __forceinline__ void add_act(const ElemGeo<R>& g, R (&G)[3][3]) {
  if constexpr (MAT == AGB_STABLE_NEO_HOOKEAN_MUSCLE) {
    G[0][0] += g.S[0];
    G[1][1] += g.S[1];
    G[2][2] += g.S[2];
    G[0][1] += g.S[3];
    G[1][0] += g.S[3];
    G[0][2] += g.S[4];
    G[2][0] += g.S[4];
    G[1][2] += g.S[5];
    G[2][1] += g.S[5];
  }
}

// correctly rounded primitives, so that every kernel that forms the PNCG
// direction or the trial point computes bit-identical values
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rcp_rn(float a) { return __frcp_rn(a); }
__device__ __forceinline__ double rcp_rn(double a) { return __drcp_rn(a); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// Solver positions are kept as an unevaluated sum hi + lo.  With FP32
// positions alone, rounding x to 2^-24 |x| caps the reachable ||g||/||g_0||
// near 1e-5 on stiff meshes (the gradient at the best representable point);
// the pair carries about 48 bits.  x += b with Knuth's two-sum, renormalised.
template <class R>
__device__ __forceinline__ void pair_add(R& hi, R& lo, R b) {
  const R s = add_rn(hi, b);
  const R bb = sub_rn(s, hi);
  const R err = add_rn(sub_rn(hi, sub_rn(s, bb)), sub_rn(b, bb));
  const R l = add_rn(lo, err);
  const R h2 = add_rn(s, l);
  lo = sub_rn(l, sub_rn(h2, s));
  hi = h2;
}

// (hi_a + lo_a) - (hi_b + lo_b) rounded once to R
template <class R>
__device__ __forceinline__ R pair_diff(R ha, R la, R hb, R lb) {
  return add_rn(sub_rn(ha, hb), sub_rn(la, lb));
}

// Jacobi preconditioner entry: 1/|d|, or 1/mean(|d| > 0) where d == 0
// (benches/bench_pncg_branching_backends.py:407-410)
template <class R>
__device__ __forceinline__ R precond(R d, R inv_mean) {
  const R ad = fabs(d);
  return ad > R(0) ? rcp_rn(ad) : inv_mean;
}

// p = -P g + beta p_prev, one component
template <class R>
__device__ __forceinline__ R pcomp(R g, R d, R po, R beta, R inv_mean) {
  return fma_rn(beta, po, -mul_rn(precond(d, inv_mean), g));
}

template <class R>
__device__ __forceinline__ void pdir(const V4<R>& g, const V4<R>& d, const V4<R>& po, R beta,
                                     R inv_mean, R (&p)[3]) {
  p[0] = pcomp(g.x, d.x, po.x, beta, inv_mean);
  p[1] = pcomp(g.y, d.y, po.y, beta, inv_mean);
  p[2] = pcomp(g.z, d.z, po.z, beta, inv_mean);
}

__device__ __forceinline__ int corner(uint32_t ids, int a) { return (int)((ids >> (8 * a)) & 0xffu); }

}  // namespace agb
