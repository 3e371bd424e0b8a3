// Per-tetrahedron element math, templated on the arithmetic type R.
//
// Restates warp/fem/func/*.py, warp/fem/_arap.py and
// warp/fem/_stable_neo_hookean.py for one element with one quadrature point.
// Inputs are the displacement gradient G = F - I = sum_a (u_a - u_0) D_a^T
// (warp/fem/func/_deformation.py:15-19 with dhdX row 0 = -(rows 1..3)) and
// the per-element constants mu' = mu dV and lambda' = lambda dV (the energy,
// its gradient and Hessian are linear in mu and lambda, so dV is folded in
// once at set-up).  Working with G instead of F keeps FP32 relative accuracy
// at small strains: J - 1, F - cof F and Psi are expanded exactly so that
// their O(1) parts cancel symbolically, not in floating point.
#pragma once

#include <cuda_runtime.h>

namespace agb {

template <class R>
struct Mat3 {
  R m[3][3];
};

template <class R>
__device__ __forceinline__ R det3(const R (&A)[3][3]) {
  return A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
         A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
         A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
}

// cofactor matrix: column j is the cross product of the other two columns
// (g3 of warp/fem/func/_gradient.py:31-40 for A = F)
template <class R>
__device__ __forceinline__ void cof3(const R (&A)[3][3], R (&C)[3][3]) {
  C[0][0] = A[1][1] * A[2][2] - A[1][2] * A[2][1];
  C[0][1] = A[1][2] * A[2][0] - A[1][0] * A[2][2];
  C[0][2] = A[1][0] * A[2][1] - A[1][1] * A[2][0];
  C[1][0] = A[0][2] * A[2][1] - A[0][1] * A[2][2];
  C[1][1] = A[0][0] * A[2][2] - A[0][2] * A[2][0];
  C[1][2] = A[0][1] * A[2][0] - A[0][0] * A[2][1];
  C[2][0] = A[0][1] * A[1][2] - A[0][2] * A[1][1];
  C[2][1] = A[0][2] * A[1][0] - A[0][0] * A[1][2];
  C[2][2] = A[0][0] * A[1][1] - A[0][1] * A[1][0];
}

template <class R>
__device__ __forceinline__ R ddot3(const R (&A)[3][3], const R (&B)[3][3]) {
  R s = R(0);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) s += A[i][j] * B[i][j];
  return s;
}

// second principal invariant i2(G) = ((tr G)^2 - tr(G^2)) / 2 = tr cof(G)
template <class R>
__device__ __forceinline__ R inv2(const R (&G)[3][3]) {
  return G[0][0] * G[1][1] + G[1][1] * G[2][2] + G[2][2] * G[0][0] - G[0][1] * G[1][0] -
         G[1][2] * G[2][1] - G[2][0] * G[0][2];
}

// Element geometry: D[a][j] = dhdX[a+1][j], a = 0..2; corner 0 is implied.
template <class R>
struct ElemGeo {
  R D[3][3];
  R mu;   // mu * dV
  R lam;  // lambda * dV
  R S[6];  // muscle: A - I = sym(a) as (S00 S11 S22 S01 S02 S12); D holds D A
};

// Gradient of a corner field w (4 corners x 3): W = sum_a (w_a - w_0) D_a^T
template <class R>
__device__ __forceinline__ void corner_gradient(const R (&w)[4][3], const R (&D)[3][3],
                                                R (&W)[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const R e1 = w[1][i] - w[0][i], e2 = w[2][i] - w[0][i], e3 = w[3][i] - w[0][i];
#pragma unroll
    for (int j = 0; j < 3; ++j) W[i][j] = e1 * D[0][j] + e2 * D[1][j] + e3 * D[2][j];
  }
}

// vjp: corner forces f_a = M D_a^T (a = 1..3), f_0 = -(f_1 + f_2 + f_3)
// (warp/fem/func/_deformation.py:28-31)
template <class R>
__device__ __forceinline__ void corner_vjp(const R (&M)[3][3], const R (&D)[3][3],
                                           R (&f)[4][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    R s = R(0);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const R v = M[i][0] * D[a][0] + M[i][1] * D[a][1] + M[i][2] * D[a][2];
      f[a + 1][i] = v;
      s += v;
    }
    f[0][i] = -s;
  }
}

// rows of dhdX for all four corners
template <class R>
__device__ __forceinline__ void corner_rows(const R (&D)[3][3], R (&Da)[4][3]) {
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    Da[1][j] = D[0][j];
    Da[2][j] = D[1][j];
    Da[3][j] = D[2][j];
    Da[0][j] = -(D[0][j] + D[1][j] + D[2][j]);
  }
}

// ---------------------------------------------------------------------------
// stable Neo-Hookean  Psi = mu/2 (I2 - 3) - mu (J - 1) + lambda/2 (J - 1)^2
// (warp/fem/_stable_neo_hookean.py:17-103)
// ---------------------------------------------------------------------------
template <class R>
struct SnhPoint {
  R G[3][3];
  R cofF[3][3];  // cof(I + G) = g3(F)
  R jm1;         // J - 1
};

template <class R>
__device__ __forceinline__ void snh_prepare(const R (&G)[3][3], SnhPoint<R>& s) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) s.G[i][j] = G[i][j];
  const R tr = G[0][0] + G[1][1] + G[2][2];
  R cG[3][3];
  cof3(G, cG);
  // det(I+G) - 1 = tr G + i2(G) + det G ; cof(I+G) = (1 + tr G) I - G^T + cof G
  s.jm1 = tr + inv2(G) + det3(G);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) s.cofF[i][j] = (i == j ? R(1) + tr : R(0)) - G[j][i] + cG[i][j];
}

template <class R>
__device__ __forceinline__ R snh_energy(const SnhPoint<R>& s, R mu, R lam) {
  // mu/2 ||G||^2 - mu (i2 + det G) + lambda/2 (J-1)^2: the linear terms of
  // mu/2 (I2 - 3) and mu (J - 1) cancel exactly
  const R gg = ddot3(s.G, s.G);
  const R q = inv2(s.G) + det3(s.G);
  return R(0.5) * mu * gg - mu * q + R(0.5) * lam * s.jm1 * s.jm1;
}

template <class R>
__device__ __forceinline__ void snh_pk1(const SnhPoint<R>& s, R mu, R lam, R (&P)[3][3]) {
  // P = mu (F - cof F) + lambda (J-1) cof F,  F - cof F = G + G^T - tr(G) I - cof(G)
  R cG[3][3];
  cof3(s.G, cG);
  const R tr = s.G[0][0] + s.G[1][1] + s.G[2][2];
  const R lj = lam * s.jm1;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const R fc = s.G[i][j] + s.G[j][i] - (i == j ? tr : R(0)) - cG[i][j];
      P[i][j] = mu * fc + lj * s.cofF[i][j];
    }
}

// diag(H_e) per corner/component: lambda (D_a . cofF_i)^2 + mu ||D_a||^2
// (h3_diag, h5_diag; h6_diag == 0: func/_hess_diag.py:29-72)
template <class R>
__device__ __forceinline__ void snh_hess_diag(const SnhPoint<R>& s, const R (&D)[3][3], R mu,
                                              R lam, R (&hd)[4][3]) {
  R Da[4][3];
  corner_rows(D, Da);
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const R nn = Da[a][0] * Da[a][0] + Da[a][1] * Da[a][1] + Da[a][2] * Da[a][2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const R w = s.cofF[i][0] * Da[a][0] + s.cofF[i][1] * Da[a][1] + s.cofF[i][2] * Da[a][2];
      hd[a][i] = lam * w * w + mu * nn;
    }
  }
}

// directional terms along dF
template <class R>
struct SnhDir {
  R a1;   // cof F : dF            (first derivative of J along dF)
  R a2;   // F : cof dF            (half the second derivative)
  R a3;   // det dF
  R ff;   // ||dF||^2
};

template <class R>
__device__ __forceinline__ void snh_dir(const SnhPoint<R>& s, const R (&dF)[3][3], SnhDir<R>& d) {
  R cdF[3][3];
  cof3(dF, cdF);
  d.a1 = ddot3(s.cofF, dF);
  d.a2 = (cdF[0][0] + cdF[1][1] + cdF[2][2]) + ddot3(s.G, cdF);
  d.a3 = det3(dF);
  d.ff = ddot3(dF, dF);
}

// p^T H_e p (h3_quad, h5_quad, h6_quad = 2 F : cof dF; func/_hess_quad.py)
template <class R>
__device__ __forceinline__ R snh_hess_quad(const SnhPoint<R>& s, const SnhDir<R>& d, R mu, R lam) {
  return lam * d.a1 * d.a1 + mu * d.ff + R(2) * (-mu + lam * s.jm1) * d.a2;
}

// Psi(F + t dF) - Psi(F) = sum_{m=1..6} c_m t^m ; returns c2..c6
// (det(F + t dF) = J + a1 t + a2 t^2 + a3 t^3)
template <class R>
__device__ __forceinline__ void snh_poly(const SnhPoint<R>& s, const SnhDir<R>& d, R mu, R lam,
                                         R (&c)[5]) {
  const R j = s.jm1;
  c[0] = R(0.5) * mu * d.ff - mu * d.a2 + lam * (j * d.a2 + R(0.5) * d.a1 * d.a1);
  c[1] = -mu * d.a3 + lam * (j * d.a3 + d.a1 * d.a2);
  c[2] = R(0.5) * lam * (d.a2 * d.a2 + R(2) * d.a1 * d.a3);
  c[3] = lam * d.a2 * d.a3;
  c[4] = R(0.5) * lam * d.a3 * d.a3;
}

// Mixed cofactor: cof(X + D) = cof(X) + mixed_cof(X, D) + cof(D); column c is
// x_{c+1} x d_{c+2} + d_{c+1} x x_{c+2} (columns of X and D, indices mod 3).
template <class R>
__device__ __forceinline__ void mixed_cof(const R (&X)[3][3], const R (&D)[3][3], R (&B)[3][3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
      B[i][c] = X[i1][c1] * D[i2][c2] - X[i2][c1] * D[i1][c2] + D[i1][c1] * X[i2][c2] - D[i2][c1] * X[i1][c2];
    }
  }
}

// P(A + D) - P(A) for stable Neo-Hookean, expanded exactly so that no O(1)
// term cancels: with F = I + A,
//   cof(A+D) - cof(A) = B(A,D) + cof(D),   cof(F+D) - cof(F) = tr(D) I - D^T + B(A,D) + cof(D),
//   J(F+D) - J(F) = cof F : D + F : cof D + det D,
//   dP = mu (D + D^T - tr(D) I - dcof(A)) + lambda ((J-1) dcof(F) + dJ cof(F+D)).
// Every term is a product with D, so FP32 keeps relative accuracy in dP.
// `s` is the state at A; `s2` receives the state at A + D (G, cof F, J - 1;
// rounded, for the diagonal and the energy).
template <class R>
__device__ __forceinline__ void snh_pk1_delta(const SnhPoint<R>& s, const R (&D)[3][3], R mu, R lam,
                                              R (&dP)[3][3], SnhPoint<R>& s2) {
  R cD[3][3], dcA[3][3];
  cof3(D, cD);
  mixed_cof(s.G, D, dcA);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) dcA[i][j] += cD[i][j];
  const R trD = D[0][0] + D[1][1] + D[2][2];
  const R a1 = ddot3(s.cofF, D);
  const R a2 = (cD[0][0] + cD[1][1] + cD[2][2]) + ddot3(s.G, cD);
  const R dJ = a1 + a2 + det3(D);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const R dcF = (i == j ? trD : R(0)) - D[j][i] + dcA[i][j];
      const R cF2 = s.cofF[i][j] + dcF;
      const R dfc = D[i][j] + D[j][i] - (i == j ? trD : R(0)) - dcA[i][j];
      dP[i][j] = mu * dfc + lam * (s.jm1 * dcF + dJ * cF2);
      s2.G[i][j] = s.G[i][j] + D[i][j];
      s2.cofF[i][j] = cF2;
    }
  s2.jm1 = s.jm1 + dJ;
}

// H_e p as a 3x3 M with corner forces M D_a^T (h3_prod, h5_prod, h6_prod)
template <class R>
__device__ __forceinline__ void snh_hess_prod(const SnhPoint<R>& s, const SnhDir<R>& d,
                                              const R (&dF)[3][3], R mu, R lam, R (&M)[3][3]) {
  // h6 matrix: derivative of cof(F) along dF, column-wise cross products
  // c0 = f1 x p2 + p1 x f2, c1 = f2 x p0 + p2 x f0, c2 = f0 x p1 + p0 x f1
  R F[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) F[i][j] = s.G[i][j] + (i == j ? R(1) : R(0));
  R H6[3][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
    // f_{c1} x p_{c2} + p_{c1} x f_{c2}
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
      H6[i][c] = F[i1][c1] * dF[i2][c2] - F[i2][c1] * dF[i1][c2] + dF[i1][c1] * F[i2][c2] -
                 dF[i2][c1] * F[i1][c2];
    }
  }
  const R s6 = -mu + lam * s.jm1;
  const R s3 = lam * d.a1;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) M[i][j] = s3 * s.cofF[i][j] + mu * dF[i][j] + s6 * H6[i][j];
}

// ---------------------------------------------------------------------------
// ARAP  Psi = mu/2 ||F - R||^2  (warp/fem/_arap.py:17-76)
//
// Rotation-variant SVD F = U diag(sigma) V^T (det U = det V = +1, sigma_2
// carries the sign of det F) from a cyclic Jacobi eigen-decomposition of the
// symmetric E = F^T F - I = G + G^T + G^T G, after the structure of
// McAdams, Selle, Tamstorf, Teran, Sifakis, "Computing the singular value
// decomposition of 3x3 matrices with minimal branching and elementary
// floating point operations" (UW-Madison CS TR1690, 2011): Jacobi on the
// normal matrix, sort with sign-preserving column swaps, then U from F V.
// Working on E (not F^T F) keeps sigma - 1 = e / (sqrt(1 + e) + 1) accurate
// at small strain.
// ---------------------------------------------------------------------------
template <class R>
struct Svd {
  R U[3][3];   // columns u_i
  R V[3][3];   // columns v_i
  R s[3];      // sigma_i (rotation-variant)
  R sm1[3];    // sigma_i - 1
};

template <class R>
__device__ __forceinline__ R rsqrt_(R x);
template <>
__device__ __forceinline__ float rsqrt_<float>(float x) {
  return rsqrtf(x);
}
template <>
__device__ __forceinline__ double rsqrt_<double>(double x) {
  return rsqrt(x);
}

// Quotients whose last bits only steer the iteration: in FP32 the fast
// division (__fdividef, within 2 ulp) and x * rsqrt(x) for x >= 1.  A Jacobi
// rotation stays orthogonal whatever its angle (c = 1 / sqrt(1 + t^2),
// s = t c), so the angle's rounding changes how fast the sweeps converge,
// not the orthogonality of V.
template <class R>
__device__ __forceinline__ R quick_div(R a, R b) {
  return a / b;
}
template <>
__device__ __forceinline__ float quick_div<float>(float a, float b) {
  return __fdividef(a, b);
}
template <class R>
__device__ __forceinline__ R sqrt_ge1(R x) {  // x >= 1
  return sqrt(x);
}
template <>
__device__ __forceinline__ float sqrt_ge1<float>(float x) {
  return x * rsqrtf(x);
}
// sqrt for x >= 0 (the singular values sqrt(1 + e)): in FP32 x * rsqrt(x),
// within a few ulp, and 0 at 0
template <class R>
__device__ __forceinline__ R sqrt_ge0(R x) {
  return sqrt(x);
}
template <>
__device__ __forceinline__ float sqrt_ge0<float>(float x) {
  return x > 0.0f ? x * rsqrtf(x) : 0.0f;
}

template <class R>
__device__ __forceinline__ void jacobi_rotate(R (&A)[3][3], R (&V)[3][3], int p, int q) {
  const R apq = A[p][q];
  if (apq == R(0)) return;
  const R theta = quick_div(A[q][q] - A[p][p], R(2) * apq);
  const R at = fabs(theta);
  R t;
  if (at > R(1e15))
    t = quick_div(R(0.5), theta);
  else
    t = quick_div(theta >= R(0) ? R(1) : R(-1), at + sqrt_ge1(theta * theta + R(1)));
  const R c = rsqrt_(t * t + R(1));
  const R sn = t * c;
  A[p][p] -= t * apq;
  A[q][q] += t * apq;
  A[p][q] = A[q][p] = R(0);
  const int r = 3 - p - q;
  const R arp = A[r][p], arq = A[r][q];
  A[r][p] = A[p][r] = c * arp - sn * arq;
  A[r][q] = A[q][r] = sn * arp + c * arq;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const R vkp = V[k][p], vkq = V[k][q];
    V[k][p] = c * vkp - sn * vkq;
    V[k][q] = sn * vkp + c * vkq;
  }
}

template <class R>
__device__ __forceinline__ void swap_cols(R (&V)[3][3], R (&e)[3], int i, int j) {
  const R te = e[i];
  e[i] = e[j];
  e[j] = te;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const R t = V[k][i];
    V[k][i] = V[k][j];
    V[k][j] = -t;  // keep det V = +1
  }
}

template <class R>
__device__ __forceinline__ void normalize3(R (&v)[3], R fallback_axis_seed) {
  const R n2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  if (n2 > R(0)) {
    const R r = rsqrt_(n2);
    v[0] *= r;
    v[1] *= r;
    v[2] *= r;
  } else {
    v[0] = fallback_axis_seed;
    v[1] = R(0);
    v[2] = R(0);
  }
}

// With WARM, the Jacobi sweeps start from the rotation `out.V` holds on entry
// (det +1): E is taken into that frame first, A = V0^T E V0, and the
// rotations accumulate onto V0.  Near a point whose V0 is known (the ARAP
// line-search trials around the base point), A is nearly diagonal and the
// sweeps stop after one or two instead of four or five.
template <class R, bool WARM = false>
__device__ void svd_rv(const R (&G)[3][3], R jm1, Svd<R>& out) {
  R A[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      R gtg = G[0][i] * G[0][j] + G[1][i] * G[1][j] + G[2][i] * G[2][j];
      A[i][j] = A[j][i] = G[i][j] + G[j][i] + gtg;
    }
  R (&V)[3][3] = out.V;
  if constexpr (WARM) {
    R EV[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) EV[i][j] = A[i][0] * V[0][j] + A[i][1] * V[1][j] + A[i][2] * V[2][j];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = i; j < 3; ++j) A[i][j] = A[j][i] = V[0][i] * EV[0][j] + V[1][i] * EV[1][j] + V[2][i] * EV[2][j];
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) V[i][j] = (i == j) ? R(1) : R(0);
  }
  const R eps = sizeof(R) == 4 ? R(1e-7) : R(1e-15);
  for (int sweep = 0; sweep < 8; ++sweep) {
    const R off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
    const R dia = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
    if (off <= eps * eps * (dia + R(1e-30))) break;
    jacobi_rotate(A, V, 0, 1);
    jacobi_rotate(A, V, 0, 2);
    jacobi_rotate(A, V, 1, 2);
  }
  R e[3] = {A[0][0], A[1][1], A[2][2]};
  if (e[0] < e[1]) swap_cols(V, e, 0, 1);
  if (e[0] < e[2]) swap_cols(V, e, 0, 2);
  if (e[1] < e[2]) swap_cols(V, e, 1, 2);
  // F v_i = v_i + G v_i
  R b0[3], b1[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    b0[k] = V[k][0] + G[k][0] * V[0][0] + G[k][1] * V[1][0] + G[k][2] * V[2][0];
    b1[k] = V[k][1] + G[k][0] * V[0][1] + G[k][1] * V[1][1] + G[k][2] * V[2][1];
  }
  normalize3(b0, R(1));
  const R proj = b0[0] * b1[0] + b0[1] * b1[1] + b0[2] * b1[2];
#pragma unroll
  for (int k = 0; k < 3; ++k) b1[k] -= proj * b0[k];
  {
    const R n2 = b1[0] * b1[0] + b1[1] * b1[1] + b1[2] * b1[2];
    if (n2 > R(1e-30)) {
      const R r = rsqrt_(n2);
      b1[0] *= r;
      b1[1] *= r;
      b1[2] *= r;
    } else {  // rank <= 1: any unit vector orthogonal to b0
      R a[3] = {R(0), R(0), R(0)};
      const int k = (fabs(b0[0]) <= fabs(b0[1]) && fabs(b0[0]) <= fabs(b0[2]))
                        ? 0
                        : (fabs(b0[1]) <= fabs(b0[2]) ? 1 : 2);
      a[k] = R(1);
      b1[0] = b0[1] * a[2] - b0[2] * a[1];
      b1[1] = b0[2] * a[0] - b0[0] * a[2];
      b1[2] = b0[0] * a[1] - b0[1] * a[0];
      normalize3(b1, R(0));
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    out.U[k][0] = b0[k];
    out.U[k][1] = b1[k];
  }
  out.U[0][2] = b0[1] * b1[2] - b0[2] * b1[1];
  out.U[1][2] = b0[2] * b1[0] - b0[0] * b1[2];
  out.U[2][2] = b0[0] * b1[1] - b0[1] * b1[0];
  const bool inverted = (R(1) + jm1) < R(0);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const R ei = fmax(e[i], R(-1));
    const R si = sqrt_ge0(R(1) + ei);
    if (i == 2 && inverted) {
      out.s[i] = -si;
      out.sm1[i] = -si - R(1);
    } else {
      out.s[i] = si;
      out.sm1[i] = quick_div(ei, si + R(1));
    }
  }
}

template <class R>
__device__ __forceinline__ R arap_energy(const Svd<R>& d, R mu) {
  return R(0.5) * mu * (d.sm1[0] * d.sm1[0] + d.sm1[1] * d.sm1[1] + d.sm1[2] * d.sm1[2]);
}

// P = mu (F - R) = mu U diag(sigma - 1) V^T
template <class R>
__device__ __forceinline__ void arap_pk1(const Svd<R>& d, R mu, R (&P)[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      P[i][j] = mu * (d.U[i][0] * d.sm1[0] * d.V[j][0] + d.U[i][1] * d.sm1[1] * d.V[j][1] +
                      d.U[i][2] * d.sm1[2] * d.V[j][2]);
}

// lambda_k = 2 / max(s_i + s_j, 2) for pairs (0,1), (1,2), (2,0)
// (func/_misc.py:31-43, clamp on)
template <class R>
__device__ __forceinline__ void arap_lambdas(const Svd<R>& d, R (&l)[3]) {
  l[0] = quick_div(R(2), fmax(d.s[0] + d.s[1], R(2)));
  l[1] = quick_div(R(2), fmax(d.s[1] + d.s[2], R(2)));
  l[2] = quick_div(R(2), fmax(d.s[2] + d.s[0], R(2)));
}

// Q_k : M for the twist modes of func/_misc.py:56-70 via W = U^T M V:
// Q0:M = (W10 - W01)/sqrt2, Q1:M = (W12 - W21)/sqrt2, Q2:M = (W02 - W20)/sqrt2
template <class R>
__device__ __forceinline__ void arap_twist_coords(const Svd<R>& d, const R (&M)[3][3], R (&q)[3]) {
  R MV[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) MV[i][j] = M[i][0] * d.V[0][j] + M[i][1] * d.V[1][j] + M[i][2] * d.V[2][j];
  auto W = [&](int i, int j) { return d.U[0][i] * MV[0][j] + d.U[1][i] * MV[1][j] + d.U[2][i] * MV[2][j]; };
  const R r2 = R(0.70710678118654752440);
  q[0] = (W(1, 0) - W(0, 1)) * r2;
  q[1] = (W(1, 2) - W(2, 1)) * r2;
  q[2] = (W(0, 2) - W(2, 0)) * r2;
}

// twist mode k as a matrix
template <class R>
__device__ __forceinline__ R arap_Q(const Svd<R>& d, int k, int i, int j) {
  const R r2 = R(0.70710678118654752440);
  const int a = (k == 0) ? 1 : (k == 1 ? 1 : 0);
  const int b = (k == 0) ? 0 : (k == 1 ? 2 : 2);
  // Q_k = (u_a v_b^T - u_b v_a^T) / sqrt2 with (a,b) = (1,0), (1,2), (0,2)
  return (d.U[i][a] * d.V[j][b] - d.U[i][b] * d.V[j][a]) * r2;
}

// p^T H_e p = mu (||dF||^2 - sum_k lambda_k (Q_k:dF)^2)
template <class R>
__device__ __forceinline__ R arap_hess_quad(const Svd<R>& d, const R (&lk)[3],
                                            const R (&dF)[3][3], R mu) {
  R q[3];
  arap_twist_coords(d, dF, q);
  return mu * (ddot3(dF, dF) - (lk[0] * q[0] * q[0] + lk[1] * q[1] * q[1] + lk[2] * q[2] * q[2]));
}

// H_e p as M = mu (dF - sum_k lambda_k (Q_k:dF) Q_k), corner forces M D_a^T
template <class R>
__device__ __forceinline__ void arap_hess_prod(const Svd<R>& d, const R (&lk)[3],
                                               const R (&dF)[3][3], R mu, R (&M)[3][3]) {
  R q[3];
  arap_twist_coords(d, dF, q);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      M[i][j] = mu * (dF[i][j] - lk[0] * q[0] * arap_Q(d, 0, i, j) -
                      lk[1] * q[1] * arap_Q(d, 1, i, j) - lk[2] * q[2] * arap_Q(d, 2, i, j));
}

// diag: mu (||D_a||^2 - sum_k lambda_k ((Q_k D_a)_i)^2)  (h4_diag, h5_diag)
template <class R>
__device__ __forceinline__ void arap_hess_diag(const Svd<R>& d, const R (&lk)[3],
                                               const R (&D)[3][3], R mu, R (&hd)[4][3]) {
  R Da[4][3];
  corner_rows(D, Da);
  const R r2 = R(0.70710678118654752440);
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const R nn = Da[a][0] * Da[a][0] + Da[a][1] * Da[a][1] + Da[a][2] * Da[a][2];
    // b = V^T D_a
    R b[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) b[k] = d.V[0][k] * Da[a][0] + d.V[1][k] * Da[a][1] + d.V[2][k] * Da[a][2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const R w0 = (d.U[i][1] * b[0] - d.U[i][0] * b[1]) * r2;
      const R w1 = (d.U[i][1] * b[2] - d.U[i][2] * b[1]) * r2;
      const R w2 = (d.U[i][0] * b[2] - d.U[i][2] * b[0]) * r2;
      hd[a][i] = mu * (nn - (lk[0] * w0 * w0 + lk[1] * w1 * w1 + lk[2] * w2 * w2));
    }
  }
}

// Energy remainder Psi(F + t dF) - Psi(F) - t P:dF for ARAP, evaluated from
// first-order quantities only: with A = F - R = R (S - I) and
// dR = R_t - R,  remainder = mu/2 (||t dF - dR||^2 + (S - I) : (dR^T dR)),
// which uses sym(R^T dR) = -dR^T dR / 2 for orthogonal R, R_t.
template <class R>
__device__ __forceinline__ R arap_remainder(const Svd<R>& base, const Svd<R>& trial, R t,
                                            const R (&dF)[3][3], R mu) {
  R dR[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const R rt = trial.U[i][0] * trial.V[j][0] + trial.U[i][1] * trial.V[j][1] + trial.U[i][2] * trial.V[j][2];
      const R r0 = base.U[i][0] * base.V[j][0] + base.U[i][1] * base.V[j][1] + base.U[i][2] * base.V[j][2];
      dR[i][j] = rt - r0;
    }
  R a = R(0);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const R v = t * dF[i][j] - dR[i][j];
      a += v * v;
    }
  // (S - I) = V diag(sm1) V^T ; (S - I) : (dR^T dR) = sum_k sm1_k ||dR v_k||^2
  R b = R(0);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    R w[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) w[i] = dR[i][0] * base.V[0][k] + dR[i][1] * base.V[1][k] + dR[i][2] * base.V[2][k];
    b += base.sm1[k] * (w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  }
  return R(0.5) * mu * (a + b);
}

// ---------------------------------------------------------------------------
// Proper rotations as unit quaternions q = (w, x, y, z), for the compact
// per-element SVD that the ARAP solver keeps between passes.
// Rotation -> quaternion by Shepperd's method (J. Guidance and Control 1(3),
// 1978): 4w^2 = 1 + tr M, 4x^2 = 1 + M00 - M11 - M22, 4y^2 = 1 - M00 + M11 -
// M22, 4z^2 = 1 - M00 - M11 + M22 sum to 4, so the largest is at least 1;
// its component comes from one reciprocal square root and the other three
// from the sums and differences of the off-diagonal pairs
// (M21 - M12 = 4wx, M02 - M20 = 4wy, M10 - M01 = 4wz, M01 + M10 = 4xy,
// M02 + M20 = 4xz, M12 + M21 = 4yz).
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ void quat_of_rotation(const R (&M)[3][3], R (&q)[4]) {
  const R tw = R(1) + M[0][0] + M[1][1] + M[2][2];
  const R tx = R(1) + M[0][0] - M[1][1] - M[2][2];
  const R ty = R(1) - M[0][0] + M[1][1] - M[2][2];
  const R tz = R(1) - M[0][0] - M[1][1] + M[2][2];
  // 4wx, 4wy, 4wz, 4xy, 4xz, 4yz
  const R dx = M[2][1] - M[1][2], dy = M[0][2] - M[2][0], dz = M[1][0] - M[0][1];
  const R sxy = M[0][1] + M[1][0], sxz = M[0][2] + M[2][0], syz = M[1][2] + M[2][1];
  // the largest of 4w^2, 4x^2, 4y^2, 4z^2 (first of equals in w, x, y, z
  // order); each component is (its product with that one, times 4) / (4
  // sqrt(t)), selected without branches so that a warp does not diverge
  const bool cw = tw >= tx && tw >= ty && tw >= tz;
  const bool cx = !cw && tx >= ty && tx >= tz;
  const bool cy = !cw && !cx && ty >= tz;
  const R t = cw ? tw : (cx ? tx : (cy ? ty : tz));
  const R h = R(0.5) * rsqrt_(t);
  q[0] = h * (cw ? t : (cx ? dx : (cy ? dy : dz)));
  q[1] = h * (cw ? dx : (cx ? t : (cy ? sxy : sxz)));
  q[2] = h * (cw ? dy : (cx ? sxy : (cy ? t : syz)));
  q[3] = h * (cw ? dz : (cx ? sxz : (cy ? syz : t)));
}

// the rotation of q / |q| (a stored quaternion is unit only to rounding):
// M = I + s [[-(y2+z2), xy-wz, xz+wy], [xy+wz, -(x2+z2), yz-wx],
//            [xz-wy, yz+wx, -(x2+y2)]],  s = 2 / |q|^2
template <class R>
__device__ __forceinline__ void rotation_of_quat(const R (&q)[4], R (&M)[3][3]) {
  const R w = q[0], x = q[1], y = q[2], z = q[3];
  const R r = rsqrt_(w * w + x * x + y * y + z * z);
  const R s = R(2) * r * r;
  const R xx = s * x * x, yy = s * y * y, zz = s * z * z;
  const R xy = s * x * y, xz = s * x * z, yz = s * y * z;
  const R wx = s * w * x, wy = s * w * y, wz = s * w * z;
  M[0][0] = R(1) - (yy + zz);
  M[0][1] = xy - wz;
  M[0][2] = xz + wy;
  M[1][0] = xy + wz;
  M[1][1] = R(1) - (xx + zz);
  M[1][2] = yz - wx;
  M[2][0] = xz - wy;
  M[2][1] = yz + wx;
  M[2][2] = R(1) - (xx + yy);
}

}  // namespace agb
