/*
 * C / OpenMP FP64 restatement of the reference's FEM kernels and PNCG loop.
 *
 * TEST INFRASTRUCTURE ONLY: the timed CPU baseline (bench.py cpu_baseline
 * and --impl reference) and a second oracle in tests/.  The product never
 * links it.
 *
 * Follows, per element and per call, the Warp kernels of liblaf/apple
 * (warp/fem/_base.py:243-383: one pass per method, dV weighting, the clamps
 * of hess_diag (317-320) and hess_quad (379-380), atomic scatter (288-289,
 * 321-322, 348-349) and scalar atomics (261, 381)), the materials
 * (warp/fem/_arap.py:17-76, warp/fem/_stable_neo_hookean.py:17-103) and the
 * PNCG iteration of benches/bench_pncg_branching_backends.py:254-456,606-679
 * with the first trial step alpha_0 = overstep * (-g.p / p.Hp).  The 3x3 SVD
 * is a cyclic Jacobi eigen-decomposition of F^T F followed by U = F V / sigma
 * with Gram-Schmidt (rotation-variant: det U = det V = +1), the published
 * structure of McAdams et al. 2011, in FP64 to full convergence.
 *
 * The reference's Warp CPU path (warp-lang) is not installed here; this port
 * is what "the reference's CPU implementation of the path" is timed as.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>

/* loops shorter than this run on one thread: small cases are then
 * deterministic (no atomic or reduction-order effects) */
#define ORC_PAR_MIN 4096
#endif

#define ORC_FUN 1u
#define ORC_GRAD 2u
#define ORC_DIAG 4u
#define ORC_PROD 8u
#define ORC_QUAD 16u

typedef struct {
  int material; /* 0 ARAP, 1 stable Neo-Hookean */
  int n_points;
  int n_cells;
  const int32_t* cells;
  const double* dhdX; /* n x 4 x 3 */
  const double* dV;
  const double* mu;
  const double* lam;
} orc_fem;

static double det3(const double A[3][3]) {
  return A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
         A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
}

/* g3: columns f1 x f2, f2 x f0, f0 x f1 (func/_gradient.py:31-40) */
static void g3(const double F[3][3], double C[3][3]) {
  for (int c = 0; c < 3; ++c) {
    int a = (c + 1) % 3, b = (c + 2) % 3;
    C[0][c] = F[1][a] * F[2][b] - F[2][a] * F[1][b];
    C[1][c] = F[2][a] * F[0][b] - F[0][a] * F[2][b];
    C[2][c] = F[0][a] * F[1][b] - F[1][a] * F[0][b];
  }
}

static double ddot(const double A[3][3], const double B[3][3]) {
  double s = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) s += A[i][j] * B[i][j];
  return s;
}

/* rotation-variant SVD */
static void svd_rv(const double F[3][3], double U[3][3], double s[3], double V[3][3]) {
  double A[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      A[i][j] = F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j];
      V[i][j] = i == j;
    }
  for (int sweep = 0; sweep < 30; ++sweep) {
    double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
    double dia = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
    if (off <= 1e-32 * dia || off == 0.0) break;
    for (int pq = 0; pq < 3; ++pq) {
      int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
      double apq = A[p][q];
      if (apq == 0.0) continue;
      double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
      double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
      double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
      A[p][p] -= t * apq;
      A[q][q] += t * apq;
      A[p][q] = A[q][p] = 0.0;
      int r = 3 - p - q;
      double arp = A[r][p], arq = A[r][q];
      A[r][p] = A[p][r] = c * arp - sn * arq;
      A[r][q] = A[q][r] = sn * arp + c * arq;
      for (int k = 0; k < 3; ++k) {
        double vkp = V[k][p], vkq = V[k][q];
        V[k][p] = c * vkp - sn * vkq;
        V[k][q] = sn * vkp + c * vkq;
      }
    }
  }
  double e[3] = {A[0][0], A[1][1], A[2][2]};
  for (int a = 0; a < 2; ++a)
    for (int b = a + 1; b < 3; ++b)
      if (e[a] < e[b]) {
        double t = e[a];
        e[a] = e[b];
        e[b] = t;
        for (int k = 0; k < 3; ++k) {
          double tv = V[k][a];
          V[k][a] = V[k][b];
          V[k][b] = -tv;
        }
      }
  double b0[3], b1[3];
  for (int k = 0; k < 3; ++k) {
    b0[k] = F[k][0] * V[0][0] + F[k][1] * V[1][0] + F[k][2] * V[2][0];
    b1[k] = F[k][0] * V[0][1] + F[k][1] * V[1][1] + F[k][2] * V[2][1];
  }
  double n0 = sqrt(b0[0] * b0[0] + b0[1] * b0[1] + b0[2] * b0[2]);
  if (n0 > 0) {
    for (int k = 0; k < 3; ++k) b0[k] /= n0;
  } else {
    b0[0] = 1; b0[1] = b0[2] = 0;
  }
  double pr = b0[0] * b1[0] + b0[1] * b1[1] + b0[2] * b1[2];
  for (int k = 0; k < 3; ++k) b1[k] -= pr * b0[k];
  double n1 = sqrt(b1[0] * b1[0] + b1[1] * b1[1] + b1[2] * b1[2]);
  if (n1 > 1e-300) {
    for (int k = 0; k < 3; ++k) b1[k] /= n1;
  } else {
    double ax[3] = {0, 0, 0};
    int k = (fabs(b0[0]) <= fabs(b0[1]) && fabs(b0[0]) <= fabs(b0[2])) ? 0 : (fabs(b0[1]) <= fabs(b0[2]) ? 1 : 2);
    ax[k] = 1;
    b1[0] = b0[1] * ax[2] - b0[2] * ax[1];
    b1[1] = b0[2] * ax[0] - b0[0] * ax[2];
    b1[2] = b0[0] * ax[1] - b0[1] * ax[0];
    double m = sqrt(b1[0] * b1[0] + b1[1] * b1[1] + b1[2] * b1[2]);
    for (int q = 0; q < 3; ++q) b1[q] /= m;
  }
  for (int k = 0; k < 3; ++k) {
    U[k][0] = b0[k];
    U[k][1] = b1[k];
  }
  U[0][2] = b0[1] * b1[2] - b0[2] * b1[1];
  U[1][2] = b0[2] * b1[0] - b0[0] * b1[2];
  U[2][2] = b0[0] * b1[1] - b0[1] * b1[0];
  for (int i = 0; i < 3; ++i) s[i] = sqrt(e[i] > 0 ? e[i] : 0.0);
  if (det3(F) < 0) s[2] = -s[2];
}

static void load(const orc_fem* m, int e, const double* u, double uc[4][3], double D[4][3]) {
  for (int a = 0; a < 4; ++a) {
    int v = m->cells[4 * e + a];
    for (int c = 0; c < 3; ++c) {
      uc[a][c] = u[3 * (size_t)v + c];
      D[a][c] = m->dhdX[12 * (size_t)e + 3 * a + c];
    }
  }
}

/* F = I + u^T dhdX ; dF = p^T dhdX */
static void defgrad(const double uc[4][3], const double D[4][3], double F[3][3], int add_identity) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int a = 0; a < 4; ++a) s += uc[a][i] * D[a][j];
      F[i][j] = s + (add_identity && i == j ? 1.0 : 0.0);
    }
}

/* vjp: out_a = M D_a^T */
static void vjp(const double D[4][3], const double M[3][3], double out[4][3]) {
  for (int a = 0; a < 4; ++a)
    for (int i = 0; i < 3; ++i) out[a][i] = M[i][0] * D[a][0] + M[i][1] * D[a][1] + M[i][2] * D[a][2];
}

static double psi(const orc_fem* m, int e, const double F[3][3]) {
  if (m->material == 0) {
    double U[3][3], s[3], V[3][3];
    svd_rv(F, U, s, V);
    double acc = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double r = U[i][0] * V[j][0] + U[i][1] * V[j][1] + U[i][2] * V[j][2];
        acc += (F[i][j] - r) * (F[i][j] - r);
      }
    return 0.5 * m->mu[e] * acc;
  }
  double J = det3(F), I2 = ddot(F, F), mu = m->mu[e], la = m->lam[e];
  return 0.5 * mu * (I2 - 3.0) - mu * (J - 1.0) + 0.5 * la * (J - 1.0) * (J - 1.0);
}

static void pk1(const orc_fem* m, int e, const double F[3][3], double P[3][3]) {
  if (m->material == 0) {
    double U[3][3], s[3], V[3][3];
    svd_rv(F, U, s, V);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        P[i][j] = m->mu[e] * (F[i][j] - (U[i][0] * V[j][0] + U[i][1] * V[j][1] + U[i][2] * V[j][2]));
    return;
  }
  double C[3][3];
  g3(F, C);
  double J = det3(F), mu = m->mu[e], la = m->lam[e];
  double d3 = -mu + la * (J - 1.0);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) P[i][j] = mu * F[i][j] + d3 * C[i][j];
}

static void twist(const double U[3][3], const double V[3][3], double Q[3][3][3], double lk[3], const double s[3]) {
  const int A[3] = {1, 1, 0}, B[3] = {0, 2, 2};
  const double r2 = 1.0 / sqrt(2.0);
  for (int k = 0; k < 3; ++k)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Q[k][i][j] = (U[i][A[k]] * V[j][B[k]] - U[i][B[k]] * V[j][A[k]]) * r2;
  double p0 = s[0] + s[1], p1 = s[1] + s[2], p2 = s[2] + s[0];
  lk[0] = 2.0 / (p0 > 2.0 ? p0 : 2.0);
  lk[1] = 2.0 / (p1 > 2.0 ? p1 : 2.0);
  lk[2] = 2.0 / (p2 > 2.0 ? p2 : 2.0);
}

static void hdiag(const orc_fem* m, int e, const double F[3][3], const double D[4][3], double h[4][3]) {
  double mu = m->mu[e];
  if (m->material == 0) {
    double U[3][3], s[3], V[3][3], Q[3][3][3], lk[3];
    svd_rv(F, U, s, V);
    twist(U, V, Q, lk, s);
    for (int a = 0; a < 4; ++a) {
      double nn = D[a][0] * D[a][0] + D[a][1] * D[a][1] + D[a][2] * D[a][2];
      for (int i = 0; i < 3; ++i) {
        double h4 = 0;
        for (int k = 0; k < 3; ++k) {
          double w = Q[k][i][0] * D[a][0] + Q[k][i][1] * D[a][1] + Q[k][i][2] * D[a][2];
          h4 += lk[k] * w * w;
        }
        h[a][i] = 0.5 * mu * (-2.0 * h4 + 2.0 * nn);
      }
    }
    return;
  }
  double C[3][3], la = m->lam[e];
  g3(F, C);
  for (int a = 0; a < 4; ++a) {
    double nn = D[a][0] * D[a][0] + D[a][1] * D[a][1] + D[a][2] * D[a][2];
    for (int i = 0; i < 3; ++i) {
      double w = C[i][0] * D[a][0] + C[i][1] * D[a][1] + C[i][2] * D[a][2];
      h[a][i] = la * w * w + 0.5 * mu * 2.0 * nn;
    }
  }
}

/* H_e p as M (corner forces M D_a^T) and p^T H_e p */
static double hprod(const orc_fem* m, int e, const double F[3][3], const double dF[3][3], double M[3][3]) {
  double mu = m->mu[e];
  if (m->material == 0) {
    double U[3][3], s[3], V[3][3], Q[3][3][3], lk[3];
    svd_rv(F, U, s, V);
    twist(U, V, Q, lk, s);
    double qd[3];
    for (int k = 0; k < 3; ++k) qd[k] = ddot(Q[k], dF);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        M[i][j] = mu * (dF[i][j] - lk[0] * qd[0] * Q[0][i][j] - lk[1] * qd[1] * Q[1][i][j] - lk[2] * qd[2] * Q[2][i][j]);
    return mu * (ddot(dF, dF) - lk[0] * qd[0] * qd[0] - lk[1] * qd[1] * qd[1] - lk[2] * qd[2] * qd[2]);
  }
  double C[3][3], H6[3][3], la = m->lam[e];
  g3(F, C);
  for (int c = 0; c < 3; ++c) {
    int a = (c + 1) % 3, b = (c + 2) % 3;
    for (int i = 0; i < 3; ++i) {
      int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
      H6[i][c] = F[i1][a] * dF[i2][b] - F[i2][a] * dF[i1][b] + dF[i1][a] * F[i2][b] - dF[i2][a] * F[i1][b];
    }
  }
  double J = det3(F), a1 = ddot(C, dF), d3 = -mu + la * (J - 1.0);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M[i][j] = la * a1 * C[i][j] + mu * dF[i][j] + d3 * H6[i][j];
  return ddot(M, dF);
}

/* one reference kernel pass; accumulates like the Warp kernels */
int orc_eval(int material, int n_points, int n_cells, const int32_t* cells, const double* dhdX, const double* dV,
             const double* mu, const double* lam, const double* u, const double* p, unsigned flags, double* energy,
             double* grad, double* diag, double* prod, double* quad) {
  orc_fem m = {material, n_points, n_cells, cells, dhdX, dV, mu, lam};
  double e_sum = 0.0, q_sum = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : e_sum, q_sum) if (n_cells >= ORC_PAR_MIN)
  for (int e = 0; e < n_cells; ++e) {
    double uc[4][3], D[4][3], F[3][3], out[4][3];
    load(&m, e, u, uc, D);
    defgrad(uc, D, F, 1);
    const double w = dV[e];
    if (flags & ORC_FUN) e_sum += psi(&m, e, F) * w;
    if (flags & ORC_GRAD) {
      double P[3][3];
      pk1(&m, e, F, P);
      vjp(D, P, out);
      for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 3; ++c) {
#pragma omp atomic
          grad[3 * (size_t)cells[4 * e + a] + c] += out[a][c] * w;
        }
    }
    if (flags & ORC_DIAG) {
      hdiag(&m, e, F, D, out);
      for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 3; ++c) {
          double v = out[a][c] * w;
          v = v > 0.0 ? v : 0.0;
#pragma omp atomic
          diag[3 * (size_t)cells[4 * e + a] + c] += v;
        }
    }
    if (flags & (ORC_PROD | ORC_QUAD)) {
      double pc[4][3], dF[3][3], M[3][3];
      load(&m, e, p, pc, D);
      defgrad(pc, D, dF, 0);
      double hq = hprod(&m, e, F, dF, M) * w;
      if (flags & ORC_QUAD) q_sum += hq > 0.0 ? hq : 0.0;
      if (flags & ORC_PROD) {
        vjp(D, M, out);
        for (int a = 0; a < 4; ++a)
          for (int c = 0; c < 3; ++c) {
#pragma omp atomic
            prod[3 * (size_t)cells[4 * e + a] + c] += out[a][c] * w;
          }
      }
    }
  }
  if (flags & ORC_FUN) *energy += e_sum;
  if (flags & ORC_QUAD) *quad += q_sum;
  return 0;
}

typedef struct {
  int max_steps;
  double rtol, atol;
  int max_bt;
  double c, overstep, beta_max;
} orc_params;

typedef struct {
  int result, n_steps;
  double grad_norm, grad_norm_first, energy;
} orc_stats;

static double dot_masked(int n3, const double* a, const double* b, const uint8_t* mask) {
  double s = 0;
#pragma omp parallel for reduction(+ : s) if (n3 >= ORC_PAR_MIN)
  for (int i = 0; i < n3; ++i)
    if (!mask[i]) s += a[i] * b[i];
  return s;
}

static double model_fun(const orc_fem* m, const double* u, const double* force) {
  double e = 0;
  orc_eval(m->material, m->n_points, m->n_cells, m->cells, m->dhdX, m->dV, m->mu, m->lam, u, NULL, ORC_FUN, &e, NULL,
           NULL, NULL, NULL);
  if (force) {
    double w = 0;
    int n3 = 3 * m->n_points;
#pragma omp parallel for reduction(+ : w) if (n3 >= ORC_PAR_MIN)
    for (int i = 0; i < n3; ++i) w -= force[i] * u[i];
    e += w;
  }
  return e;
}

/* PNCG on the full vector with fixed components masked (the free-space
 * vectors of forward/_problem.py are the unmasked components).  `mask` is
 * n_points*3 bytes; u holds the fixed values on entry. */
int orc_pncg(int material, int n_points, int n_cells, const int32_t* cells, const double* dhdX, const double* dV,
             const double* mu, const double* lam, const uint8_t* mask, const double* force, double* u,
             const orc_params* prm, orc_stats* st) {
  orc_fem m = {material, n_points, n_cells, cells, dhdX, dV, mu, lam};
  const int n3 = 3 * n_points;
  double* g = calloc(n3, sizeof(double));
  double* gp = calloc(n3, sizeof(double));
  double* d = calloc(n3, sizeof(double));
  double* P = calloc(n3, sizeof(double));
  double* dir = calloc(n3, sizeof(double));
  double* pd = calloc(n3, sizeof(double));
  double* trial = calloc(n3, sizeof(double));
  double* Py = calloc(n3, sizeof(double));
  double gnorm0 = 0, value = 0;
  st->result = 1;
  st->n_steps = 0;
  for (int it = 0;; ++it) {
    value = model_fun(&m, u, force);
    memset(g, 0, n3 * sizeof(double));
    memset(d, 0, n3 * sizeof(double));
    orc_eval(material, n_points, n_cells, cells, dhdX, dV, mu, lam, u, NULL, ORC_GRAD, NULL, g, NULL, NULL, NULL);
    orc_eval(material, n_points, n_cells, cells, dhdX, dV, mu, lam, u, NULL, ORC_DIAG, NULL, NULL, d, NULL, NULL);
    if (force)
      for (int i = 0; i < n3; ++i) g[i] -= force[i];
    for (int i = 0; i < n3; ++i)
      if (mask[i]) g[i] = d[i] = 0.0;
    double gnorm = sqrt(dot_masked(n3, g, g, mask));
    if (it == 0) gnorm0 = gnorm;
    st->grad_norm = gnorm;
    st->grad_norm_first = gnorm0;
    st->energy = value;
    if (!(isfinite(gnorm) && isfinite(value))) {
      st->result = 3;
      break;
    }
    if (gnorm <= fmax(prm->atol, prm->rtol * gnorm0)) {
      st->result = 0;
      break;
    }
    if (it >= prm->max_steps) {
      st->result = 1;
      break;
    }
    /* preconditioner: 1/|d|, zeros -> mean of positive entries (proxy :407-410) */
    double sum = 0;
    long cnt = 0;
    for (int i = 0; i < n3; ++i)
      if (!mask[i] && fabs(d[i]) > 0) {
        sum += fabs(d[i]);
        ++cnt;
      }
    double mean = cnt ? sum / cnt : 1.0;
    for (int i = 0; i < n3; ++i) P[i] = mask[i] ? 0.0 : 1.0 / (fabs(d[i]) > 0 ? fabs(d[i]) : mean);
    double beta = 0.0;
    if (it > 0) {
      double yp = 0, gpy = 0, ypy = 0, pg = 0;
      for (int i = 0; i < n3; ++i) {
        if (mask[i]) continue;
        double y = g[i] - gp[i];
        yp += y * pd[i];
        gpy += g[i] * P[i] * y;
        ypy += y * P[i] * y;
        pg += pd[i] * g[i];
      }
      beta = fabs(yp) > 1e-12 ? gpy / yp - (ypy / yp) * (pg / yp) : INFINITY;
      if (!(isfinite(beta) && fabs(beta) <= prm->beta_max)) beta = 0.0;
    }
    for (int i = 0; i < n3; ++i) dir[i] = -P[i] * g[i] + beta * pd[i];
    double gd = dot_masked(n3, g, dir, mask);
    if (!(isfinite(gd) && gd < 0)) {
      beta = 0;
      for (int i = 0; i < n3; ++i) dir[i] = -P[i] * g[i];
      gd = dot_masked(n3, g, dir, mask);
    }
    double hq = 0;
    orc_eval(material, n_points, n_cells, cells, dhdX, dV, mu, lam, u, dir, ORC_QUAD, NULL, NULL, NULL, NULL, &hq);
    double alpha = -gd / hq;
    if (isnan(alpha)) alpha = 0;
    if (isinf(alpha)) alpha = alpha > 0 ? 1.0 : 0.0;
    if (!(alpha > 0 && isfinite(alpha))) alpha = 1.0;
    alpha *= prm->overstep;
    int ok = 0, ls = 0;
    for (;;) {
      for (int i = 0; i < n3; ++i) trial[i] = u[i] + alpha * dir[i];
      double tv = model_fun(&m, trial, force);
      ok = isfinite(tv) && tv <= value + prm->c * alpha * gd;
      if (ok || ls >= prm->max_bt || !(alpha > 0)) break;
      alpha *= 0.5;
      ++ls;
    }
    st->n_steps = it + 1;
    if (ok) {
      memcpy(u, trial, n3 * sizeof(double));
    } else if (beta == 0.0) {
      st->result = 2;
      break;
    }
    memcpy(gp, g, n3 * sizeof(double));
    memcpy(pd, dir, n3 * sizeof(double));
  }
  free(g); free(gp); free(d); free(P); free(dir); free(pd); free(trial); free(Py);
  return 0;
}

int orc_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
