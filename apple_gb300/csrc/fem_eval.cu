// Evaluation API kernels: the five WarpPotential methods as one fused,
// tiled pass over the mesh (warp/fem/_base.py:243-383).
//
// One CTA per tile: the tile's vertices (<= kTileVerts) are staged in
// shared memory, each thread evaluates elements of the tile, the
// element-to-vertex scatter (the reference's 4 x vec3 global atomics per tet,
// _base.py:288-289, 321-322, 348-349) becomes shared-memory accumulation,
// and each tile writes one slot per vertex that a vertex pass sums in a
// fixed order.  Scalar outputs (energy, p^T H p) are reduced in float-float
// and finished by the last block, replacing the single-address scalar
// atomics of _base.py:261, 381.
#include "kernels.h"
#include "tile.cuh"

namespace agb {

template <class R>
__global__ void __launch_bounds__(256) pack_kernel(int n, const int32_t* __restrict__ uoi,
                                                   const R* __restrict__ u, V4<R>* __restrict__ ui,
                                                   const R* __restrict__ p, V4<R>* __restrict__ pi) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const size_t k = 3 * (size_t)uoi[i];
    ui[i] = V4<R>{u[k], u[k + 1], u[k + 2], R(0)};
    if (p) pi[i] = V4<R>{p[k], p[k + 1], p[k + 2], R(0)};
  }
}

template <class R, int MAT>
__global__ void __launch_bounds__(kElemThreads) fem_eval_kernel(
    FemView fv, unsigned flags, const V4<R>* __restrict__ u, const V4<R>* __restrict__ p,
    const int32_t* __restrict__ slot_of_tv, V4<R>* __restrict__ slots, int n_slots,
    AccStore<R>* __restrict__ partials, unsigned* counter, double* energy, double* quad) {
  __shared__ R sx[3][kTileVerts];
  __shared__ R sp[3][kTileVerts];
  __shared__ R acc[9][kTileVerts];
  __shared__ Acc<R> red[(kElemThreads / 32) * 2];

  const bool do_fun = flags & AGB_FUN, do_grad = flags & AGB_GRAD, do_diag = flags & AGB_HESS_DIAG;
  const bool do_prod = flags & AGB_HESS_PROD, do_quad = flags & AGB_HESS_QUAD;
  const bool need_p = do_prod || do_quad;

  const int tile = blockIdx.x;
  const int vs = fv.tile_vstart[tile], nv = fv.tile_vstart[tile + 1] - vs;
  const int es = fv.tile_estart[tile], ee = fv.tile_estart[tile + 1];

  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    const int v = fv.tv_vid[vs + i];
    const V4<R> a = ldg4(u + v);
    sx[0][i] = a.x;
    sx[1][i] = a.y;
    sx[2][i] = a.z;
    if (need_p) {
      const V4<R> b = ldg4(p + v);
      sp[0][i] = b.x;
      sp[1][i] = b.y;
      sp[2][i] = b.z;
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) acc[q][i] = R(0);
  }
  __syncthreads();

  Acc<R> sums[2] = {};
  for (int e = es + threadIdx.x; e < ee; e += blockDim.x) {
    ElemGeo<R> geo;
    uint32_t ids;
    load_elem_m<R, MAT>(fv, e, geo, ids);
    int l[4];
    R uc[4][3];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      l[a] = corner(ids, a);
#pragma unroll
      for (int c = 0; c < 3; ++c) uc[a][c] = sx[c][l[a]];
    }
    R G[3][3];
    corner_gradient(uc, geo.D, G);
    add_act<MAT>(geo, G);
    R dF[3][3];
    if (need_p) {
      R pc[4][3];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) pc[a][c] = sp[c][l[a]];
      corner_gradient(pc, geo.D, dF);
    }
    R f[4][3];
    if constexpr (snh_family(MAT)) {
      SnhPoint<R> s;
      snh_prepare(G, s);
      if (do_fun) sums[0].add(snh_energy(s, geo.mu, geo.lam));
      if (do_grad) {
        R P[3][3];
        snh_pk1(s, geo.mu, geo.lam, P);
        corner_vjp(P, geo.D, f);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int c = 0; c < 3; ++c) atomicAdd(&acc[c][l[a]], f[a][c]);
      }
      if (do_diag) {
        snh_hess_diag(s, geo.D, geo.mu, geo.lam, f);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int c = 0; c < 3; ++c) atomicAdd(&acc[3 + c][l[a]], fmax(f[a][c], R(0)));
      }
      if (need_p) {
        SnhDir<R> d;
        snh_dir(s, dF, d);
        if (do_quad) sums[1].add(fmax(snh_hess_quad(s, d, geo.mu, geo.lam), R(0)));
        if (do_prod) {
          R M[3][3];
          snh_hess_prod(s, d, dF, geo.mu, geo.lam, M);
          corner_vjp(M, geo.D, f);
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int c = 0; c < 3; ++c) atomicAdd(&acc[6 + c][l[a]], f[a][c]);
        }
      }
    } else {
      const R jm1 = (G[0][0] + G[1][1] + G[2][2]) + inv2(G) + det3(G);
      Svd<R> sv;
      svd_rv(G, jm1, sv);
      if (do_fun) sums[0].add(arap_energy(sv, geo.mu));
      if (do_grad) {
        R P[3][3];
        arap_pk1(sv, geo.mu, P);
        corner_vjp(P, geo.D, f);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int c = 0; c < 3; ++c) atomicAdd(&acc[c][l[a]], f[a][c]);
      }
      R lk[3];
      arap_lambdas(sv, lk);
      if (do_diag) {
        arap_hess_diag(sv, lk, geo.D, geo.mu, f);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int c = 0; c < 3; ++c) atomicAdd(&acc[3 + c][l[a]], fmax(f[a][c], R(0)));
      }
      if (do_quad) sums[1].add(fmax(arap_hess_quad(sv, lk, dF, geo.mu), R(0)));
      if (do_prod) {
        R M[3][3];
        arap_hess_prod(sv, lk, dF, geo.mu, M);
        corner_vjp(M, geo.D, f);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int c = 0; c < 3; ++c) atomicAdd(&acc[6 + c][l[a]], f[a][c]);
      }
    }
  }
  __syncthreads();

  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    const int s = slot_of_tv[vs + i];
    if (do_grad) slots[s] = V4<R>{acc[0][i], acc[1][i], acc[2][i], R(0)};
    if (do_diag) slots[(size_t)n_slots + s] = V4<R>{acc[3][i], acc[4][i], acc[5][i], R(0)};
    if (do_prod) slots[2 * (size_t)n_slots + s] = V4<R>{acc[6][i], acc[7][i], acc[8][i], R(0)};
  }

  if (do_fun || do_quad) {
    double tot[2];
    if (grid_reduce<2, R>(sums, partials, counter, gridDim.x, red, tot) && threadIdx.x == 0) {
      if (do_fun) *energy += tot[0];
      if (do_quad) *quad += tot[1];
    }
  }
}

constexpr int kUnpackThreads = 256;

int unpack_blocks(int n_points) {
  int b = (n_points + kUnpackThreads - 1) / kUnpackThreads;
  return b < 1 ? 1 : (b > 1216 ? 1216 : b);
}

template <class R>
__global__ void __launch_bounds__(kUnpackThreads) unpack_kernel(
    int n, const int32_t* __restrict__ uoi, const int32_t* __restrict__ off,
    const V4<R>* __restrict__ slots, int n_slots, unsigned flags, R* grad, R* diag, R* prod,
    const V4<R>* __restrict__ force, const V4<R>* __restrict__ u, AccStore<R>* partials,
    unsigned* counter, double* energy) {
  __shared__ Acc<R> red[kUnpackThreads / 32];
  Acc<R> ext[1] = {};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const size_t k = 3 * (size_t)uoi[i];
    const int s0 = off[i], s1 = off[i + 1];
    R* outs[3] = {grad, diag, prod};
    const unsigned fl[3] = {AGB_GRAD, AGB_HESS_DIAG, AGB_HESS_PROD};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      if (!(flags & fl[q])) continue;
      R sx = R(0), sy = R(0), sz = R(0);
      for (int s = s0; s < s1; ++s) {
        const V4<R> v = slots[(size_t)q * n_slots + s];
        sx += v.x;
        sy += v.y;
        sz += v.z;
      }
      if (q == 0 && force) {
        const V4<R> f = ldg4(force + i);
        sx -= f.x;
        sy -= f.y;
        sz -= f.z;
      }
      outs[q][k] += sx;
      outs[q][k + 1] += sy;
      outs[q][k + 2] += sz;
    }
    if ((flags & AGB_FUN) && force) {
      const V4<R> f = ldg4(force + i);
      const V4<R> x = ldg4(u + i);
      ext[0].add(-(f.x * x.x + f.y * x.y + f.z * x.z));
    }
  }
  if ((flags & AGB_FUN) && force) {
    double tot[1];
    if (grid_reduce<1, R>(ext, partials, counter, gridDim.x, red, tot) && threadIdx.x == 0)
      *energy += tot[0];
  }
}

cudaError_t launch_pack(int precision, int n, const int32_t* uoi, const void* u, void* ui,
                        const void* p, void* pi, cudaStream_t stream) {
  const int blocks = unpack_blocks(n);
  if (precision == AGB_F64)
    pack_kernel<double><<<blocks, 256, 0, stream>>>(n, uoi, (const double*)u, (V4<double>*)ui,
                                                    (const double*)p, (V4<double>*)pi);
  else
    pack_kernel<float><<<blocks, 256, 0, stream>>>(n, uoi, (const float*)u, (V4<float>*)ui,
                                                   (const float*)p, (V4<float>*)pi);
  return cudaGetLastError();
}

cudaError_t launch_fem_eval(int precision, const FemView& fv, unsigned flags, const void* u,
                            const void* p, const int32_t* slot_of_tv, void* slots, int32_t n_slots,
                            void* partials, unsigned* counter, double* energy, double* quad,
                            cudaStream_t stream) {
  if (fv.n_tiles == 0) return cudaSuccess;
  const dim3 grid(fv.n_tiles), block(kElemThreads);
#define AGB_EVAL_LAUNCH(R, MAT)                                                                \
  fem_eval_kernel<R, MAT><<<grid, block, 0, stream>>>(                                        \
      fv, flags, (const V4<R>*)u, (const V4<R>*)p, slot_of_tv, (V4<R>*)slots, n_slots,          \
      (AccStore<R>*)partials, counter, energy, quad)
  if (precision == AGB_F64) {
    if (fv.material == AGB_ARAP)
      AGB_EVAL_LAUNCH(double, AGB_ARAP);
    else if (fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE)
      AGB_EVAL_LAUNCH(double, AGB_STABLE_NEO_HOOKEAN_MUSCLE);
    else
      AGB_EVAL_LAUNCH(double, AGB_STABLE_NEO_HOOKEAN);
  } else {
    if (fv.material == AGB_ARAP)
      AGB_EVAL_LAUNCH(float, AGB_ARAP);
    else if (fv.material == AGB_STABLE_NEO_HOOKEAN_MUSCLE)
      AGB_EVAL_LAUNCH(float, AGB_STABLE_NEO_HOOKEAN_MUSCLE);
    else
      AGB_EVAL_LAUNCH(float, AGB_STABLE_NEO_HOOKEAN);
  }
#undef AGB_EVAL_LAUNCH
  return cudaGetLastError();
}

cudaError_t launch_unpack(int precision, int n, const int32_t* uoi, const int32_t* off,
                          const void* slots, int32_t n_slots, unsigned flags, void* grad,
                          void* diag, void* prod, const void* force, const void* u, void* partials,
                          unsigned* counter, double* energy, cudaStream_t stream) {
  const int blocks = unpack_blocks(n);
  if (precision == AGB_F64)
    unpack_kernel<double><<<blocks, kUnpackThreads, 0, stream>>>(
        n, uoi, off, (const V4<double>*)slots, n_slots, flags, (double*)grad, (double*)diag,
        (double*)prod, (const V4<double>*)force, (const V4<double>*)u,
        (AccStore<double>*)partials, counter, energy);
  else
    unpack_kernel<float><<<blocks, kUnpackThreads, 0, stream>>>(
        n, uoi, off, (const V4<float>*)slots, n_slots, flags, (float*)grad, (float*)diag,
        (float*)prod, (const V4<float>*)force, (const V4<float>*)u, (AccStore<float>*)partials,
        counter, energy);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// free/fixed DOF maps (forward/dof_map/_dof_map.py:30-50): one gather each,
// with coalesced writes; to_full reads a full-length slot map (free index or
// -1) instead of scattering the free and the fixed values separately
// ---------------------------------------------------------------------------
template <class R>
__global__ void dof_to_free_kernel(int64_t n, const int64_t* __restrict__ idx, const R* __restrict__ full,
                                   R* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = full[idx[i]];
}

template <class R>
__global__ void dof_to_full_kernel(int64_t n, const int32_t* __restrict__ slot, const R* __restrict__ free_in,
                                   const R* __restrict__ fill, R* __restrict__ out) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = slot[j];
    out[j] = k >= 0 ? free_in[k] : (fill ? fill[j] : R(0));
  }
}

static int dof_blocks(int64_t n) {
  const int64_t b = (n + 255) / 256;
  const int64_t cap = 152 * 8;  // 8 resident 256-thread CTAs on each of the 152 SMs
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

cudaError_t launch_dof_to_free(int precision, int64_t n, const int64_t* idx, const void* full, void* out,
                               cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (precision == AGB_F64)
    dof_to_free_kernel<double><<<dof_blocks(n), 256, 0, s>>>(n, idx, (const double*)full, (double*)out);
  else
    dof_to_free_kernel<float><<<dof_blocks(n), 256, 0, s>>>(n, idx, (const float*)full, (float*)out);
  return cudaGetLastError();
}

cudaError_t launch_dof_to_full(int precision, int64_t n, const int32_t* slot, const void* free_in,
                               const void* fill, void* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (precision == AGB_F64)
    dof_to_full_kernel<double><<<dof_blocks(n), 256, 0, s>>>(n, slot, (const double*)free_in,
                                                            (const double*)fill, (double*)out);
  else
    dof_to_full_kernel<float><<<dof_blocks(n), 256, 0, s>>>(n, slot, (const float*)free_in,
                                                           (const float*)fill, (float*)out);
  return cudaGetLastError();
}

}  // namespace agb
