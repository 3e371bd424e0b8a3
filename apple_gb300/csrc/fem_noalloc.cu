// agb_fem_fun_noalloc: the energy of a potential without any device
// allocation on the caller's side.
//
// Who needs it: code that runs under a device allocator it does not own and
// must not call cudaMalloc itself -- for example an XLA/JAX FFI handler
// (the reference reaches its energies through one, warp/model/_adapter.py),
// where XLA reserves most of the device memory up front, or a real-time
// loop with a fixed memory budget.  The potential handle and the caller's
// input and output buffers already exist; the per-call scratch that the
// regular entry point keeps in its handle (a packed copy of u, per-block
// partial sums and a completion counter) is replaced here by reading u in
// the caller's order and by one file-scope device array.
//
// The array holds kNoAllocMaxTiles float-float partials (8 bytes each) and
// one counter: 512 KiB + 256 bytes, held by every GPU that loads this
// library until the process exits.  Meshes with more tiles (about 40
// million tets at the ~625 elements per tile of a structured grid) are
// rejected with AGB_E_INVALID.  Every call on a device shares the array and
// it keeps the last call's contents: the counter is cleared before each
// launch and every partial is written before it is read.  Calls that overlap
// on the GPU (concurrent streams) race on the array.
#include "kernels.h"
#include "tile.cuh"

namespace agb {

constexpr int kNoAllocMaxTiles = 65536;
constexpr size_t kNoAllocPartialBytes = (size_t)kNoAllocMaxTiles * 8;

static __device__ __align__(256) unsigned char g_fun_noalloc_scratch[kNoAllocPartialBytes + 256];

template <class R, int MAT>
__global__ void __launch_bounds__(kElemThreads)
    fem_fun_noalloc_kernel(FemView fv, const int32_t* __restrict__ user_of_internal,
                           const R* __restrict__ u, unsigned char* scratch, double* out) {
  __shared__ R sx[3][kTileVerts];
  __shared__ Acc<R> red[kElemThreads / 32];
  const int tile = blockIdx.x;
  const int vs = fv.tile_vstart[tile], nv = fv.tile_vstart[tile + 1] - vs;
  const int es = fv.tile_estart[tile], ee = fv.tile_estart[tile + 1];
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    const size_t k = 3 * (size_t)user_of_internal[fv.tv_vid[vs + i]];
    sx[0][i] = u[k];
    sx[1][i] = u[k + 1];
    sx[2][i] = u[k + 2];
  }
  __syncthreads();
  Acc<R> sums[1] = {};
  for (int e = es + threadIdx.x; e < ee; e += blockDim.x) {
    ElemGeo<R> geo;
    uint32_t ids;
    load_elem<R>(fv, e, geo, ids);
    R w[4][3], G[3][3];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) w[a][c] = sx[c][corner(ids, a)];
    corner_gradient(w, geo.D, G);
    if constexpr (MAT == AGB_STABLE_NEO_HOOKEAN) {
      SnhPoint<R> s;
      snh_prepare(G, s);
      sums[0].add(snh_energy(s, geo.mu, geo.lam));
    } else {
      Svd<R> sv;
      svd_rv(G, (G[0][0] + G[1][1] + G[2][2]) + inv2(G) + det3(G), sv);
      sums[0].add(arap_energy(sv, geo.mu));
    }
  }
  double tot[1];
  if (grid_reduce<1, R>(sums, (AccStore<R>*)scratch, (unsigned*)(scratch + kNoAllocPartialBytes),
                        gridDim.x, red, tot) &&
      threadIdx.x == 0)
    *out += tot[0];
}

// Device address of the scratch array.  The array's name is only a host-side
// stand-in, so the address is looked up with the caller's device current, on
// every call: the lookup is cheap once the module is loaded, and a cached
// address would dangle after cudaDeviceReset reloads the module.
static int noalloc_scratch(unsigned char** ptr) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_fun_noalloc_scratch);
  AGB_REQUIRE(e == cudaSuccess && p, AGB_E_CUDA, "agb_fem_fun_noalloc: cudaGetSymbolAddress: %s",
              cudaGetErrorString(e));
  *ptr = (unsigned char*)p;
  return AGB_OK;
}

}  // namespace agb

using namespace agb;

extern "C" int agb_fem_fun_noalloc(agb_fem* fem, const void* u, double* output, void* stream) {
  clear_error();
  AGB_REQUIRE(fem && u && output, AGB_E_INVALID, "agb_fem_fun_noalloc: null argument");
  const FemView fv = fem->view();
  AGB_REQUIRE(fv.material != AGB_STABLE_NEO_HOOKEAN_MUSCLE, AGB_E_INVALID,
              "agb_fem_fun_noalloc: muscle potentials are not supported; use agb_fem_fun");
  AGB_REQUIRE(fv.n_tiles <= kNoAllocMaxTiles, AGB_E_INVALID,
              "agb_fem_fun_noalloc: the mesh has %d tiles; this entry point holds partial sums for at "
              "most %d (use agb_fem_fun)",
              fv.n_tiles, kNoAllocMaxTiles);
  if (fv.n_tiles == 0) return AGB_OK;
  unsigned char* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  AGB_CHECK_CUDA(cudaMemsetAsync(scratch + kNoAllocPartialBytes, 0, sizeof(unsigned), s));
  const int32_t* uoi = fem->space->d_user_of_internal;
  const dim3 grid(fv.n_tiles), block(kElemThreads);
  if (fem->precision == AGB_F64) {
    if (fv.material == AGB_ARAP)
      fem_fun_noalloc_kernel<double, AGB_ARAP><<<grid, block, 0, s>>>(fv, uoi, (const double*)u, scratch, output);
    else
      fem_fun_noalloc_kernel<double, AGB_STABLE_NEO_HOOKEAN>
          <<<grid, block, 0, s>>>(fv, uoi, (const double*)u, scratch, output);
  } else {
    if (fv.material == AGB_ARAP)
      fem_fun_noalloc_kernel<float, AGB_ARAP><<<grid, block, 0, s>>>(fv, uoi, (const float*)u, scratch, output);
    else
      fem_fun_noalloc_kernel<float, AGB_STABLE_NEO_HOOKEAN>
          <<<grid, block, 0, s>>>(fv, uoi, (const float*)u, scratch, output);
  }
  AGB_CHECK_CUDA(cudaGetLastError());
  return AGB_OK;
}
