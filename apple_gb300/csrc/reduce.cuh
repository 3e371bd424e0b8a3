// Global sums for the PNCG scalars (energy, p^T H p, dot products).
//
// GB300's FP64 rate is about 1/64 of its FP32 rate, so per-element FP64
// adds would cost more than the memory pass they sit in.  Leaves therefore
// accumulate in float-float form (hi + lo, error-free two-sum, about 44
// significant bits), warps and blocks combine float-float pairs in a fixed
// order, and each block writes one pair per quantity.  The last block to
// finish (detected with a counter after a fence, no spinning) adds the block
// partials in a fixed order and hands FP64 values to the scalar logic, so
// every sum is deterministic for a given grid.  The FP64 build (R = double)
// accumulates plain doubles.
#pragma once

#include <cuda_runtime.h>

namespace agb {

template <class R>
struct Acc;

template <>
struct Acc<float> {
  float hi, lo;  // no initialisers: usable in __shared__; value-initialise with {}
  __device__ __forceinline__ void add(float b) {
    const float s = hi + b;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (b - bb);
    hi = s;
    lo += err;
  }
  __device__ __forceinline__ void add(const Acc<float>& o) {
    const float s = hi + o.hi;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (o.hi - bb);
    hi = s;
    lo = lo + o.lo + err;
  }
  __device__ __forceinline__ Acc<float> shfl_down(int off) const {
    Acc<float> r{};
    r.hi = __shfl_down_sync(0xffffffffu, hi, off);
    r.lo = __shfl_down_sync(0xffffffffu, lo, off);
    return r;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
  // lane 0 gets the float sum of hi + lo over the warp
  __device__ __forceinline__ void warp_plain_sum() {
    float v = hi + lo;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    hi = v;
    lo = 0.f;
  }
};

template <>
struct Acc<double> {
  double v;
  __device__ __forceinline__ void add(double b) { v += b; }
  __device__ __forceinline__ void add(const Acc<double>& o) { v += o.v; }
  __device__ __forceinline__ Acc<double> shfl_down(int off) const {
    Acc<double> r{};
    r.v = __shfl_down_sync(0xffffffffu, v, off);
    return r;
  }
  __device__ __forceinline__ double value() const { return v; }
  __device__ __forceinline__ void warp_plain_sum() {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  }
};

// Storage of one partial in global memory.
template <class R>
struct AccStore;
template <>
struct AccStore<float> {
  float2 p;
};
template <>
struct AccStore<double> {
  double p;
};

template <class R>
__device__ __forceinline__ AccStore<R> acc_store(const Acc<R>& a);
template <>
__device__ __forceinline__ AccStore<float> acc_store<float>(const Acc<float>& a) {
  return AccStore<float>{make_float2(a.hi, a.lo)};
}
template <>
__device__ __forceinline__ AccStore<double> acc_store<double>(const Acc<double>& a) {
  return AccStore<double>{a.v};
}

template <class R>
__device__ __forceinline__ Acc<R> acc_load(const AccStore<R>* s);
template <>
__device__ __forceinline__ Acc<float> acc_load<float>(const AccStore<float>* s) {
  const float2 v = __ldcg(&s->p);
  Acc<float> a{};
  a.hi = v.x;
  a.lo = v.y;
  return a;
}
template <>
__device__ __forceinline__ Acc<double> acc_load<double>(const AccStore<double>* s) {
  Acc<double> a{};
  a.v = __ldcg(&s->p);
  return a;
}

// Block-wide reduction of N accumulators.  Result valid in thread 0.
// `scratch` must hold (blockDim/32) * N entries.  Warps reduce by shuffles:
// quantities whose bit is set in FF (sums whose terms change sign) keep the
// float-float pair through the warp tree, the others (sums of same-sign
// terms, counts) use a plain float tree (relative error <= 5 ulp); then
// thread k < N adds quantity k across warps in float-float (fixed order).
template <int N, unsigned FF = 0xffffffffu, class R>
__device__ __forceinline__ void block_reduce(Acc<R> (&a)[N], Acc<R>* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    if ((FF >> k) & 1u) {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) a[k].add(a[k].shfl_down(off));
    } else {
      a[k].warp_plain_sum();
    }
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) scratch[warp * N + k] = a[k];
  }
  __syncthreads();
  if (threadIdx.x < N) {
    Acc<R> s = scratch[threadIdx.x];
    for (int w = 1; w < nw; ++w) s.add(scratch[w * N + threadIdx.x]);
    scratch[threadIdx.x] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) a[k] = scratch[k];
  }
  __syncthreads();
}

// Two-level completion tree: blocks report in groups of 32; the last block
// of a group adds the group's partials (fixed order) into a group partial,
// and the last group to finish adds the group partials.  The critical path
// is two partial loads instead of one pass over every block's partial.
// cnt holds ceil(nblocks/32) + 1 zeroed counters; each finisher resets the
// counter it completed.  Returns true in the final block, where `total`
// (thread 0) holds the sums.
template <int N, unsigned FF = 0xffffffffu, class R>
__device__ __forceinline__ bool grid_reduce2(Acc<R> (&a)[N], AccStore<R>* partials,
                                             AccStore<R>* gpartials, unsigned* cnt, int nblocks,
                                             Acc<R>* scratch, double (&total)[N]) {
  __shared__ bool s_last;
  block_reduce<N, FF, R>(a, scratch);
  const int grp = blockIdx.x >> 5, ngroups = (nblocks + 31) >> 5;
  const int gsize = min(32, nblocks - (grp << 5));
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) partials[(size_t)blockIdx.x * N + k] = acc_store(a[k]);
    __threadfence();
    s_last = atomicAdd(&cnt[grp], 1u) == (unsigned)gsize - 1u;
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  Acc<R> b[N] = {};
  if (threadIdx.x < gsize) {
#pragma unroll
    for (int k = 0; k < N; ++k) b[k] = acc_load<R>(partials + (size_t)((grp << 5) + threadIdx.x) * N + k);
  }
  block_reduce<N, 0xffffffffu, R>(b, scratch);
  if (threadIdx.x == 0) {
    cnt[grp] = 0u;
#pragma unroll
    for (int k = 0; k < N; ++k) gpartials[(size_t)grp * N + k] = acc_store(b[k]);
    __threadfence();
    s_last = atomicAdd(&cnt[ngroups], 1u) == (unsigned)ngroups - 1u;
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  Acc<R> c[N] = {};
  for (int i = threadIdx.x; i < ngroups; i += blockDim.x) {
#pragma unroll
    for (int k = 0; k < N; ++k) c[k].add(acc_load<R>(gpartials + (size_t)i * N + k));
  }
  block_reduce<N, 0xffffffffu, R>(c, scratch);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) total[k] = c[k].value();
    cnt[ngroups] = 0u;
  }
  return true;
}

// Write this block's N partials; return true in the last block to finish,
// in which `total` (thread 0 only) holds the fixed-order sums over all
// `nblocks` partials.  Resets the counter for the next launch.
template <int N, unsigned FF, class R>
__device__ __forceinline__ bool grid_reduce_masked(Acc<R> (&a)[N], AccStore<R>* partials,
                                                   unsigned* counter, int nblocks, Acc<R>* scratch,
                                                   double (&total)[N]) {
  __shared__ bool s_last;
  block_reduce<N, FF, R>(a, scratch);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) partials[(size_t)blockIdx.x * N + k] = acc_store(a[k]);
    __threadfence();
    const unsigned prev = atomicAdd(counter, 1u);
    s_last = (prev == (unsigned)nblocks - 1u);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  Acc<R> b[N] = {};
#pragma unroll 2
  for (int blk = threadIdx.x; blk < nblocks; blk += blockDim.x) {
    Acc<R> v[N];
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = acc_load<R>(partials + (size_t)blk * N + k);
#pragma unroll
    for (int k = 0; k < N; ++k) b[k].add(v[k]);
  }
  block_reduce<N, 0xffffffffu, R>(b, scratch);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) total[k] = b[k].value();
    *counter = 0u;
  }
  return true;
}

// grid_reduce_masked, and the last block also copies `words` 32-bit words of
// `src` (the solver's scalar state) into shared `dst` in the same round trip
// as the partials, so that its scalar logic reads shared memory instead of
// making one dependent global load per field.  `dst` is complete in every
// thread of the last block on return.
template <int N, unsigned FF, class R>
__device__ __forceinline__ bool grid_reduce_masked_state(Acc<R> (&a)[N], AccStore<R>* partials,
                                                         unsigned* counter, int nblocks, Acc<R>* scratch,
                                                         double (&total)[N], const uint32_t* src,
                                                         uint32_t* dst, int words) {
  __shared__ bool s_last;
  block_reduce<N, FF, R>(a, scratch);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) partials[(size_t)blockIdx.x * N + k] = acc_store(a[k]);
    __threadfence();
    const unsigned prev = atomicAdd(counter, 1u);
    s_last = (prev == (unsigned)nblocks - 1u);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  uint32_t w = 0;
  if ((int)threadIdx.x < words) w = __ldcg(src + threadIdx.x);
  Acc<R> b[N] = {};
#pragma unroll 2
  for (int blk = threadIdx.x; blk < nblocks; blk += blockDim.x) {
    Acc<R> v[N];
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = acc_load<R>(partials + (size_t)blk * N + k);
#pragma unroll
    for (int k = 0; k < N; ++k) b[k].add(v[k]);
  }
  if ((int)threadIdx.x < words) dst[threadIdx.x] = w;
  block_reduce<N, 0xffffffffu, R>(b, scratch);  // ends with a barrier: dst is complete
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) total[k] = b[k].value();
    *counter = 0u;
  }
  return true;
}

template <int N, class R>
__device__ __forceinline__ bool grid_reduce(Acc<R> (&a)[N], AccStore<R>* partials, unsigned* counter,
                                            int nblocks, Acc<R>* scratch, double (&total)[N]) {
  return grid_reduce_masked<N, 0xffffffffu, R>(a, partials, counter, nblocks, scratch, total);
}

// Sum a range of stored partials inside one block (thread 0 gets the value).
template <class R>
__device__ __forceinline__ double block_sum_partials(const AccStore<R>* partials, int n, int stride,
                                                     Acc<R>* scratch) {
  Acc<R> b[1] = {};
  for (int i = threadIdx.x; i < n; i += blockDim.x) b[0].add(acc_load<R>(partials + (size_t)i * stride));
  block_reduce<1, 0xffffffffu, R>(b, scratch);
  return b[0].value();
}

}  // namespace agb
