// CUDA helpers shared by the device translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <vector>

#include "topt_internal.h"

#define TOPT_CUDA(call)                                              \
  do {                                                               \
    cudaError_t e_ = (call);                                         \
    if (e_ != cudaSuccess) return topt::fail_cuda((int)e_, #call);   \
  } while (0)

#define TOPT_CHECK_LAUNCH(name)                                      \
  do {                                                               \
    cudaError_t e_ = cudaGetLastError();                             \
    if (e_ != cudaSuccess) return topt::fail_cuda((int)e_, name);    \
  } while (0)

namespace topt {

// Launch counter of this translation unit's kernels: thread 0 of block 0 of
// every launch increments it; topt_launch_count() sums the units.
static __device__ unsigned long long g_kernel_launches;
#define TOPT_KERNEL_COUNT()                                              \
  do {                                                                   \
    if (blockIdx.x == 0 && threadIdx.x == 0)                             \
      atomicAdd(&topt::g_kernel_launches, 1ull);                         \
  } while (0)

// Number of SMs of the current device (GB300: 152), queried once per call site.
int device_sm_count();

// Owning device allocation.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  int alloc(size_t n) {
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      p = nullptr;
      return fail(TOPT_NO_MEMORY, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
    }
    bytes = n;
    return TOPT_OK;
  }
  template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

template <typename T>
int upload(DevBuf& b, const T* host, size_t n, cudaStream_t s) {
  int rc = b.alloc(n * sizeof(T));
  if (rc) return rc;
  if (n) TOPT_CUDA(cudaMemcpyAsync(b.p, host, n * sizeof(T), cudaMemcpyHostToDevice, s));
  return TOPT_OK;
}

inline int grid_for(int64_t n, int block, int cap = 1 << 30) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

// Warp sum of a value.
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// Deterministic block sum of L values per thread (blockDim.x multiple of 32,
// <= 1024).  Result valid in thread 0.  `sh` needs 32*L elements.
template <typename T, int L>
__device__ __forceinline__ void block_sum(T (&v)[L], T* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
#pragma unroll
  for (int j = 0; j < L; ++j) v[j] = warp_sum(v[j]);
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < L; ++j) sh[wid * L + j] = v[j];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int j = 0; j < L; ++j) {
      T x = lane < nw ? sh[lane * L + j] : T(0);
      v[j] = warp_sum(x);
    }
  }
  __syncthreads();
}

// Deterministic cross-block finish: every block stores its L partials; the
// last block to arrive sums them (fixed thread-strided assignment, then the
// fixed block tree: the same order every call) into out[0..L) and re-arms
// the counter.  Call from all threads after block_sum (partials in thread 0).
template <typename T, int L>
__device__ __forceinline__ bool grid_finish(T (&v)[L], T* partials, unsigned* counter,
                                            T* out) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < L; ++j) partials[blockIdx.x * L + j] = v[j];
    __threadfence();
    unsigned t = atomicAdd(counter, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // the whole last block sums the partials: thread-strided partial sums (the
  // L2 loads of a thread are independent and issued back to back), then the
  // fixed block tree
  T acc[L];
#pragma unroll
  for (int j = 0; j < L; ++j) acc[j] = T(0);
  const int nb = (int)gridDim.x;
  int b = threadIdx.x;
  for (; b + 3 * (int)blockDim.x < nb; b += 4 * blockDim.x) {
    T v[4][L];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int j = 0; j < L; ++j) v[u][j] = __ldcg(partials + (b + u * blockDim.x) * L + j);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int j = 0; j < L; ++j) acc[j] += v[u][j];
  }
  for (; b < nb; b += blockDim.x) {
#pragma unroll
    for (int j = 0; j < L; ++j) acc[j] += __ldcg(partials + b * L + j);
  }
  __shared__ T shf[32 * L];
  block_sum<T, L>(acc, shf);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < L; ++j) out[j] = acc[j];
    *counter = 0u;
  }
  return true;
}

// Cross-block maximum of non-negative values, NaN-propagating (a NaN in any
// block gives NaN): call from all threads with the thread's running maximum
// m and NaN flag; the last block to arrive combines the block maxima with
// all its threads and writes *out (max is order-free, so the result is
// deterministic) and re-arms the counter.
__device__ __forceinline__ void grid_max_finish(double m, bool nan, double* partials,
                                                unsigned* counter, double* out) {
  __shared__ double shm[32];
  __shared__ int anynan;
  __shared__ bool last;
  if (threadIdx.x == 0) anynan = 0;
  __syncthreads();
  if (nan) anynan = 1;
  double v = warp_max(m);
  if ((threadIdx.x & 31) == 0) shm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double u = threadIdx.x < (int)(blockDim.x >> 5) ? shm[threadIdx.x] : 0.0;
    u = warp_max(u);
    if (threadIdx.x == 0) {
      partials[blockIdx.x] = anynan ? NAN : u;
      __threadfence();
      last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double r = 0.0;
  bool bad = false;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    const double pv = __ldcg(partials + b);
    if (pv != pv) bad = true;
    r = pv > r ? pv : r;
  }
  __syncthreads();   // shm / anynan reuse
  if (threadIdx.x == 0) anynan = 0;
  __syncthreads();
  if (bad) anynan = 1;
  v = warp_max(r);
  if ((threadIdx.x & 31) == 0) shm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double u = threadIdx.x < (int)(blockDim.x >> 5) ? shm[threadIdx.x] : 0.0;
    u = warp_max(u);
    if (threadIdx.x == 0) {
      *out = anynan ? NAN : u;
      *counter = 0u;
    }
  }
}

}  // namespace topt
