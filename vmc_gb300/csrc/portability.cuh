// portability.cuh -- lets the engine's device code also compile as plain C++.
//
// The production build is nvcc for sm_103a.  With VMC_HOST_EMULATION defined
// the same sources compile with g++ into a host library in which every CTA
// runs with a single thread (blockDim.x == 1): barriers become no-ops and
// warp shuffles become identities.  That build exists only so the CPU test
// suite can check the engine's index maps and control flow against the
// oracle; the Python package never loads it.
#pragma once

#ifdef VMC_HOST_EMULATION

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __noinline__
#define __grid_constant__
#define __align__(n) __attribute__((aligned(n)))
#define __restrict__
#define __launch_bounds__(...)
#define VMC_SHARED static
using std::isfinite;

struct vmc_dim3 {
  unsigned x = 0, y = 0, z = 0;
};
extern thread_local vmc_dim3 threadIdx, blockIdx, blockDim, gridDim;

inline void __syncthreads() {}
inline void __syncwarp(unsigned = 0xffffffffu) {}
inline float __shfl_xor_sync(unsigned, float v, int, int = 32) { return v; }
inline double __shfl_xor_sync(unsigned, double v, int, int = 32) { return v; }
inline unsigned __ballot_sync(unsigned, int pred) { return pred ? 1u : 0u; }
inline int __popc(unsigned v) { return __builtin_popcount(v); }
inline float __shfl_sync(unsigned, float v, int, int = 32) { return v; }
inline int __shfl_sync(unsigned, int v, int, int = 32) { return v; }
inline float __fdividef(float a, float b) { return a / b; }
inline int atomicOr(int* p, int v) {
  int o = *p;
  *p |= v;
  return o;
}
inline int atomicAdd(int* p, int v) {
  int o = *p;
  *p += v;
  return o;
}
inline double atomicAdd(double* p, double v) {
  double o = *p;
  *p += v;
  return o;
}
typedef void* cudaStream_t;
typedef int cudaError_t;
#define cudaSuccess 0

#define VMC_LAUNCH(kernel, grid, block, smem, stream, ...)            \
  do {                                                                \
    gridDim.x = (unsigned)(grid);                                     \
    blockDim.x = 1;                                                   \
    threadIdx.x = 0;                                                  \
    for (unsigned _b = 0; _b < (unsigned)(grid); ++_b) {              \
      blockIdx.x = _b;                                                \
      kernel(__VA_ARGS__);                                            \
    }                                                                 \
  } while (0)

inline cudaError_t vmc_alloc(void** p, size_t n) {
  *p = std::malloc(n ? n : 1);
  return *p ? 0 : 1;
}
inline void vmc_free(void* p) { std::free(p); }
inline cudaError_t vmc_h2d(void* dst, const void* src, size_t n, cudaStream_t) {
  std::memcpy(dst, src, n);
  return 0;
}
inline cudaError_t vmc_d2h(void* dst, const void* src, size_t n, cudaStream_t) {
  std::memcpy(dst, src, n);
  return 0;
}
inline cudaError_t vmc_memset(void* dst, int v, size_t n, cudaStream_t) {
  std::memset(dst, v, n);
  return 0;
}
inline cudaError_t vmc_last_error() { return 0; }
inline cudaError_t vmc_sync(cudaStream_t) { return 0; }
inline int vmc_num_sms() { return 4; }

#else  // CUDA build

#include <cuda_runtime.h>

#define VMC_SHARED __shared__

#define VMC_LAUNCH(kernel, grid, block, smem, stream, ...) \
  kernel<<<(grid), (block), (smem), (cudaStream_t)(stream)>>>(__VA_ARGS__)

inline cudaError_t vmc_alloc(void** p, size_t n) { return cudaMalloc(p, n ? n : 1); }
inline void vmc_free(void* p) { cudaFree(p); }
inline cudaError_t vmc_h2d(void* dst, const void* src, size_t n, cudaStream_t s) {
  return cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, s);
}
inline cudaError_t vmc_d2h(void* dst, const void* src, size_t n, cudaStream_t s) {
  return cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, s);
}
inline cudaError_t vmc_memset(void* dst, int v, size_t n, cudaStream_t s) {
  return cudaMemsetAsync(dst, v, n, s);
}
inline cudaError_t vmc_last_error() { return cudaGetLastError(); }
inline cudaError_t vmc_sync(cudaStream_t s) { return cudaStreamSynchronize(s); }
inline int vmc_num_sms() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

#endif
