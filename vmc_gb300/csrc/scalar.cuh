// scalar.cuh -- scalar helpers that let the CTA linear-algebra routines run in
// FP32 (the plain engine) or FP64 (the boundary-MPS chain of mixed-precision
// plans) from one template.  Each overload maps to the native instruction of
// its type; the FP32 overloads are the ones the FP32 code always used.
#pragma once

#include "portability.cuh"

namespace vmc {

__device__ __forceinline__ float vfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double vfma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float vsqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ double vsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ float vabs(float a) { return fabsf(a); }
__device__ __forceinline__ double vabs(double a) { return fabs(a); }
__device__ __forceinline__ float vcopysign(float a, float b) { return copysignf(a, b); }
__device__ __forceinline__ double vcopysign(double a, double b) { return copysign(a, b); }
__device__ __forceinline__ float vmax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double vmax(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ float vmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double vmin(double a, double b) { return fmin(a, b); }
// quotient inside the Sturm recurrence: the fast approximate divide in FP32
__device__ __forceinline__ float vfdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double vfdiv(double a, double b) { return a / b; }

// Tolerances of the eigensolver per precision (relative to the unit roundoff).
template <typename T>
struct Tol;
template <>
struct Tol<float> {
  static constexpr float big = 3.4e38f;          // larger than any value
  static constexpr float bisect_rtol = 2.5e-7f;  // relative width of a converged bisection interval
  static constexpr int bisect_iter_scale = 1;    // multisection rounds: base count times this
  static constexpr float inv_tiny = 1.2e-7f;     // smallest pivot of inverse iteration, relative to |T|
  static constexpr float chol_min = 1e-10f;      // CholQR gives up below this diagonal
  static constexpr float cluster = 1e-3f;        // eigenvalues closer than this * |T| form a cluster
  static constexpr int inv_iters = 2;            // inverse-iteration steps per eigenvector
};
template <>
struct Tol<double> {
  static constexpr double big = 1.7e308;
  static constexpr double bisect_rtol = 4e-16;
  static constexpr int bisect_iter_scale = 2;
  static constexpr double inv_tiny = 2.3e-16;
  static constexpr double chol_min = 1e-24;
  static constexpr double cluster = 1e-6;
  static constexpr int inv_iters = 2;
};

// lane exchange of a value of any of the scalar types (identity in the host build)
__device__ __forceinline__ float shfl_xor_t(unsigned mask, float v, int o, int width = 32) {
#ifndef VMC_HOST_EMULATION
  return __shfl_xor_sync(mask, v, o, width);
#else
  (void)mask; (void)o; (void)width;
  return v;
#endif
}
__device__ __forceinline__ double shfl_xor_t(unsigned mask, double v, int o, int width = 32) {
#ifndef VMC_HOST_EMULATION
  return __shfl_xor_sync(mask, v, o, width);
#else
  (void)mask; (void)o; (void)width;
  return v;
#endif
}

__device__ __forceinline__ float warp_sum_t(float v) {
#ifndef VMC_HOST_EMULATION
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
#endif
  return v;
}
__device__ __forceinline__ double warp_sum_t(double v) {
#ifndef VMC_HOST_EMULATION
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
#endif
  return v;
}

}  // namespace vmc
