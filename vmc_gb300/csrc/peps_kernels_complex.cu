// peps_kernels_complex.cu -- the fused kernel (peps_device.cuh) and its
// launchers for complex64 elements, stored as interleaved (re, im) floats.
#include "peps_plan.cuh"

namespace vmc {
namespace ck {
constexpr bool kCplx = true;
constexpr int kEs = 2;
#include "peps_device.cuh"
#include "peps_launch.cuh"
}  // namespace ck
}  // namespace vmc
