// peps_kernels_gi.cu -- the gauge-invariant plans' fused kernel (gi_device.cuh) and its launchers,
// for real FP32 and complex64 elements: a translation unit of its own, so that the standard kernels
// keep their code generation.
#define VMC_GI_TU 1
#include "peps_plan.cuh"

namespace vmc {
namespace gr {
constexpr bool kCplx = false;
constexpr int kEs = 1;
#include "peps_device.cuh"
#include "peps_launch.cuh"
}  // namespace gr
namespace gc {
constexpr bool kCplx = true;
constexpr int kEs = 2;
#include "peps_device.cuh"
#include "peps_launch.cuh"
}  // namespace gc
}  // namespace vmc
