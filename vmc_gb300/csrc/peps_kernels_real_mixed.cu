// peps_kernels_real_mixed.cu -- the mixed-precision fused kernel: real
// elements, the boundary-MPS chain (zip-up, truncation, stored boundary
// tensors) in FP64 (chain_f64.cuh), environments, Metropolis, gradients and
// energies in FP32.  The kernel of plans created with VMC_PRECISION_MIXED; a
// translation unit of its own so the FP32 kernels keep their code generation.
#define VMC_CHAIN_F64 1
#include "peps_plan.cuh"

namespace vmc {
namespace rm {
constexpr bool kCplx = false;
constexpr int kEs = 1;
#include "peps_device.cuh"
#include "peps_launch.cuh"
}  // namespace rm
}  // namespace vmc
