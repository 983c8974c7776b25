// peps_kernels_real_tc.cu -- the real FP32 fused kernel with its CTA GEMMs of at least 16 x 8 x 8 on the
// tensor cores (3xTF32 mma.sync, FP32 accuracy): the kernel of plans with tile_policy 3.  A translation
// unit of its own, so that the default kernel keeps its code generation (registers, spills) and these
// GEMMs stay inlined, with their index maps specialised, at every call site.
#define VMC_GEMM_TENSOR_CORES 1
#include "peps_plan.cuh"

namespace vmc {
namespace rt {
constexpr bool kCplx = false;
constexpr int kEs = 1;
#include "peps_device.cuh"
#include "peps_launch.cuh"
}  // namespace rt
}  // namespace vmc
