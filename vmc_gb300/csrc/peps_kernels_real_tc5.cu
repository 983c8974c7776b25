// peps_kernels_real_tc5.cu -- the real FP32 fused kernel with its large CTA GEMMs (M >= 64, N >= 16,
// K >= 16, M N K >= 2^17) on the 5th-generation tensor cores: tcgen05.mma kind::tf32 in the 3xTF32 split
// (FP32 accuracy), operands staged in shared memory, accumulators in tensor memory.  The kernel of plans
// with tile_policy 4; a translation unit of its own so the other kernels keep their code generation.
#define VMC_GEMM_TCGEN05 1
#include "peps_plan.cuh"

namespace vmc {
namespace rq {
constexpr bool kCplx = false;
constexpr int kEs = 1;
#include "peps_device.cuh"
#include "peps_launch.cuh"
}  // namespace rq
}  // namespace vmc
