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

#ifdef VMC_PHASE_TIMERS
// Debug-only (not part of the product ABI): read and reset the phase counters
// of the mixed-precision kernel.
extern "C" int vmc_debug_phase_timers_mixed(unsigned long long* host_out) {
  using namespace vmc;
#ifdef VMC_HOST_EMULATION
  for (int i = 0; i < PH_COUNT; ++i) { host_out[i] = g_phase[i]; g_phase[i] = 0; }
  return PH_COUNT;
#else
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return -(int)e;
  e = cudaMemcpyFromSymbol(host_out, g_phase, sizeof(unsigned long long) * PH_COUNT);
  if (e != cudaSuccess) return -1000 - (int)e;
  unsigned long long z[PH_COUNT] = {0};
  e = cudaMemcpyToSymbol(g_phase, z, sizeof(z));
  if (e != cudaSuccess) return -2000 - (int)e;
  return PH_COUNT;
#endif
}
#endif
