// peps_kernels_real.cu -- the fused kernel (peps_device.cuh) and its launchers
// for real FP32 elements.  The complex64 build is peps_kernels_complex.cu; the
// two compile in parallel.
#include "peps_plan.cuh"

namespace vmc {
namespace rk {
constexpr bool kCplx = false;
constexpr int kEs = 1;
#include "peps_device.cuh"
#include "peps_launch.cuh"
}  // namespace rk
}  // namespace vmc

#ifdef VMC_PHASE_TIMERS
// Debug-only (not part of the product ABI): read and reset the phase counters
// of the real-element kernel.
extern "C" int vmc_debug_phase_timers(unsigned long long* host_out) {
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
