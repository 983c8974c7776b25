// phase_timers.cuh -- optional per-phase cycle counters for profiling the
// fused kernel (build with -DVMC_PHASE_TIMERS; compiled out otherwise).
#pragma once

#include "portability.cuh"

namespace vmc {

// Optional per-phase cycle counters (build with -DVMC_PHASE_TIMERS); thread 0
// of every CTA accumulates clock64() deltas.  Off in the product build.
enum Phase { PH_T_RENV = 0, PH_T_METRO, PH_T_ZIP, PH_JACOBI, PH_E_RENV, PH_E_LEFT, PH_E_VERT, PH_B_ZIP, PH_CHAIN,
             PH_GRAM, PH_TRIDIAG, PH_BISECT, PH_INVIT, PH_CHOLQR, PH_BACK, PH_CARRY, PH_V_RIGHT, PH_V_LEFT,
             PH_THETA, PH_COUNT };
#if defined(VMC_PHASE_TIMERS) && !defined(VMC_HOST_EMULATION)
static __device__ unsigned long long g_phase[PH_COUNT];
#define VMC_TSTART(v) long long v = clock64()
#define VMC_TSTOP(v, ph) \
  do { if (threadIdx.x == 0) atomicAdd(&g_phase[ph], (unsigned long long)(clock64() - (v))); } while (0)
#elif defined(VMC_PHASE_TIMERS) && defined(VMC_HOST_EMULATION)
}  // namespace vmc
#include <chrono>
namespace vmc {
static unsigned long long g_phase[PH_COUNT];
inline long long host_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch()).count();
}
#define VMC_TSTART(v) long long v = host_ns()
#define VMC_TSTOP(v, ph) (g_phase[ph] += (unsigned long long)(host_ns() - (v)))
#else
#define VMC_TSTART(v) (void)0
#define VMC_TSTOP(v, ph) (void)0
#endif

}  // namespace vmc
