// uniforms.cu -- counter-based uniform draws for the Metropolis accept tests
// of a TDVP step that runs as one CUDA graph.
//
// The reference splits a JAX key per accept test (kernels.py:189-190); the
// engine takes explicit uniforms instead.  A captured graph replays its
// kernels with the arguments it was captured with, so the draw counter lives
// in device memory: every call fills out[0..n) from (seed, *counter) and then
// increments *counter, and each replay draws fresh numbers.  Eager and
// replayed calls with the same (seed, counter) draw the same numbers.
//
// Generator: SplitMix64 (Steele, Lea, Flood, "Fast splittable pseudorandom
// number generators", OOPSLA 2014).  The stream key is
// mix(seed + (counter + 1) * gamma) and draw i is the top 53 bits of
// mix(key + (i + 1) * gamma) times 2^-53, with mix the SplitMix64 output
// function and gamma = 0x9E3779B97F4A7C15.
#include <cstdint>

#include "portability.cuh"
#include "../../include/vmc_gb300.h"

namespace vmc {
namespace rng {

constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ull;

__device__ __host__ inline uint64_t mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void fill_kernel(double* out, long long n, uint64_t seed, const uint64_t* counter) {
  const uint64_t key = mix(seed + (*counter + 1) * kGamma);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (double)(mix(key + (uint64_t)(i + 1) * kGamma) >> 11) * (1.0 / 9007199254740992.0);
}

__global__ void bump_kernel(uint64_t* counter) {
  if (blockIdx.x == 0 && threadIdx.x == 0) *counter += 1;
}

}  // namespace rng
}  // namespace vmc

extern "C" vmc_status vmc_uniforms(void* stream, double* out, int64_t n, uint64_t seed, uint64_t* counter) {
  if (n < 0 || !counter || (n > 0 && !out)) return VMC_ERR_INVALID;
  if (n > 0) {
    const long long blocks = (n + 255) / 256;
    VMC_LAUNCH(vmc::rng::fill_kernel, (int)(blocks < 4096 ? blocks : 4096), 256, 0, stream, out, (long long)n, seed,
               counter);
  }
  VMC_LAUNCH(vmc::rng::bump_kernel, 1, 32, 0, stream, counter);
  return vmc_last_error() == cudaSuccess ? VMC_OK : VMC_ERR_CUDA;
}
