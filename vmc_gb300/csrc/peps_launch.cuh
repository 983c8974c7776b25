// peps_launch.cuh -- the launchers of one element type's kernels, exported to
// the host code as a KernelSet (included inside namespace vmc::rk or vmc::ck,
// after peps_device.cuh).

static cudaError_t launch_permute(const DevPlan* dplan, int n_sites, const float* tensors, float* perm,
                                  void* stream) {
  VMC_LAUNCH(permute_tensors_kernel, std::min(n_sites, 1024), kThreads, 0, stream, dplan, tensors, perm);
  return vmc_last_error();
}

#ifdef VMC_GI_TU
#define VMC_FUSED_KERNEL gi_kernel
#else
#define VMC_FUSED_KERNEL peps_kernel
#endif

static cudaError_t opt_in_smem(size_t smem) {
#ifndef VMC_HOST_EMULATION
  // static (~5 KB) + dynamic shared memory may exceed the 48 KB default: always opt in
  if (smem > 0)
    return cudaFuncSetAttribute(VMC_FUSED_KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
#endif
  (void)smem;
  return cudaSuccess;
}

static cudaError_t prepare_peps(int threads, size_t smem, int* per_sm) {
  const cudaError_t e = opt_in_smem(smem);
  if (e != cudaSuccess) return e;
#ifdef VMC_HOST_EMULATION
  (void)threads;
  *per_sm = 4;
  return cudaSuccess;
#else
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, VMC_FUSED_KERNEL, threads, smem);
#endif
}

static cudaError_t launch_peps(const BatchJobs& jobs, int grid, int threads, size_t smem, void* stream,
                               float* slots, int32_t* next, int32_t* status) {
  const cudaError_t e = opt_in_smem(smem);
  if (e != cudaSuccess) return e;
  VMC_LAUNCH(VMC_FUSED_KERNEL, grid, threads, smem, stream, jobs, slots, next, status);
  return vmc_last_error();
}

const KernelSet& kernels() {
  static const KernelSet k{&launch_permute, &prepare_peps, &launch_peps};
  return k;
}

#undef VMC_FUSED_KERNEL
