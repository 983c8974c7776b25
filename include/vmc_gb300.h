/*
 * vmc_gb300.h -- C ABI of the GB300 (sm_103a) PEPS evaluation engine.
 *
 * Plain C: pointers, sizes and integer status codes; no CUDA, torch or JAX
 * types cross this boundary.  Device pointers are CUDA device addresses;
 * `stream` is a cudaStream_t passed as void*.  Every compute entry point is
 * stream-ordered and allocates nothing: the caller owns all buffers and
 * passes a workspace sized by vmc_workspace_size().  A call over zero chains
 * (n == 0) returns VMC_OK and reads or writes none of its buffers, which may
 * then be null (vmc_peps_vjp still zeroes out_grad: a sum over no samples).
 * Configuration values index the site tensors on the device unchecked: they
 * must lie in [0, d) (gauge links of a GI plan in [0, N)); the Python layer
 * (vmc_gb300.engine) refuses others before it launches.
 *
 * The entry points replace, for a batch of chains, the reference's PEPS
 * kernels (fliingelephant/VMC, Python/JAX):
 *   - vmc_peps_plan / vmc_peps_plan_set_operator: the static closure built by
 *     build_mc_kernels (src/vmc/peps/standard/kernels.py:91-114) -- shape,
 *     strategy, params_per_site and bucket_terms(operator.terms)
 *     (src/vmc/operators/local_terms.py:165-200);
 *   - vmc_peps_init_cache: init_cache (kernels.py:115-129);
 *   - vmc_peps_sweep: one make_mc_sampler step, i.e. vmap(transition then
 *     estimate) over chains (src/vmc/core/sampling.py:28-38,
 *     kernels.py:131-245), fused into one launch;
 *   - vmc_peps_amp_grad: _value_and_grad / peps_apply forward + hand-written
 *     adjoint (src/vmc/peps/standard/compat.py:31-64,94-133);
 *   - vmc_peps_local_energy: local_estimate (compat.py:136-194).
 *
 * Numerics: FP32 contractions with FP64 log-scales and FP64 energy
 * accumulation.  Amplitudes are returned as (log|psi|, sign); log-derivatives
 * O_k = dpsi/dA / psi are returned directly, so nothing underflows.
 *
 * Complex plans (VMC_DTYPE_C64, complex64 site tensors as in the reference's
 * complex PEPS): every complex array is interleaved (re, im) -- the packed
 * tensors and out_O as float pairs, out_E as double pairs, the operator
 * tables of vmc_peps_plan_set_operator as double pairs -- and the "sign"
 * arrays hold the phase of psi in radians (psi = exp(logamp + i phase)).
 */
#ifndef VMC_GB300_H_
#define VMC_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int vmc_status;

enum {
  VMC_OK = 0,
  VMC_ERR_INVALID = 1,     /* bad shape / dimension / null pointer */
  VMC_ERR_UNSUPPORTED = 2, /* valid request the engine does not implement */
  VMC_ERR_WORKSPACE = 3,   /* workspace smaller than vmc_workspace_size() */
  VMC_ERR_CUDA = 4,        /* a CUDA runtime call failed */
  VMC_ERR_NONFINITE = 5,   /* device status word reported NaN/Inf */
  VMC_ERR_TIMEOUT = 6,     /* a bounded device wait gave up */
  VMC_ERR_SCRATCH = 7      /* plan needs more than the fixed scratch of vmc_peps_amp_grad_noalloc */
};

/* dtype of the site tensors: real FP32, or complex64 (FP32 real and imaginary parts). */
enum { VMC_DTYPE_F32 = 0, VMC_DTYPE_C64 = 1 };

/* Boundary-MPS strategy: strategy.py:44-92. */
enum {
  VMC_STRATEGY_NO_TRUNCATION = 0,
  VMC_STRATEGY_ZIP_UP = 1,
  VMC_STRATEGY_DENSITY_MATRIX = 2,
  VMC_STRATEGY_VARIATIONAL = 3
};

/* Device status word bits (written by kernels, read with cudaMemcpy). */
enum { VMC_DEV_NONFINITE = 1, VMC_DEV_TIMEOUT = 2 };

typedef struct vmc_shape {
  int n_rows;
  int n_cols;
} vmc_shape;

typedef struct vmc_plan vmc_plan;

/* Version and error strings. */
const char* vmc_version(void);
const char* vmc_status_string(vmc_status s);

/*
 * Create an immutable plan for an open-boundary n_rows x n_cols PEPS with
 * bond dimension `bond_dim`, physical dimension `phys_dim` and boundary
 * bond `chi` (truncate_bond_dimension).  `n_sweeps` is used by the
 * variational strategy only.  Replaces the closure of
 * build_mc_kernels (kernels.py:104-113) and PEPS.site_dims (model.py:27-35).
 */
vmc_status vmc_peps_plan(const vmc_shape* shape, int bond_dim, int chi, int phys_dim,
                         int dtype, int strategy, int n_sweeps, vmc_plan** out_plan);

/* Arithmetic of a plan (vmc_plan_options.precision). */
enum {
  /* every contraction, truncation and stored tensor in FP32 */
  VMC_PRECISION_FP32 = 0,
  /* the boundary-MPS chain -- zip-up theta, its truncation and the stored
   * boundary tensors that feed the next row's zip -- in double-float (pairs
   * of FP32 values, ~48 significant bits, on the FP32 units; the
   * eigenvalues' refinement and inverse iteration in FP64); environments,
   * Metropolis ratios, gradients and energies in FP32.  Real ZipUp,
   * DensityMatrix and NoTruncation plans.  Truncated amplitudes are
   * ill-conditioned (the kept subspace moves by the relative error of the
   * decomposition divided by the relative singular-value gap at the cut), so
   * an FP32 truncation puts the batch-mean energy ~6e-5 of the energy scale
   * off the FP64 result at 8x8, D=4, chi=16; this tier brings it to ~1e-7. */
  VMC_PRECISION_MIXED = 1
};

/*
 * Options of a plan -- the launch configuration the autotuner
 * (vmc_gb300.autotune) picks per (lattice, D, chi, dtype, strategy), and the
 * arithmetic.  No reference counterpart (XLA picks its own kernels).  A
 * zero-initialised struct except smem_kb = -1 gives the defaults, which is
 * what vmc_peps_plan uses; nothing is read from the environment.
 *   threads      CTA size, a multiple of 32 in [64, 256]; 0: 128
 *   smem_kb      dynamic shared memory per CTA for the truncation arena and
 *                the 1-row intermediates, 0..52 KB (FP32) or 0..200 KB
 *                (mixed precision); -1: the precision's default (0: all in
 *                the CTA's workspace slot, L1-cached)
 *   tile_policy  register tiles of the CTA GEMMs: 0 default, 1 smaller, 2 larger, 3 real GEMMs of at
 *                least 16 x 8 x 8 on the tensor cores (3xTF32, FP32 accuracy; faster from D = 6, chi = 36
 *                on), the rest as 0
 *   precision    VMC_PRECISION_FP32 or VMC_PRECISION_MIXED
 *   trunc_method 0: Gram matrix + tridiagonal eigensolver; 1: one-sided
 *                Jacobi on theta (real FP32 plans; a cross-check of 0)
 *   vchunk       bond values per vertical-energy chunk; 0: all at once
 *   vert_smem    1: vertical-energy buffers in the shared-memory arena,
 *                chunked to fit; 0: in the workspace slot
 * Every choice but precision computes the same quantities and differs in
 * FP32 rounding only (GEMM and reduction order).
 */
typedef struct {
  int threads;
  int smem_kb;
  int tile_policy;
  int precision;
  int trunc_method;
  int vchunk;
  int vert_smem;
} vmc_plan_options;
vmc_status vmc_peps_plan_ex(const vmc_shape* shape, int bond_dim, int chi, int phys_dim, int dtype,
                            int strategy, int n_sweeps, const vmc_plan_options* options,
                            vmc_plan** out_plan);

/*
 * Attach the bucketed LocalHamiltonian (local_terms.py:165-200).  Terms of
 * the same kind and location are summed by the caller.  All arrays are HOST
 * arrays of float64, copied into the plan:
 *   onesite[n_rows*n_cols][d][d], onesite_mask[n_rows*n_cols]
 *   horiz[n_rows*(n_cols-1)][d*d][d*d], horiz_mask[...]
 *   vert[(n_rows-1)*n_cols][d*d][d*d], vert_mask[...]
 *   diagonal terms: n_diag terms; term t touches diag_nsites[t] sites listed
 *   (row-major site ids) in diag_sites[diag_site_off[t] ...] and its table of
 *   d^diag_nsites[t] values starts at diag_values[diag_value_off[t]].
 * The local-energy convention is the reference's: an off-diagonal term adds
 * sum_j op[j, s] psi(j) / psi (energy.py:176-200).  For a complex plan the
 * onesite / horiz / vert tables hold (re, im) double pairs per element;
 * diagonal tables stay real.
 */
vmc_status vmc_peps_plan_set_operator(vmc_plan* plan,
                                      const double* onesite, const int* onesite_mask,
                                      const double* horiz, const int* horiz_mask,
                                      const double* vert, const int* vert_mask,
                                      int n_diag, const int* diag_nsites,
                                      const int* diag_site_off, const int* diag_sites,
                                      const int* diag_value_off, const double* diag_values);

/*
 * Gauge-invariant PEPS for pure Z_N lattice gauge theory (phys_dim = 1):
 * GIPEPS / GIPEPSConfig of src/vmc/peps/gi/model.py:41-119 with equal
 * degeneracy per charge (bond dimension dmax per sector), and its kernels
 * (src/vmc/peps/gi/kernels.py:17-126).  The plan is a standard plan whose
 * "physical" index is a site's gauge configuration (its slice,
 * model.py:308-347): phys_dim = the largest count N^(links - 1).  The site
 * tensors are packed as (slice, up, down, left, right) per site, slices past a
 * site's own count zero.  With a GI plan the calls above take:
 *   configs[n][n_state] int32, n_state = R*C + R*(C-1) + (R-1)*C: the
 *     flattened (sites, h links, v links) sample (model.py:121-144), sites 0;
 *   uniforms[n][(R-1)*(C-1)] and deltas[n][(R-1)*(C-1)] (in [1, N), NULL for
 *     N = 2): the per-plaquette accept draws and flip offsets of the
 *     plaquette sweep (model.py:629-703, 901-957);
 *   out_p: the slice index of every parameter (kernels.py:101-118);
 *   out_E: link-diagonal plus plaquette energies (model.py:392-617).
 * Slices per site are at most 27 (N <= 3); larger N returns VMC_ERR_UNSUPPORTED.
 * vmc_gi_set_operator: host FP64 arrays hdiag[R*(C-1)][N], vdiag[(R-1)*C][N]
 * (energy of a link with value k: LinkDiagonalTerm, gi/local_terms.py:12-39)
 * and plaq[(R-1)*(C-1)] (coefficient of P + P^dag, PlaquetteTerm).
 */
vmc_status vmc_gi_plan(const vmc_shape* shape, int N, int dmax, int chi, int dtype, int strategy,
                       int n_sweeps, const vmc_plan_options* options, vmc_plan** out_plan);
vmc_status vmc_gi_set_operator(vmc_plan* plan, const double* hdiag, const double* vdiag,
                               const double* plaq);

void vmc_plan_destroy(vmc_plan* plan);

/* Number of parameters per sample of the sliced log-derivative (sum of
 * params_per_site, src/vmc/utils/smallo.py:23-35) and of the full tensors. */
int64_t vmc_peps_n_params_sliced(const vmc_plan* plan);
int64_t vmc_peps_n_params_full(const vmc_plan* plan);

/* Chains a launch runs at once: resident CTAs per SM (for the plan's CTA size
 * and shared memory) times the SM count; the workspace holds one slot each. */
int vmc_plan_resident_ctas(const vmc_plan* plan);

/* Bytes of the per-chain bottom-environment cache (Cache.bottom_envs,
 * kernels.py:32-35) for n_chains chains, and of the scratch workspace one
 * call needs.  The cache persists between sweeps; the workspace does not. */
size_t vmc_cache_size(const vmc_plan* plan, int n_chains);
size_t vmc_workspace_size(const vmc_plan* plan, int n_chains);

/*
 * init_cache (kernels.py:115-129): bottom environments of every row for
 * configs[n_chains][n_sites] (int32 occupancies 0..d-1).
 * tensors: FP32 site tensors packed site-major, each (d, up, down, left,
 * right) C-order (the order of ravel_pytree over model.tensors).
 */
vmc_status vmc_peps_init_cache(const vmc_plan* plan, void* stream, const float* tensors,
                               const int32_t* configs, int n_chains, void* cache,
                               void* workspace, size_t workspace_bytes, int32_t* status_dev);

/*
 * One Monte-Carlo sweep for n_chains chains: transition (kernels.py:131-209)
 * followed by estimate (kernels.py:211-245).
 *   configs_inout[n_chains][n_sites] int32: updated in place.
 *   uniforms[n_chains][n_sites] float64 in [0,1): the reference's per-site
 *     jax.random.uniform(accept_key) draws (kernels.py:189-190).
 *   deltas[n_chains][n_sites] int32 or NULL when d <= 2: the flip offsets of
 *     kernels.py:170-175, new = (s + delta) mod d with Python's non-negative
 *     modulo, so any integer offset is valid (the reference draws [1, d)).
 *   cache_inout: the bottom-environment cache (read by the transition,
 *     rewritten by the estimate).
 * Outputs (any may be NULL except out_E):
 *   out_O[n_chains][n_params] FP32 log-derivatives dpsi/dA / psi, sliced
 *     (full_gradient=0) or scattered into d x params (full_gradient=1)
 *     (_assemble_log_derivatives, kernels.py:54-88);
 *   out_p[n_chains][n_params_sliced] int8 active slice indices;
 *   out_E[n_chains] FP64 local energies;
 *   out_logamp[n_chains] FP64 log|psi| and out_sign[n_chains] FP64 sign;
 *   out_margin[n_chains] FP32 min over sites of |min(1, ratio) - u| (the
 *     distance of each accept decision from its threshold);
 *   out_gap[n_chains] FP32 min over truncating cuts of the relative gap
 *     (l_k - l_{k+1}) / l_k of the eigenvalues of theta theta^T (small values
 *     mark samples whose kept subspace is ill-conditioned).
 */
vmc_status vmc_peps_sweep(const vmc_plan* plan, void* stream, const float* tensors,
                          int32_t* configs_inout, const double* uniforms, const int32_t* deltas,
                          int n_chains, void* cache_inout, int full_gradient, float* out_O,
                          int8_t* out_p, double* out_E, double* out_logamp, double* out_sign,
                          float* out_margin, float* out_gap, void* workspace,
                          size_t workspace_bytes, int32_t* status_dev);

/*
 * vmc_peps_sweep without a per-chain cache: each chain's bottom environments
 * are recomputed at the start of its sweep, in one cache entry per resident
 * CTA inside the workspace, and dropped after it.  The same results as
 * vmc_peps_init_cache followed by vmc_peps_sweep, bit for bit, for one extra
 * bottom-up pass per chain; memory grows with the resident CTAs instead of the
 * chains (the reference recomputes them every call: init_cache,
 * kernels.py:115-129, runs on each sampler call).  Workspace:
 * vmc_sweep_recompute_workspace_size(plan, n_chains) bytes.
 */
size_t vmc_sweep_recompute_workspace_size(const vmc_plan* plan, int n_chains);
vmc_status vmc_peps_sweep_recompute(const vmc_plan* plan, void* stream, const float* tensors,
                                    int32_t* configs_inout, const double* uniforms, const int32_t* deltas,
                                    int n_chains, int full_gradient, float* out_O, int8_t* out_p,
                                    double* out_E, double* out_logamp, double* out_sign, float* out_margin,
                                    float* out_gap, void* workspace, size_t workspace_bytes,
                                    int32_t* status_dev);

/*
 * Amplitude and hand-written adjoint for samples[n][n_sites]
 * (compat.py:31-64 peps_apply custom_vjp; compat.py:94-133 _value_and_grad;
 * energy.py:276-301 _compute_all_gradients): log|psi|, sign and
 * out_O = (dpsi/dA)/psi (sliced or full).  out_O may be NULL for values only.
 */
vmc_status vmc_peps_amp_grad(const vmc_plan* plan, void* stream, const float* tensors,
                             const int32_t* samples, int n, int full_gradient, float* out_O,
                             double* out_logamp, double* out_sign, float* out_gap, void* workspace,
                             size_t workspace_bytes, int32_t* status_dev);

/*
 * Vector-Jacobian product of the amplitudes: the adjoint of peps_apply
 * (compat.py:49-61, whose backward scatters g * env_grad into the gradient,
 * energy.py:276-301).  out_grad[k] = sum_i w_i O_i[k] over the FULL
 * parameter layout (n_params_full elements; O_i = (dpsi_i / dtheta) / psi_i,
 * the rows vmc_peps_amp_grad writes).  The kernel builds each sample's
 * gradient environments as amp_grad does and adds w_i O_i into out_grad in
 * FP64 (atomics), so no n x n_params matrix exists: memory is the workspace
 * plus the one gradient.  For the backward of amp_i = sign_i exp(logamp_i)
 * with output cotangents g_i, pass w_i = g_i amp_i (real plans) or
 * w_i = conj(g_i) amp_i and conjugate the result (complex plans, where w and
 * out_grad hold (re, im) pairs).  out_grad is zeroed by the call (stream
 * ordered); workspace: vmc_workspace_size(plan, n).  Standard (not
 * gauge-invariant) plans.
 */
vmc_status vmc_peps_vjp(const vmc_plan* plan, void* stream, const float* tensors, const int32_t* samples, int n,
                        const double* weights, double* out_grad, void* workspace, size_t workspace_bytes,
                        int32_t* status_dev);

/*
 * vmc_peps_amp_grad without a caller workspace.  No counterpart in the
 * reference: it exists for callers that cannot hand the engine scratch memory,
 * e.g. a framework that has reserved the device memory in a pool of its own
 * and offers no scratch allocation where it calls out, or host code that must
 * not trigger an allocation (allocations synchronise the device) at the call.
 *
 * Scratch is one fixed array of this library in device memory,
 * VMC_NOALLOC_SCRATCH_BYTES (64 MiB) per device.  A plan needs the permuted
 * tensors plus at least one CTA slot in it (vmc_workspace_size(plan, 1)
 * bytes); larger plans are rejected with VMC_ERR_SCRATCH and nothing is
 * launched.  Chains are then processed by as many CTAs as fit, so results are
 * identical to vmc_peps_amp_grad's but throughput drops for large plans.
 *
 * The array is a static device variable of this library: it takes 64 MiB of
 * device memory in every CUDA context that loads the library, whether or not
 * this entry point is ever called.
 *
 * The first call on a device looks up the array's address on the current
 * device (cudaGetSymbolAddress) and caches it; make that first call before any
 * stream capture begins.  The cached address belongs to the device's primary
 * context: after cudaDeviceReset (or anything else that destroys and recreates
 * that context) the process must not call this entry point again.  Nothing in the scratch needs to start at zero: the
 * kernels write every word before reading it.  All calls on a device share
 * the one array, so calls that overlap in time (different streams or threads)
 * race on it and corrupt each other's results: serialise them.  The call
 * allocates no device or host memory.
 */
#define VMC_NOALLOC_SCRATCH_BYTES (64ull << 20)
vmc_status vmc_peps_amp_grad_noalloc(const vmc_plan* plan, void* stream, const float* tensors,
                                     const int32_t* samples, int n, int full_gradient, float* out_O,
                                     double* out_logamp, double* out_sign, float* out_gap,
                                     int32_t* status_dev);

/*
 * local_estimate (compat.py:136-194): E_loc for samples[n][n_sites] with the
 * caller's amplitudes (amp = sign * exp(logamp)) as denominators.
 */
vmc_status vmc_peps_local_energy(const vmc_plan* plan, void* stream, const float* tensors,
                                 const int32_t* samples, int n, const double* logamp,
                                 const double* sign, double* out_E, void* workspace,
                                 size_t workspace_bytes, int32_t* status_dev);

/*
 * Uneven batches: up to VMC_MAX_BATCH_JOBS jobs, each one of the calls above
 * on its own plan (lattice, bond dimension, strategy, operator), in ONE
 * persistent launch.  No single counterpart in the reference, where every
 * model runs through its own jitted sampler and evaluator
 * (src/vmc/peps/standard/kernels.py:91-247, one call per model); a job has the
 * arguments and the results of the call it names:
 *   VMC_JOB_INIT_CACHE   vmc_peps_init_cache   (tensors, configs, cache)
 *   VMC_JOB_SWEEP        vmc_peps_sweep        (all fields; deltas when d > 2;
 *                                               cache NULL: vmc_peps_sweep_recompute)
 *   VMC_JOB_AMP_GRAD     vmc_peps_amp_grad     (configs = samples; logamp, sign
 *                                               are outputs; out_O, out_gap optional)
 *   VMC_JOB_LOCAL_ENERGY vmc_peps_local_energy (logamp, sign are inputs; out_E)
 * Fields a kind does not use are ignored.  Every plan of a batch has the same
 * element type, CTA size and kernel (standard or gauge-invariant; tile policy 3
 * or not), else VMC_ERR_UNSUPPORTED.  Each chain's results are bit-identical to the
 * single call's: the same device code runs every chain.  CTAs take
 * (job, chain) items from a device counter, jobs in decreasing order of cost
 * per chain, so the lattices that take longest start first.
 *
 * vmc_batch_workspace_size: bytes of workspace for these jobs (0 if the batch
 * is invalid).  The workspace needs no initial value.  The call launches one
 * permutation kernel per job, one memset and the batch kernel on `stream`,
 * and allocates nothing; the pointers in jobs[] are read at the call, so
 * a captured launch replays with the same buffers.
 */
#define VMC_MAX_BATCH_JOBS 16
typedef enum {
  VMC_JOB_INIT_CACHE = 0,
  VMC_JOB_SWEEP = 1,
  VMC_JOB_AMP_GRAD = 2,
  VMC_JOB_LOCAL_ENERGY = 3
} vmc_job_kind;

typedef struct {
  const vmc_plan* plan;
  int kind; /* vmc_job_kind */
  int n_chains;
  int full_gradient;
  const float* tensors;
  int32_t* configs;
  const double* uniforms;
  const int32_t* deltas;
  void* cache;
  float* out_O;
  int8_t* out_p;
  double* out_E;
  double* logamp;
  double* sign;
  float* out_margin;
  float* out_gap;
} vmc_peps_job;

size_t vmc_batch_workspace_size(const vmc_peps_job* jobs, int n_jobs);
vmc_status vmc_peps_batch(const vmc_peps_job* jobs, int n_jobs, void* stream, void* workspace,
                          size_t workspace_bytes, int32_t* status_dev);

/*
 * The same batch with an explicit buffer placement.  Shared memory and L1
 * share one array per SM, so a batch runs all its plans either with their
 * own placement (VMC_BATCH_LAYOUT_PLAN: truncation arena and 1-row
 * intermediates in shared memory where they fit) or with every buffer in
 * the CTA's workspace slot (VMC_BATCH_LAYOUT_SLOT), which leaves the whole
 * array to L1 for plans too large for shared memory.  VMC_BATCH_LAYOUT_AUTO
 * (what vmc_peps_batch does) takes the slot placement when plans whose arena
 * lives in the slot carry more than half of the batch's work.  The placement
 * moves data, not arithmetic: results are the same bits either way.
 */
enum { VMC_BATCH_LAYOUT_AUTO = -1, VMC_BATCH_LAYOUT_PLAN = 0, VMC_BATCH_LAYOUT_SLOT = 1 };
size_t vmc_batch_workspace_size_ex(const vmc_peps_job* jobs, int n_jobs, int layout);
vmc_status vmc_peps_batch_ex(const vmc_peps_job* jobs, int n_jobs, int layout, void* stream, void* workspace,
                             size_t workspace_bytes, int32_t* status_dev);

/*
 * Column-pivoted Householder QR, A P = Q R, in FP64 (complex_elements = 0) or
 * complex128 (interleaved (re, im) doubles): the factorisation of the SR QR
 * solve, jax.lax.linalg.qr(o_centered, full_matrices=False, pivoting=True)
 * (src/vmc/preconditioners/preconditioners.py:178-180; LAPACK/MAGMA xGEQP3).
 *   a: column-major m x (n + nrhs), leading dimension lda >= m.  The first n
 *      columns are factorised; the last nrhs are right-hand sides b, returned
 *      as Q^H b.
 * On return, as xGEQP3 leaves them: R in the upper triangle of the first
 * min(m, n) rows, the reflectors v (v[0] = 1 implied) below the diagonal,
 * tau[min(m, n)], and jpvt[n] the 0-based original index of each column of R.
 * Pivots follow xLAQP2 (the unblocked xGEQP3): largest partial column norm,
 * the first on ties, with xLAQP2's norm downdating and recomputation.
 * workspace: vmc_qr_pivoted_workspace_size(n) bytes, no initial value.  The
 * call launches 2 min(m, n) + 1 kernels on `stream` and allocates nothing.
 */
/*
 * Uniform draws in [0, 1) for the Metropolis accept tests (in place of the
 * reference's per-site jax.random.uniform(accept_key), kernels.py:189-190),
 * for callers that replay a whole TDVP step as one CUDA graph: fills out[n]
 * (device FP64) from (seed, *counter) and increments the device word
 * *counter, so every replay draws fresh numbers and a replay equals the eager
 * call with the same counter.  SplitMix64 (Steele, Lea, Flood, OOPSLA 2014):
 * key = mix(seed + (counter + 1) gamma), out[i] = (mix(key + (i + 1) gamma)
 * >> 11) 2^-53, gamma = 0x9E3779B97F4A7C15.  Two kernels on `stream`.
 */
vmc_status vmc_uniforms(void* stream, double* out, int64_t n, uint64_t seed, uint64_t* counter);

size_t vmc_qr_pivoted_workspace_size(int n);
vmc_status vmc_qr_pivoted(void* stream, int complex_elements, double* a, int64_t lda, int m, int n, int nrhs,
                          double* tau, int32_t* jpvt, void* workspace, size_t workspace_bytes);

/*
 * The sample-space Gram matrix of a real sliced Jacobian in FP64, the matrix
 * the SampleSpace SR solve factorises before its centring terms
 * (src/vmc/qgt/qgt.py:173-223 sums it over the expanded slice blocks,
 * sum_k (O o [p == k]) (O o [p == k])^T; src/vmc/qgt/jacobian.py:56-93):
 *     out[i n + j] = sum_c [p[i ld + c] == p[j ld + c]] o[i ld + c] o[j ld + c]
 *   o: n x ncols FP32 log-derivatives (the engine's out_O, sliced layout);
 *   p: n x ncols active slice indices (the engine's out_p); both row-major
 *      with row stride ld >= ncols elements;
 *   out: n x n FP64, row-major; every entry is written (the matrix is
 *      symmetric).
 * The products are exact (FP32 inputs) and are summed in double-float on the
 * FP32 units, flushed into FP64 every 256 columns.  One kernel on `stream`;
 * allocates nothing.
 */
vmc_status vmc_sliced_gram(void* stream, const float* o, const int8_t* p, int n, int ncols, int64_t ld,
                           double* out);

/*
 * The parameter-space Gram matrix of the same sliced Jacobian, O_exp^T O_exp,
 * in FP64: the matrix of the ParameterSpace SR solve before its centring term
 * (src/vmc/qgt/qgt.py:173-223 on the expanded blocks in slice order,
 * jacobian.py:21-33):
 *     out[(k ncols + c) W + (k' ncols + c')] =
 *         sum_i [p[i ld + c] == k][p[i ld + c'] == k'] o[i ld + c] o[i ld + c']
 * with W = d ncols; o, p as for vmc_sliced_gram; out: W x W FP64 row-major,
 * every entry written.  d = 2 slices (VMC_ERR_UNSUPPORTED otherwise).  Exact
 * products summed in double-float, flushed into FP64 every 256 samples.  One
 * kernel on `stream`; allocates nothing.
 */
vmc_status vmc_sliced_gram_params(void* stream, const float* o, const int8_t* p, int n, int ncols, int64_t ld,
                                  int d, double* out);

#ifdef __cplusplus
}
#endif

#endif /* VMC_GB300_H_ */
