// peps_plan.cuh -- what the host code and the two element-type builds of the
// fused kernel (peps_kernels_real.cu, peps_kernels_complex.cu) share: limits,
// the device plan, the workspace-slot and shared-memory layouts, the job table
// of a launch, and the launchers each build exports.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "device_common.cuh"
#include "phase_timers.cuh"
#include "truncation.cuh"
#include "householder.cuh"
#include "../../include/vmc_gb300.h"

namespace vmc {

// Largest CTA the fused kernel is compiled for, and the CTAs of that size an
// SM must hold (__launch_bounds__): 256 x 2 caps registers at 128 per thread.
#ifndef VMC_MAX_THREADS
#define VMC_MAX_THREADS 256
#endif
#ifndef VMC_MIN_CTAS
#define VMC_MIN_CTAS 2
#endif
constexpr int kThreads = VMC_MAX_THREADS;
constexpr int kDefaultThreads = 128;  // one chain per 4 warps: more chains resident per SM
constexpr int kMaxVec = 512;   // max vectors in one truncation (chi * D)
constexpr int kMaxCols = 64;   // max lattice columns
constexpr int kMaxD = 27;      // max slices per site: physical dimension (<= 4), or gauge configurations (Z3: 27)
constexpr int kMaxPhys = 4;    // max physical dimension of a standard plan (its energy paths size d x d)
constexpr int kPermKinds = 6;  // permuted copies of every site tensor
constexpr float kJacobiTol = 5e-7f;  // stop when every |a_p.a_q| <= tol |a_p||a_q|
constexpr int kJacobiSweeps = 16;
// dynamic shared memory per chain; 52 KB keeps 4 chains of 128 threads on an SM
constexpr long long kMaxArenaSmemBytes = 52 * 1024;
// mixed precision: largest and default dynamic shared memory per CTA for the FP64 arena
constexpr long long kMaxArenaSmemBytesF64 = 200 * 1024;
constexpr long long kDefaultArenaSmemBytesF64 = 52 * 1024;
enum PermKind { P_ZIPT = 0, P_ZIPB = 1, P_RENV = 2, P_LENV = 3, P_R2 = 4, P_VRB = 5 };
enum Mode { MODE_INIT = 0, MODE_SWEEP = 1, MODE_AMPGRAD = 2, MODE_ENERGY = 3, MODE_VJP = 4 };


// Device-side plan: scalars plus device pointers into one allocation.
struct DevPlan {
  int R, C, D, d, chi, strategy, n_sweeps, n_sites;
  int es;                 // floats per element: 1 real FP32, 2 complex64 (re, im)
  int np_sliced;          // sum of params_per_site
  int TS, ES, E2S, SCR, MM;  // buffer sizes (floats)
  int nmax, kmax;         // largest truncation matrix side / kept bond
  int trunc_method;       // 0: Gram + tridiagonal eigensolver, 1: one-sided Jacobi
  int chain64;            // mixed precision: the boundary-MPS chain in double-float (chain_f64.cuh), the rest FP32
  int arena_in_smem;      // truncation arena in dynamic shared memory
  int mat_in_smem;        // theta matrix inside the arena (else in a separate global slot region)
  int threads;            // CTA size of the fused kernel
  int tile_policy;        // register-tile policy of the CTA GEMMs (cta_gemm)
  long long arena_floats;
  long long arena_g_floats;  // floats of the truncation arena that live in the CTA's slot
  long long dyn_smem_bytes;  // dynamic shared memory per CTA (the arena's, or tcgen05 staging for tile policy 4)
  int scr1;               // size of one 1-row GEMM intermediate (floats)
  int vchunk, vbuf;       // vertical-energy chunk (bond values) and buffer size (floats)
  int vert_in_smem;       // vertical-energy buffers live in the shared-memory arena
  int onerow_in_smem;     // 1-row intermediates share the shared-memory arena
  int n_scr;              // number of SCR scratch buffers per slot
  int VS;                 // one variational environment (floats); 0 unless Variational
  long long slot_floats;  // floats per workspace slot
  long long perm_floats;  // floats of the permuted tensor pack
  long long cache_floats_per_chain;  // bottom env tensors per chain
  // per-site (n_sites)
  const int* sdim;        // [n_sites][4] up, down, left, right
  const int* site_off;    // packed params offset
  const int* site_osl;    // offset in the sliced O vector
  const int* perm_off;    // offset in the permuted pack
  // bond dims
  const int* tb;          // [(R+1)][(C+1)] top env bonds (row r = before row r)
  const int* bb;          // [R][(C+1)] bottom env bonds (row r = rows r+1.. from below)
  // operator
  const float* onesite;   // [n_sites][d][d]
  const int* onesite_mask;
  const float* horiz;     // [R*(C-1)][d*d][d*d]
  const int* horiz_mask;
  const float* vert;      // [(R-1)*C][d*d][d*d]
  const int* vert_mask;
  const int* row_has_h;   // [R] any horizontal term in row
  const int* row_has_v;   // [R] any vertical term between r and r+1
  int n_diag;
  const int* diag_nsites;
  const int* diag_site_off;
  const int* diag_sites;
  const int* diag_value_off;
  const double* diag_values;
  // gauge-invariant PEPS (pure Z_N gauge, gi != 0): the "physical" index of a site is its gauge
  // configuration (slice), selected by the link values; a chain's state is (sites, h links, v links)
  int gi, gi_N, n_state;          // n_state: ints per chain (n_sites for a standard plan)
  const double* gi_hdiag;         // [R*(C-1)][N] energy of a horizontal link with value k
  const double* gi_vdiag;         // [(R-1)*C][N] energy of a vertical link with value k
  const double* gi_plaq;          // [(R-1)*(C-1)] plaquette coefficient (P + P^dag)
};

struct Slot {
  float* topc;   // (R+1)*C*TS
  double* lt;    // R+1
  double* rl;    // [q][c] log-scale of right environment renv[q][c]
  double* r2l;   // [c] log-scale of 2-row right environment r2[c]
  float* brow[3];
  float* renv;   // d*C*ES  [q][c]
  float* lenv;   // (d+1)*ES
  float* r2;     // C*E2S
  float* l2[2];  // E2S
  float* arena;  // truncation arena when it does not fit shared memory
  float* venv;   // Variational: left envs C*VS, then right envs C*VS
  double* h64;   // mixed precision: the df64 boundary-MPS chain (chain_f64_doubles 8-byte elements), else null
  float* scr[11 + 2 * kMaxPhys + 5];  // n_scr = 11 + 2 kMaxPhys buffers (GI plans use the first 12)
};

__host__ __device__ inline long long al64(long long n) { return (n + 63) & ~63LL; }
__host__ __device__ inline long long al32(long long n) { return (n + 31) & ~31LL; }
__host__ __device__ inline int min_i(int a, int b) { return a < b ? a : b; }

__device__ inline Slot make_slot(const DevPlan& P, float* base) {
  Slot s;
  float* p = base;
  s.topc = p; p += al64((long long)(P.R + 1) * P.C * P.TS);
  s.lt = reinterpret_cast<double*>(p); p += al64(2 * (P.R + 2));
  s.rl = reinterpret_cast<double*>(p); p += al64(2LL * P.d * P.C);
  s.r2l = reinterpret_cast<double*>(p); p += al64(2LL * P.C);
  for (int i = 0; i < 3; ++i) { s.brow[i] = p; p += al64((long long)P.C * P.TS); }
  s.renv = p; p += al64((long long)P.d * P.C * P.ES);
  s.lenv = p; p += al64((long long)(P.d + 1) * P.ES);
  s.r2 = p; p += al64((long long)P.C * P.E2S);
  for (int i = 0; i < 2; ++i) { s.l2[i] = p; p += al64(P.E2S); }
  s.arena = p; p += al64(P.arena_g_floats);
  for (int i = 0; i < P.n_scr; ++i) { s.scr[i] = p; p += al64(P.SCR); }
  s.venv = p; p += al64(2LL * P.C * P.VS);
  s.h64 = P.chain64 ? reinterpret_cast<double*>(p) : nullptr;
  return s;
}

struct Shared {
  double red[32];
  int flag;
  int sel[kMaxVec];
  float sig[kMaxVec];
  int spins[2][kMaxCols];
  int vb[kMaxCols + 1];  // Variational: current bond dimensions of the row being compressed
  double bcast[8];
};

// Floats of the truncation arena (layout: make_arena); es = floats per element.
__host__ __device__ inline long long arena_floats(int nmax, int kmax, int trunc_method, int es) {
  const int ld = nmax | 1;
  return 2 * al64((long long)es * nmax * ld) + al64((long long)es * nmax * (trunc_method == 1 ? ld : kmax)) +
         al64((long long)kmax * kmax) + al64(4LL * kmax * nmax) + al64(((long long)kmax * nmax + 3) / 4) +
         3 * al64(nmax) + 3 * al64((long long)es * nmax) + al64(nmax + 1) + al64(2LL * es * nmax) +
         al64(nmax + 64) + 64 + (es == 2 ? al64((long long)nmax * kmax) : 0);
}

// Doubles of the FP64 truncation arena of a mixed-precision plan (layout:
// make_arena_d in chain_f64.cuh), and of the part that can be split out into
// the CTA's slot when the rest must fit shared memory: theta (read by the Gram
// and carry GEMMs) and the inverse-iteration factors (one thread each, in
// sequence).
__host__ __device__ inline long long arena_doubles(int nmax, int kmax) {
  const int ld = nmax | 1;
  return 2 * al32((long long)nmax * ld) + al32((long long)nmax * kmax) + al32((long long)kmax * kmax) +
         al32(4LL * kmax * nmax) + al32(((long long)kmax * nmax + 7) / 8) + 6 * al32(nmax) + al32(nmax + 1) +
         al32(2LL * nmax) + al32(nmax + 64) + 32;
}
__host__ __device__ inline long long arena_split_doubles(int nmax, int kmax) {
  return al32((long long)nmax * (nmax | 1)) + al32(4LL * kmax * nmax);
}
// 8-byte elements of the df64 chain buffers in a slot (make_chain_d): two boundary
// rows, two carries and the Z1 intermediate.  The FP64 arena takes the place
// of the FP32 one (shared memory or the slot's arena region).
__host__ __device__ inline long long chain_f64_doubles(int C, long long TS, long long SCR) {
  return 2 * al32((long long)C * TS) + 3 * al32(SCR);
}

// Arguments of one job: the chains of one plan in one mode.
struct ChainJob {
  const DevPlan* P;
  int mode;
  int n_chains;
  int full_gradient;
  // 0: cache holds one entry per chain (the caller's bottom-environment
  // cache); 1: cache holds one entry per CTA and a sweep first recomputes the
  // chain's bottom environments there (nothing is kept between sweeps)
  int cache_per_cta;
  const float* tensors;
  const float* perm;
  int32_t* configs;
  const double* uniforms;
  const int32_t* deltas;
  float* cache;
  float* out_O;
  int8_t* out_p;
  double* out_E;
  double* logamp_io;
  double* sign_io;
  float* out_margin;
  float* out_gap;
  // MODE_VJP: per-chain weights (kEs doubles each) and the FP64 gradient they accumulate into
  const double* vjp_w;
  double* vjp_grad;
};

// The job table of one launch of the fused kernel (a kernel parameter).  Work
// item i is chain i - first[j] of job j, for first[j] <= i < first[j+1]; every
// CTA owns one workspace slot of slot_floats floats.
constexpr int kMaxBatchJobs = VMC_MAX_BATCH_JOBS;
struct BatchJobs {
  ChainJob job[kMaxBatchJobs];
  int first[kMaxBatchJobs + 1];
  int n_jobs;
  long long slot_floats;
};

// Launchers of one element type's kernels, on `stream`.
struct KernelSet {
  // permuted tensor copies of one plan into perm (a workspace region)
  cudaError_t (*permute)(const DevPlan* dplan, int n_sites, const float* tensors, float* perm, void* stream);
  // opt in to smem bytes of dynamic shared memory; *per_sm := resident CTAs per SM
  cudaError_t (*prepare)(int threads, size_t smem, int* per_sm);
  // the fused kernel over jobs; next = NULL: CTA b runs items b, b + grid, ...;
  // else CTAs take items from the counter *next, which must be zero at launch
  cudaError_t (*run)(const BatchJobs& jobs, int grid, int threads, size_t smem, void* stream, float* slots,
                     int32_t* next, int32_t* status);
};
namespace rk { const KernelSet& kernels(); }  // real FP32 elements
namespace rt { const KernelSet& kernels(); }  // real FP32 elements, tensor-core GEMMs (tile_policy 3)
namespace rq { const KernelSet& kernels(); }  // real FP32 elements, tcgen05 GEMMs (tile_policy 4)
namespace rm { const KernelSet& kernels(); }  // real, mixed precision: df64 boundary-MPS chain
namespace ck { const KernelSet& kernels(); }  // complex64 elements
namespace gr { const KernelSet& kernels(); }  // gauge-invariant plans, real FP32
namespace gc { const KernelSet& kernels(); }  // gauge-invariant plans, complex64
inline const KernelSet& kernels_of(const DevPlan& P) {
  if (P.gi) return P.es == 2 ? gc::kernels() : gr::kernels();
  if (P.es == 2) return ck::kernels();
  if (P.chain64) return rm::kernels();
  if (P.tile_policy == 4) return rq::kernels();
  return P.tile_policy == 3 ? rt::kernels() : rk::kernels();
}

}  // namespace vmc
