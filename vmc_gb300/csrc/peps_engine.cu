// peps_engine.cu -- fused per-sample PEPS evaluation on GB300 (sm_103a).
//
// One CTA owns one chain at a time (persistent grid over chains) and runs the
// whole reference sweep for it -- transition (kernels.py:131-209) and estimate
// (kernels.py:211-245) -- from one launch.  All tensor contractions are CTA
// GEMMs (device_common.cuh); the boundary-MPS truncation is a CTA-level
// one-sided Jacobi SVD.  Boundary MPSs are renormalised tensor by tensor and
// their log-norms are carried in FP64, so nothing underflows for any lattice.
//
// Layouts (row-major, last index fastest):
//   site tensor A[p][u][v][l][r]           (d, up, down, left, right)
//   boundary MPS tensor [left][phys][right]
//   1-row environment   [top][mpo][bottom]
//   2-row environment   [top][mpo row r][mpo row r+1][bottom]
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>
#include <algorithm>
#include <cstdlib>
#include <mutex>

#include "peps_plan.cuh"

#ifdef VMC_HOST_EMULATION
thread_local vmc_dim3 threadIdx, blockIdx, blockDim, gridDim;
#endif

namespace vmc {

// ===========================================================================
// Host side: plan construction.
// ===========================================================================
struct HostOp {
  std::vector<float> onesite, horiz, vert;
  std::vector<int> onesite_mask, horiz_mask, vert_mask, row_has_h, row_has_v;
  std::vector<int> diag_nsites, diag_site_off, diag_sites, diag_value_off;
  std::vector<double> diag_values;
  std::vector<double> gi_hdiag, gi_vdiag, gi_plaq;  // gauge-invariant plans
};

}  // namespace vmc

struct vmc_plan {
  vmc::DevPlan hp;          // host copy with device pointers
  vmc::DevPlan* dplan = nullptr;  // device copy
  vmc::DevPlan hpg;         // buffer placement with no shared memory (layout fields only are used)
  vmc::DevPlan* dplan_g = nullptr;  // device copy of hp with hpg's buffer placement
  void* dbuf = nullptr;     // device arrays
  std::vector<int> sdim, site_off, site_osl, perm_off, tb, bb;
  vmc::HostOp op;
  bool op_set = false;
  int slots_max = 0;
};

namespace vmc {

// Bond dimensions produced by applying one row MPO to a boundary MPS
// (strategy.py:118-150; dims depend on shapes only).
static std::vector<int> apply_bonds(const std::vector<int>& bin, const std::vector<int>& wb, int pout, int chi,
                                    int strategy, int n_sweeps) {
  const int C = (int)bin.size() - 1;
  std::vector<int> out(C + 1, 1);
  if (strategy == VMC_STRATEGY_NO_TRUNCATION) {
    for (int i = 0; i <= C; ++i) out[i] = bin[i] * wb[i];
    return out;
  }
  int left = bin[0] * wb[0];
  out[0] = left;
  for (int i = 0; i < C - 1; ++i) {
    const int m = left * pout, n = bin[i + 1] * wb[i + 1];
    // ZipUp / Variational keep min(chi, rank bound); DensityMatrix keeps min(chi, columns) eigenvectors of
    // the column Gram (strategy.py:167)
    const int k = strategy == VMC_STRATEGY_DENSITY_MATRIX ? std::min(chi, n) : std::min(chi, std::min(m, n));
    out[i + 1] = k;
    left = k;
  }
  out[C] = bin[C] * wb[C];
  if (strategy == VMC_STRATEGY_VARIATIONAL && n_sweeps > 0) {
    // the right-to-left sweep's LQ keeps min(left, phys * right) (strategy.py:403-410)
    for (int i = C - 1; i >= 1; --i) out[i] = std::min(out[i], pout * out[i + 1]);
  }
  return out;
}

static vmc_status upload_plan(vmc_plan* pl) {
  DevPlan& P = pl->hp;
  HostOp& op = pl->op;
  // gather all arrays into one device buffer
  std::vector<char> blob;
  auto push = [&](const void* data, size_t bytes) -> size_t {
    size_t off = (blob.size() + 15) & ~size_t(15);
    blob.resize(off + bytes);
    if (data && bytes) std::memcpy(blob.data() + off, data, bytes);
    return off;
  };
  const size_t o_sdim = push(pl->sdim.data(), pl->sdim.size() * 4);
  const size_t o_soff = push(pl->site_off.data(), pl->site_off.size() * 4);
  const size_t o_sosl = push(pl->site_osl.data(), pl->site_osl.size() * 4);
  const size_t o_poff = push(pl->perm_off.data(), pl->perm_off.size() * 4);
  const size_t o_tb = push(pl->tb.data(), pl->tb.size() * 4);
  const size_t o_bb = push(pl->bb.data(), pl->bb.size() * 4);
  const size_t o_os = push(op.onesite.data(), op.onesite.size() * 4);
  const size_t o_osm = push(op.onesite_mask.data(), op.onesite_mask.size() * 4);
  const size_t o_hz = push(op.horiz.data(), op.horiz.size() * 4);
  const size_t o_hzm = push(op.horiz_mask.data(), op.horiz_mask.size() * 4);
  const size_t o_vt = push(op.vert.data(), op.vert.size() * 4);
  const size_t o_vtm = push(op.vert_mask.data(), op.vert_mask.size() * 4);
  const size_t o_rh = push(op.row_has_h.data(), op.row_has_h.size() * 4);
  const size_t o_rv = push(op.row_has_v.data(), op.row_has_v.size() * 4);
  const size_t o_dn = push(op.diag_nsites.data(), op.diag_nsites.size() * 4);
  const size_t o_dso = push(op.diag_site_off.data(), op.diag_site_off.size() * 4);
  const size_t o_ds = push(op.diag_sites.data(), op.diag_sites.size() * 4);
  const size_t o_dvo = push(op.diag_value_off.data(), op.diag_value_off.size() * 4);
  const size_t o_dv = push(op.diag_values.data(), op.diag_values.size() * 8);
  const size_t o_gh = push(op.gi_hdiag.data(), op.gi_hdiag.size() * 8);
  const size_t o_gv = push(op.gi_vdiag.data(), op.gi_vdiag.size() * 8);
  const size_t o_gp = push(op.gi_plaq.data(), op.gi_plaq.size() * 8);
  const size_t o_plan = push(nullptr, sizeof(DevPlan));
  const size_t o_plan_g = push(nullptr, sizeof(DevPlan));
  if (pl->dbuf) vmc_free(pl->dbuf);
  pl->dbuf = nullptr;
  if (vmc_alloc(&pl->dbuf, blob.size()) != cudaSuccess) return VMC_ERR_CUDA;
  char* base = static_cast<char*>(pl->dbuf);
  P.sdim = reinterpret_cast<const int*>(base + o_sdim);
  P.site_off = reinterpret_cast<const int*>(base + o_soff);
  P.site_osl = reinterpret_cast<const int*>(base + o_sosl);
  P.perm_off = reinterpret_cast<const int*>(base + o_poff);
  P.tb = reinterpret_cast<const int*>(base + o_tb);
  P.bb = reinterpret_cast<const int*>(base + o_bb);
  P.onesite = reinterpret_cast<const float*>(base + o_os);
  P.onesite_mask = reinterpret_cast<const int*>(base + o_osm);
  P.horiz = reinterpret_cast<const float*>(base + o_hz);
  P.horiz_mask = reinterpret_cast<const int*>(base + o_hzm);
  P.vert = reinterpret_cast<const float*>(base + o_vt);
  P.vert_mask = reinterpret_cast<const int*>(base + o_vtm);
  P.row_has_h = reinterpret_cast<const int*>(base + o_rh);
  P.row_has_v = reinterpret_cast<const int*>(base + o_rv);
  P.diag_nsites = reinterpret_cast<const int*>(base + o_dn);
  P.diag_site_off = reinterpret_cast<const int*>(base + o_dso);
  P.diag_sites = reinterpret_cast<const int*>(base + o_ds);
  P.diag_value_off = reinterpret_cast<const int*>(base + o_dvo);
  P.diag_values = reinterpret_cast<const double*>(base + o_dv);
  P.gi_hdiag = reinterpret_cast<const double*>(base + o_gh);
  P.gi_vdiag = reinterpret_cast<const double*>(base + o_gv);
  P.gi_plaq = reinterpret_cast<const double*>(base + o_gp);
  std::memcpy(blob.data() + o_plan, &P, sizeof(DevPlan));
  pl->dplan = reinterpret_cast<DevPlan*>(base + o_plan);
  {
    DevPlan G = P;  // arrays and operator of P, buffer placement of the no-shared-memory layout
    const DevPlan& L = pl->hpg;
    G.arena_in_smem = L.arena_in_smem;
    G.mat_in_smem = L.mat_in_smem;
    G.arena_floats = L.arena_floats;
    G.arena_g_floats = L.arena_g_floats;
    G.dyn_smem_bytes = L.dyn_smem_bytes;
    G.scr1 = L.scr1;
    G.vchunk = L.vchunk;
    G.vbuf = L.vbuf;
    G.vert_in_smem = L.vert_in_smem;
    G.onerow_in_smem = L.onerow_in_smem;
    G.slot_floats = L.slot_floats;
    std::memcpy(blob.data() + o_plan_g, &G, sizeof(DevPlan));
    pl->dplan_g = reinterpret_cast<DevPlan*>(base + o_plan_g);
  }
  if (vmc_h2d(pl->dbuf, blob.data(), blob.size(), nullptr) != cudaSuccess) return VMC_ERR_CUDA;
  if (vmc_sync(nullptr) != cudaSuccess) return VMC_ERR_CUDA;
  return VMC_OK;
}

// Sweeps of this plan need explicit flip offsets: d > 2 site flips, or Z_N plaquette flips with N > 2.
static bool needs_deltas(const DevPlan& P) { return P.gi ? P.gi_N > 2 : P.d > 2; }

static void default_operator(vmc_plan* pl) {
  DevPlan& P = pl->hp;
  HostOp& op = pl->op;
  const int d2 = P.d * P.d;
  op.onesite.assign((size_t)P.es * P.n_sites * P.d * P.d, 0.f);
  op.onesite_mask.assign(P.n_sites, 0);
  op.horiz.assign((size_t)P.es * std::max(P.R * (P.C - 1), 1) * d2 * d2, 0.f);
  op.horiz_mask.assign(std::max(P.R * (P.C - 1), 1), 0);
  op.vert.assign((size_t)P.es * std::max((P.R - 1) * P.C, 1) * d2 * d2, 0.f);
  op.vert_mask.assign(std::max((P.R - 1) * P.C, 1), 0);
  op.row_has_h.assign(P.R, 0);
  op.row_has_v.assign(P.R, 0);
  op.diag_nsites.assign(1, 0);
  op.diag_site_off.assign(1, 0);
  op.diag_sites.assign(1, 0);
  op.diag_value_off.assign(1, 0);
  op.diag_values.assign(1, 0.0);
  P.n_diag = 0;
  const size_t N = P.gi ? (size_t)P.gi_N : 1;
  op.gi_hdiag.assign(std::max(P.R * (P.C - 1), 1) * N, 0.0);
  op.gi_vdiag.assign(std::max((P.R - 1) * P.C, 1) * N, 0.0);
  op.gi_plaq.assign(std::max((P.R - 1) * (P.C - 1), 1), 0.0);
}

}  // namespace vmc

using namespace vmc;

extern "C" {

const char* vmc_version(void) { return "vmc_gb300 0.1 (sm_103a)"; }

const char* vmc_status_string(vmc_status s) {
  switch (s) {
    case VMC_OK: return "ok";
    case VMC_ERR_INVALID: return "invalid argument";
    case VMC_ERR_UNSUPPORTED: return "unsupported configuration";
    case VMC_ERR_WORKSPACE: return "workspace too small";
    case VMC_ERR_CUDA: return "CUDA runtime error";
    case VMC_ERR_NONFINITE: return "non-finite result";
    case VMC_ERR_TIMEOUT: return "device wait timed out";
    case VMC_ERR_SCRATCH: return "plan needs more than the fixed 64 MiB no-alloc scratch";
    default: return "unknown status";
  }
}

vmc_status vmc_peps_plan(const vmc_shape* shape, int bond_dim, int chi, int phys_dim, int dtype, int strategy,
                         int n_sweeps, vmc_plan** out_plan) {
  return vmc_peps_plan_ex(shape, bond_dim, chi, phys_dim, dtype, strategy, n_sweeps, nullptr, out_plan);
}

// A plan; gi_N > 0 makes it the gauge-invariant pure-Z_N-gauge plan whose "physical" index is a
// site's gauge configuration (phys_dim = the largest number of configurations of a site).
static vmc_status create_plan(const vmc_shape* shape, int bond_dim, int chi, int phys_dim, int dtype, int strategy,
                              int n_sweeps, const vmc_plan_options* opts, int gi_N, vmc_plan** out_plan);

vmc_status vmc_peps_plan_ex(const vmc_shape* shape, int bond_dim, int chi, int phys_dim, int dtype, int strategy,
                            int n_sweeps, const vmc_plan_options* opts, vmc_plan** out_plan) {
  return create_plan(shape, bond_dim, chi, phys_dim, dtype, strategy, n_sweeps, opts, 0, out_plan);
}

vmc_status vmc_gi_plan(const vmc_shape* shape, int N, int dmax, int chi, int dtype, int strategy, int n_sweeps,
                       const vmc_plan_options* opts, vmc_plan** out_plan) {
  if (!shape || !out_plan || N < 2 || dmax < 1) return VMC_ERR_INVALID;
  const int R = shape->n_rows, C = shape->n_cols;
  if (R < 2 || C < 2) return VMC_ERR_UNSUPPORTED;  // no plaquette to sweep
  // configurations per site: N^(links - 1) (model.py:99-101); the plan's slices are the largest count
  int slices = 1;
  for (int r = 0; r < R; ++r)
    for (int c = 0; c < C; ++c) {
      const int links = (r > 0) + (r < R - 1) + (c > 0) + (c < C - 1);
      int n = 1;
      for (int k = 1; k < links; ++k) n *= N;
      slices = std::max(slices, n);
    }
  if (slices > kMaxD) return VMC_ERR_UNSUPPORTED;
  return create_plan(shape, dmax, chi, slices, dtype, strategy, n_sweeps, opts, N, out_plan);
}

static vmc_status create_plan(const vmc_shape* shape, int bond_dim, int chi, int phys_dim, int dtype, int strategy,
                              int n_sweeps, const vmc_plan_options* opts, int gi_N, vmc_plan** out_plan) {
  if (!shape || !out_plan) return VMC_ERR_INVALID;
  if (opts && (opts->threads != 0 && (opts->threads < 64 || opts->threads > kThreads || opts->threads % 32 != 0)))
    return VMC_ERR_INVALID;
  if (opts && (opts->tile_policy < 0 || opts->tile_policy > 4 || opts->smem_kb < -1)) return VMC_ERR_INVALID;
  if (opts && (opts->precision < VMC_PRECISION_FP32 || opts->precision > VMC_PRECISION_MIXED ||
               opts->trunc_method < 0 || opts->trunc_method > 1 || opts->vchunk < 0 || opts->vert_smem < 0))
    return VMC_ERR_INVALID;
  // tile policy 4 (tcgen05 GEMMs): real FP32 standard plans, CTAs of at least 4 warps (one per TMEM lane quadrant)
  if (opts && opts->tile_policy == 4 &&
      (dtype != VMC_DTYPE_F32 || gi_N > 0 || opts->precision != VMC_PRECISION_FP32 ||
       (opts->threads != 0 && opts->threads < 128)))
    return VMC_ERR_UNSUPPORTED;
  const int precision = opts ? opts->precision : VMC_PRECISION_FP32;
  // the high-precision chain exists for real ZipUp / NoTruncation / DensityMatrix plans with the Gram
  // eigensolver and FFMA tiles
  if (precision == VMC_PRECISION_MIXED &&
      (dtype != VMC_DTYPE_F32 || gi_N > 0 || strategy == VMC_STRATEGY_VARIATIONAL || opts->trunc_method != 0 ||
       opts->tile_policy >= 3))
    return VMC_ERR_UNSUPPORTED;
  *out_plan = nullptr;
  const int R = shape->n_rows, C = shape->n_cols;
  if (R < 1 || C < 1 || C > kMaxCols || bond_dim < 1 || phys_dim < 1 || chi < 1) return VMC_ERR_INVALID;
  if (phys_dim > (gi_N ? kMaxD : kMaxPhys)) return VMC_ERR_UNSUPPORTED;
  if (dtype != VMC_DTYPE_F32 && dtype != VMC_DTYPE_C64) return VMC_ERR_UNSUPPORTED;
  if (strategy < 0 || strategy > VMC_STRATEGY_VARIATIONAL || n_sweeps < 0) return VMC_ERR_INVALID;
  // DensityMatrix (strategy.py:153-176) carries V_k^H: with the Gram eigensolver only (it is one), and
  // not on gauge-invariant plans
  if (strategy == VMC_STRATEGY_DENSITY_MATRIX && (gi_N > 0 || (opts && opts->trunc_method != 0)))
    return VMC_ERR_UNSUPPORTED;
  vmc_plan* pl = new (std::nothrow) vmc_plan();
  if (!pl) return VMC_ERR_INVALID;
  DevPlan& P = pl->hp;
  std::memset(&P, 0, sizeof(P));
  P.R = R; P.C = C; P.D = bond_dim; P.d = phys_dim; P.chi = chi; P.strategy = strategy;
  P.es = dtype == VMC_DTYPE_C64 ? 2 : 1;
  P.n_sweeps = n_sweeps; P.n_sites = R * C;
  P.gi = gi_N > 0;
  P.gi_N = gi_N;
  P.n_state = P.gi ? R * C + R * (C - 1) + (R - 1) * C : R * C;
  const int D = bond_dim, d = phys_dim;
  pl->sdim.resize(4 * R * C);
  pl->site_off.resize(R * C);
  pl->site_osl.resize(R * C);
  pl->perm_off.resize(R * C);
  long long off = 0, osl = 0, poff = 0;
  for (int r = 0; r < R; ++r)
    for (int c = 0; c < C; ++c) {
      const int s = r * C + c;
      const int u = r == 0 ? 1 : D, v = r == R - 1 ? 1 : D, l = c == 0 ? 1 : D, rr = c == C - 1 ? 1 : D;
      pl->sdim[4 * s] = u; pl->sdim[4 * s + 1] = v; pl->sdim[4 * s + 2] = l; pl->sdim[4 * s + 3] = rr;
      const int sz = u * v * l * rr;
      pl->site_off[s] = (int)off;
      pl->site_osl[s] = (int)osl;
      pl->perm_off[s] = (int)poff;
      off += (long long)d * sz;
      osl += sz;
      poff += (long long)kPermKinds * d * sz;
    }
  P.np_sliced = (int)osl;
  P.perm_floats = (poff * P.es + 63) & ~63LL;
  // bond dims
  pl->tb.assign((size_t)(R + 1) * (C + 1), 1);
  pl->bb.assign((size_t)R * (C + 1), 1);
  std::vector<int> wb(C + 1, 1);
  for (int i = 1; i < C; ++i) wb[i] = D;
  // Variational rows pass through their QR-initialisation bonds (never
  // clamped) before the sweeps: size the tensor buffers for those as well
  long long TS_init = 1, chi_init = 1;
  auto account_init = [&](const std::vector<int>& cur, int pout) {
    const std::vector<int> init = apply_bonds(cur, wb, pout, chi, strategy, 0);
    for (int c = 0; c < C; ++c) {
      TS_init = std::max(TS_init, (long long)init[c] * pout * init[c + 1]);
      chi_init = std::max(chi_init, (long long)std::max(init[c], init[c + 1]));
    }
  };
  {
    std::vector<int> cur(C + 1, 1);
    for (int r = 0; r < R; ++r) {
      for (int i = 0; i <= C; ++i) pl->tb[(size_t)r * (C + 1) + i] = cur[i];
      const int pout = r == R - 1 ? 1 : D;
      account_init(cur, pout);
      cur = apply_bonds(cur, wb, pout, chi, strategy, n_sweeps);
    }
    for (int i = 0; i <= C; ++i) pl->tb[(size_t)R * (C + 1) + i] = cur[i];
  }
  {
    std::vector<int> cur(C + 1, 1);
    for (int r = R - 1; r >= 0; --r) {
      for (int i = 0; i <= C; ++i) pl->bb[(size_t)r * (C + 1) + i] = cur[i];
      const int pout = r == 0 ? 1 : D;
      account_init(cur, pout);
      cur = apply_bonds(cur, wb, pout, chi, strategy, n_sweeps);
    }
  }
  // buffer sizes
  long long TS = 1, ES = 1, E2S = 1, chimax = 1, MM = 1;
  auto phys_top = [&](int r) { return r == 0 ? 1 : D; };   // phys of top env row r = up leg of row r
  auto phys_bot = [&](int r) { return r == R - 1 ? 1 : D; };
  for (int r = 0; r <= R; ++r)
    for (int c = 0; c < C; ++c) {
      const long long a = pl->tb[(size_t)r * (C + 1) + c], b = pl->tb[(size_t)r * (C + 1) + c + 1];
      const int ph = r < R ? phys_top(r) : 1;
      TS = std::max(TS, a * ph * b);
      chimax = std::max(chimax, std::max(a, b));
    }
  for (int r = 0; r < R; ++r)
    for (int c = 0; c < C; ++c) {
      const long long a = pl->bb[(size_t)r * (C + 1) + c], b = pl->bb[(size_t)r * (C + 1) + c + 1];
      TS = std::max(TS, a * phys_bot(r) * b);
      chimax = std::max(chimax, std::max(a, b));
    }
  for (int r = 0; r < R; ++r)
    for (int c = 0; c <= C; ++c) {
      const long long t = pl->tb[(size_t)r * (C + 1) + c], b = pl->bb[(size_t)r * (C + 1) + c];
      ES = std::max(ES, t * D * b);
      if (r + 1 < R) E2S = std::max(E2S, t * D * D * (long long)pl->bb[(size_t)(r + 1) * (C + 1) + c]);
    }
  TS = std::max(TS, TS_init);
  chimax = std::max(chimax, chi_init);
  // truncation matrices: rows kc*pout <= chimax*D, cols <= chimax*D
  MM = (chimax * D + 1) * (chimax * D + 1);
  // element counts above; every DevPlan buffer size below counts floats (es per element)
  const long long es = P.es;
  // (>= 8 * kMaxVec floats: contract_bottom keeps 2 x kMaxVec complex doubles in scr[0])
  const long long SCR = std::max(es * std::max({chimax * chimax * D * D * D, TS * D * D, MM}), 8LL * kMaxVec);
  TS *= es;
  ES *= es;
  E2S *= es;
  P.nmax = (int)(chimax * D);
  P.kmax = (int)std::min<long long>(chi, chimax * D);
  // the one-sided Jacobi cross-check exists for real elements only
  P.trunc_method = (opts && opts->trunc_method == 1 && es == 1) ? 1 : 0;
  P.chain64 = precision == VMC_PRECISION_MIXED;
  P.threads = (opts && opts->threads) ? opts->threads : kDefaultThreads;
  P.tile_policy = opts ? opts->tile_policy : 0;
  // shared memory per CTA: the FP64 arena of a mixed plan is twice the FP32 one
  const long long smem_cap = P.chain64 ? kMaxArenaSmemBytesF64 : kMaxArenaSmemBytes;
  long long budget = P.chain64 ? kDefaultArenaSmemBytesF64 : kMaxArenaSmemBytes;
  if (opts && opts->smem_kb >= 0) budget = std::min<long long>(opts->smem_kb * 1024LL, smem_cap);
  // tile policy 4: the dynamic shared memory is the tcgen05 staging area; every other buffer in the slot
  if (P.tile_policy == 4) budget = 0;
  const int opt_vchunk = opts ? opts->vchunk : 0;
  const int opt_vert_smem = opts ? opts->vert_smem : 0;
  // Buffer placement for a shared-memory budget (bytes per CTA): truncation
  // arena, 1-row intermediates and vertical-energy buffers go to shared memory
  // when they fit, else to the CTA's workspace slot.
  auto lay_out = [&](DevPlan& Q, long long budget) {
    const long long mat_floats = al64(es * Q.nmax * (Q.nmax | 1));
    // a mixed plan's arena holds FP64 values: two floats each
    const long long trunc_all =
        Q.chain64 ? 2 * arena_doubles(Q.nmax, Q.kmax) : arena_floats(Q.nmax, Q.kmax, Q.trunc_method, Q.es);
    Q.arena_in_smem = 0;
    Q.mat_in_smem = 1;  // "theta lives inside the arena" (arena itself may be global)
    Q.arena_floats = trunc_all;
    // a mixed plan splits out theta and the inverse-iteration factors (FP64)
    const long long split_floats = Q.chain64 ? 2 * arena_split_doubles(Q.nmax, Q.kmax) : mat_floats;
    if (trunc_all * 4 <= budget) {
      Q.arena_in_smem = 1;
      Q.mat_in_smem = 1;
    } else if ((trunc_all - split_floats) * 4 <= budget && Q.trunc_method == 0) {
      Q.arena_in_smem = 1;
      Q.mat_in_smem = 0;
      Q.arena_floats = trunc_all - split_floats;
    }
    Q.arena_g_floats = Q.arena_in_smem ? (Q.mat_in_smem ? 0 : split_floats) : Q.arena_floats;
    Q.scr1 = (int)al64(es * std::max(chimax * chimax * D * D, (long long)D * D * D * D));
    {
      // one bond value of a vertical-energy intermediate holds <= chimax * D^3 floats
      const long long unit = es * chimax * D * D * D;
      const long long nbuf = 1 + 2LL * d;
      long long ch = (budget / 4) / (nbuf * unit);
      ch = std::max(1LL, std::min(ch, chimax));
      if (opt_vchunk > 0) ch = std::max(1LL, std::min(ch, (long long)opt_vchunk));
      Q.vchunk = (int)ch;
      Q.vbuf = (int)al64(ch * unit);
      // The vertical-energy buffers live in (L1-cached) global scratch with the
      // whole bond range in one chunk: fewer, larger GEMMs beat shared-memory
      // chunks of a few bond values (measured +5 % at 8x8, D=4, chi=16).
      // The vert_smem option puts them in the shared-memory arena, chunked.
      Q.vert_in_smem = 0;
      if (opt_vert_smem != 0 && !Q.gi && Q.arena_in_smem && nbuf * Q.vbuf * 4 <= budget) Q.vert_in_smem = 1;
    }
    Q.onerow_in_smem = 0;
    if (Q.arena_in_smem && std::max(Q.arena_floats, 4LL * Q.scr1) * 4 <= budget) {
      Q.onerow_in_smem = 1;
      Q.arena_floats = std::max(Q.arena_floats, 4LL * Q.scr1);
    }
    if (Q.vert_in_smem) {
      Q.arena_floats = std::max(Q.arena_floats, (1 + 2LL * d) * Q.vbuf);
    } else {
      Q.vchunk = (int)chimax;
      Q.vbuf = (int)SCR;
    }
    Q.TS = (int)TS; Q.ES = (int)ES; Q.E2S = (int)E2S; Q.MM = (int)MM; Q.SCR = (int)SCR;
    Q.n_scr = 11 + 2 * kMaxPhys;
    Q.VS = strategy == VMC_STRATEGY_VARIATIONAL ? (int)(es * chimax * D * chimax) : 0;
    Q.slot_floats = al64((long long)(R + 1) * C * TS) + al64(2 * (R + 2)) + al64(2LL * d * C) + al64(2LL * C) +
                    3 * al64((long long)C * TS) +
                    al64((long long)d * C * ES) + al64((long long)(d + 1) * ES) + al64((long long)C * E2S) +
                    2 * al64(E2S) +
                    al64(Q.arena_g_floats) +
                    (long long)Q.n_scr * al64(SCR) + al64(2LL * C * Q.VS) +
                    (Q.chain64 ? 2 * chain_f64_doubles(C, TS, SCR) : 0);
  };
  lay_out(P, budget);
  P.dyn_smem_bytes = P.tile_policy == 4 ? kTcStageBytes : (P.arena_in_smem ? P.arena_floats * 4 : 0);
  // The same plan with everything in the slot (no dynamic shared memory): an
  // uneven batch dominated by plans too large for shared memory runs them all
  // this way, so those keep the whole L1 (shared memory and L1 share one array).
  pl->hpg = P;
  lay_out(pl->hpg, 0);
  pl->hpg.dyn_smem_bytes = P.tile_policy == 4 ? kTcStageBytes : 0;
  P.cache_floats_per_chain = al64((long long)R * C * TS);
  if (chimax * D > kMaxVec) {
    delete pl;
    return VMC_ERR_UNSUPPORTED;
  }
  default_operator(pl);
  vmc_status st = upload_plan(pl);
  if (st != VMC_OK) {
    vmc_plan_destroy(pl);
    return st;
  }
  {
    const size_t smem = (size_t)P.dyn_smem_bytes;
    int per_sm = 4, occ = 0;
    if (kernels_of(P).prepare(P.threads, smem, &occ) == cudaSuccess && occ > 0) per_sm = occ;
    pl->slots_max = vmc_num_sms() * per_sm;
  }
  *out_plan = pl;
  return VMC_OK;
}

vmc_status vmc_peps_plan_set_operator(vmc_plan* pl, const double* onesite, const int* onesite_mask,
                                      const double* horiz, const int* horiz_mask, const double* vert,
                                      const int* vert_mask, int n_diag, const int* diag_nsites,
                                      const int* diag_site_off, const int* diag_sites, const int* diag_value_off,
                                      const double* diag_values) {
  if (!pl) return VMC_ERR_INVALID;
  DevPlan& P = pl->hp;
  HostOp& op = pl->op;
  default_operator(pl);
  const int d = P.d, d2 = d * d, R = P.R, C = P.C;
  // complex plans read (re, im) pairs for every matrix element
  const size_t es = (size_t)P.es;
  if (onesite && onesite_mask) {
    for (int s = 0; s < P.n_sites; ++s) {
      op.onesite_mask[s] = onesite_mask[s] != 0;
      for (size_t i = 0; i < es * d * d; ++i) op.onesite[es * s * d * d + i] = (float)onesite[es * s * d * d + i];
    }
  }
  if (horiz && horiz_mask && C > 1) {
    for (int t = 0; t < R * (C - 1); ++t) {
      op.horiz_mask[t] = horiz_mask[t] != 0;
      if (op.horiz_mask[t]) op.row_has_h[t / (C - 1)] = 1;
      for (size_t i = 0; i < es * d2 * d2; ++i) op.horiz[es * t * d2 * d2 + i] = (float)horiz[es * t * d2 * d2 + i];
    }
  }
  if (vert && vert_mask && R > 1) {
    for (int t = 0; t < (R - 1) * C; ++t) {
      op.vert_mask[t] = vert_mask[t] != 0;
      if (op.vert_mask[t]) op.row_has_v[t / C] = 1;
      for (size_t i = 0; i < es * d2 * d2; ++i) op.vert[es * t * d2 * d2 + i] = (float)vert[es * t * d2 * d2 + i];
    }
  }
  if (n_diag > 0) {
    if (!diag_nsites || !diag_site_off || !diag_sites || !diag_value_off || !diag_values) return VMC_ERR_INVALID;
    op.diag_nsites.assign(diag_nsites, diag_nsites + n_diag);
    op.diag_site_off.assign(diag_site_off, diag_site_off + n_diag);
    op.diag_value_off.assign(diag_value_off, diag_value_off + n_diag);
    int n_sites_total = 0, n_values = 0;
    for (int t = 0; t < n_diag; ++t) {
      if (diag_nsites[t] < 1) return VMC_ERR_INVALID;
      n_sites_total = std::max(n_sites_total, diag_site_off[t] + diag_nsites[t]);
      int nv = 1;
      for (int k = 0; k < diag_nsites[t]; ++k) nv *= d;
      n_values = std::max(n_values, diag_value_off[t] + nv);
    }
    op.diag_sites.assign(diag_sites, diag_sites + n_sites_total);
    for (int v : op.diag_sites)
      if (v < 0 || v >= P.n_sites) return VMC_ERR_INVALID;
    op.diag_values.assign(diag_values, diag_values + n_values);
  }
  P.n_diag = n_diag;
  pl->op_set = true;
  return upload_plan(pl);
}

vmc_status vmc_gi_set_operator(vmc_plan* pl, const double* hdiag, const double* vdiag, const double* plaq) {
  if (!pl || !pl->hp.gi) return VMC_ERR_INVALID;
  const DevPlan& P = pl->hp;
  HostOp& op = pl->op;
  default_operator(pl);
  const size_t N = (size_t)P.gi_N;
  if (hdiag) op.gi_hdiag.assign(hdiag, hdiag + (size_t)P.R * (P.C - 1) * N);
  if (vdiag) op.gi_vdiag.assign(vdiag, vdiag + (size_t)(P.R - 1) * P.C * N);
  if (plaq) op.gi_plaq.assign(plaq, plaq + (size_t)(P.R - 1) * (P.C - 1));
  pl->op_set = true;
  return upload_plan(pl);
}

void vmc_plan_destroy(vmc_plan* pl) {
  if (!pl) return;
  if (pl->dbuf) vmc_free(pl->dbuf);
  delete pl;
}

int64_t vmc_peps_n_params_sliced(const vmc_plan* pl) { return pl ? pl->hp.np_sliced : 0; }
int vmc_plan_resident_ctas(const vmc_plan* pl) { return pl ? pl->slots_max : 0; }
int64_t vmc_peps_n_params_full(const vmc_plan* pl) { return pl ? (int64_t)pl->hp.np_sliced * pl->hp.d : 0; }

size_t vmc_cache_size(const vmc_plan* pl, int n_chains) {
  if (!pl || n_chains < 0) return 0;
  return (size_t)n_chains * (pl->hp.cache_floats_per_chain * 4 + (size_t)pl->hp.R * 8);
}

static int n_slots(const vmc_plan* pl, int n_chains) { return std::max(1, std::min(n_chains, pl->slots_max)); }

size_t vmc_workspace_size(const vmc_plan* pl, int n_chains) {
  if (!pl || n_chains < 0) return 0;
  return ((size_t)pl->hp.perm_floats + (size_t)n_slots(pl, n_chains) * pl->hp.slot_floats) * 4;
}

// One job of a plan: the arguments of one C-ABI call.
static ChainJob chain_job(const vmc_plan* pl, int mode, const float* tensors, float* perm, int32_t* configs,
                          const double* uniforms, const int32_t* deltas, int n, void* cache, int full_gradient,
                          float* out_O, int8_t* out_p, double* out_E, double* logamp, double* sign, float* margin,
                          float* gap) {
  return ChainJob{pl->dplan, mode, n, full_gradient, 0, tensors, perm, configs, uniforms, deltas,
                  static_cast<float*>(cache), out_O, out_p, out_E, logamp, sign, margin, gap};
}

// The fused kernel over the n_chains of one job J on grid CTAs: the permuted
// tensors at the start of wsf, the CTA slots after them.
static vmc_status run_job(const vmc_plan* pl, void* stream, ChainJob J, float* wsf, int grid, int32_t* status) {
  const KernelSet& K = kernels_of(pl->hp);
  if (K.permute(pl->dplan, pl->hp.n_sites, J.tensors, wsf, stream) != cudaSuccess) return VMC_ERR_CUDA;
  J.perm = wsf;
  BatchJobs bj;
  std::memset(&bj, 0, sizeof(bj));
  bj.job[0] = J;
  bj.first[0] = 0;
  bj.first[1] = J.n_chains;
  bj.n_jobs = 1;
  bj.slot_floats = pl->hp.slot_floats;
  const size_t smem = (size_t)pl->hp.dyn_smem_bytes;
  return K.run(bj, grid, pl->hp.threads, smem, stream, wsf + pl->hp.perm_floats, nullptr, status) == cudaSuccess
             ? VMC_OK
             : VMC_ERR_CUDA;
}

static vmc_status launch(const vmc_plan* pl, void* stream, int mode, const float* tensors, int32_t* configs,
                         const double* uniforms, const int32_t* deltas, int n, void* cache, int full_gradient,
                         float* out_O, int8_t* out_p, double* out_E, double* logamp, double* sign, float* margin,
                         float* gap, void* ws, size_t ws_bytes, int32_t* status) {
  if (!pl || n < 0) return VMC_ERR_INVALID;
  if (n == 0) return VMC_OK;  // no chain: no buffer is read or written
  if (!tensors || !configs || !ws || !status) return VMC_ERR_INVALID;
  if (ws_bytes < vmc_workspace_size(pl, n)) return VMC_ERR_WORKSPACE;
  return run_job(pl, stream,
                 chain_job(pl, mode, tensors, nullptr, configs, uniforms, deltas, n, cache, full_gradient, out_O,
                           out_p, out_E, logamp, sign, margin, gap),
                 static_cast<float*>(ws), n_slots(pl, n), status);
}

vmc_status vmc_peps_init_cache(const vmc_plan* pl, void* stream, const float* tensors, const int32_t* configs,
                               int n_chains, void* cache, void* workspace, size_t workspace_bytes,
                               int32_t* status_dev) {
  if (!cache && n_chains > 0) return VMC_ERR_INVALID;
  return launch(pl, stream, MODE_INIT, tensors, const_cast<int32_t*>(configs), nullptr, nullptr, n_chains, cache, 0,
                nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, workspace, workspace_bytes,
                status_dev);
}

vmc_status vmc_peps_sweep(const vmc_plan* pl, void* stream, const float* tensors, int32_t* configs_inout,
                          const double* uniforms, const int32_t* deltas, int n_chains, void* cache_inout,
                          int full_gradient, float* out_O, int8_t* out_p, double* out_E, double* out_logamp,
                          double* out_sign, float* out_margin, float* out_gap, void* workspace,
                          size_t workspace_bytes, int32_t* status_dev) {
  if (!pl || (n_chains > 0 && (!uniforms || !cache_inout || !out_E || !out_logamp || !out_sign)))
    return VMC_ERR_INVALID;
  if (n_chains > 0 && needs_deltas(pl->hp) && !deltas) return VMC_ERR_INVALID;
  return launch(pl, stream, MODE_SWEEP, tensors, configs_inout, uniforms, deltas, n_chains, cache_inout,
                full_gradient, out_O, out_p, out_E, out_logamp, out_sign, out_margin, out_gap, workspace,
                workspace_bytes, status_dev);
}

vmc_status vmc_peps_vjp(const vmc_plan* pl, void* stream, const float* tensors, const int32_t* samples, int n,
                        const double* weights, double* out_grad, void* workspace, size_t workspace_bytes,
                        int32_t* status_dev) {
  if (!pl || n < 0 || !out_grad || (n > 0 && (!tensors || !samples || !weights || !workspace || !status_dev)))
    return VMC_ERR_INVALID;
  if (pl->hp.gi) return VMC_ERR_UNSUPPORTED;
  const size_t grad_bytes = (size_t)pl->hp.np_sliced * pl->hp.d * pl->hp.es * sizeof(double);
  if (vmc_memset(out_grad, 0, grad_bytes, static_cast<cudaStream_t>(stream)) != cudaSuccess) return VMC_ERR_CUDA;
  if (n == 0) return VMC_OK;
  if (workspace_bytes < vmc_workspace_size(pl, n)) return VMC_ERR_WORKSPACE;
  ChainJob J = chain_job(pl, MODE_VJP, tensors, nullptr, const_cast<int32_t*>(samples), nullptr, nullptr, n,
                         nullptr, 1, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
  J.vjp_w = weights;
  J.vjp_grad = out_grad;
  return run_job(pl, stream, J, static_cast<float*>(workspace), n_slots(pl, n), status_dev);
}

// Floats of the per-CTA cache entries of a recomputing sweep on grid CTAs.
static size_t recompute_cache_floats(const DevPlan& P, int grid) {
  return (size_t)grid * P.cache_floats_per_chain + 2 * (size_t)grid * P.R;
}

size_t vmc_sweep_recompute_workspace_size(const vmc_plan* pl, int n_chains) {
  if (!pl || n_chains < 0) return 0;
  return vmc_workspace_size(pl, n_chains) + recompute_cache_floats(pl->hp, n_slots(pl, n_chains)) * 4;
}

vmc_status vmc_peps_sweep_recompute(const vmc_plan* pl, void* stream, const float* tensors, int32_t* configs_inout,
                                    const double* uniforms, const int32_t* deltas, int n_chains, int full_gradient,
                                    float* out_O, int8_t* out_p, double* out_E, double* out_logamp,
                                    double* out_sign, float* out_margin, float* out_gap, void* workspace,
                                    size_t workspace_bytes, int32_t* status_dev) {
  if (!pl || n_chains < 0) return VMC_ERR_INVALID;
  if (n_chains == 0) return VMC_OK;
  if (!tensors || !configs_inout || !uniforms || !out_E || !out_logamp || !out_sign || !workspace || !status_dev)
    return VMC_ERR_INVALID;
  if (needs_deltas(pl->hp) && !deltas) return VMC_ERR_INVALID;
  if (workspace_bytes < vmc_sweep_recompute_workspace_size(pl, n_chains)) return VMC_ERR_WORKSPACE;
  const int grid = n_slots(pl, n_chains);
  float* wsf = static_cast<float*>(workspace);
  float* entries = wsf + pl->hp.perm_floats + (size_t)grid * pl->hp.slot_floats;
  ChainJob J = chain_job(pl, MODE_SWEEP, tensors, nullptr, configs_inout, uniforms, deltas, n_chains, entries,
                         full_gradient, out_O, out_p, out_E, out_logamp, out_sign, out_margin, out_gap);
  J.cache_per_cta = 1;
  return run_job(pl, stream, J, wsf, grid, status_dev);
}

// ---------------------------------------------------------------------------
// vmc_peps_amp_grad_noalloc: the amp_grad launch with its workspace in a fixed
// device array of this library (sized by VMC_NOALLOC_SCRATCH_BYTES).
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[VMC_NOALLOC_SCRATCH_BYTES];

#ifndef VMC_HOST_EMULATION
constexpr int kNoAllocMaxDevices = 64;
static void* g_noalloc_ptr[kNoAllocMaxDevices];
static std::mutex g_noalloc_mutex;
#endif

// Address of the scratch array on the current device, looked up once per device.
static vmc_status noalloc_scratch(void** out) {
#ifdef VMC_HOST_EMULATION
  *out = g_noalloc_scratch;
  return VMC_OK;
#else
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return VMC_ERR_CUDA;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return VMC_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return VMC_ERR_CUDA;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return VMC_OK;
#endif
}

vmc_status vmc_peps_amp_grad_noalloc(const vmc_plan* pl, void* stream, const float* tensors,
                                     const int32_t* samples, int n, int full_gradient, float* out_O,
                                     double* out_logamp, double* out_sign, float* out_gap, int32_t* status_dev) {
  if (!pl || n < 0 || (n > 0 && (!tensors || !samples || !out_logamp || !out_sign || !status_dev)))
    return VMC_ERR_INVALID;
  const size_t perm_bytes = (size_t)pl->hp.perm_floats * 4, slot_bytes = (size_t)pl->hp.slot_floats * 4;
  if (perm_bytes + slot_bytes > VMC_NOALLOC_SCRATCH_BYTES) return VMC_ERR_SCRATCH;
  if (n == 0) return VMC_OK;
  void* ws = nullptr;
  const vmc_status st = noalloc_scratch(&ws);
  if (st != VMC_OK) return st;
  const size_t fit = (VMC_NOALLOC_SCRATCH_BYTES - perm_bytes) / slot_bytes;
  const int grid = (int)std::min<size_t>({fit, (size_t)n, (size_t)pl->slots_max});
  return run_job(pl, stream,
                 chain_job(pl, MODE_AMPGRAD, tensors, nullptr, const_cast<int32_t*>(samples), nullptr, nullptr, n,
                           nullptr, full_gradient, out_O, nullptr, nullptr, out_logamp, out_sign, nullptr, out_gap),
                 static_cast<float*>(ws), grid, status_dev);
}

vmc_status vmc_peps_amp_grad(const vmc_plan* pl, void* stream, const float* tensors, const int32_t* samples, int n,
                             int full_gradient, float* out_O, double* out_logamp, double* out_sign, float* out_gap,
                             void* workspace, size_t workspace_bytes, int32_t* status_dev) {
  if (!pl || (n > 0 && (!out_logamp || !out_sign))) return VMC_ERR_INVALID;
  return launch(pl, stream, MODE_AMPGRAD, tensors, const_cast<int32_t*>(samples), nullptr, nullptr, n, nullptr,
                full_gradient, out_O, nullptr, nullptr, out_logamp, out_sign, nullptr, out_gap, workspace,
                workspace_bytes, status_dev);
}

vmc_status vmc_peps_local_energy(const vmc_plan* pl, void* stream, const float* tensors, const int32_t* samples,
                                 int n, const double* logamp, const double* sign, double* out_E, void* workspace,
                                 size_t workspace_bytes, int32_t* status_dev) {
  if (!pl || (n > 0 && (!logamp || !sign || !out_E))) return VMC_ERR_INVALID;
  return launch(pl, stream, MODE_ENERGY, tensors, const_cast<int32_t*>(samples), nullptr, nullptr, n, nullptr, 0,
                nullptr, nullptr, out_E, const_cast<double*>(logamp), const_cast<double*>(sign), nullptr, nullptr,
                workspace, workspace_bytes, status_dev);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Uneven batches.  Workspace: [item counter, 256 B][permuted tensors of each
// job, in the caller's order][grid slots of the largest slot_floats].
// ---------------------------------------------------------------------------
struct BatchLayout {
  int n = 0;                           // non-empty jobs
  int order[VMC_MAX_BATCH_JOBS];       // caller indices, decreasing cost per chain
  size_t perm_off[VMC_MAX_BATCH_JOBS]; // floats from the workspace start, by caller index
  size_t entry_off[VMC_MAX_BATCH_JOBS];  // per-CTA cache entries of recomputing sweeps (0: none)
  long long slot_floats = 0;
  size_t slots_off = 0;  // floats
  int grid = 0, threads = 0, es = 0, total = 0;
  int slot_layout = 0;  // 1: every plan with its no-shared-memory buffer placement
  const KernelSet* K = nullptr;  // one fused kernel for the whole table (standard or GI, one element type)
  size_t smem = 0, bytes = 0;
};

static bool job_valid(const vmc_peps_job& j) {
  if (!j.plan || j.n_chains < 0) return false;
  if (j.n_chains == 0) return true;
  if (!j.tensors || !j.configs) return false;
  switch (j.kind) {
    case VMC_JOB_INIT_CACHE: return j.cache != nullptr;
    case VMC_JOB_SWEEP:  // no cache: the sweep recomputes the bottom environments
      return j.uniforms && j.out_E && j.logamp && j.sign && (!needs_deltas(j.plan->hp) || j.deltas);
    case VMC_JOB_AMP_GRAD: return j.logamp && j.sign;
    case VMC_JOB_LOCAL_ENERGY: return j.logamp && j.sign && j.out_E;
    default: return false;
  }
}

static vmc_status batch_layout(const vmc_peps_job* jobs, int n_jobs, int layout, BatchLayout* L) {
  if (!jobs || n_jobs < 1) return VMC_ERR_INVALID;
  if (n_jobs > VMC_MAX_BATCH_JOBS) return VMC_ERR_UNSUPPORTED;
  if (layout < VMC_BATCH_LAYOUT_AUTO || layout > VMC_BATCH_LAYOUT_SLOT) return VMC_ERR_INVALID;
  size_t off = 64;  // the item counter
  long long total = 0;
  double cost[VMC_MAX_BATCH_JOBS];
  // Shared memory and L1 share one array per SM: when plans whose arena does
  // not fit shared memory (they lean on L1) carry most of the work, the whole
  // batch runs with no dynamic shared memory, every plan in its slot layout.
  double w_all = 0.0, w_slot = 0.0;
  for (int i = 0; i < n_jobs; ++i) {
    if (!job_valid(jobs[i])) return VMC_ERR_INVALID;
    const DevPlan& P = jobs[i].plan->hp;
    cost[i] = (double)P.n_sites * P.nmax * P.nmax * P.nmax * P.es * P.es;
    w_all += cost[i] * jobs[i].n_chains;
    if (!P.arena_in_smem) w_slot += cost[i] * jobs[i].n_chains;
  }
  L->slot_layout = layout == VMC_BATCH_LAYOUT_AUTO ? w_slot > 0.5 * w_all : layout == VMC_BATCH_LAYOUT_SLOT;
  for (int i = 0; i < n_jobs; ++i) {
    const vmc_peps_job& j = jobs[i];
    const DevPlan& P = L->slot_layout ? j.plan->hpg : j.plan->hp;
    if (L->threads == 0) {
      L->threads = P.threads;
      L->es = P.es;
      L->K = &kernels_of(P);
    } else if (P.threads != L->threads || P.es != L->es || &kernels_of(P) != L->K) {
      return VMC_ERR_UNSUPPORTED;
    }
    L->perm_off[i] = off;
    off += al64(P.perm_floats);
    if (j.n_chains == 0) continue;
    total += j.n_chains;
    L->slot_floats = std::max(L->slot_floats, P.slot_floats);
    L->smem = std::max(L->smem, (size_t)P.dyn_smem_bytes);
    L->order[L->n++] = i;
  }
  if (total > 0x7fffffffLL) return VMC_ERR_UNSUPPORTED;
  std::stable_sort(L->order, L->order + L->n, [&](int a, int b) { return cost[a] > cost[b]; });
  L->total = (int)total;
  L->slots_off = off;
  int per_sm = 4;
  if (L->n > 0) {
    if (L->K->prepare(L->threads, L->smem, &per_sm) != cudaSuccess) return VMC_ERR_CUDA;
    if (per_sm < 1) return VMC_ERR_UNSUPPORTED;
  }
  L->grid = (int)std::min<long long>(total, (long long)vmc_num_sms() * per_sm);
  off += (size_t)L->grid * (size_t)L->slot_floats;
  for (int i = 0; i < n_jobs; ++i) {
    L->entry_off[i] = 0;
    if (jobs[i].kind == VMC_JOB_SWEEP && !jobs[i].cache && jobs[i].n_chains > 0) {
      L->entry_off[i] = off;
      off += al64((long long)recompute_cache_floats(jobs[i].plan->hp, L->grid));
    }
  }
  L->bytes = off * 4;
  return VMC_OK;
}

static vmc_status launch_batch(const vmc_peps_job* jobs, const BatchLayout& L, void* stream, float* wsf,
                               int32_t* status) {
  static const int kMode[4] = {MODE_INIT, MODE_SWEEP, MODE_AMPGRAD, MODE_ENERGY};
  const KernelSet& K = *L.K;
  BatchJobs bj;
  std::memset(&bj, 0, sizeof(bj));
  bj.n_jobs = L.n;
  bj.slot_floats = L.slot_floats;
  bj.first[0] = 0;
  for (int k = 0; k < L.n; ++k) {
    const vmc_peps_job& j = jobs[L.order[k]];
    const int kind = j.kind;
    const bool sweep = kind == VMC_JOB_SWEEP, grad = sweep || kind == VMC_JOB_AMP_GRAD;
    bj.job[k] = chain_job(j.plan, kMode[kind], j.tensors, wsf + L.perm_off[L.order[k]], j.configs,
                          sweep ? j.uniforms : nullptr, sweep && needs_deltas(j.plan->hp) ? j.deltas : nullptr,
                          j.n_chains,
                          sweep && L.entry_off[L.order[k]] ? static_cast<void*>(wsf + L.entry_off[L.order[k]])
                          : (sweep || kind == VMC_JOB_INIT_CACHE) ? j.cache : nullptr,
                          j.full_gradient,
                          grad ? j.out_O : nullptr, sweep ? j.out_p : nullptr,
                          (sweep || kind == VMC_JOB_LOCAL_ENERGY) ? j.out_E : nullptr,
                          kind == VMC_JOB_INIT_CACHE ? nullptr : j.logamp,
                          kind == VMC_JOB_INIT_CACHE ? nullptr : j.sign, sweep ? j.out_margin : nullptr,
                          grad ? j.out_gap : nullptr);
    bj.job[k].cache_per_cta = sweep && L.entry_off[L.order[k]] ? 1 : 0;
    if (L.slot_layout) bj.job[k].P = j.plan->dplan_g;
    bj.first[k + 1] = bj.first[k] + j.n_chains;
    if (K.permute(j.plan->dplan, j.plan->hp.n_sites, j.tensors, wsf + L.perm_off[L.order[k]], stream) !=
        cudaSuccess)
      return VMC_ERR_CUDA;
  }
  int32_t* next = reinterpret_cast<int32_t*>(wsf);
  if (vmc_memset(next, 0, sizeof(int32_t), static_cast<cudaStream_t>(stream)) != cudaSuccess) return VMC_ERR_CUDA;
  return K.run(bj, L.grid, L.threads, L.smem, stream, wsf + L.slots_off, next, status) == cudaSuccess
             ? VMC_OK
             : VMC_ERR_CUDA;
}

extern "C" {

size_t vmc_batch_workspace_size_ex(const vmc_peps_job* jobs, int n_jobs, int layout) {
  BatchLayout L;
  return batch_layout(jobs, n_jobs, layout, &L) == VMC_OK ? L.bytes : 0;
}

size_t vmc_batch_workspace_size(const vmc_peps_job* jobs, int n_jobs) {
  return vmc_batch_workspace_size_ex(jobs, n_jobs, VMC_BATCH_LAYOUT_AUTO);
}

vmc_status vmc_peps_batch(const vmc_peps_job* jobs, int n_jobs, void* stream, void* workspace,
                          size_t workspace_bytes, int32_t* status_dev) {
  return vmc_peps_batch_ex(jobs, n_jobs, VMC_BATCH_LAYOUT_AUTO, stream, workspace, workspace_bytes, status_dev);
}

vmc_status vmc_peps_batch_ex(const vmc_peps_job* jobs, int n_jobs, int layout, void* stream, void* workspace,
                             size_t workspace_bytes, int32_t* status_dev) {
  if (!workspace || !status_dev) return VMC_ERR_INVALID;
  BatchLayout L;
  const vmc_status st = batch_layout(jobs, n_jobs, layout, &L);
  if (st != VMC_OK) return st;
  if (L.total == 0) return VMC_OK;
  if (workspace_bytes < L.bytes) return VMC_ERR_WORKSPACE;
  float* wsf = static_cast<float*>(workspace);
  return launch_batch(jobs, L, stream, wsf, status_dev);
}

}  // extern "C"
