// gi_device.cuh -- device side of the gauge-invariant PEPS in pure Z_N gauge
// theory (src/vmc/peps/gi/model.py, phys_dim = 1): slices selected by link
// values, plaquette Metropolis sweeps over row pairs and plaquette energies.
// Included by peps_device.cuh inside the element-type namespace, after the
// contraction helpers.
//
// A chain's state is the reference's flattened sample (model.py:121-144):
// sites[R][C] (all 0 without matter), h[R][C-1], v[R-1][C].  The "physical"
// index of a site is its slice: the base-N digits of its independent links
// (model.py:308-347), so the standard contraction, gradient and bottom-up
// machinery run unchanged on slices.

__device__ inline int gi_link(const DevPlan& P, const int32_t* st, bool horizontal, int r, int c) {
  return horizontal ? st[P.n_sites + r * (P.C - 1) + c] : st[P.n_sites + P.R * (P.C - 1) + r * P.C + c];
}

// Link value with the plaquette (fr, fc) flipped by delta (model.py:369-389); delta 0: no flip.
__device__ inline int gi_link_flipped(const DevPlan& P, const int32_t* st, bool horizontal, int r, int c, int fr,
                                      int fc, int delta) {
  int k = gi_link(P, st, horizontal, r, c);
  if (delta) {
    if (horizontal && c == fc && r == fr) k += delta;
    if (horizontal && c == fc && r == fr + 1) k -= delta;
    if (!horizontal && r == fr && c == fc) k += delta;
    if (!horizontal && r == fr && c == fc + 1) k -= delta;
    k %= P.gi_N;
    if (k < 0) k += P.gi_N;
  }
  return k;
}

// Slice of site (r, c) (model.py:308-347): digits of the active links in the order left, up, down,
// right, skipping the first active of right, down, up, left (fixed by Gauss law).
__device__ inline int gi_slice(const DevPlan& P, const int32_t* st, int r, int c, int fr = -1, int fc = -1,
                               int delta = 0) {
  const int R = P.R, C = P.C;
  const bool left = c > 0, right = c < C - 1, up = r > 0, down = r < R - 1;
  const int dependent = right ? 3 : down ? 2 : up ? 1 : left ? 0 : -1;  // 0 left, 1 up, 2 down, 3 right
  int idx = 0;
  if (left && dependent != 0) idx = idx * P.gi_N + gi_link_flipped(P, st, true, r, c - 1, fr, fc, delta);
  if (up && dependent != 1) idx = idx * P.gi_N + gi_link_flipped(P, st, false, r - 1, c, fr, fc, delta);
  if (down && dependent != 2) idx = idx * P.gi_N + gi_link_flipped(P, st, false, r, c, fr, fc, delta);
  if (right && dependent != 3) idx = idx * P.gi_N + gi_link_flipped(P, st, true, r, c, fr, fc, delta);
  return idx;
}

__device__ inline void gi_row_slices(const DevPlan& P, const int32_t* st, int r, int* dst) {
  for (int c = threadIdx.x; c < P.C; c += blockDim.x) dst[c] = gi_slice(P, st, r, c);
}

// Right 2-row environments of rows (r, r+1) between top row `top` and the bottom environment `bot`
// below row r+1 (energy.py:24-44), slices sp0 / sp1: S.r2[c] for c = C-1 .. 0, log-scales S.r2l.
__device__ __noinline__ void gi_right_envs_2row(const DevPlan& P, const Slot& S, Shared& sh, const float* perm,
                                          const float* top, const int* tbond, const float* bot, const int* bbond,
                                          int r, const int* sp0, const int* sp1, float* const* vb) {
  const int C = P.C;
  if (threadIdx.x == 0) {
    set_elem(S.r2 + (size_t)(C - 1) * P.E2S, 0, 1.f);
    S.r2l[C - 1] = 0.0;
  }
  __syncthreads();
  for (int c = C - 1; c >= 1; --c) {
    const int s0 = site_id(P, r, c), s1 = site_id(P, r + 1, c);
    const int U = P.sdim[4 * s0], V = P.sdim[4 * s0 + 1], Lb = P.sdim[4 * s0 + 2], Rb = P.sdim[4 * s0 + 3];
    const int V1 = P.sdim[4 * s1 + 1], Lb1 = P.sdim[4 * s1 + 2], Rb1 = P.sdim[4 * s1 + 3];
    const int ta = tbond[c], tb = tbond[c + 1], ba = bbond[c], bb = bbond[c + 1];
    const float* T = top + (size_t)c * P.TS;
    const float* B = bot + (size_t)c * P.TS;
    const float* Rin = S.r2 + (size_t)c * P.E2S;
    float* Rout = S.r2 + (size_t)(c - 1) * P.E2S;
    // P1[a][u][rr][y][f] = sum_b T[a][u][b] R2[b][rr][y][f]
    gemm(make_gemm(T, lin(tb), 1, Rin, lin(1), Rb * Rb1 * bb, vb[0], lin(Rb * Rb1 * bb), lin(1), ta * U,
                   Rb * Rb1 * bb, tb));
    // P2[a][l][f][v][y] = sum_{u,rr} P1 A(u,v,l,rr)
    gemm(make_gemm(vb[0], two(Rb1 * bb, U * Rb * Rb1 * bb, 1), Rb1 * bb, perm_of(P, perm, s0, P_RENV, sp0[c]),
                   lin(1), Lb * V, vb[1], three(Rb1, bb, Lb * bb * V * Rb1, 1, V * Rb1), two(V, bb * V * Rb1, Rb1),
                   ta * Rb1 * bb, Lb * V, U * Rb));
    // P3[a][l][x][w][f] = sum_{v,y} P2 A'(v,w,x,y)
    gemm(make_gemm(vb[1], lin(V * Rb1), 1, perm_of(P, perm, s1, P_R2, sp1[c]), lin(1), V1 * Lb1, vb[0],
                   two(bb, Lb1 * V1 * bb, 1), two(Lb1, bb, V1 * bb), ta * Lb * bb, V1 * Lb1, V * Rb1));
    // R2'[a][l][x][e] = sum_{w,f} P3 B[e][w][f]
    gemm(make_gemm(vb[0], lin(V1 * bb), 1, B, lin(V1 * bb), 1, Rout, lin(ba), lin(1), ta * Lb * Lb1, ba, V1 * bb));
    const double lg = cta_normalize(Rout, ta * Lb * Lb1 * ba * kEs, sh.red);
    if (threadIdx.x == 0) S.r2l[c - 1] = S.r2l[c] + lg;
  }
}

// Lout = Lin extended by column c of rows (r, r+1) with slices s0 (row r) and s1 (row r+1)
// (model.py:695-699, "alxe,aub,lruv,xyvw,ewf->bryf").  Lin: [a][l][x][e] at column c's left bonds;
// Lout: [b][rr][y][f] at its right bonds.  vb[0], vb[1]: scratch.
__device__ __noinline__ void gi_left_column(const DevPlan& P, const float* perm, const float* top, const int* tbond,
                                      const float* bot, const int* bbond, int r, int c, int s0slice, int s1slice,
                                      const float* Lin, float* Lout, float* const* vb) {
  const int s0 = site_id(P, r, c), s1 = site_id(P, r + 1, c);
  const int U = P.sdim[4 * s0], V = P.sdim[4 * s0 + 1], Lb = P.sdim[4 * s0 + 2], Rb = P.sdim[4 * s0 + 3];
  const int V1 = P.sdim[4 * s1 + 1], Lb1 = P.sdim[4 * s1 + 2], Rb1 = P.sdim[4 * s1 + 3];
  const int ta = tbond[c], tb = tbond[c + 1], ba = bbond[c], bb = bbond[c + 1];
  const float* T = top + (size_t)c * P.TS;
  const float* B = bot + (size_t)c * P.TS;
  // Q1[x][e][b][l][u] = sum_a L[a][(l,x,e)] T[a][u][b]
  gemm(make_gemm(Lin, lin(1), Lb * Lb1 * ba, T, two(tb, tb, 1), U * tb, vb[0], two(Lb1 * ba, U, tb * Lb * U),
                 two(tb, 1, Lb * U), Lb * Lb1 * ba, U * tb, ta));
  // Q2[e][b][rr][x][v] = sum_{l,u} Q1 A[s0](u,v,l,rr)
  gemm(make_gemm(vb[0], lin(Lb * U), 1, perm_of(P, perm, s0, P_LENV, s0slice), lin(1), Rb * V, vb[1],
                 two(ba * tb, V, Rb * Lb1 * V), two(V, Lb1 * V, 1), Lb1 * ba * tb, Rb * V, Lb * U));
  // Q3[b][rr][y][e][w] = sum_{x,v} Q2 A'[s1](v,w,x,y)
  gemm(make_gemm(vb[1], lin(Lb1 * V), 1, perm_of(P, perm, s1, P_ZIPT, s1slice), lin(1), V1 * Rb1, vb[0],
                 two(tb * Rb, V1, Rb1 * ba * V1), two(Rb1, 1, ba * V1), ba * tb * Rb, V1 * Rb1, Lb1 * V));
  // L'[b][rr][y][f] = sum_{e,w} Q3 B[e][w][f]
  gemm(make_gemm(vb[0], lin(ba * V1), 1, B, lin(1), bb, Lout, lin(bb), lin(1), tb * Rb * Rb1, bb, ba * V1));
}

// Elements of a 2-row environment at the left bonds of column c (c = C: the closing scalar).
__device__ inline int gi_env2_size(const DevPlan& P, const int* tbond, const int* bbond, int r, int c) {
  if (c >= P.C) return 1;
  const int s0 = site_id(P, r, c), s1 = site_id(P, r + 1, c);
  return tbond[c] * P.sdim[4 * s0 + 2] * P.sdim[4 * s1 + 2] * bbond[c];
}

// Plaquette Metropolis sweep of rows (r, r+1) (model.py:629-703): top = the top environment above
// row r, bot = the bottom environment below row r+1.  Updates the links in st; sh.spins[0] and
// [1] hold the slices of rows r and r+1 on return.
__device__ __noinline__ void gi_sweep_pair(const DevPlan& P, const Slot& S, Shared& sh, const float* perm, const float* top,
                              const int* tbond, const float* bot, const int* bbond, int r, int32_t* st,
                              const double* u, const int32_t* deltas, float* const* vb, float* min_margin) {
  const int C = P.C;
  gi_row_slices(P, st, r, sh.spins[0]);
  gi_row_slices(P, st, r + 1, sh.spins[1]);
  __syncthreads();
  gi_right_envs_2row(P, S, sh, perm, top, tbond, bot, bbond, r, sh.spins[0], sh.spins[1], vb);
  // L: left environment before column c; La: L extended by column c with its current slices (carried
  // from the previous plaquette); Lb: La extended by column c+1; Pa / Pb: the proposal's extensions
  float* L = S.l2[0];
  float* La = S.l2[1];
  float* Lb = S.scr[9];
  float* Pa = S.scr[10];
  float* Pb = S.scr[11];
  if (threadIdx.x == 0) set_elem(L, 0, 1.f);
  __syncthreads();
  if (C > 1) gi_left_column(P, perm, top, tbond, bot, bbond, r, 0, sh.spins[0][0], sh.spins[1][0], L, La, vb);
  for (int c = 0; c + 1 < C; ++c) {
    const int k = r * (C - 1) + c;
    const int delta = deltas ? deltas[k] : 1;
    // current and proposed slices of the plaquette's four sites
    const int c01 = sh.spins[0][c + 1], c11 = sh.spins[1][c + 1];
    const int p00 = gi_slice(P, st, r, c, r, c, delta), p01 = gi_slice(P, st, r, c + 1, r, c, delta);
    const int p10 = gi_slice(P, st, r + 1, c, r, c, delta), p11 = gi_slice(P, st, r + 1, c + 1, r, c, delta);
    const float* Rn = S.r2 + (size_t)(c + 1) * P.E2S;
    const int n2 = gi_env2_size(P, tbond, bbond, r, c + 2);
    gi_left_column(P, perm, top, tbond, bot, bbond, r, c + 1, c01, c11, La, Lb, vb);
    const double pc = abs2_dot(Lb, Rn, n2, sh.red);
    gi_left_column(P, perm, top, tbond, bot, bbond, r, c, p00, p10, L, Pa, vb);
    gi_left_column(P, perm, top, tbond, bot, bbond, r, c + 1, p01, p11, Pa, Pb, vb);
    const double pp = abs2_dot(Pb, Rn, n2, sh.red);
    // contraction.py:88-94
    const double ratio = pc > 0.0 ? pp / pc : (pp > 0.0 ? INFINITY : 0.0);
    const double thr = ratio < 1.0 ? ratio : 1.0;
    const bool accept = u[k] < thr;
    const float m = (float)fabs(thr - u[k]);
    if (m < *min_margin) *min_margin = m;
    __syncthreads();  // every thread has its slices and the dot products before the links change
    if (accept && threadIdx.x == 0) {
      const int N = P.gi_N;
      int* hl = st + P.n_sites;
      int* vl = st + P.n_sites + P.R * (C - 1);
      hl[r * (C - 1) + c] = ((hl[r * (C - 1) + c] + delta) % N + N) % N;
      hl[(r + 1) * (C - 1) + c] = ((hl[(r + 1) * (C - 1) + c] - delta) % N + N) % N;
      vl[r * C + c] = ((vl[r * C + c] + delta) % N + N) % N;
      vl[r * C + c + 1] = ((vl[r * C + c + 1] - delta) % N + N) % N;
      sh.spins[0][c] = p00;
      sh.spins[0][c + 1] = p01;
      sh.spins[1][c] = p10;
      sh.spins[1][c + 1] = p11;
    }
    __syncthreads();
    // the kept branch: the left environment past column c, renormalised by 2^-e, and its extension by
    // column c+1 (the next plaquette's La) scaled by the same exact power of two
    float* next = accept ? Pa : La;
    float* next_a = accept ? Pb : Lb;
    float* free0 = accept ? La : Pa;
    float* free1 = accept ? Lb : Pb;
    const double lg = cta_normalize(next, gi_env2_size(P, tbond, bbond, r, c + 1) * kEs, sh.red);
    const int e = (int)lrint(lg / 0.69314718055994530942);
    if (e != 0) {
      const float sc = ldexpf(1.f, -e);
      const int na = n2 * kEs;
      for (int i = threadIdx.x; i < na; i += blockDim.x) next_a[i] *= sc;
      __syncthreads();
    }
    float* old_L = L;
    L = next;
    La = next_a;
    Lb = old_L;
    Pa = free0;
    Pb = free1;
  }
}

// Plaquette energies of rows (r, r+1) (model.py:544-608): sum over plaquettes of
// coeff (psi(+1 flip) + psi(-1 flip)) / psi; sp0 / sp1 are the rows' slices, vsc the factor
// exp(log-scales of top and bottom - log psi) / sign.
__device__ __noinline__ void gi_plaquette_energy(const DevPlan& P, const Slot& S, Shared& sh, const float* perm,
                                    const float* top, const int* tbond, const float* bot, const int* bbond, int r,
                                    const int32_t* st, const int* sp0, const int* sp1, const double* vsc,
                                    float* const* vb, double* energy) {
  const int C = P.C;
  bool any = false;
  for (int c = 0; c + 1 < C; ++c) any = any || P.gi_plaq[r * (C - 1) + c] != 0.0;
  if (!any) return;
  gi_right_envs_2row(P, S, sh, perm, top, tbond, bot, bbond, r, sp0, sp1, vb);
  float* L = S.l2[0];
  float* Ln = S.l2[1];
  float* Pa = S.scr[10];
  float* Pb = S.scr[11];
  if (threadIdx.x == 0) set_elem(L, 0, 1.f);
  __syncthreads();
  double l2log = 0.0;
  for (int c = 0; c + 1 < C; ++c) {
    const double coeff = P.gi_plaq[r * (C - 1) + c];
    if (coeff != 0.0) {
      const float* Rn = S.r2 + (size_t)(c + 1) * P.E2S;
      const int n2 = gi_env2_size(P, tbond, bbond, r, c + 2);
      double s_re = 0.0, s_im = 0.0;
      // +1 and -1 flips; for N = 2 they are the same configuration
      const int n_delta = P.gi_N == 2 ? 1 : 2;
      for (int i = 0; i < n_delta; ++i) {
        const int delta = i == 0 ? 1 : -1;
        const int p00 = gi_slice(P, st, r, c, r, c, delta), p01 = gi_slice(P, st, r, c + 1, r, c, delta);
        const int p10 = gi_slice(P, st, r + 1, c, r, c, delta), p11 = gi_slice(P, st, r + 1, c + 1, r, c, delta);
        gi_left_column(P, perm, top, tbond, bot, bbond, r, c, p00, p10, L, Pa, vb);
        gi_left_column(P, perm, top, tbond, bot, bbond, r, c + 1, p01, p11, Pa, Pb, vb);
        double im = 0.0;
        s_re += elem_dot(Pb, Rn, n2, sh.red, &im);
        s_im += im;
      }
      if (P.gi_N == 2) {
        s_re *= 2.0;
        s_im *= 2.0;
      }
      const double f = exp(l2log + S.r2l[c + 1]);
      acc3(energy, coeff, 0.0, s_re, s_im, vsc[0] * f, vsc[1] * f);
    }
    gi_left_column(P, perm, top, tbond, bot, bbond, r, c, sp0[c], sp1[c], L, Ln, vb);
    l2log += cta_normalize(Ln, gi_env2_size(P, tbond, bbond, r, c + 1) * kEs, sh.red);
    float* t = L;
    L = Ln;
    Ln = t;
  }
}

// Link-diagonal energies (gi/local_terms.py:12-39): sum over links of diag[value].
__device__ __noinline__ double gi_link_energy(const DevPlan& P, const int32_t* st) {
  double e = 0.0;
  const int R = P.R, C = P.C, N = P.gi_N;
  for (int r = 0; r < R; ++r)
    for (int c = 0; c + 1 < C; ++c) e += P.gi_hdiag[(r * (C - 1) + c) * N + gi_link(P, st, true, r, c)];
  for (int r = 0; r + 1 < R; ++r)
    for (int c = 0; c < C; ++c) e += P.gi_vdiag[(r * C + c) * N + gi_link(P, st, false, r, c)];
  return e;
}

// One chain of a GI plan (gi/kernels.py:33-124): init_cache (bottom environments of the selected
// slices), transition (plaquette sweeps, model.py:901-957), estimate (O_k of the active slices,
// link-diagonal and plaquette energies, model.py:392-617), or the amplitude / gradient / energy
// evaluations on given samples; the CTA's workspace slot at slot_base.
__device__ __forceinline__ void gi_chain(const ChainJob& J, int chain, float* slot_base, int32_t* status) {
  const DevPlan& P = *J.P;
  VMC_SHARED Shared sh;
#ifdef VMC_HOST_EMULATION
  float* dyn_smem = emu_dyn_smem(P.arena_in_smem ? P.arena_floats : 0);
  std::memset(&sh, 0xff, sizeof(sh));
#else
  extern __shared__ float dyn_smem[];
#endif
  Slot S = make_slot(P, slot_base);
  if (threadIdx.x == 0) g_tile_policy = P.tile_policy;  // read by cta_gemm after the next barrier
  const Arena ar = make_arena(P, P.arena_in_smem ? dyn_smem : S.arena, S.arena);
  if (P.onerow_in_smem)
    for (int i = 0; i < 4; ++i) S.scr[3 + i] = dyn_smem + (size_t)i * P.scr1;
  float* vbuf[2] = {S.scr[7], S.scr[8]};  // GEMM scratch of the 2-row environment steps
  const int mode = J.mode, n_chains = J.n_chains, full_gradient = J.full_gradient;
  const float* perm = J.perm;
  float* cache = J.cache;
  const int R = P.R, C = P.C;
  const size_t n_plaq = (size_t)(R - 1) * (C - 1);
  const int n_params = full_gradient ? P.d * P.np_sliced : P.np_sliced;
  int32_t* st = J.configs + (size_t)chain * P.n_state;
  float min_gap = INFINITY;
  const bool own_entry = J.cache_per_cta != 0;
  const int ce = own_entry ? (int)blockIdx.x : chain, ce_n = own_entry ? (int)gridDim.x : n_chains;

  if (mode == MODE_INIT || (own_entry && mode == MODE_SWEEP)) {
    // gi/kernels.py:33-49: bottom environments from the bottom up
    double* lb = cache_logs(P, cache, ce_n, ce);
    fill_ones_row(P, cache_row(P, cache, ce, R - 1));
    if (threadIdx.x == 0) lb[R - 1] = 0.0;
    for (int r = R - 1; r >= 1; --r) {
      gi_row_slices(P, st, r, sh.spins[0]);
      __syncthreads();
      const double ls = apply_row(P, S, sh, perm, cache_row(P, cache, ce, r), bbonds(P, r),
                                  cache_row(P, cache, ce, r - 1), bbonds(P, r - 1), r, sh.spins[0], true, ar,
                                  &min_gap);
      if (threadIdx.x == 0) lb[r - 1] = lb[r] + ls;
      __syncthreads();
    }
    if (mode == MODE_INIT) return;
    min_gap = INFINITY;
  }

  // top-down: plaquette sweep of rows (r, r+1) against the cached bottom environment, then row r
  // into the top environment (model.py:928-957)
  float min_margin = INFINITY;
  fill_ones_row(P, S.topc);
  if (threadIdx.x == 0) S.lt[0] = 0.0;
  __syncthreads();
  for (int r = 0; r < R; ++r) {
    float* top = S.topc + (size_t)r * C * P.TS;
    if (mode == MODE_SWEEP && r + 1 < R)
      gi_sweep_pair(P, S, sh, perm, top, tbonds(P, r), cache_row(P, cache, ce, r + 1), bbonds(P, r + 1), r, st,
                    J.uniforms + chain * n_plaq, J.deltas ? J.deltas + chain * n_plaq : nullptr, vbuf, &min_margin);
    gi_row_slices(P, st, r, sh.spins[0]);
    __syncthreads();
    const double ls = apply_row(P, S, sh, perm, top, tbonds(P, r), S.topc + (size_t)(r + 1) * C * P.TS,
                                tbonds(P, r + 1), r, sh.spins[0], false, ar, &min_gap);
    if (threadIdx.x == 0) S.lt[r + 1] = S.lt[r] + ls;
    __syncthreads();
  }
  double sgn = 1.0;
  double logamp = S.lt[R] + contract_bottom(P, S.topc + (size_t)R * C * P.TS, tbonds(P, R), sh,
                                           reinterpret_cast<double*>(S.scr[0]), &sgn);
  if (mode == MODE_ENERGY) {
    logamp = J.logamp_io[chain];
    sgn = J.sign_io[chain];
  } else if (threadIdx.x == 0) {
    J.logamp_io[chain] = logamp;
    J.sign_io[chain] = sgn;
    if (J.out_margin && mode == MODE_SWEEP) J.out_margin[chain] = min_margin;
  }
  if (!isfinite(logamp) && threadIdx.x == 0) atomicOr(status, VMC_DEV_NONFINITE);

  // bottom-up estimate
  const bool want_grad = (mode == MODE_SWEEP || mode == MODE_AMPGRAD);
  const bool want_energy = (mode == MODE_SWEEP || mode == MODE_ENERGY);
  float* Orow = J.out_O ? elem(J.out_O, (size_t)chain * n_params) : nullptr;
  if (Orow && full_gradient) {
    for (int i = threadIdx.x; i < n_params * kEs; i += blockDim.x) Orow[i] = 0.f;
    __syncthreads();
  }
  double energy[2] = {0.0, 0.0};
  if (want_energy && threadIdx.x == 0) energy[0] = gi_link_energy(P, st);
  const double inv_re = kCplx ? cos(sgn) : sgn, inv_im = kCplx ? -sin(sgn) : 0.0;
  double* lbc = (mode == MODE_SWEEP) ? cache_logs(P, cache, ce_n, ce) : nullptr;
  double lb_cur = 0.0, lb_prev = 0.0;
  int ib_cur = 0, ib_prev = 1, ib_next = 2;
  fill_ones_row(P, S.brow[ib_cur]);
  for (int r = R - 1; r >= 0; --r) {
    gi_row_slices(P, st, r, sh.spins[0]);
    if (r + 1 < R) gi_row_slices(P, st, r + 1, sh.spins[1]);
    __syncthreads();
    float* bcur = S.brow[ib_cur];
    if (mode == MODE_SWEEP) {
      cta_copy(cache_row(P, cache, ce, r), bcur, C * P.TS);
      if (threadIdx.x == 0) lbc[r] = lb_cur;
    }
    const float* top = S.topc + (size_t)r * C * P.TS;
    if (want_grad) {
      const double om = exp(S.lt[r] + lb_cur - logamp);
      const double osc[2] = {inv_re * om, inv_im * om};
      estimate_row(P, S, sh, perm, J.tensors, top, tbonds(P, r), bcur, bbonds(P, r), r, sh.spins[0], osc, Orow,
                   full_gradient, true, false, energy);
    }
    if (want_energy && r + 1 < R) {
      const double vm = exp(S.lt[r] + lb_prev - logamp);
      const double vsc[2] = {inv_re * vm, inv_im * vm};
      gi_plaquette_energy(P, S, sh, perm, top, tbonds(P, r), S.brow[ib_prev], bbonds(P, r + 1), r, st,
                          sh.spins[0], sh.spins[1], vsc, vbuf, energy);
    }
    if (r > 0) {
      const double ls = apply_row(P, S, sh, perm, bcur, bbonds(P, r), S.brow[ib_next], bbonds(P, r - 1), r,
                                  sh.spins[0], true, ar, &min_gap);
      lb_prev = lb_cur;
      lb_cur = lb_cur + ls;
      const int t = ib_prev;
      ib_prev = ib_cur;
      ib_cur = ib_next;
      ib_next = t;
    }
  }
  if (J.out_gap && threadIdx.x == 0) J.out_gap[chain] = min_gap;
  if (want_energy && threadIdx.x == 0) {
    J.out_E[kEs * chain] = energy[0];
    if (kCplx) J.out_E[kEs * chain + 1] = energy[1];
    if (!isfinite(energy[0]) || !isfinite(energy[1])) atomicOr(status, VMC_DEV_NONFINITE);
  }
  if (J.out_p && mode == MODE_SWEEP) {
    // the slice index of every parameter (gi/kernels.py:101-118; the pure-gauge site index is 0)
    for (int s = 0; s < P.n_sites; ++s) {
      const int sz = ssize(P, s);
      const int8_t v = (int8_t)gi_slice(P, st, s / C, s % C);
      for (int i = threadIdx.x; i < sz; i += blockDim.x) J.out_p[(size_t)chain * P.np_sliced + P.site_osl[s] + i] = v;
    }
  }
  __syncthreads();
}
