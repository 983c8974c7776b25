// chain_f64.cuh -- the boundary-MPS chain of mixed-precision plans in
// double-float (df64.cuh: hi + lo in FP32, about 48 significant bits).
//
// Included by peps_device.cuh inside the real-element namespace of the
// mixed-precision kernel (VMC_CHAIN_F64).  Every tensor a boundary MPS is
// built from -- the zip-up carry, theta = carry . m . w, its Gram matrix, the
// eigensolver, the kept vectors and the stored boundary tensors that feed the
// next row's zip -- is held in df64.  Each new boundary tensor is also written
// as an FP32 copy for the environments, Metropolis ratios, gradients and
// energies, which stay FP32.
//
// Why the precision: ZipUp keeps the top-chi singular subspace of theta at
// every cut (strategy.py:128-150).  At 8x8, D=4, chi=16 the relative gap
// (s_chi - s_chi+1) / s_chi at the smallest cut of a sample is below 1e-2 for
// nearly every sample and reaches 2e-4, and the kept subspace moves by the
// relative error of the decomposition divided by that gap.  Measured against
// the FP64 oracle (24 chains, batch-mean E relative to mean|E_loc|, O_k
// Frobenius over the batch): an FP32 Gram eigensolver gives 1.2e-4 / 4.6e-4;
// an exact decomposition of FP32-rounded theta 1.0e-6 / 7.7e-6; FP32-rounded
// stored tensors and carry 5.2e-6 / 1.7e-5, and both roundings together
// 7.7e-6 / 2.7e-5.  The decomposition's arithmetic is what needs the precision;
// keeping the whole chain above FP32 gives 1.0e-6 / 4.9e-7, clear of the
// 1e-5 / 1e-4 bars, where FP32 storage alone would sit at the edge of the first.
//
// Why df64 and not FP64: this GPU issues FP64 at 1/64 of its FP32 rate, so a
// chain in FP64 keeps the FP64 pipe busy (56 % in the profile of the FP64
// version) in GEMM-shaped steps -- theta, its Gram matrix, the carry, the
// back-transform.  Here each GEMM product is an error-free FP32 product
// (fl(a_hi b_hi) plus its fmaf residual) with the cross terms, summed by
// Knuth's two-sum into an FP32 pair: FP32 instructions only.  The eigenvalue
// refinement and inverse iteration on the tridiagonal matrix stay FP64
// (O(n k) sequential work, cta_sym_topk_df).  Values are renormalised by
// powers of two at every cut, so the FP32 exponent range of hi and lo is ample.
#pragma once

// ---------------------------------------------------------------------------
// CTA GEMM with df64 accumulation: C (df64) = A B, A and B df64 or FP32 (the
// site tensors).  Same index maps and thread-tile interleaving as the FP32
// GEMM.  A product loses only the lo*lo term and the rounding of its residual
// (~2^-47 relative); the running sum is renormalised every 16 steps.
// ---------------------------------------------------------------------------
template <typename TA, typename TB>
struct GemmD {
  const TA* A;
  const TB* B;
  df64* C;
  int M, N, K;
  IMap am;
  int sak;
  IMap bn;
  int sbk;
  IMap cm, cn;
};

template <typename TA, typename TB>
__device__ inline GemmD<TA, TB> make_gemm_d(const TA* A, IMap am, int sak, const TB* B, IMap bn, int sbk, df64* C,
                                             IMap cm, IMap cn, int M, int N, int K) {
  GemmD<TA, TB> g;
  g.A = A; g.B = B; g.C = C; g.M = M; g.N = N; g.K = K;
  g.am = am; g.sak = sak; g.bn = bn; g.sbk = sbk; g.cm = cm; g.cn = cn;
  return g;
}

__device__ __forceinline__ void df_ld(const df64* p, float& h, float& l) {
  const df64 v = *p;
  h = v.hi;
  l = v.lo;
}
__device__ __forceinline__ void df_ld(const float* p, float& h, float& l) {
  h = *p;
  l = 0.f;
}

template <typename TA, typename TB, int TM, int TN>
__device__ __forceinline__ void gemm_tiles_d(const GemmD<TA, TB>& g) {
  constexpr bool AL = std::is_same<TA, df64>::value, BL = std::is_same<TB, df64>::value;
  const int tiles_m = (g.M + TM - 1) / TM;
  const int tiles_n = (g.N + TN - 1) / TN;
  const int n_tiles = tiles_m * tiles_n;
  for (int t = threadIdx.x; t < n_tiles; t += blockDim.x) {
    const int tn = t % tiles_n;
    const int tm = t / tiles_n;
    int aoff[TM], boff[TN];
    bool mv[TM], nv[TN];
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int m = tm + i * tiles_m;
      mv[i] = m < g.M;
      aoff[i] = imap(g.am, mv[i] ? m : 0);
    }
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int n = tn + j * tiles_n;
      nv[j] = n < g.N;
      boff[j] = imap(g.bn, nv[j] ? n : 0);
    }
    float sh[TM][TN], sl[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) sh[i][j] = sl[i][j] = 0.f;
    for (int k = 0; k < g.K; ++k) {
      float ah[TM], al[TM], bh[TN], bl[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) df_ld(g.A + aoff[i] + (size_t)k * g.sak, ah[i], al[i]);
#pragma unroll
      for (int j = 0; j < TN; ++j) df_ld(g.B + boff[j] + (size_t)k * g.sbk, bh[j], bl[j]);
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) df_mac<AL, BL>(sh[i][j], sl[i][j], ah[i], al[i], bh[j], bl[j]);
      if ((k & 15) == 15) {
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) df_renorm(sh[i][j], sl[i][j]);
      }
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      if (!mv[i]) continue;
      const int co = imap(g.cm, tm + i * tiles_m);
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        if (!nv[j]) continue;
        df_renorm(sh[i][j], sl[i][j]);
        g.C[co + imap(g.cn, tn + j * tiles_n)] = df64(sh[i][j], sl[i][j]);
      }
    }
  }
}

// CTA-wide df64 GEMM; ends with a barrier.
template <typename TA, typename TB>
__device__ inline void cta_gemm_d(const GemmD<TA, TB>& g) {
  const int work = g.M * g.N;
  const int nt = blockDim.x;
  if (g.M >= 4 && g.N >= 4 && work >= nt * 16) {
    gemm_tiles_d<TA, TB, 4, 4>(g);
  } else if (g.M >= 2 && g.N >= 2 && work >= nt * 4) {
    gemm_tiles_d<TA, TB, 2, 2>(g);
  } else {
    gemm_tiles_d<TA, TB, 1, 1>(g);
  }
  __syncthreads();
}

struct ArenaD {
  df64* mat;
  df64* G;
  df64* Y;
  EigScratchT<double> eig;
};

// Layout mirrored by arena_doubles() / arena_split_doubles() in
// peps_plan.cuh (a df64 takes the 8 bytes of a double).  With
// P.mat_in_smem == 0, theta and the inverse-iteration factors live at g (the
// slot) and the rest at p (shared memory).
__device__ inline ArenaD make_arena_d(const DevPlan& P, double* p, double* g) {
  ArenaD a;
  const int nmax = P.nmax, ld = P.nmax | 1, kmax = P.kmax;
  double*& q = P.mat_in_smem ? p : g;
  a.mat = reinterpret_cast<df64*>(q); q += al32((long long)nmax * ld);
  a.eig.lu = q; q += al32(4LL * kmax * nmax);
  a.G = reinterpret_cast<df64*>(p); p += al32((long long)nmax * ld);
  a.Y = reinterpret_cast<df64*>(p); p += al32((long long)nmax * kmax);
  a.eig.S = p; p += al32((long long)kmax * kmax);
  a.eig.sw = reinterpret_cast<unsigned char*>(p); p += al32(((long long)kmax * nmax + 7) / 8);
  a.eig.d = p; p += al32(nmax);
  a.eig.e = p; p += al32(nmax);
  a.eig.e2 = p; p += al32(nmax);
  a.eig.tau = p; p += al32(nmax);
  a.eig.v = p; p += al32(nmax);
  a.eig.p = p; p += al32(nmax);
  a.eig.lam = p; p += al32(nmax + 1);
  a.eig.cvec = p; p += al32(2LL * nmax);
  a.eig.part = p; p += al32(nmax + 64);
  a.eig.flag = reinterpret_cast<int*>(p); p += 32;
  a.eig.yr = nullptr;
  return a;
}

// Rescale x[0..n) by the power of two that brings max|x| into [0.5, 1) (exact
// on hi and lo); returns the log of the factor taken out.
__device__ inline double cta_normalize_df(df64* x, int n, double* red) {
  float m = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, fabsf(x[i].hi));
#ifndef VMC_HOST_EMULATION
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
#endif
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = (double)m;
  __syncthreads();
  m = 0.f;
  for (int w = 0; w < nw; ++w) m = fmaxf(m, (float)red[w]);
  __syncthreads();
  if (!(m > 0.f) || !isfinite(m)) return 0.0;
  int e = 0;
  frexpf(m, &e);
  if (e == 0) return 0.0;
  const float sc = ldexpf(1.f, -e);
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = df64(x[i].hi * sc, x[i].lo * sc);
  __syncthreads();
  return (double)e * 0.69314718055994530942;
}

// dst32[i] = the FP32 value of src[i]: the copy a boundary tensor's consumers read.
__device__ inline void cta_round_copy(float* dst, const df64* src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i].to_float();
  __syncthreads();
}

__device__ inline void fill_ones_row_d(const DevPlan& P, df64* row) {
  for (int c = threadIdx.x; c < P.C; c += blockDim.x) row[(size_t)c * P.TS] = df64(1.f, 0.f);
  __syncthreads();
}

// The df64 buffers of one chain's boundary-MPS chain: rows, carries and Z1
// carved from the slot's FP64-sized region (layout mirrored by
// chain_f64_doubles() in peps_plan.cuh), the arena at `arena` (shared memory or
// the slot's arena region) with its split-out part at `arena_g` (the slot's
// arena region).
struct ChainD {
  df64* row[2];  // current and next boundary MPS (C tensors at stride TS)
  df64* carry[2];
  df64* z1;
  ArenaD ar;
};

__device__ inline ChainD make_chain_d(const DevPlan& P, double* p, double* arena, double* arena_g) {
  ChainD c;
  for (int i = 0; i < 2; ++i) { c.row[i] = reinterpret_cast<df64*>(p); p += al32((long long)P.C * P.TS); }
  for (int i = 0; i < 2; ++i) { c.carry[i] = reinterpret_cast<df64*>(p); p += al32(P.SCR); }
  c.z1 = reinterpret_cast<df64*>(p);
  c.ar = make_arena_d(P, arena, arena_g);
  return c;
}

// Boundary-MPS row application (strategy.py:118-176, contraction.py:59-65) in
// df64: src and dst hold C tensors at stride TS; dst32 receives the FP32 copy
// of dst.  Returns the sum of the log-norms divided out of the new tensors.
// *min_gap receives the smallest relative eigen-gap (l_k - l_{k+1}) / l_k of
// the Gram matrix at a truncating cut.  ZipUp, DensityMatrix and NoTruncation.
__device__ __noinline__ double apply_row_hp(const DevPlan& P, Shared& sh, const float* perm, const df64* src,
                                            const int* bin, df64* dst, float* dst32, const int* bout, int row,
                                            const int* spins, bool from_below, const ChainD& ch, float* min_gap) {
  const int C = P.C;
  const ArenaD& ar = ch.ar;
  double logsum = 0.0;
  df64* carry = ch.carry[0];
  df64* carry_next = ch.carry[1];
  df64* Z1 = ch.z1;
  const df64 one(1.f, 0.f), zero(0.f, 0.f);
  if (threadIdx.x == 0) carry[0] = one;
  __syncthreads();
  int kc = 1;
  for (int c = 0; c < C; ++c) {
    const int s = site_id(P, row, c);
    const int U = P.sdim[4 * s], V = P.sdim[4 * s + 1], Lb = P.sdim[4 * s + 2], Rb = P.sdim[4 * s + 3];
    const int pin = from_below ? V : U;
    const int pout = from_below ? U : V;
    const float* Ap = perm_of(P, perm, s, from_below ? P_ZIPB : P_ZIPT, spins[c]);
    const int din = bin[c], dn = bin[c + 1];
    const df64* m = src + (size_t)c * P.TS;
    df64* out = dst + (size_t)c * P.TS;
    float* out32 = dst32 + (size_t)c * P.TS;
    if (P.strategy == VMC_STRATEGY_NO_TRUNCATION) {
      // out[d][l][q][r'][w] = sum_p m[d][p][r'] A(p, q, l, w)
      const int ncol = dn * Rb;
      cta_gemm_d(make_gemm_d(m, two(dn, pin * dn, 1), dn, Ap, three(pout, Rb, pin * pout * Rb, Rb, 1), pout * Rb,
                             out, two(dn, Lb * pout * ncol, Rb), three(pout, Rb, pout * ncol, ncol, 1), din * dn,
                             Lb * pout * Rb, pin));
      const int n_el = din * Lb * pout * ncol;
      logsum += cta_normalize_df(out, n_el, sh.red);
      cta_round_copy(out32, out, n_el);
      continue;
    }
    VMC_TSTART(tth);
    // Z1[k][l][p][r'] = sum_d carry[k][l][d] m[d][p][r']
    cta_gemm_d(make_gemm_d(static_cast<const df64*>(carry), lin(din), 1, m, lin(1), pin * dn, Z1, lin(pin * dn),
                           lin(1), kc * Lb, pin * dn, din));
    const int mrows = kc * pout;
    const int ncols = dn * Rb;
    if (c == C - 1) {
      // last site: untruncated, out[k][q][(r',w)]
      cta_gemm_d(make_gemm_d(static_cast<const df64*>(Z1), two(dn, Lb * pin * dn, 1), dn, Ap, lin(1), pout * Rb,
                             out, two(dn, pout * ncols, Rb), two(Rb, ncols, 1), kc * dn, pout * Rb, Lb * pin));
      const int n_el = mrows * ncols;
      logsum += cta_normalize_df(out, n_el, sh.red);
      cta_round_copy(out32, out, n_el);
      break;
    }
    const int kout = bout[c + 1];
    // theta as a row-major matrix: mat[(k,q)][(r',w)], odd leading dimension
    const int ldm = ncols | 1;
    df64* mat = ar.mat;
    const df64* cm = mat;
    cta_gemm_d(make_gemm_d(static_cast<const df64*>(Z1), two(dn, Lb * pin * dn, 1), dn, Ap, lin(1), pout * Rb, mat,
                           two(dn, pout * ldm, Rb), two(Rb, ldm, 1), kc * dn, pout * Rb, Lb * pin));
    VMC_TSTOP(tth, PH_THETA);
    if (P.strategy == VMC_STRATEGY_DENSITY_MATRIX) {
      // DensityMatrix (strategy.py:153-176): new tensor theta V, carry V^T, V = the top-kout eigenvectors
      // of rho = theta^T theta (V = I when every column is kept)
      if (kout >= ncols) {
        for (int e = threadIdx.x; e < ncols * kout; e += blockDim.x) ar.Y[e] = (e / kout == e % kout) ? one : zero;
        __syncthreads();
      } else {
        const int ldg = ncols | 1;
        cta_gemm_d(make_gemm_d(cm, lin(1), ldm, cm, lin(1), ldm, ar.G, lin(ldg), lin(1), ncols, ncols, mrows));
        cta_sym_topk_df(ar.G, ncols, ldg, kout, ar.Y, kout, ar.eig, sh.red);
        if (threadIdx.x == 0) {
          const double lk = ar.eig.lam[kout - 1], lk1 = ar.eig.lam[kout];
          const float gap = lk > 0.0 ? (float)fmax((lk - lk1) / lk, 0.0) : 0.f;
          if (gap < *min_gap) *min_gap = gap;
        }
      }
      cta_gemm_d(make_gemm_d(cm, lin(ldm), 1, static_cast<const df64*>(ar.Y), lin(1), kout, out, lin(kout), lin(1),
                             mrows, kout, ncols));
      for (int e = threadIdx.x; e < kout * ncols; e += blockDim.x) {
        const int kk = e / ncols, col = e % ncols;
        carry_next[(size_t)kk * ncols + (col % Rb) * dn + col / Rb] = ar.Y[(size_t)col * kout + kk];
      }
      __syncthreads();
    } else if (mrows <= ncols && kout >= mrows) {
      // every row direction is kept: U = I, carry = theta
      for (int e = threadIdx.x; e < mrows * mrows; e += blockDim.x) out[e] = (e / mrows == e % mrows) ? one : zero;
      for (int e = threadIdx.x; e < mrows * ncols; e += blockDim.x) {
        const int i = e / ncols, col = e % ncols;
        carry_next[(size_t)i * ncols + (col % Rb) * dn + col / Rb] = mat[(size_t)i * ldm + col];
      }
      __syncthreads();
    } else if (mrows > ncols && kout >= ncols) {
      // every column is kept: U = Q of the leading kout columns (an orthonormal basis of the column
      // space, exact for rank-deficient theta), carry = Q^T theta
      cta_householder_q<df64>(mat, mrows, kout, ldm, 1, out, kout, 1, ar.G, kout | 1,
                              reinterpret_cast<df64*>(ar.eig.tau));
      cta_gemm_d(make_gemm_d(static_cast<const df64*>(out), lin(1), kout, cm, lin(1), ldm, carry_next, lin(ncols),
                             two(Rb, 1, dn), kout, ncols, mrows));
    } else {
      // ---- Gram + tridiagonal eigensolver on the smaller side ----
      const bool rows_side = mrows <= ncols;
      const int nG = rows_side ? mrows : ncols;
      const int ldg = nG | 1;
      VMC_TSTART(tg);
      if (rows_side)  // G = theta theta^T
        cta_gemm_d(make_gemm_d(cm, lin(ldm), 1, cm, lin(ldm), 1, ar.G, lin(ldg), lin(1), nG, nG, ncols));
      else  // G = theta^T theta
        cta_gemm_d(make_gemm_d(cm, lin(1), ldm, cm, lin(1), ldm, ar.G, lin(ldg), lin(1), nG, nG, mrows));
      VMC_TSTOP(tg, PH_GRAM);
      cta_sym_topk_df(ar.G, nG, ldg, kout, ar.Y, kout, ar.eig, sh.red);
      if (threadIdx.x == 0 && kout < nG) {
        const double lk = ar.eig.lam[kout - 1], lk1 = ar.eig.lam[kout];
        const float gap = lk > 0.0 ? (float)((lk - lk1) / lk) : 0.f;
        if (gap < *min_gap) *min_gap = gap;
      }
      if (rows_side) {
        for (int e = threadIdx.x; e < mrows * kout; e += blockDim.x) out[e] = ar.Y[e];
        __syncthreads();
      } else {
        // U = theta V / |theta V| column-wise
        cta_gemm_d(make_gemm_d(cm, lin(ldm), 1, static_cast<const df64*>(ar.Y), lin(1), kout, out, lin(kout),
                               lin(1), mrows, kout, ncols));
        df64* nrm = reinterpret_cast<df64*>(ar.eig.cvec);
        for (int t = threadIdx.x; t < kout; t += blockDim.x) {
          df64 a = zero;
          for (int i = 0; i < mrows; ++i) a = vfma(out[(size_t)i * kout + t], out[(size_t)i * kout + t], a);
          nrm[t] = a;
        }
        __syncthreads();
        double* scale = ar.eig.v;  // free after the eigensolver
        for (int t = threadIdx.x; t < kout; t += blockDim.x) {
          double smax = 0.0;
          for (int q = 0; q < kout; ++q) smax = fmax(smax, nrm[q].to_double());
          const double s2 = nrm[t].to_double();
          scale[t] = (s2 > 1e-60 * smax && s2 > 0.0) ? 1.0 / sqrt(s2) : 0.0;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < mrows * kout; e += blockDim.x) out[e] = out[e] * df64(scale[e % kout]);
        __syncthreads();
      }
      // carry'[k'][w][r'] = sum_i U[i][k'] theta[i][(r',w)]
      VMC_TSTART(tc);
      cta_gemm_d(make_gemm_d(static_cast<const df64*>(out), lin(1), kout, cm, lin(1), ldm, carry_next, lin(ncols),
                             two(Rb, 1, dn), kout, ncols, mrows));
      VMC_TSTOP(tc, PH_CARRY);
    }
    logsum += cta_normalize_df(carry_next, kout * ncols, sh.red);
    logsum += cta_normalize_df(out, mrows * kout, sh.red);
    cta_round_copy(out32, out, mrows * kout);
    df64* t = carry;
    carry = carry_next;
    carry_next = t;
    kc = kout;
  }
  return logsum;
}

// contract_bottom (contraction.py:30-35) of a df64 boundary row: log|psi| and
// *sign_or_phase the sign.  One thread, FP64.
__device__ __noinline__ double contract_bottom_d(const DevPlan& P, const df64* row, const int* bonds, Shared& sh,
                                                 df64* tmp, double* sign_out) {
  if (threadIdx.x == 0) {
    double* v = reinterpret_cast<double*>(tmp);
    double* w = v + kMaxVec;
    v[0] = 1.0;
    for (int c = 0; c < P.C; ++c) {
      const int l = bonds[c], r = bonds[c + 1];
      const df64* t = row + (size_t)c * P.TS;
      for (int j = 0; j < r; ++j) {
        double a = 0.0;
        for (int i = 0; i < l; ++i) a = fma(v[i], t[(size_t)i * r + j].to_double(), a);
        w[j] = a;
      }
      for (int j = 0; j < r; ++j) v[j] = w[j];
    }
    sh.bcast[0] = v[0];
  }
  __syncthreads();
  const double vr = sh.bcast[0];
  __syncthreads();
  *sign_out = vr < 0 ? -1.0 : 1.0;
  return vr == 0.0 ? -INFINITY : log(fabs(vr));
}
