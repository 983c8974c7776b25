// peps_device.cuh -- the device side of the PEPS engine: contraction steps,
// boundary-MPS row application (ZipUp / Variational / NoTruncation),
// environments, Metropolis, estimate (O_k, E_loc) and the fused persistent
// kernel.
//
// Included by each kernel translation unit (peps_kernels_*.cu) inside a
// namespace that defines kCplx (complex elements) and kEs (floats per element:
// 1 for real FP32, 2 for complex64 stored as interleaved (re, im) floats).
// Every buffer size in the DevPlan counts floats; every tensor dimension counts
// elements.

// Code a gauge-invariant plan never runs (GI plans refuse DensityMatrix and the VJP mode) is left out of
// the GI kernel's translation unit, whose register allocation it would otherwise burden.
#ifdef VMC_GI_TU
constexpr bool kDensityMatrixCode = false, kVjpCode = false;
#else
constexpr bool kDensityMatrixCode = true, kVjpCode = true;
#endif

// GEMMs on this file's element type.  The conjugating variants are the
// conj(.) of the reference's complex contractions (no-ops for real elements).
__device__ inline void gemm(Gemm g) {
  g.cplx = kCplx;
  cta_gemm(g);
}
__device__ inline void gemm_ca(Gemm g) {
  g.cplx = kCplx;
  g.conja = kCplx;
  cta_gemm(g);
}
__device__ inline void gemm_cb(Gemm g) {
  g.cplx = kCplx;
  g.conjb = kCplx;
  cta_gemm(g);
}
// |<x, y>|^2 of the bilinear dot over n elements
__device__ inline double abs2_dot(const float* x, const float* y, int n, double* red) {
  if (kCplx) {
    double im = 0.0;
    const double re = cta_cdot(x, y, n, red, &im);
    return re * re + im * im;
  }
  const double v = cta_dot(x, y, n, red);
  return v * v;
}
// bilinear dot over n elements: (re, im)
__device__ inline double elem_dot(const float* x, const float* y, int n, double* red, double* im) {
  if (kCplx) return cta_cdot(x, y, n, red, im);
  *im = 0.0;
  return cta_dot(x, y, n, red);
}

// element e of a buffer of this file's element type
__device__ __forceinline__ float* elem(float* p, size_t e) { return p + kEs * e; }
__device__ __forceinline__ const float* elem(const float* p, size_t e) { return p + kEs * e; }
// x[e] = re (+ i 0)
__device__ __forceinline__ void set_elem(float* p, size_t e, float re) {
  p[kEs * e] = re;
  if (kCplx) p[kEs * e + 1] = 0.f;
}

__device__ inline int site_id(const DevPlan& P, int r, int c) { return r * P.C + c; }
__device__ inline int ssize(const DevPlan& P, int s) {
  const int* d4 = P.sdim + 4 * s;
  return d4[0] * d4[1] * d4[2] * d4[3];
}
__device__ inline const float* perm_of(const DevPlan& P, const float* perm, int s, int kind, int p) {
  return elem(perm, P.perm_off[s] + (size_t)(kind * P.d + p) * ssize(P, s));
}
__device__ inline const float* slice_of(const DevPlan& P, const float* tensors, int s, int p) {
  return elem(tensors, P.site_off[s] + (size_t)p * ssize(P, s));
}

// ---------------------------------------------------------------------------
// Permuted copies of the site tensors (shared by all chains).
// ---------------------------------------------------------------------------
__global__ void permute_tensors_kernel(const DevPlan* __restrict__ Pp, const float* __restrict__ tensors,
                                       float* __restrict__ perm) {
  const DevPlan& P = *Pp;
  for (int s = blockIdx.x; s < P.n_sites; s += gridDim.x) {
    const int U = P.sdim[4 * s], V = P.sdim[4 * s + 1], L = P.sdim[4 * s + 2], Rr = P.sdim[4 * s + 3];
    const int sz = U * V * L * Rr;
    const int total = P.d * sz;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
      const int p = i / sz;
      int t = i % sz;
      const int r = t % Rr; t /= Rr;
      const int l = t % L; t /= L;
      const int v = t % V;
      const int u = t / V;
      const float* x = elem(tensors, P.site_off[s] + i);
      float* base = elem(perm, P.perm_off[s]);
      const size_t dst[kPermKinds] = {
          (size_t)(P_ZIPT * P.d + p) * sz + ((l * U + u) * V + v) * Rr + r,   // [l][u][v][r]
          (size_t)(P_ZIPB * P.d + p) * sz + ((l * V + v) * U + u) * Rr + r,   // [l][v][u][r]
          (size_t)(P_RENV * P.d + p) * sz + ((u * Rr + r) * L + l) * V + v,   // [u][r][l][v]
          (size_t)(P_LENV * P.d + p) * sz + ((l * U + u) * Rr + r) * V + v,   // [l][u][r][v]
          (size_t)(P_R2 * P.d + p) * sz + ((u * Rr + r) * V + v) * L + l,     // [u][r][v][l]
          (size_t)(P_VRB * P.d + p) * sz + ((v * Rr + r) * L + l) * U + u};   // [v][r][l][u]
#pragma unroll
      for (int k = 0; k < kPermKinds; ++k)
#pragma unroll
        for (int f = 0; f < kEs; ++f) elem(base, dst[k])[f] = x[f];
    }
  }
}

// ---------------------------------------------------------------------------
// Contraction steps.  Dimension names: ta/tb top-MPS bonds left/right of the
// column, ba/bb bottom-MPS bonds, U/V up/down legs, Lb/Rb left/right legs.
// ---------------------------------------------------------------------------

// X1[a][u][rr][f] = sum_b T[a][u][b] R[b][rr][f]
__device__ inline void renv_step1(const float* T, const float* Rin, float* X1, int ta, int U, int tb, int Rb,
                                  int bb) {
  gemm(make_gemm(T, lin(tb), 1, Rin, lin(1), Rb * bb, X1, lin(Rb * bb), lin(1), ta * U, Rb * bb, tb));
}
// R'[a][l][e] = sum_{u,rr,v,f} X1[a][u][rr][f] A(u,v,l,rr) B[e][v][f]
__device__ inline void renv_step23(const float* X1, const float* Aperm_renv, const float* B, float* X2, float* Rout,
                                   int ta, int U, int Rb, int bb, int Lb, int V, int ba) {
  gemm(make_gemm(X1, two(bb, U * Rb * bb, 1), bb, Aperm_renv, lin(1), Lb * V, X2, two(bb, Lb * V * bb, 1),
                     lin(bb), ta * bb, Lb * V, U * Rb));
  gemm(make_gemm(X2, lin(V * bb), 1, B, lin(V * bb), 1, Rout, lin(ba), lin(1), ta * Lb, ba, V * bb));
}
// Y1[e][b][l][u] = sum_a L[a][l][e] T[a][u][b]
__device__ inline void lenv_step1(const float* Lin, const float* T, float* Y1, int ta, int Lb, int ba, int U,
                                  int tb) {
  gemm(make_gemm(Lin, lin(1), Lb * ba, T, lin(1), U * tb, Y1, two(ba, U, tb * Lb * U), two(tb, 1, Lb * U),
                     Lb * ba, U * tb, ta));
}
// L'[b][rr][f] = sum_{e,l,u,v} Y1[e][b][l][u] A(u,v,l,rr) B[e][v][f]
__device__ inline void lenv_step23(const float* Y1, const float* Aperm_lenv, const float* B, float* Y2, float* Lout,
                                   int ba, int tb, int Lb, int U, int Rb, int V, int bb) {
  gemm(make_gemm(Y1, lin(Lb * U), 1, Aperm_lenv, lin(1), Rb * V, Y2, two(tb, V, Rb * ba * V),
                     two(V, ba * V, 1), ba * tb, Rb * V, Lb * U));
  gemm(make_gemm(Y2, lin(ba * V), 1, B, lin(1), bb, Lout, lin(bb), lin(1), tb * Rb, bb, ba * V));
}
// G[u][v][l][rr] = alpha * sum Y1[e][b][l][u] B[e][v][f] R[b][rr][f]  (alpha = alpha_re + i alpha_im)
__device__ inline void grad_env(const float* Y1, const float* B, const float* Rc, float* W, float* G, int ba,
                                int V, int bb, int tb, int Rb, int Lb, int U, float alpha_re, float alpha_im) {
  gemm(make_gemm(B, lin(bb), 1, Rc, lin(bb), 1, W, two(V, tb * V * Rb, Rb), two(Rb, V * Rb, 1), ba * V,
                     tb * Rb, bb));
  Gemm g = make_gemm(Y1, lin(1), Lb * U, W, lin(1), V * Rb, G, two(U, Rb, V * Lb * Rb), two(Rb, Lb * Rb, 1),
                     Lb * U, V * Rb, ba * tb, alpha_re);
  g.alpha_im = alpha_im;
  gemm(g);
}

// ---------------------------------------------------------------------------
// Boundary-MPS row application (strategy.apply of strategy.py:118-150 and
// contraction.py:59-65).  src/dst hold C tensors at stride TS.  Returns the
// sum of log-norms divided out of the new tensors.  The truncation matrices
// live in `arena` (shared memory when they fit).  *min_gap receives the
// smallest relative eigen-gap (l_k - l_{k+1}) / l_k of theta theta^T seen at
// a truncating cut.
// ---------------------------------------------------------------------------
struct Arena {
  float* mat;
  float* G;
  float* Y;
  EigScratch eig;
};

__device__ inline Arena make_arena(const DevPlan& P, float* base, float* global_mat) {
  Arena a;
  const int nmax = P.nmax, ld = P.nmax | 1, kmax = P.kmax;
  // layout mirrored by arena_floats(); complex buffers hold kEs floats per element
  float* p = base;
  if (P.mat_in_smem) {
    a.mat = p;
    p += al64((long long)kEs * nmax * ld);
  } else {
    a.mat = global_mat;
  }
  a.G = p; p += al64((long long)kEs * nmax * ld);
  a.Y = p; p += al64((long long)kEs * nmax * (P.trunc_method == 1 ? ld : kmax));
  a.eig.S = p; p += al64((long long)kmax * kmax);
  a.eig.lu = p; p += al64(4LL * kmax * nmax);
  a.eig.sw = reinterpret_cast<unsigned char*>(p); p += al64(((long long)kmax * nmax + 3) / 4);
  a.eig.d = p; p += al64(nmax);
  a.eig.e = p; p += al64(nmax);
  a.eig.e2 = p; p += al64(nmax);
  a.eig.tau = p; p += al64((long long)kEs * nmax);
  a.eig.v = p; p += al64((long long)kEs * nmax);
  a.eig.p = p; p += al64((long long)kEs * nmax);
  a.eig.lam = p; p += al64(nmax + 1);
  a.eig.cvec = p; p += al64(2LL * kEs * nmax);
  a.eig.part = p; p += al64(nmax + 64);
  a.eig.flag = reinterpret_cast<int*>(p); p += 64;
  a.eig.yr = nullptr;
  if (kCplx) {
    a.eig.yr = p;
    p += al64((long long)nmax * kmax);
  }
  return a;
}


// Select the kout largest of sig[0..nv) into sh.sel (ties by index).
__device__ inline void select_topk(Shared& sh, int nv, int kout) {
  for (int j = threadIdx.x; j < nv; j += blockDim.x) {
    int rank = 0;
    const float sj = sh.sig[j];
    for (int i = 0; i < nv; ++i) {
      const float si = sh.sig[i];
      rank += (si > sj) || (si == sj && i < j);
    }
    if (rank < kout) sh.sel[rank] = j;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Variational compression sweeps (strategy.py:179-219 with the environments
// of :257-289 and the sweeps of :292-427).  On entry dst holds the
// QR-initialised result with the bond dimensions in sh.vb; on exit dst holds
// the result of n_sweeps (left-to-right, right-to-left) pairs, every tensor
// Frobenius-normalised, and the return value is the log of the scale taken
// out.  The bonds end at bout (the right-to-left sweep's LQ clamps a bond to
// phys * right).  Index names: src MPS m[d][p][r], row MPO W[l][p][q][w]
// (p = pin, q = pout), result T[a][q][b]; left environments LE[d][l][a],
// right environments RE[r][w][b].
//   lr site i:  X[a][l][p][r] = LE.m,  Y[a][q][r][w] = X.W,
//               optimal[a][q][b] = Y.RE,  T = Q of optimal,  LE' = Y.T
//   rl site i:  Z1[d][p][w][b] = m.RE,  Z2[d][l][q][b] = Z1.W',
//               optimal[a][(q,b)] = LE.Z2,  T = Q^T of optimal^T,  RE' = Z2.T
// Only the final right-to-left sweep's scales reach the state: its site-0
// tensor is the unnormalised optimum, built from right environments that
// were renormalised on the way.
// ---------------------------------------------------------------------------
// Q of the Householder QR of the leading k columns (real or complex elements)
__device__ inline void qr_q(const float* A, int m, int k, int ars, int acs, float* Q, int qrs, int qcs, float* H,
                            int ldh, float* tau) {
  if (kCplx)
    cta_householder_q_c(A, m, k, ars, acs, Q, qrs, qcs, H, ldh, tau);
  else
    cta_householder_q(A, m, k, ars, acs, Q, qrs, qcs, H, ldh, tau);
}

struct VSite {
  int din, dn, pin, pout, Lb, Rb;
  const float* m;
  const float* W;   // [l][p][q][w]
  const float* W2;  // [p][w][l][q]
};

__device__ inline VSite vsite(const DevPlan& P, const float* perm, const float* src, const int* bin, int row, int c,
                              const int* spins, bool from_below) {
  VSite v;
  const int s = site_id(P, row, c);
  const int U = P.sdim[4 * s], V = P.sdim[4 * s + 1];
  v.Lb = P.sdim[4 * s + 2];
  v.Rb = P.sdim[4 * s + 3];
  v.pin = from_below ? V : U;
  v.pout = from_below ? U : V;
  v.din = bin[c];
  v.dn = bin[c + 1];
  v.m = src + (size_t)c * P.TS;
  v.W = perm_of(P, perm, s, from_below ? P_ZIPB : P_ZIPT, spins[c]);
  v.W2 = perm_of(P, perm, s, from_below ? P_VRB : P_RENV, spins[c]);
  return v;
}

// Z2[d][l][q][b] (via Z1) for site v and right environment RE of bond kb.
__device__ inline void vright_z2(const VSite& v, const float* RE, int kb, float* Z1, float* Z2) {
  gemm(make_gemm(v.m, lin(v.dn), 1, RE, lin(1), v.Rb * kb, Z1, lin(v.Rb * kb), lin(1), v.din * v.pin, v.Rb * kb,
                     v.dn));
  gemm(make_gemm(Z1, two(kb, v.pin * v.Rb * kb, 1), kb, v.W2, lin(1), v.Lb * v.pout, Z2,
                     two(kb, v.Lb * v.pout * kb, 1), lin(kb), v.din * kb, v.Lb * v.pout, v.pin * v.Rb));
}

// RE'[d][l][c] = sum_{q,b} Z2[d][l][q][b] conj(T[c][q][b]), renormalised; returns log of its norm.
__device__ inline double vright_env(const VSite& v, const float* Z2, const float* T, int kb, int kt, float* REn,
                                    double* red) {
  const int qb = v.pout * kb;
  gemm_cb(make_gemm(Z2, lin(qb), 1, T, lin(qb), 1, REn, lin(kt), lin(1), v.din * v.Lb, kt, qb));
  const int n = v.din * v.Lb * kt;
  return cta_normalize(REn, n * kEs, red);
}

__device__ __noinline__ double variational_sweeps(const DevPlan& P, const Slot& S, Shared& sh, const float* perm,
                                                  const float* src, const int* bin, float* dst, int row,
                                                  const int* spins, bool from_below, const Arena& ar) {
  const int C = P.C;
  const size_t VS = (size_t)P.VS;
  float* LE = S.venv;
  float* RE = S.venv + (size_t)C * VS;
  float* X = S.scr[7];
  float* Y = S.scr[8];
  float* O = S.scr[9];
  int* vb = sh.vb;
  // right environments of the initial result
  if (threadIdx.x == 0) set_elem(RE + (size_t)(C - 1) * VS, 0, 1.f);
  __syncthreads();
  for (int i = C - 1; i >= 1; --i) {
    const VSite v = vsite(P, perm, src, bin, row, i, spins, from_below);
    vright_z2(v, RE + (size_t)i * VS, vb[i + 1], X, Y);
    vright_env(v, Y, dst + (size_t)i * P.TS, vb[i + 1], vb[i], RE + (size_t)(i - 1) * VS, sh.red);
  }
  double logsum = 0.0;
  for (int sweep = 0; sweep < P.n_sweeps; ++sweep) {
    // ---- left to right (strategy.py:292-356); the last site is recomputed by the next sweep ----
    if (threadIdx.x == 0) set_elem(LE, 0, 1.f);
    __syncthreads();
    for (int i = 0; i + 1 < C; ++i) {
      const VSite v = vsite(P, perm, src, bin, row, i, spins, from_below);
      const int ka = vb[i], kb = vb[i + 1];
      const float* LEi = LE + (size_t)i * VS;
      gemm(make_gemm(LEi, lin(1), v.Lb * ka, v.m, lin(1), v.pin * v.dn, X,
                         two(ka, v.pin * v.dn, v.Lb * v.pin * v.dn), lin(1), v.Lb * ka, v.pin * v.dn, v.din));
      gemm(make_gemm(X, two(v.dn, v.Lb * v.pin * v.dn, 1), v.dn, v.W, lin(1), v.pout * v.Rb, Y,
                         two(v.dn, v.pout * v.dn * v.Rb, v.Rb), two(v.Rb, v.dn * v.Rb, 1), ka * v.dn,
                         v.pout * v.Rb, v.Lb * v.pin));
      gemm(make_gemm(Y, lin(v.dn * v.Rb), 1, RE + (size_t)i * VS, lin(1), kb, O, lin(kb), lin(1), ka * v.pout, kb,
                         v.dn * v.Rb));
      const int mr = ka * v.pout;
      const int kt = kb < mr ? kb : mr;
      float* T = dst + (size_t)i * P.TS;
      qr_q(O, mr, kt, kb, 1, T, kt, 1, ar.G, kt | 1, ar.eig.tau);
      if (threadIdx.x == 0) vb[i + 1] = kt;
      float* LEn = LE + (size_t)(i + 1) * VS;
      // LE'[r][w][b] = sum_{a,q} Y[a][q][r][w] conj(T[a][q][b])
      gemm_cb(make_gemm(Y, lin(1), v.dn * v.Rb, T, lin(1), kt, LEn, lin(kt), lin(1), v.dn * v.Rb, kt, mr));
      const int n = v.dn * v.Rb * kt;
      cta_normalize(LEn, n * kEs, sh.red);
    }
    // ---- right to left (strategy.py:359-427) ----
    logsum = 0.0;
    if (threadIdx.x == 0) set_elem(RE + (size_t)(C - 1) * VS, 0, 1.f);
    __syncthreads();
    for (int i = C - 1; i >= 0; --i) {
      const VSite v = vsite(P, perm, src, bin, row, i, spins, from_below);
      const int ka = vb[i], kb = vb[i + 1];
      vright_z2(v, RE + (size_t)i * VS, kb, X, Y);
      const int qb = v.pout * kb;
      float* T = dst + (size_t)i * P.TS;
      float* opt = (i == 0) ? T : O;
      gemm(make_gemm(LE + (size_t)i * VS, lin(1), ka, Y, lin(1), qb, opt, lin(qb), lin(1), ka, qb, v.din * v.Lb));
      if (i == 0) {
        const int n = ka * qb;
        logsum += cta_normalize(T, n * kEs, sh.red);
        break;
      }
      // LQ through the QR of optimal^T (transpose, not adjoint): T[c][(q,b)] = Q[(q,b)][c]
      const int kt = ka < qb ? ka : qb;
      qr_q(O, qb, kt, 1, qb, T, 1, qb, ar.G, kt | 1, ar.eig.tau);
      if (threadIdx.x == 0) vb[i] = kt;
      logsum += vright_env(v, Y, T, kb, kt, RE + (size_t)(i - 1) * VS, sh.red);
      logsum += cta_normalize(T, kt * qb * kEs, sh.red);
    }
  }
  return logsum;
}

__device__ __noinline__ double apply_row(const DevPlan& P, const Slot& S, Shared& sh, const float* perm,
                                         const float* src, const int* bin, float* dst, const int* bout, int row,
                                         const int* spins, bool from_below, const Arena& ar, float* min_gap) {
  const int C = P.C;
  double logsum = 0.0;
  float* carry = S.scr[0];
  float* carry_next = S.scr[1];
  float* Z1 = S.scr[2];
  if (threadIdx.x == 0) {
    set_elem(carry, 0, 1.f);
    sh.vb[0] = bout[0];
    sh.vb[C] = bout[C];
  }
  __syncthreads();
  int kc = 1;
  for (int c = 0; c < C; ++c) {
    const int s = site_id(P, row, c);
    const int U = P.sdim[4 * s], V = P.sdim[4 * s + 1], Lb = P.sdim[4 * s + 2], Rb = P.sdim[4 * s + 3];
    const int pin = from_below ? V : U;
    const int pout = from_below ? U : V;
    const float* Ap = perm_of(P, perm, s, from_below ? P_ZIPB : P_ZIPT, spins[c]);
    const int din = bin[c], dn = bin[c + 1];
    const float* m = src + (size_t)c * P.TS;
    float* out = dst + (size_t)c * P.TS;
    if (P.strategy == VMC_STRATEGY_NO_TRUNCATION) {
      // out[d][l][q][r'][w] = sum_p m[d][p][r'] A(p, q, l, w)
      const int ncol = dn * Rb;
      gemm(make_gemm(m, two(dn, pin * dn, 1), dn, Ap, three(pout, Rb, pin * pout * Rb, Rb, 1), pout * Rb, out,
                         two(dn, Lb * pout * ncol, Rb), three(pout, Rb, pout * ncol, ncol, 1), din * dn,
                         Lb * pout * Rb, pin));
      const int n_el = din * Lb * pout * ncol;
      logsum += cta_normalize(out, n_el * kEs, sh.red);
      continue;
    }
    // Z1[k][l][p][r'] = sum_d carry[k][l][d] m[d][p][r']
    gemm(make_gemm(carry, lin(din), 1, m, lin(1), pin * dn, Z1, lin(pin * dn), lin(1), kc * Lb, pin * dn, din));
    const int mrows = kc * pout;
    const int ncols = dn * Rb;
    if (c == C - 1) {
      // last site: untruncated, out[k][q][(r',w)]
      gemm(make_gemm(Z1, two(dn, Lb * pin * dn, 1), dn, Ap, lin(1), pout * Rb, out, two(dn, pout * ncols, Rb),
                         two(Rb, ncols, 1), kc * dn, pout * Rb, Lb * pin));
      const int n_el = mrows * ncols;
      logsum += cta_normalize(out, n_el * kEs, sh.red);
      break;
    }
    // Variational: initialisation bonds min(chi, rows, cols) (strategy.py:244-246)
    const int kout = (P.strategy == VMC_STRATEGY_VARIATIONAL) ? min_i(P.chi, min_i(mrows, ncols)) : bout[c + 1];
    if (threadIdx.x == 0) sh.vb[c + 1] = kout;
    // theta as a row-major matrix: mat[(k,q)][(r',w)], odd leading dimension
    const int ldm = ncols | 1;
    float* mat = ar.mat;
    gemm(make_gemm(Z1, two(dn, Lb * pin * dn, 1), dn, Ap, lin(1), pout * Rb, mat, two(dn, pout * ldm, Rb),
                       two(Rb, ldm, 1), kc * dn, pout * Rb, Lb * pin));
    if (kDensityMatrixCode && P.strategy == VMC_STRATEGY_DENSITY_MATRIX) {
      // ---- DensityMatrix (strategy.py:153-176): rho = theta^H theta and its top-kout eigenvectors V;
      // the new tensor is theta V (columns not normalised) and the carry V^H.  With every column kept,
      // V = I: rho's eigenbasis is then any unitary, which the carry undoes in the next theta, and the
      // later column Grams (theta'^H theta') do not see it ----
      if (kout >= ncols) {
        for (int e = threadIdx.x; e < ncols * kout; e += blockDim.x) set_elem(ar.Y, e, (e / kout == e % kout) ? 1.f : 0.f);
        __syncthreads();
      } else {
        const int ldg = ncols | 1;
        gemm_ca(make_gemm(mat, lin(1), ldm, mat, lin(1), ldm, ar.G, lin(ldg), lin(1), ncols, ncols, mrows));
        if (kCplx)
          cta_herm_topk(ar.G, ncols, ldg, kout, ar.Y, kout, ar.eig, sh.red);
        else
          cta_sym_topk(ar.G, ncols, ldg, kout, ar.Y, kout, ar.eig, sh.red);
        if (threadIdx.x == 0) {
          // a kept eigenvalue at the rounding level of a null space: no gap (kept vectors arbitrary)
          const float lk = ar.eig.lam[kout - 1], lk1 = ar.eig.lam[kout];
          const float gap = lk > 0.f ? fmaxf((lk - lk1) / lk, 0.f) : 0.f;
          if (gap < *min_gap) *min_gap = gap;
        }
      }
      gemm(make_gemm(mat, lin(ldm), 1, ar.Y, lin(1), kout, out, lin(kout), lin(1), mrows, kout, ncols));
      // carry'[k'][w][r'] = conj(V[(r', w)][k'])
      for (int e = threadIdx.x; e < kout * ncols; e += blockDim.x) {
        const int kk = e / ncols, col = e % ncols;
        const float* y = elem(ar.Y, (size_t)col * kout + kk);
        float* c = elem(carry_next, (size_t)kk * ncols + (col % Rb) * dn + col / Rb);
        c[0] = y[0];
        if (kCplx) c[1] = -y[1];
      }
      __syncthreads();
    } else if (mrows <= ncols && kout >= mrows) {
      // every row direction is kept: U = I, carry = theta
      for (int e = threadIdx.x; e < mrows * mrows; e += blockDim.x) set_elem(out, e, (e / mrows == e % mrows) ? 1.f : 0.f);
      for (int e = threadIdx.x; e < mrows * ncols; e += blockDim.x) {
        const int i = e / ncols, col = e % ncols;
        const float* x = elem(mat, (size_t)i * ldm + col);
        float* y = elem(carry_next, (size_t)i * ncols + (col % Rb) * dn + col / Rb);
#pragma unroll
        for (int f = 0; f < kEs; ++f) y[f] = x[f];
      }
      __syncthreads();
    } else if (P.strategy == VMC_STRATEGY_VARIATIONAL || (mrows > ncols && kout >= ncols)) {
      // ---- QR: Variational initialisation (strategy.py:222-254), or a ZipUp cut that keeps every
      // column (U S V^T = theta exactly; an orthonormal basis of the column space is all that is
      // needed, and theta V / sigma would not be one for near-zero sigma).  U = Q of the leading
      // kout columns, carry = Q^H theta ----
      qr_q(mat, mrows, kout, ldm, 1, out, kout, 1, ar.G, kout | 1, ar.eig.tau);
      gemm_ca(make_gemm(out, lin(1), kout, mat, lin(1), ldm, carry_next, lin(ncols), two(Rb, 1, dn), kout, ncols,
                        mrows));
    } else if (!kCplx && P.trunc_method == 1) {
      // ---- reference path: one-sided Jacobi on the smaller set of vectors ----
      if (mrows >= ncols) {
        // vectors = columns: transpose into G (column j at G + j*ldc), keep theta in mat
        const int ldc = mrows | 1;
        float* V = ar.G;
        for (int e = threadIdx.x; e < mrows * ncols; e += blockDim.x) {
          const int i = e / ncols, j = e % ncols;
          V[(size_t)j * ldc + i] = mat[(size_t)i * ldm + j];
        }
        __syncthreads();
        {
          VMC_TSTART(tj);
          jacobi_orthogonalize(V, ncols, mrows, ldc, nullptr, 0, 0, kJacobiTol, kJacobiSweeps, &sh.flag);
          VMC_TSTOP(tj, PH_JACOBI);
        }
        for (int j = threadIdx.x; j < ncols; j += blockDim.x) {
          float a = 0.f;
          for (int i = 0; i < mrows; ++i) a = fmaf(V[(size_t)j * ldc + i], V[(size_t)j * ldc + i], a);
          sh.sig[j] = a;
        }
        __syncthreads();
        select_topk(sh, ncols, kout);
        float smax = 0.f;
        for (int i = 0; i < ncols; ++i) smax = fmaxf(smax, sh.sig[i]);
        for (int e = threadIdx.x; e < mrows * kout; e += blockDim.x) {
          const int i = e / kout, kk = e % kout;
          const int j = sh.sel[kk];
          const float s2 = sh.sig[j];
          out[e] = (s2 > 1e-30f * smax && s2 > 0.f) ? V[(size_t)j * ldc + i] / sqrtf(s2) : 0.f;
        }
        __syncthreads();
        gemm(make_gemm(out, lin(1), kout, mat, lin(1), ldm, carry_next, lin(ncols), two(Rb, 1, dn), kout, ncols,
                           mrows));
      } else {
        float* Q = ar.Y;
        const int ldq = mrows;
        for (int e = threadIdx.x; e < mrows * mrows; e += blockDim.x) Q[e] = (e / mrows == e % mrows) ? 1.f : 0.f;
        __syncthreads();
        VMC_TSTART(tj);
        jacobi_orthogonalize(mat, mrows, ncols, ldm, Q, mrows, ldq, kJacobiTol, kJacobiSweeps, &sh.flag);
        VMC_TSTOP(tj, PH_JACOBI);
        for (int j = threadIdx.x; j < mrows; j += blockDim.x) {
          float a = 0.f;
          for (int i = 0; i < ncols; ++i) a = fmaf(mat[(size_t)j * ldm + i], mat[(size_t)j * ldm + i], a);
          sh.sig[j] = a;
        }
        __syncthreads();
        select_topk(sh, mrows, kout);
        for (int e = threadIdx.x; e < mrows * kout; e += blockDim.x) {
          const int i = e / kout, kk = e % kout;
          out[e] = Q[(size_t)sh.sel[kk] * ldq + i];
        }
        for (int e = threadIdx.x; e < kout * ncols; e += blockDim.x) {
          const int kk = e / ncols, col = e % ncols;
          carry_next[(size_t)kk * ncols + (col % Rb) * dn + col / Rb] = mat[(size_t)sh.sel[kk] * ldm + col];
        }
        __syncthreads();
      }
    } else {
      // ---- Gram + tridiagonal eigensolver on the smaller side ----
      VMC_TSTART(tj);
      const bool rows_side = mrows <= ncols;
      const int nG = rows_side ? mrows : ncols;
      const int ldg = nG | 1;
      VMC_TSTART(tg);
      if (rows_side) {
        // G = theta theta^H
        gemm_cb(make_gemm(mat, lin(ldm), 1, mat, lin(ldm), 1, ar.G, lin(ldg), lin(1), nG, nG, ncols));
      } else {
        // G = theta^H theta
        gemm_ca(make_gemm(mat, lin(1), ldm, mat, lin(1), ldm, ar.G, lin(ldg), lin(1), nG, nG, mrows));
      }
      VMC_TSTOP(tg, PH_GRAM);
      if (kCplx)
        cta_herm_topk(ar.G, nG, ldg, kout, ar.Y, kout, ar.eig, sh.red);
      else
        cta_sym_topk(ar.G, nG, ldg, kout, ar.Y, kout, ar.eig, sh.red);
      if (threadIdx.x == 0 && kout < nG) {
        const float lk = ar.eig.lam[kout - 1], lk1 = ar.eig.lam[kout];
        const float gap = lk > 0.f ? (lk - lk1) / lk : 0.f;
        if (gap < *min_gap) *min_gap = gap;
      }
      if (rows_side) {
        for (int e = threadIdx.x; e < mrows * kout * kEs; e += blockDim.x) out[e] = ar.Y[e];
        __syncthreads();
      } else {
        // U = theta V / |theta V| column-wise
        gemm(make_gemm(mat, lin(ldm), 1, ar.Y, lin(1), kout, out, lin(kout), lin(1), mrows, kout, ncols));
        for (int t = threadIdx.x; t < kout; t += blockDim.x) {
          float a = 0.f;
          for (int i = 0; i < mrows; ++i) {
            const float* u = elem(out, (size_t)i * kout + t);
#pragma unroll
            for (int f = 0; f < kEs; ++f) a = fmaf(u[f], u[f], a);
          }
          sh.sig[t] = a;
        }
        __syncthreads();
        float smax = 0.f;
        for (int t = 0; t < kout; ++t) smax = fmaxf(smax, sh.sig[t]);
        for (int e = threadIdx.x; e < mrows * kout; e += blockDim.x) {
          const float s2 = sh.sig[e % kout];
          const float sc = (s2 > 1e-30f * smax && s2 > 0.f) ? 1.f / sqrtf(s2) : 0.f;
          float* u = elem(out, e);
#pragma unroll
          for (int f = 0; f < kEs; ++f) u[f] *= sc;
        }
        __syncthreads();
      }
      // carry'[k'][w][r'] = sum_i conj(U[i][k']) theta[i][(r',w)]
      VMC_TSTART(tc);
      gemm_ca(make_gemm(out, lin(1), kout, mat, lin(1), ldm, carry_next, lin(ncols), two(Rb, 1, dn), kout, ncols,
                        mrows));
      VMC_TSTOP(tc, PH_CARRY);
      VMC_TSTOP(tj, PH_JACOBI);
    }
    // renormalise the carry: its norm shrinks by the contraction at every
    // site, and a Gram matrix of a tiny theta underflows FP32 a few sites on
    {
      const int n_el = kout * ncols;
      logsum += cta_normalize(carry_next, n_el * kEs, sh.red);
    }
    // renormalise the new tensor
    {
      const int n_el = mrows * kout;
      logsum += cta_normalize(out, n_el * kEs, sh.red);
    }
    float* t = carry;
    carry = carry_next;
    carry_next = t;
    kc = kout;
  }
  if (P.strategy == VMC_STRATEGY_VARIATIONAL && P.n_sweeps > 0 && C > 1)
    logsum = variational_sweeps(P, S, sh, perm, src, bin, dst, row, spins, from_below, ar);
  return logsum;
}

// contract_bottom (contraction.py:30-35): product of the row's matrices
// t[:, 0, :], evaluated by one thread in FP64 using `tmp` (>= 2*max bond
// doubles of workspace).
// Amplitude of the final top row: the product of its matrices t[:, 0, :],
// evaluated by one thread in FP64 using `tmp` (>= 4 * kMaxVec doubles).
// Returns log|psi|; *sign_or_phase receives the sign (real elements) or the
// phase in radians (complex elements).
__device__ __noinline__ double contract_bottom(const DevPlan& P, const float* row, const int* bonds, Shared& sh,
                                               double* tmp, double* sign_or_phase) {
  if (threadIdx.x == 0) {
    double* v = tmp;
    double* w = tmp + 2 * kMaxVec;
    v[0] = 1.0;
    v[1] = 0.0;
    for (int c = 0; c < P.C; ++c) {
      const int l = bonds[c], r = bonds[c + 1];
      const float* t = row + (size_t)c * P.TS;
      for (int j = 0; j < r; ++j) {
        double ar = 0.0, ai = 0.0;
        for (int i = 0; i < l; ++i) {
          const float* x = elem(t, (size_t)i * r + j);
          if (kCplx) {
            ar += v[2 * i] * (double)x[0] - v[2 * i + 1] * (double)x[1];
            ai += v[2 * i] * (double)x[1] + v[2 * i + 1] * (double)x[0];
          } else {
            ar += v[2 * i] * (double)x[0];
          }
        }
        w[2 * j] = ar;
        w[2 * j + 1] = ai;
      }
      for (int j = 0; j < 2 * r; ++j) v[j] = w[j];
    }
    sh.bcast[0] = v[0];
    sh.bcast[1] = v[1];
  }
  __syncthreads();
  const double vr = sh.bcast[0], vi = sh.bcast[1];
  __syncthreads();
  if (kCplx) {
    *sign_or_phase = atan2(vi, vr);
    const double mag = hypot(vr, vi);
    return mag == 0.0 ? -INFINITY : log(mag);
  }
  *sign_or_phase = vr < 0 ? -1.0 : 1.0;
  return vr == 0.0 ? -INFINITY : log(fabs(vr));
}

__device__ inline void fill_ones_row(const DevPlan& P, float* row) {
  for (int c = threadIdx.x; c < P.C; c += blockDim.x) set_elem(row + (size_t)c * P.TS, 0, 1.f);
  __syncthreads();
}

#ifndef VMC_CHAIN_F64
#define VMC_CHAIN_F64 0
#endif
#if VMC_CHAIN_F64
#include "chain_f64.cuh"
#endif

// op element (re, im) of a real or complex operator table
__device__ __forceinline__ void op_elem(const float* table, size_t e, double* re, double* im) {
  const float* x = elem(table, e);
  *re = x[0];
  *im = kCplx ? (double)x[1] : 0.0;
}

// Pairs (p, q), as bit p*d + q, whose coefficient in column `col` of the d^2 x d^2 two-site operator
// `op` (element (j, col) at j*d*d + col) is nonzero: the only amplitudes psi(p, q) that E_loc uses.
// For a Heisenberg bond with parallel spins that is the configuration's own pair alone.
__device__ __forceinline__ unsigned nonzero_pairs(const float* op, int d, int col) {
  unsigned m = 0;
  for (int j = 0; j < d * d; ++j) {
    double re, im;
    op_elem(op, (size_t)j * d * d + col, &re, &im);
    if (re != 0.0 || im != 0.0) m |= 1u << j;
  }
  return m;
}

// Right environments of one row: R[q][c] for c = C-1..0 (R_c covers columns
// > c), at renv[q][c] for the current spin q of site c+1 (read through
// renv_cur()).  With open_q, also for every other q that the horizontal term
// of the bond (c, c+1) meets with a nonzero coefficient.
__device__ __noinline__ void right_envs(const DevPlan& P, const Slot& S, Shared& sh, const float* perm,
                                       const float* top, const int* tbond, const float* bot, const int* bbond, int row,
                                       const int* spins, bool open_q) {
  const int C = P.C;
  float* X1 = S.scr[3];
  float* X2 = S.scr[4];
  // R_{C-1} = [1] for every q slot
  for (int q = threadIdx.x; q < P.d; q += blockDim.x) {
    set_elem(S.renv + ((size_t)q * C + (C - 1)) * P.ES, 0, 1.f);
    S.rl[(size_t)q * C + (C - 1)] = 0.0;
  }
  __syncthreads();
  for (int c = C - 1; c >= 1; --c) {
    // absorb site c into R_c -> R_{c-1}
    const int s = site_id(P, row, c);
    const int U = P.sdim[4 * s], V = P.sdim[4 * s + 1], Lb = P.sdim[4 * s + 2], Rb = P.sdim[4 * s + 3];
    const int ta = tbond[c], tb = tbond[c + 1], ba = bbond[c], bb = bbond[c + 1];
    const float* T = top + (size_t)c * P.TS;
    const float* B = bot + (size_t)c * P.TS;
    // R_c (current spin of site c+1) lives in slot spin(c+1); for c = C-1 all slots hold [1]
    const int qin = (c == C - 1) ? 0 : spins[c + 1];
    const float* Rin = S.renv + ((size_t)qin * C + c) * P.ES;
    const double lin_c = S.rl[(size_t)qin * C + c];
    renv_step1(T, Rin, X1, ta, U, tb, Rb, bb);
    // R_{c-1}^(q) for the configuration's spin of site c and, when the bond (c-1, c) carries a term, for
    // every q that meets a nonzero coefficient of its operator
    unsigned qm = 0;
    if (open_q && P.horiz_mask[row * (C - 1) + c - 1]) {
      const unsigned jm = nonzero_pairs(elem(P.horiz, (size_t)(row * (C - 1) + c - 1) * P.d * P.d * P.d * P.d),
                                        P.d, spins[c - 1] * P.d + spins[c]);
      for (int p = 0; p < P.d; ++p) qm |= (jm >> (p * P.d)) & ((1u << P.d) - 1u);
    }
    for (int q = 0; q < P.d; ++q) {
      if (q != spins[c] && !((qm >> q) & 1u)) continue;
      float* Rout = S.renv + ((size_t)q * C + (c - 1)) * P.ES;
      renv_step23(X1, perm_of(P, perm, s, P_RENV, q), B, X2, Rout, ta, U, Rb, bb, Lb, V, ba);
      const double lg = cta_normalize(Rout, ta * Lb * ba * kEs, sh.red);
      if (threadIdx.x == 0) S.rl[(size_t)q * C + (c - 1)] = lin_c + lg;
    }
  }
}

__device__ inline const float* renv_cur(const DevPlan& P, const Slot& S, const int* spins, int c) {
  const int q = (c == P.C - 1) ? 0 : spins[c + 1];
  return S.renv + ((size_t)q * P.C + c) * P.ES;
}
__device__ inline double rlog_cur(const DevPlan& P, const Slot& S, const int* spins, int c) {
  const int q = (c == P.C - 1) ? 0 : spins[c + 1];
  return S.rl[(size_t)q * P.C + c];
}


// ---------------------------------------------------------------------------
// Transition of one row (kernels.py:142-206): Metropolis along the row.
// ---------------------------------------------------------------------------
__device__ __noinline__ void metropolis_row(const DevPlan& P, const Slot& S, Shared& sh, const float* perm, const float* top,
                               const int* tbond, const float* bot, const int* bbond, int row, int* spins,
                               const double* uniforms, const int32_t* deltas, float* min_margin) {
  const int C = P.C;
  VMC_TSTART(tr);
  right_envs(P, S, sh, perm, top, tbond, bot, bbond, row, spins, false);
  VMC_TSTOP(tr, PH_T_RENV);
  VMC_TSTART(tm);
  float* Lc = S.lenv;                  // current left env
  float* Lp0 = S.lenv + P.ES;          // L' for the current spin
  float* Lp1 = S.lenv + 2 * P.ES;      // L' for the proposed spin
  float* Y1 = S.scr[3];
  float* Y2 = S.scr[4];
  if (threadIdx.x == 0) set_elem(Lc, 0, 1.f);
  __syncthreads();
  double amp_cur = 0.0;  // |psi|^2 in this column's scale
  for (int c = 0; c < C; ++c) {
    const int s = site_id(P, row, c);
    const int U = P.sdim[4 * s], V = P.sdim[4 * s + 1], Lb = P.sdim[4 * s + 2], Rb = P.sdim[4 * s + 3];
    const int ta = tbond[c], tb = tbond[c + 1], ba = bbond[c], bb = bbond[c + 1];
    const float* T = top + (size_t)c * P.TS;
    const float* B = bot + (size_t)c * P.TS;
    const float* Rc = renv_cur(P, S, spins, c);
    const int cur = spins[c];
    int flip = cur;
    if (P.d == 2) flip = 1 - cur;
    else if (P.d > 2) flip = ((cur + deltas[row * C + c]) % P.d + P.d) % P.d;  // Python's modulo: any offset
    lenv_step1(Lc, T, Y1, ta, Lb, ba, U, tb);
    lenv_step23(Y1, perm_of(P, perm, s, P_LENV, cur), B, Y2, Lp0, ba, tb, Lb, U, Rb, V, bb);
    const int n_env = tb * Rb * bb;
    // L and R are renormalised per column, so psi is recomputed at every
    // column in that column's scale; the ratio is scale-free
    amp_cur = abs2_dot(Lp0, Rc, n_env, sh.red);
    double amp_flip = amp_cur;
    if (flip != cur) {
      lenv_step23(Y1, perm_of(P, perm, s, P_LENV, flip), B, Y2, Lp1, ba, tb, Lb, U, Rb, V, bb);
      amp_flip = abs2_dot(Lp1, Rc, n_env, sh.red);
    }
    // _metropolis_ratio (contraction.py:88-94) and accept (kernels.py:188-193)
    const double pc = amp_cur, pf = amp_flip;
    double ratio;
    if (pc > 0.0) ratio = pf / pc;
    else ratio = pf > 0.0 ? INFINITY : 0.0;
    const double thr = ratio < 1.0 ? ratio : 1.0;
    const double u = uniforms[row * C + c];
    const bool accept = (flip != cur) && (u < thr);
    const float margin = (float)fabs(thr - u);
    if (threadIdx.x == 0 && margin < *min_margin) *min_margin = margin;
    if (accept) {
      amp_cur = amp_flip;
      if (threadIdx.x == 0) spins[c] = flip;
    }
    __syncthreads();
    float* sel = accept ? Lp1 : Lp0;
    cta_copy(Lc, sel, n_env * kEs);
    cta_normalize(Lc, n_env * kEs, sh.red);
  }
  VMC_TSTOP(tm, PH_T_METRO);
}

// ---------------------------------------------------------------------------
// Estimate of one row (energy.py:158-205): gradient envs, one-site and
// horizontal energies.  `oscale` = exp(lt + lb - logamp) * sign(amp).
// ---------------------------------------------------------------------------
// energy += (ar + i ai) * (br + i bi) * (cr + i ci)
__device__ __forceinline__ void acc3(double* energy, double ar, double ai, double br, double bi, double cr,
                                     double ci) {
  const double xr = ar * br - ai * bi, xi = ar * bi + ai * br;
  energy[0] += xr * cr - xi * ci;
  energy[1] += xr * ci + xi * cr;
}

// Gradient environments, one-site and horizontal E_loc of one row
// (energy.py:158-205).  osc = (re, im) of exp(lt + lb - log|psi|) / phase(psi);
// energy[0..1] accumulates (re, im).
__device__ __noinline__ void estimate_row(const DevPlan& P, const Slot& S, Shared& sh, const float* perm,
                                          const float* tensors, const float* top, const int* tbond, const float* bot,
                                          const int* bbond, int row, const int* spins, const double* osc,
                                          float* Orow, int full_gradient, bool want_grad, bool want_energy,
                                          double* energy, const double* vjp_w = nullptr,
                                          double* vjp_grad = nullptr) {
  const int C = P.C;
  const bool has_h = want_energy && P.row_has_h[row];
  VMC_TSTART(tr);
  right_envs(P, S, sh, perm, top, tbond, bot, bbond, row, spins, has_h);
  VMC_TSTOP(tr, PH_E_RENV);
  VMC_TSTART(tl);
  float* Lc = S.lenv;
  float* Y1 = S.scr[3];
  float* Y2 = S.scr[4];
  float* W = S.scr[5];
  float* Gtmp = S.scr[6];
  if (threadIdx.x == 0) set_elem(Lc, 0, 1.f);
  __syncthreads();
  double llog = 0.0;  // log-scale taken out of the left environment
  for (int c = 0; c < C; ++c) {
    const int s = site_id(P, row, c);
    const int U = P.sdim[4 * s], V = P.sdim[4 * s + 1], Lb = P.sdim[4 * s + 2], Rb = P.sdim[4 * s + 3];
    const int ta = tbond[c], tb = tbond[c + 1], ba = bbond[c], bb = bbond[c + 1];
    const float* T = top + (size_t)c * P.TS;
    const float* B = bot + (size_t)c * P.TS;
    const float* Rc = renv_cur(P, S, spins, c);
    const int cur = spins[c];
    const int sz = U * V * Lb * Rb;
    // column scale: psi-normalised amplitude factor times the environments' log-scales
    const double f = exp(llog + rlog_cur(P, S, spins, c));
    const double cs_re = osc[0] * f, cs_im = osc[1] * f;
    lenv_step1(Lc, T, Y1, ta, Lb, ba, U, tb);
    const bool os = want_energy && P.onesite_mask[s];
    if (want_grad || os) {
      float* G = Gtmp;
      if (want_grad && Orow != nullptr) {
        G = elem(Orow, full_gradient ? (size_t)P.d * P.site_osl[s] + (size_t)cur * sz : (size_t)P.site_osl[s]);
      }
      grad_env(Y1, B, Rc, W, G, ba, V, bb, tb, Rb, Lb, U, (float)cs_re, (float)cs_im);
      if (kVjpCode && vjp_grad) {
        // vector-Jacobian product: grad[full layout of site s, slice cur] += w * O (FP64), with G this
        // site's O for the chain; the weight stays out of the FP32 G, where a tiny amplitude would underflow
        double* dst = vjp_grad + (size_t)kEs * ((size_t)P.d * P.site_osl[s] + (size_t)cur * sz);
        for (int i = threadIdx.x; i < sz; i += blockDim.x) {
          if (kCplx) {
            const double gr = G[2 * i], gi = G[2 * i + 1];
            atomicAdd(dst + 2 * i, vjp_w[0] * gr - vjp_w[1] * gi);
            atomicAdd(dst + 2 * i + 1, vjp_w[0] * gi + vjp_w[1] * gr);
          } else {
            atomicAdd(dst + i, vjp_w[0] * (double)G[i]);
          }
        }
        __syncthreads();  // G (scratch) is rewritten at the next column
      }
      if (os) {
        // amps_site[p] = sum A[p] . G  (already divided by psi); E += sum_p op[p, s] amps[p]
        for (int p = 0; p < P.d; ++p) {
          double ai = 0.0;
          const double ar = elem_dot(slice_of(P, tensors, s, p), G, sz, sh.red, &ai);
          double orr, oi;
          op_elem(P.onesite, ((size_t)s * P.d + p) * P.d + cur, &orr, &oi);
          acc3(energy, orr, oi, ar, ai, 1.0, 0.0);
        }
      }
    }
    const int n_env = tb * Rb * bb;
    const bool hz = has_h && c < C - 1 && P.horiz_mask[row * (C - 1) + c];
    if (hz) {
      // L'^{(p)} for every p, R_c^{(q)} for every q: psi(p,q) = <L'^p, R^q>
      const int cur1 = spins[c + 1];
      const size_t op0 = (size_t)(row * (C - 1) + c) * P.d * P.d * P.d * P.d;
      const int col = cur * P.d + cur1;
      const unsigned jm = nonzero_pairs(elem(P.horiz, op0), P.d, col);
      for (int p = 0; p < P.d; ++p) {
        // L'^(p) for the configuration's own spin (the next environment) and for every p with a nonzero
        // coefficient; psi(p, q) only where the coefficient is nonzero
        const unsigned qm = (jm >> (p * P.d)) & ((1u << P.d) - 1u);
        if (p != cur && qm == 0) continue;
        float* Lp = S.lenv + (size_t)(1 + p) * P.ES;
        lenv_step23(Y1, perm_of(P, perm, s, P_LENV, p), B, Y2, Lp, ba, tb, Lb, U, Rb, V, bb);
        for (int q = 0; q < P.d; ++q) {
          if (!((qm >> q) & 1u)) continue;
          const float* Rq = S.renv + ((size_t)q * C + c) * P.ES;
          double pi = 0.0;
          const double pr = elem_dot(Lp, Rq, n_env, sh.red, &pi);
          const double fq = exp(llog + S.rl[(size_t)q * C + c]);
          double orr, oi;
          op_elem(P.horiz, op0 + (size_t)(p * P.d + q) * P.d * P.d + col, &orr, &oi);
          acc3(energy, orr, oi, pr, pi, osc[0] * fq, osc[1] * fq);
        }
      }
      cta_copy(Lc, S.lenv + (size_t)(1 + cur) * P.ES, n_env * kEs);
      llog += cta_normalize(Lc, n_env * kEs, sh.red);
    } else if (c < C - 1) {
      float* Lp = S.lenv + P.ES;
      lenv_step23(Y1, perm_of(P, perm, s, P_LENV, cur), B, Y2, Lp, ba, tb, Lb, U, Rb, V, bb);
      cta_copy(Lc, Lp, n_env * kEs);
      llog += cta_normalize(Lc, n_env * kEs, sh.red);
    }
  }
  VMC_TSTOP(tl, PH_E_LEFT);
}

// ---------------------------------------------------------------------------
// Vertical energy of the row pair (r, r+1) (energy.py:24-95).
// top: top env of row r; bot: bottom env of row r+1.  Every step is chunked
// over one bond index (`vc` values at a time) so its intermediates fit the
// buffers vb[0..1+2d) of P.vbuf floats (shared memory when it fits).
// ---------------------------------------------------------------------------
__device__ __noinline__ void vertical_energy(const DevPlan& P, const Slot& S, Shared& sh, const float* perm,
                                               const float* top, const int* tbond, const float* bot,
                                               const int* bbond, int r, const int* sp0, const int* sp1,
                                               const double* vsc, float* const* vb, double* energy) {
  const int C = P.C, d = P.d;
  VMC_TSTART(tvr);
  // R2_{C-1} = [1]
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
    const float* A0 = perm_of(P, perm, s0, P_RENV, sp0[c]);
    const float* A1 = perm_of(P, perm, s1, P_R2, sp1[c]);
    for (int a0 = 0; a0 < ta; a0 += P.vchunk) {
      const int na = P.vchunk < ta - a0 ? P.vchunk : ta - a0;
      // P1[a][u][rr][y][f] = sum_b T[a][u][b] R2[b][rr][y][f]
      gemm(make_gemm(elem(T, (size_t)a0 * U * tb), lin(tb), 1, Rin, lin(1), Rb * Rb1 * bb, vb[0], lin(Rb * Rb1 * bb),
                         lin(1), na * U, Rb * Rb1 * bb, tb));
      // P2[a][l][f][v][y] = sum_{u,rr} P1[a][u][rr][(y,f)] A(u,v,l,rr)
      gemm(make_gemm(vb[0], two(Rb1 * bb, U * Rb * Rb1 * bb, 1), Rb1 * bb, A0, lin(1), Lb * V, vb[1],
                         three(Rb1, bb, Lb * bb * V * Rb1, 1, V * Rb1), two(V, bb * V * Rb1, Rb1), na * Rb1 * bb,
                         Lb * V, U * Rb));
      // P3[a][l][x][w][f] = sum_{v,y} P2[a][l][f][v][y] A'(v,w,x,y)
      gemm(make_gemm(vb[1], lin(V * Rb1), 1, A1, lin(1), V1 * Lb1, vb[0], two(bb, Lb1 * V1 * bb, 1),
                         two(Lb1, bb, V1 * bb), na * Lb * bb, V1 * Lb1, V * Rb1));
      // R2'[a][l][x][e] = sum_{w,f} P3[a][l][x][w][f] B[e][w][f]
      gemm(make_gemm(vb[0], lin(V1 * bb), 1, B, lin(V1 * bb), 1, elem(Rout, (size_t)a0 * Lb * Lb1 * ba), lin(ba),
                         lin(1), na * Lb * Lb1, ba, V1 * bb));
    }
    const double lg = cta_normalize(Rout, ta * Lb * Lb1 * ba * kEs, sh.red);
    if (threadIdx.x == 0) S.r2l[c - 1] = S.r2l[c] + lg;
  }
  VMC_TSTOP(tvr, PH_V_RIGHT);
  VMC_TSTART(tvl);
  float* Lc = S.l2[0];
  float* Ln = S.l2[1];
  if (threadIdx.x == 0) set_elem(Lc, 0, 1.f);
  __syncthreads();
  double l2log = 0.0;  // log-scale taken out of the 2-row left environment
  for (int c = 0; c < C; ++c) {
    const int s0 = site_id(P, r, c), s1 = site_id(P, r + 1, c);
    const int U = P.sdim[4 * s0], V = P.sdim[4 * s0 + 1], Lb = P.sdim[4 * s0 + 2], Rb = P.sdim[4 * s0 + 3];
    const int V1 = P.sdim[4 * s1 + 1], Lb1 = P.sdim[4 * s1 + 2], Rb1 = P.sdim[4 * s1 + 3];
    const int ta = tbond[c], tb = tbond[c + 1], ba = bbond[c], bb = bbond[c + 1];
    const float* T = top + (size_t)c * P.TS;
    const float* B = bot + (size_t)c * P.TS;
    const float* Rc = S.r2 + (size_t)c * P.E2S;
    const int s_cur = sp0[c];
    // pairs (p, q) with a nonzero coefficient in the configuration's column of the bond operator; when
    // that is the configuration's own pair alone (a Heisenberg bond with parallel spins), psi comes from
    // the slices the environment update forms anyway
    const unsigned jm = P.vert_mask[r * C + c]
                            ? nonzero_pairs(elem(P.vert, (size_t)(r * C + c) * d * d * d * d), d, s_cur * d + sp1[c])
                            : 0u;
    const bool vt = jm != 0;
    const bool own_only = jm == (1u << (s_cur * d + sp1[c]));
    const bool last = (c == C - 1);
    if (!vt && last) break;
    double psi[kMaxPhys * kMaxPhys], psi_im[kMaxPhys * kMaxPhys];  // standard plans only: d <= kMaxPhys
    for (int i = 0; i < d * d; ++i) psi[i] = psi_im[i] = 0.0;
    const int sz0 = ssize(P, s0), sz1 = ssize(P, s1);
    const int vstride = (int)(vb[2] - vb[1]) / kEs;  // buffer spacing in elements
    for (int b0 = 0; b0 < tb; b0 += P.vchunk) {
      const int nb = P.vchunk < tb - b0 ? P.vchunk : tb - b0;
      float* Q1 = vb[0];
      // Q1[x][e][b][l][u] = sum_a L2[a][(l,x,e)] T[a][u][b0+b]
      gemm(make_gemm(Lc, lin(1), Lb * Lb1 * ba, elem(T, b0), two(nb, tb, 1), U * tb, Q1,
                         two(Lb1 * ba, U, nb * Lb * U), two(nb, 1, Lb * U), Lb * Lb1 * ba, U * nb, ta));
      // Q2[p][e][b][rr][x][v] = sum_{l,u} Q1[x][e][b][l][u] A[p](u,v,l,rr); with a vertical term every
      // p at once (the spin slices of A are contiguous, the buffers vb[1+p] equally spaced)
      if (vt && !own_only) {
        gemm(make_gemm(Q1, lin(Lb * U), 1, perm_of(P, perm, s0, P_LENV, 0), two(Rb * V, sz0, 1), Rb * V,
                           vb[1], two(ba * nb, V, Rb * Lb1 * V), three(Rb, V, vstride, Lb1 * V, 1),
                           Lb1 * ba * nb, d * Rb * V, Lb * U));
      } else {
        gemm(make_gemm(Q1, lin(Lb * U), 1, perm_of(P, perm, s0, P_LENV, s_cur), lin(1), Rb * V, vb[1 + s_cur],
                           two(ba * nb, V, Rb * Lb1 * V), two(V, Lb1 * V, 1), Lb1 * ba * nb, Rb * V, Lb * U));
      }
      if (vt) {
        float* W2 = vb[0];
        // W2[e][b][rr][w][y] = sum_f B[e][w][f] R2[b0+b][rr][y][f]
        gemm(make_gemm(B, lin(bb), 1, elem(Rc, (size_t)b0 * Rb * Rb1 * bb), lin(bb), 1, W2,
                           two(V1, nb * Rb * V1 * Rb1, Rb1), three(Rb, Rb1, Rb * V1 * Rb1, V1 * Rb1, 1), ba * V1,
                           nb * Rb * Rb1, bb));
        const int q2n = Lb1 * ba * nb * Rb * V;
        if (own_only) {
          // Vq for q = the configuration's spin only; psi(cur, cur1) += <Q2[cur], Vq>
          const int q = sp1[c];
          gemm(make_gemm(perm_of(P, perm, s1, P_ZIPT, q), lin(V1 * Rb1), 1, W2, lin(V1 * Rb1), 1, vb[1 + d + q],
                             lin(1), lin(Lb1 * V), Lb1 * V, ba * nb * Rb, V1 * Rb1));
          if (kCplx) {
            double im = 0.0;
            psi[s_cur * d + q] += cta_cdot(vb[1 + s_cur], vb[1 + d + q], q2n, sh.red, &im);
            psi_im[s_cur * d + q] += im;
          } else {
            psi[s_cur * d + q] += cta_dot(vb[1 + s_cur], vb[1 + d + q], q2n, sh.red);
          }
        } else {
          // Vq[e][b][rr][x][v] = sum_{w,y} A'[q][x][v][w][y] W2[e][b][rr][w][y], every q in one GEMM
          gemm(make_gemm(perm_of(P, perm, s1, P_ZIPT, 0), two(Lb1 * V, sz1, V1 * Rb1), 1, W2, lin(V1 * Rb1), 1,
                             vb[1 + d], two(Lb1 * V, vstride, 1), lin(Lb1 * V), d * Lb1 * V, ba * nb * Rb,
                             V1 * Rb1));
          // psi(p, q) += <Q2[p], Vq> for all d*d pairs in one pass and one reduction
          if (kCplx) {
            for (int pp = 0; pp < d; ++pp)
              for (int q = 0; q < d; ++q) {
                double im = 0.0;
                psi[pp * d + q] += cta_cdot(vb[1 + pp], vb[1 + d + q], q2n, sh.red, &im);
                psi_im[pp * d + q] += im;
              }
          } else {
            cta_dots_all(vb + 1, vb + 1 + d, d, q2n, psi, sh.red);
          }
        }
      }
      if (!last) {
        float* Q3 = vb[0];
        // Q3[b][rr][y][e][w] = sum_{x,v} Q2[s][e][b][rr][x][v] A'(v,w,x,y)
        gemm(make_gemm(vb[1 + s_cur], lin(Lb1 * V), 1, perm_of(P, perm, s1, P_ZIPT, sp1[c]), lin(1), V1 * Rb1,
                           Q3, two(nb * Rb, V1, Rb1 * ba * V1), two(Rb1, 1, ba * V1), ba * nb * Rb, V1 * Rb1,
                           Lb1 * V));
        // L2'[b0+b][rr][y][f] = sum_{e,w} Q3 B[e][w][f]
        gemm(make_gemm(Q3, lin(ba * V1), 1, B, lin(1), bb, elem(Ln, (size_t)b0 * Rb * Rb1 * bb), lin(bb), lin(1),
                           nb * Rb * Rb1, bb, ba * V1));
      }
    }
    if (vt) {
      const float* op = elem(P.vert, (size_t)(r * C + c) * d * d * d * d);
      const int col = s_cur * d + sp1[c];
      const double f = exp(l2log + S.r2l[c]);
      for (int j = 0; j < d * d; ++j) {
        double orr, oi;
        op_elem(op, (size_t)j * d * d + col, &orr, &oi);
        acc3(energy, orr, oi, psi[j], psi_im[j], vsc[0] * f, vsc[1] * f);
      }
    }
    if (!last) {
      l2log += cta_normalize(Ln, tb * Rb * Rb1 * bb * kEs, sh.red);
      float* t = Lc;
      Lc = Ln;
      Ln = t;
    }
  }
  VMC_TSTOP(tvl, PH_V_LEFT);
}

__device__ inline const int* tbonds(const DevPlan& P, int r) { return P.tb + (size_t)r * (P.C + 1); }
__device__ inline const int* bbonds(const DevPlan& P, int r) { return P.bb + (size_t)r * (P.C + 1); }

__device__ inline float* cache_row(const DevPlan& P, float* cache, int chain, int r) {
  return cache + (size_t)chain * P.cache_floats_per_chain + (size_t)r * P.C * P.TS;
}
__device__ inline double* cache_logs(const DevPlan& P, float* cache, int n_chains, int chain) {
  double* base = reinterpret_cast<double*>(cache + (size_t)n_chains * P.cache_floats_per_chain);
  return base + (size_t)chain * P.R;
}

// ---------------------------------------------------------------------------
// The fused kernel.
// ---------------------------------------------------------------------------
#ifdef VMC_HOST_EMULATION
// Shared memory starts with whatever an earlier chain left: the host build
// poisons it so that a read before write shows up as NaN in the host tests.
inline float* emu_dyn_smem(long long floats) {
  static float* buf = nullptr;
  static long long have = 0;
  if (floats > have) {
    std::free(buf);
    buf = static_cast<float*>(std::malloc(sizeof(float) * floats));
    have = floats;
  }
  if (buf) std::memset(buf, 0xff, sizeof(float) * have);
  return buf;
}
#endif

// One chain of a job, on this CTA, with the CTA's workspace slot at slot_base.
__device__ __forceinline__ void run_chain(const ChainJob& J, int chain, float* slot_base, int32_t* status) {
  const DevPlan& P = *J.P;
  VMC_SHARED Shared sh;
#ifdef VMC_HOST_EMULATION
  float* dyn_smem = emu_dyn_smem(P.arena_in_smem ? P.arena_floats : 0);
  std::memset(&sh, 0xff, sizeof(sh));
#else
  extern __shared__ __align__(16) float dyn_smem[];
#endif
  const int mode = J.mode, n_chains = J.n_chains, full_gradient = J.full_gradient;
  const float* tensors = J.tensors;
  const float* perm = J.perm;
  int32_t* configs = J.configs;
  const double* uniforms = J.uniforms;
  const int32_t* deltas = J.deltas;
  float* cache = J.cache;
  float* out_O = J.out_O;
  int8_t* out_p = J.out_p;
  double* out_E = J.out_E;
  double* logamp_io = J.logamp_io;
  double* sign_io = J.sign_io;
  float* out_margin = J.out_margin;
  float* out_gap = J.out_gap;
  Slot S = make_slot(P, slot_base);
  if (threadIdx.x == 0) g_tile_policy = P.tile_policy;  // read by cta_gemm after the next barrier
#if VMC_CHAIN_F64
  // the high-precision chain's arena (8-byte df64 elements) takes the place of the FP32 truncation arena
  const ChainD ch = make_chain_d(P, S.h64, reinterpret_cast<double*>(P.arena_in_smem ? dyn_smem : S.arena),
                                 reinterpret_cast<double*>(S.arena));
#else
  const Arena ar = make_arena(P, P.arena_in_smem ? dyn_smem : S.arena, S.arena);
#endif
  if (P.onerow_in_smem) {
    // the 1-row environment GEMM intermediates are never live during a truncation
    for (int i = 0; i < 4; ++i) S.scr[3 + i] = dyn_smem + (size_t)i * P.scr1;
  }
  // vertical-energy buffers (standard plans, d <= kMaxPhys); a GI plan uses the first two as scratch
  float* vbuf[1 + 2 * kMaxPhys];
  for (int i = 0; i < 1 + 2 * (P.d < kMaxPhys ? P.d : kMaxPhys); ++i)
    vbuf[i] = P.vert_in_smem ? dyn_smem + (size_t)i * P.vbuf : S.scr[7 + i];

  const int R = P.R, C = P.C;
  const int n_params = full_gradient ? P.d * P.np_sliced : P.np_sliced;

  int32_t* cfg = configs + (size_t)chain * P.n_sites;
  float min_gap = INFINITY;
  // this chain's cache entry: its own, or (recompute) the CTA's
  const bool own_entry = J.cache_per_cta != 0;
  const int ce = own_entry ? (int)blockIdx.x : chain, ce_n = own_entry ? (int)gridDim.x : n_chains;

  if (mode == MODE_INIT || (own_entry && mode == MODE_SWEEP)) {
    // init_cache (kernels.py:115-129): bottom envs from the bottom up
    double* lb = cache_logs(P, cache, ce_n, ce);
    float* b = cache_row(P, cache, ce, R - 1);
    fill_ones_row(P, b);
    if (threadIdx.x == 0) lb[R - 1] = 0.0;
#if VMC_CHAIN_F64
    int hc = 0;
    fill_ones_row_d(P, ch.row[0]);
#endif
    for (int r = R - 1; r >= 1; --r) {
      for (int c = threadIdx.x; c < C; c += blockDim.x) sh.spins[0][c] = cfg[r * C + c];
      __syncthreads();
#if VMC_CHAIN_F64
      const double ls = apply_row_hp(P, sh, perm, ch.row[hc], bbonds(P, r), ch.row[hc ^ 1],
                                     cache_row(P, cache, ce, r - 1), bbonds(P, r - 1), r, sh.spins[0], true, ch,
                                     &min_gap);
      hc ^= 1;
#else
      const double ls = apply_row(P, S, sh, perm, cache_row(P, cache, ce, r), bbonds(P, r),
                                  cache_row(P, cache, ce, r - 1), bbonds(P, r - 1), r, sh.spins[0], true, ar,
                                  &min_gap);
#endif
      if (threadIdx.x == 0) lb[r - 1] = lb[r] + ls;
      __syncthreads();
    }
    if (mode == MODE_INIT) return;
    min_gap = INFINITY;  // the sweep reports its own cuts, as after a separate init_cache
  }

  // ---------------- top-down pass: transition or forward ----------------
  VMC_TSTART(tchain);
  float min_margin = INFINITY;
#if VMC_CHAIN_F64
  int ht = 0;
  fill_ones_row_d(P, ch.row[0]);
#endif
  fill_ones_row(P, S.topc);
  if (threadIdx.x == 0) S.lt[0] = 0.0;
  __syncthreads();
  for (int r = 0; r < R; ++r) {
    for (int c = threadIdx.x; c < C; c += blockDim.x) sh.spins[0][c] = cfg[r * C + c];
    __syncthreads();
    float* top = S.topc + (size_t)r * C * P.TS;
    if (mode == MODE_SWEEP) {
      const float* bot = cache_row(P, cache, ce, r);
      metropolis_row(P, S, sh, perm, top, tbonds(P, r), bot, bbonds(P, r), r, sh.spins[0],
                     uniforms + (size_t)chain * P.n_sites, deltas ? deltas + (size_t)chain * P.n_sites : nullptr,
                     &min_margin);
      for (int c = threadIdx.x; c < C; c += blockDim.x) cfg[r * C + c] = sh.spins[0][c];
      __syncthreads();
    }
    VMC_TSTART(tz);
#if VMC_CHAIN_F64
    const double ls = apply_row_hp(P, sh, perm, ch.row[ht], tbonds(P, r), ch.row[ht ^ 1],
                                   S.topc + (size_t)(r + 1) * C * P.TS, tbonds(P, r + 1), r, sh.spins[0], false, ch,
                                   &min_gap);
    ht ^= 1;
#else
    const double ls = apply_row(P, S, sh, perm, top, tbonds(P, r), S.topc + (size_t)(r + 1) * C * P.TS,
                                tbonds(P, r + 1), r, sh.spins[0], false, ar, &min_gap);
#endif
    VMC_TSTOP(tz, PH_T_ZIP);
    if (threadIdx.x == 0) S.lt[r + 1] = S.lt[r] + ls;
    __syncthreads();
  }
  double sgn = 1.0;
#if VMC_CHAIN_F64
  double logamp = S.lt[R] + contract_bottom_d(P, ch.row[ht], tbonds(P, R), sh, ch.z1, &sgn);
#else
  double logamp = S.lt[R] + contract_bottom(P, S.topc + (size_t)R * C * P.TS, tbonds(P, R), sh,
                                           reinterpret_cast<double*>(S.scr[0]), &sgn);
#endif
  if (mode == MODE_ENERGY) {
    logamp = logamp_io[chain];
    sgn = sign_io[chain];
  } else if (threadIdx.x == 0 && logamp_io) {
    logamp_io[chain] = logamp;
    sign_io[chain] = sgn;
    if (out_margin && mode == MODE_SWEEP) out_margin[chain] = min_margin;
  }
  if (!isfinite(logamp) && threadIdx.x == 0) atomicOr(status, VMC_DEV_NONFINITE);

  // ---------------- bottom-up estimate ----------------
  const bool want_grad = (mode == MODE_SWEEP || mode == MODE_AMPGRAD || mode == MODE_VJP);
  const bool want_energy = (mode == MODE_SWEEP || mode == MODE_ENERGY);
  float* Orow = out_O ? elem(out_O, (size_t)chain * n_params) : nullptr;
  const double* vjp_w = (mode == MODE_VJP) ? J.vjp_w + (size_t)kEs * chain : nullptr;
  double* vjp_grad = (mode == MODE_VJP) ? J.vjp_grad : nullptr;
  if (Orow && full_gradient) {
    for (int i = threadIdx.x; i < n_params * kEs; i += blockDim.x) Orow[i] = 0.f;
    __syncthreads();
  }
  double energy[2] = {0.0, 0.0};
  if (want_energy) {
    // diagonal terms (energy.py:150-156)
    if (threadIdx.x == 0) {
      for (int t = 0; t < P.n_diag; ++t) {
        int idx = 0;
        for (int k = 0; k < P.diag_nsites[t]; ++k) idx = idx * P.d + cfg[P.diag_sites[P.diag_site_off[t] + k]];
        energy[0] += P.diag_values[P.diag_value_off[t] + idx];
      }
    }
  }
  // 1 / (sign or phase of psi): multiplies every psi-normalised quantity
  const double inv_re = kCplx ? cos(sgn) : sgn, inv_im = kCplx ? -sin(sgn) : 0.0;
  double* lbc = (mode == MODE_SWEEP) ? cache_logs(P, cache, ce_n, ce) : nullptr;
  double lb_cur = 0.0, lb_prev = 0.0;
  int ib_cur = 0, ib_prev = 1, ib_next = 2;
#if VMC_CHAIN_F64
  int hb = 0;
  fill_ones_row_d(P, ch.row[0]);
#endif
  fill_ones_row(P, S.brow[ib_cur]);
  for (int r = R - 1; r >= 0; --r) {
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
      sh.spins[0][c] = cfg[r * C + c];
      if (r + 1 < R) sh.spins[1][c] = cfg[(r + 1) * C + c];
    }
    __syncthreads();
    float* bcur = S.brow[ib_cur];
    if (mode == MODE_SWEEP) {
      cta_copy(cache_row(P, cache, ce, r), bcur, C * P.TS);
      if (threadIdx.x == 0) lbc[r] = lb_cur;
    }
    const float* top = S.topc + (size_t)r * C * P.TS;
    const double om = exp(S.lt[r] + lb_cur - logamp);
    const double osc[2] = {inv_re * om, inv_im * om};
    estimate_row(P, S, sh, perm, tensors, top, tbonds(P, r), bcur, bbonds(P, r), r, sh.spins[0], osc, Orow,
                 full_gradient, want_grad, want_energy, energy, vjp_w, vjp_grad);
    if (want_energy && r < R - 1 && P.row_has_v[r]) {
      const double vm = exp(S.lt[r] + lb_prev - logamp);
      const double vsc[2] = {inv_re * vm, inv_im * vm};
      VMC_TSTART(tv);
      vertical_energy(P, S, sh, perm, top, tbonds(P, r), S.brow[ib_prev], bbonds(P, r + 1), r, sh.spins[0],
                      sh.spins[1], vsc, vbuf, energy);
      VMC_TSTOP(tv, PH_E_VERT);
    }
    if (r > 0) {
      VMC_TSTART(tb);
#if VMC_CHAIN_F64
      const double ls = apply_row_hp(P, sh, perm, ch.row[hb], bbonds(P, r), ch.row[hb ^ 1], S.brow[ib_next],
                                     bbonds(P, r - 1), r, sh.spins[0], true, ch, &min_gap);
      hb ^= 1;
#else
      const double ls = apply_row(P, S, sh, perm, bcur, bbonds(P, r), S.brow[ib_next], bbonds(P, r - 1), r,
                                  sh.spins[0], true, ar, &min_gap);
#endif
      VMC_TSTOP(tb, PH_B_ZIP);
      lb_prev = lb_cur;
      lb_cur = lb_cur + ls;
      const int t = ib_prev;
      ib_prev = ib_cur;
      ib_cur = ib_next;
      ib_next = t;
    }
  }
  if (out_gap && threadIdx.x == 0) out_gap[chain] = min_gap;
  if (want_energy && threadIdx.x == 0) {
    out_E[kEs * chain] = energy[0];
    if (kCplx) out_E[kEs * chain + 1] = energy[1];
    if (!isfinite(energy[0]) || !isfinite(energy[1])) atomicOr(status, VMC_DEV_NONFINITE);
  }
  if (out_p && mode == MODE_SWEEP) {
    // active_slice_indices = repeat(config, params_per_site) (kernels.py:82-87)
    for (int s = 0; s < P.n_sites; ++s) {
      const int sz = ssize(P, s);
      const int8_t v = (int8_t)cfg[s];
      for (int i = threadIdx.x; i < sz; i += blockDim.x) out_p[(size_t)chain * P.np_sliced + P.site_osl[s] + i] = v;
    }
  }
  __syncthreads();
  VMC_TSTOP(tchain, PH_CHAIN);}

#ifndef VMC_GI_TU
// The fused persistent kernel over the (job, chain) items of a job table
// (uneven batches: lattices, bond dimensions, modes).  next == NULL: CTA b runs
// items b, b + grid, ...  Otherwise CTAs take items from the counter *next
// (zero at launch) until none is left; with the jobs ordered by decreasing cost
// per chain the slowest chains start first and the fast ones fill in.  Every
// CTA keeps its workspace slot at slots + blockIdx.x * slot_floats.
// At most 128 registers per thread (two 256-thread CTAs, or four of the default
// 128 threads, per SM): left free, the compiler takes all 255 and halves occupancy.
__global__ void __launch_bounds__(kThreads, VMC_MIN_CTAS) peps_kernel(const __grid_constant__ BatchJobs jobs, float* slots,
                                                           int32_t* next, int32_t* status) {
  VMC_SHARED int item;
  float* slot = slots + (size_t)blockIdx.x * jobs.slot_floats;
  const int total = jobs.first[jobs.n_jobs];
#if VMC_GEMM_TCGEN05 && !defined(VMC_HOST_EMULATION)
  tc_setup(status);
#endif
  for (int i = blockIdx.x;; i += gridDim.x) {
    if (next) {
      if (threadIdx.x == 0) item = atomicAdd(next, 1);
      __syncthreads();
      i = item;
      __syncthreads();
    }
    if (i >= total) break;
    int j = 0;
    while (j + 1 < jobs.n_jobs && i >= jobs.first[j + 1]) ++j;
    run_chain(jobs.job[j], i - jobs.first[j], slot, status);
  }
#if VMC_GEMM_TCGEN05 && !defined(VMC_HOST_EMULATION)
  tc_teardown();
#endif
}
#else  // the gauge-invariant translation unit

#include "gi_device.cuh"

// The gauge-invariant plans' kernel: the same job-table walk over gi_chain (a separate kernel, so the
// standard chain code keeps its register allocation).  A job table holds GI plans only.
__global__ void __launch_bounds__(kThreads, VMC_MIN_CTAS) gi_kernel(const __grid_constant__ BatchJobs jobs,
                                                                     float* slots, int32_t* next, int32_t* status) {
  VMC_SHARED int item;
  float* slot = slots + (size_t)blockIdx.x * jobs.slot_floats;
  const int total = jobs.first[jobs.n_jobs];
  for (int i = blockIdx.x;; i += gridDim.x) {
    if (next) {
      if (threadIdx.x == 0) item = atomicAdd(next, 1);
      __syncthreads();
      i = item;
      __syncthreads();
    }
    if (i >= total) break;
    int j = 0;
    while (j + 1 < jobs.n_jobs && i >= jobs.first[j + 1]) ++j;
    gi_chain(jobs.job[j], i - jobs.first[j], slot, status);
  }
}
#endif
