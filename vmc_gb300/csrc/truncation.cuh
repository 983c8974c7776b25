// truncation.cuh -- CTA-level dominant invariant subspace of a small symmetric
// matrix, for the boundary-MPS truncation (strategy.py:128-150: keep the top-k
// left singular vectors of theta).
//
// The amplitude only depends on the kept subspace, so the truncation works on
// the Gram matrix G = M M^T (or M^T M) of the theta matrix M:
//   1. Householder tridiagonalisation  G = Q T Q^T   (3 barriers per column),
//   2. multisection bisection with Sturm counts for the k (+1) largest
//      eigenvalues of T (groups of 8 lanes per eigenvalue),
//   3. inverse iteration on the tridiagonal T for each eigenvalue (one thread
//      per eigenvector, LU with partial pivoting),
//   4. CholQR2 re-orthonormalisation of the k vectors (warp Cholesky),
//   5. back-transformation with the stored reflectors: U = Q Y.
// All arrays may live in shared or global memory.
#pragma once

#include "device_common.cuh"
#include "phase_timers.cuh"
#include "scalar.cuh"
#include "df64.cuh"

#include <type_traits>

namespace vmc {

__device__ __forceinline__ float warp_sum_f(float v) {
#ifndef VMC_HOST_EMULATION
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
#endif
  return v;
}

__device__ __forceinline__ void warp_sync() {
#ifndef VMC_HOST_EMULATION
  __syncwarp();
#endif
}

// In-place Householder tridiagonalisation of the symmetric n x n matrix A
// (row-major, leading dimension lda).  On exit d[0..n-1], e[0..n-2] hold T,
// tau[j] and A[j+1+i][j] (i >= 1; v_j[0] = 1 implicit) the reflectors
// H_j = I - tau_j v_j v_j^T with G = H_0 ... H_{n-3} T H_{n-3} ... H_0.
// `v`, `p` are n floats of scratch; `part` holds >= 64 floats.
// Per column: 3 barriers; the matrix-vector product uses `rg` threads per row
// and the rank-2 update a 2-D thread grid (no integer division).
template <typename T>
__device__ inline void cta_tridiagonalize(T* A, int n, int lda, T* d, T* e, T* tau, T* v,
                                          T* p, T* part) {
  constexpr bool kDF = std::is_same<T, df64>::value;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = (nt + 31) >> 5;
  if (n == 1) {
    if (tid == 0) d[0] = A[0];
    __syncthreads();
    return;
  }
  // threads per row in the matvec (power of two, <= 32)
  int rg = 1;
  while (rg * 2 <= 32 && rg * 2 * n <= nt) rg *= 2;
  const int rrow = tid / rg, rlane = tid % rg, nrow_thr = nt / rg;
  const unsigned rmask = (rg == 32) ? 0xffffffffu : (((1u << rg) - 1u) << ((tid & 31) & ~(rg - 1)));
  // 2-D grid for the update: gx columns x gy rows
  int gx = 1;
  while (gx * gx < nt) gx *= 2;
  if (gx > nt) gx = nt;
  const int gy = nt / gx;
  const int ux = tid % gx, uy = tid / gx;
  {
    T s = T(0.);
    for (int i = 2 + tid; i < n; i += nt) s = vfma(A[(size_t)i * lda], A[(size_t)i * lda], s);
    s = warp_sum_t(s);
    if (lane == 0) part[warp] = s;
  }
  __syncthreads();
  for (int j = 0; j < n - 2; ++j) {
    const int m = n - j - 1;
    T xn2 = T(0.);
    for (int w = 0; w < nwarps; ++w) xn2 += part[w];
    const T alpha = A[(size_t)(j + 1) * lda + j];
    T tj = T(0.), beta = alpha, scal = T(0.);
    if (xn2 > T(0.)) {
      beta = -vcopysign(vsqrt(alpha * alpha + xn2), alpha);
      tj = (beta - alpha) / beta;
      scal = T(1.) / (alpha - beta);
    }
    // column j stays unscaled until barrier (2): the matrix-vector product
    // below rebuilds v from it, so v needs no barrier of its own (df64: a
    // product per element costs more than the barrier, so v is read back)
    const T* colj = A + (size_t)(j + 1) * lda + j;
    for (int i = tid; i < m; i += nt) v[i] = (i == 0) ? T(1.) : colj[(size_t)i * lda] * scal;
    if (tid == 0) {
      d[j] = A[(size_t)j * lda + j];
      e[j] = beta;
      tau[j] = tj;
    }
    T* As = A + (size_t)(j + 1) * lda + (j + 1);
    if (tj == T(0.)) {
      __syncthreads();  // v visible
      T s = T(0.);
      for (int i = 2 + tid; i < m; i += nt) s = vfma(As[(size_t)i * lda], As[(size_t)i * lda], s);
      s = warp_sum_t(s);
      if (lane == 0) part[warp] = s;
      __syncthreads();
      continue;
    }
    if constexpr (kDF) __syncthreads();  // v visible
    // p = tau * A_sub v, rg threads per row; partial p.v per warp
    T pv = T(0.);
    if constexpr (kDF) {
      for (int i = rrow; i < m; i += nrow_thr) {
        const T* row = As + (size_t)i * lda;
        T s0 = T(0.), s1 = T(0.), s2 = T(0.), s3 = T(0.);
        int l = rlane;
        for (; l + 3 * rg < m; l += 4 * rg) {
          acc_mac(s0, row[l], v[l]);
          acc_mac(s1, row[l + rg], v[l + rg]);
          acc_mac(s2, row[l + 2 * rg], v[l + 2 * rg]);
          acc_mac(s3, row[l + 3 * rg], v[l + 3 * rg]);
        }
        for (; l < m; l += rg) acc_mac(s0, row[l], v[l]);
        T s = (df_norm(s0) + df_norm(s1)) + (df_norm(s2) + df_norm(s3));
#ifndef VMC_HOST_EMULATION
        for (int o = rg / 2; o > 0; o >>= 1) s += shfl_xor_t(rmask, s, o, rg);
#endif
        const T pi = tj * s;
        if (rlane == 0) {
          p[i] = pi;
          pv = vfma(pi, v[i], pv);
        }
      }
    } else {
    for (int i = rrow; i < m; i += nrow_thr) {
      const T* row = As + (size_t)i * lda;
      T s0 = T(0.), s1 = T(0.), s2 = T(0.), s3 = T(0.);
      int l = rlane;
      for (; l + 3 * rg < m; l += 4 * rg) {
        const T a0 = row[l], a1 = row[l + rg], a2 = row[l + 2 * rg], a3 = row[l + 3 * rg];
        const T b0 = l == 0 ? T(1.) : colj[(size_t)l * lda] * scal;
        const T b1 = colj[(size_t)(l + rg) * lda] * scal;
        const T b2 = colj[(size_t)(l + 2 * rg) * lda] * scal;
        const T b3 = colj[(size_t)(l + 3 * rg) * lda] * scal;
        s0 = vfma(a0, b0, s0);
        s1 = vfma(a1, b1, s1);
        s2 = vfma(a2, b2, s2);
        s3 = vfma(a3, b3, s3);
      }
      for (; l < m; l += rg) s0 = vfma(row[l], l == 0 ? T(1.) : colj[(size_t)l * lda] * scal, s0);
      T s = (s0 + s1) + (s2 + s3);
#ifndef VMC_HOST_EMULATION
      for (int o = rg / 2; o > 0; o >>= 1) s += shfl_xor_t(rmask, s, o, rg);
#endif
      const T pi = tj * s;
      if (rlane == 0) {
        p[i] = pi;
        pv = vfma(pi, i == 0 ? T(1.) : colj[(size_t)i * lda] * scal, pv);
      }
    }
    }
    pv = warp_sum_t(pv);
    if (lane == 0) part[32 + warp] = pv;
    __syncthreads();  // (2) p and v visible
    // store the reflector in column j (nothing reads column j any more)
    for (int i = 1 + tid; i < m; i += nt) A[(size_t)(j + 1 + i) * lda + j] = v[i];
    T ptv = T(0.);
    for (int w = 0; w < nwarps; ++w) ptv += part[32 + w];
    const T K = T(0.5) * tj * ptv;
    // A_sub -= v w^T + w v^T, w = p - K v
    T s = T(0.);
    // columns l = l0 + q*gx (q < 4) of this thread: v_l, w_l kept in registers
    for (int l0 = ux; l0 < m; l0 += 4 * gx) {
      T vl[4], wl[4];
      int nl = 0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int l = l0 + q * gx;
        vl[q] = l < m ? v[l] : T(0.);
        wl[q] = l < m ? p[l] - K * vl[q] : T(0.);
        nl += l < m;
      }
      for (int i = uy; i < m; i += gy) {
        const T vi = v[i], wi = p[i] - K * vi;
        T* arow = As + (size_t)i * lda;
        T a[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) a[q] = q < nl ? arow[l0 + q * gx] : T(0.);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (q < nl) {
            T nv;
            if constexpr (kDF)
              nv = df_sub2(a[q], vi, wl[q], wi, vl[q]);
            else
              nv = a[q] - vi * wl[q] - wi * vl[q];
            arow[l0 + q * gx] = nv;
            if (l0 + q * gx == 0 && i >= 2) s = vfma(nv, nv, s);
          }
        }
      }
    }
    s = warp_sum_t(s);
    if (lane == 0) part[warp] = s;
    __syncthreads();  // (3) trailing matrix updated
  }
  if (tid == 0) {
    d[n - 2] = A[(size_t)(n - 2) * lda + n - 2];
    e[n - 2] = A[(size_t)(n - 1) * lda + n - 2];
    d[n - 1] = A[(size_t)(n - 1) * lda + n - 1];
  }
  __syncthreads();
  (void)rmask;
}

// Number of eigenvalues of T (d, e2 = e^2) smaller than x.
template <typename T>
__device__ __forceinline__ int sturm_count(const T* d, const T* e2, int n, T x, T pivmin) {
  T q = d[0] - x;
  if (vabs(q) < pivmin) q = -pivmin;
  int cnt = q < T(0.);
#pragma unroll 4
  for (int i = 1; i < n; ++i) {
    q = (d[i] - x) - vfdiv(e2[i - 1], q);
    if (vabs(q) < pivmin) q = -pivmin;
    cnt += q < T(0.);
  }
  return cnt;
}

// The kk largest eigenvalues of T, descending, into lam[0..kk-1].
// e2 receives e^2 (n-1 floats of scratch).  Returns the Gershgorin scale |T|.
template <typename T>
__device__ inline T cta_top_eigenvalues(const T* d, const T* e, T* e2, int n, int kk, T* lam) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < n - 1; i += nt) e2[i] = e[i] * e[i];
  __syncthreads();
  // Gershgorin interval and the largest e^2: every warp reduces over all rows (strided over its lanes,
  // then shuffles; min and max are exact, so each thread ends with the same values without a barrier)
  T lo = Tol<T>::big, hi = -Tol<T>::big, e2max = T(0.);
  for (int i = tid & 31; i < n; i += (nt < 32 ? nt : 32)) {
    const T r = (i > 0 ? vabs(e[i - 1]) : T(0.)) + (i < n - 1 ? vabs(e[i]) : T(0.));
    lo = vmin(lo, d[i] - r);
    hi = vmax(hi, d[i] + r);
    if (i < n - 1) e2max = vmax(e2max, e2[i]);
  }
#ifndef VMC_HOST_EMULATION
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = vmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = vmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    e2max = vmax(e2max, __shfl_xor_sync(0xffffffffu, e2max, o));
  }
#endif
  const T tnorm = vmax(vabs(lo), vabs(hi));
  const T pivmin = T(1e-30) * vmax(T(1.), e2max);
  const T span = hi - lo;
  lo -= T(1e-6) * span + T(1e-30);
  hi += T(1e-6) * span + T(1e-30);
  // lanes per eigenvalue: 8 (9-way multisection) unless fewer lanes let every
  // wanted eigenvalue run in one round
  int G = nt >= 8 ? 8 : 1;
  while (G > 2 && nt / G < kk) G >>= 1;
  const int ngroups = nt / G;
  const int l = tid % G;
  const int base = (tid & 31) & ~(G - 1);
  // exactly this group's lanes: groups leave the loop independently
  const unsigned gmask = (((1u << G) - 1u) << base);
  const int npts = G > 1 ? G - 1 : 1;
  const int rounds = (kk + ngroups - 1) / ngroups;
  for (int rd = 0; rd < rounds; ++rd) {
    const int t = rd * ngroups + tid / G;
    const bool valid = t < kk && tid / G < ngroups;
    const int idx = n - 1 - (valid ? t : 0);
    T a = lo, b = hi;
    const int max_it = Tol<T>::bisect_iter_scale * (npts >= 7 ? 14 : (npts >= 3 ? 20 : (npts >= 2 ? 26 : 64)));
    for (int it = 0; it < max_it; ++it) {
      const T step = (b - a) / T(npts + 1);
      int pred = 0;
      if (l < npts) pred = sturm_count(d, e2, n, a + T(l + 1) * step, pivmin) <= idx;
#ifdef VMC_HOST_EMULATION
      const unsigned bits = (unsigned)pred;
#else
      const unsigned bits = (__ballot_sync(gmask, pred) >> base) & ((1u << G) - 1u);
#endif
      const int L = __popc(bits);
      const T na = (L == 0) ? a : a + T(L) * step;
      const T nb = (L == npts) ? b : a + T(L + 1) * step;
      a = na;
      b = nb;
      if (b - a <= Tol<T>::bisect_rtol * vmax(vabs(a), vabs(b)) + pivmin) break;
    }
    if (valid && l == 0) lam[t] = T(0.5) * (a + b);
  }
  __syncthreads();
  return tnorm;
}

// One eigenvector of T for eigenvalue lam by inverse iteration (serial; one
// thread).  x receives the normalised vector with stride xs.  u0/u1/u2/mul
// are n floats each and sw n bytes of private scratch.
// If n_orth > 0, every iterate is orthogonalised against the n_orth vectors
// `orth` (stride xs, column offset 1 apart) -- used for clusters of nearly
// equal eigenvalues.
template <typename T>
__device__ inline void tri_inverse_iteration(const T* d, const T* e, int n, T lam, T tnorm, T* x,
                                             int xs, T* u0, T* u1, T* u2, T* mul,
                                             unsigned char* sw, unsigned seed, const T* orth = nullptr,
                                             int n_orth = 0) {
  const T tiny = Tol<T>::inv_tiny * vmax(tnorm, T(1e-30));
  // FP64: u0 holds the pivots' reciprocals (one division per row instead of
  // one per row and iteration; FP64 division costs many FP64 multiply-adds)
  constexpr bool kRecip = std::is_same<T, double>::value;
  T al = d[0] - lam;
  T be = n > 1 ? e[0] : T(0.);
#pragma unroll 4
  for (int i = 0; i < n - 1; ++i) {
    const T c = e[i];
    const T a1 = d[i + 1] - lam;
    const T b1 = (i + 1 < n - 1) ? e[i + 1] : T(0.);
    if (vabs(al) >= vabs(c)) {
      T piv = al;
      if (vabs(piv) < tiny) piv = vcopysign(tiny, piv == T(0.) ? T(1.) : piv);
      T m;
      if constexpr (kRecip) {
        const T r = T(1.) / piv;
        m = c * r;
        u0[i] = r;
      } else {
        m = c / piv;
        u0[i] = piv;
      }
      sw[i] = 0;
      u1[i] = be;
      u2[i] = T(0.);
      mul[i] = m;
      al = a1 - m * be;
      be = b1;
    } else {
      T m;
      if constexpr (kRecip) {
        const T r = T(1.) / c;
        m = al * r;
        u0[i] = r;
      } else {
        m = al / c;
        u0[i] = c;
      }
      sw[i] = 1;
      u1[i] = a1;
      u2[i] = b1;
      mul[i] = m;
      al = be - m * a1;
      be = -m * b1;
    }
  }
  if (vabs(al) < tiny) al = vcopysign(tiny, al == T(0.) ? T(1.) : al);
  u0[n - 1] = kRecip ? T(1.) / al : al;
  // the back substitution reads these (times zero) at i = n-1: they must not hold stale data
  u1[n - 1] = T(0.);
  u2[n - 1] = T(0.);
  // start vector: deterministic pseudo-random entries in [0.5, 1.5)
  unsigned h = seed * 2654435761u + 12345u;
  for (int i = 0; i < n; ++i) {
    h = h * 1664525u + 1013904223u;
    x[(size_t)i * xs] = T(0.5) + T(h >> 8) * T(1.0 / 16777216.0);
  }
  for (int iter = 0; iter < Tol<T>::inv_iters; ++iter) {
    // forward: apply the row operations to the right-hand side (in x)
    T act = x[0];
    #pragma unroll 4
    for (int i = 0; i < n - 1; ++i) {
      const T r1 = x[(size_t)(i + 1) * xs];
      if (!sw[i]) {
        x[(size_t)i * xs] = act;
        act = r1 - mul[i] * act;
      } else {
        x[(size_t)i * xs] = r1;
        act = act - mul[i] * r1;
      }
    }
    x[(size_t)(n - 1) * xs] = act;
    // back substitution
    T xn1 = T(0.), xn2 = T(0.), amax = T(0.);
    #pragma unroll 4
    for (int i = n - 1; i >= 0; --i) {
      const T num = x[(size_t)i * xs] - u1[i] * xn1 - u2[i] * xn2;
      const T xi = kRecip ? num * u0[i] : num / u0[i];
      x[(size_t)i * xs] = xi;
      xn2 = xn1;
      xn1 = xi;
      amax = vmax(amax, vabs(xi));
    }
    const T sc = amax > T(0.) ? T(1.) / amax : T(1.);
    for (int i = 0; i < n; ++i) x[(size_t)i * xs] *= sc;
    for (int o = 0; o < n_orth; ++o) {
      const T* y = orth + o;
      T dot = T(0.), yy = T(0.);
      for (int i = 0; i < n; ++i) {
        dot = vfma(y[(size_t)i * xs], x[(size_t)i * xs], dot);
        yy = vfma(y[(size_t)i * xs], y[(size_t)i * xs], yy);
      }
      const T c = yy > T(0.) ? dot / yy : T(0.);
      for (int i = 0; i < n; ++i) x[(size_t)i * xs] -= c * y[(size_t)i * xs];
    }
  }
  T nrm = T(0.);
  for (int i = 0; i < n; ++i) nrm = vfma(x[(size_t)i * xs], x[(size_t)i * xs], nrm);
  const T sc = nrm > T(0.) ? T(1.) / vsqrt(nrm) : T(0.);
  for (int i = 0; i < n; ++i) x[(size_t)i * xs] *= sc;
}

// Orthonormalise the k columns of Y (n x k, row stride ldy) by CholQR: S = Y^T Y,
// S = R^T R (warp 0), Y <- Y R^-1.  Returns false if S is numerically singular.
template <typename T>
__device__ inline bool cta_cholqr(T* Y, int n, int k, int ldy, T* S, int* flag) {
  const int tid = threadIdx.x;
  cta_gram_t(Y, n, k, ldy, S);
  if (tid == 0) *flag = 0;
  __syncthreads();
  const int nl = blockDim.x < 32 ? blockDim.x : 32;
  if (tid < 32) {
    for (int j = 0; j < k; ++j) {
      const T sjj = S[j * k + j];
      if (!(sjj > Tol<T>::chol_min)) {
        if (tid == 0) *flag = 1;
        break;
      }
      const T rjj = vsqrt(sjj);
      warp_sync();
      for (int c = j + 1 + tid; c < k; c += nl) S[j * k + c] /= rjj;
      if (tid == 0) S[j * k + j] = rjj;
      warp_sync();
      for (int c = j + 1 + tid; c < k; c += nl) {
        const T rjc = S[j * k + c];
        for (int i = j + 1; i <= c; ++i) S[i * k + c] -= S[j * k + i] * rjc;
      }
      warp_sync();
    }
  }
  __syncthreads();
  if (*flag) return false;
  // FP64: R's diagonal replaced by its reciprocals (k divisions instead of n k)
  constexpr bool kRecip = std::is_same<T, double>::value;
  if constexpr (kRecip) {
    for (int t = tid; t < k; t += blockDim.x) S[t * k + t] = T(1.) / S[t * k + t];
    __syncthreads();
  }
  // Y <- Y R^-1, one row per thread
  for (int i = tid; i < n; i += blockDim.x) {
    T* y = Y + (size_t)i * ldy;
    for (int t = 0; t < k; ++t) {
      T v = y[t];
      for (int s = 0; s < t; ++s) v -= y[s] * S[s * k + t];
      y[t] = kRecip ? v * S[t * k + t] : v / S[t * k + t];
    }
  }
  __syncthreads();
  return true;
}

// Modified Gram-Schmidt fallback (serial over columns, parallel over rows).
template <typename T>
__device__ inline void cta_mgs(T* Y, int n, int k, int ldy, double* red) {
  for (int t = 0; t < k; ++t) {
    for (int s = 0; s < t; ++s) {
      double dot = 0.0;
      for (int i = threadIdx.x; i < n; i += blockDim.x) dot += (double)Y[(size_t)i * ldy + s] * Y[(size_t)i * ldy + t];
      dot = cta_sum(dot, red);
      for (int i = threadIdx.x; i < n; i += blockDim.x) Y[(size_t)i * ldy + t] -= T(dot) * Y[(size_t)i * ldy + s];
      __syncthreads();
    }
    double nn = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) nn += (double)Y[(size_t)i * ldy + t] * Y[(size_t)i * ldy + t];
    nn = cta_sum(nn, red);
    const T sc = nn > 0.0 ? T(1.0 / sqrt(nn)) : T(0.);
    for (int i = threadIdx.x; i < n; i += blockDim.x) Y[(size_t)i * ldy + t] *= sc;
    __syncthreads();
  }
}

// Apply Q = H_0 ... H_{n-3} to Y (n x k):  Y <- Q Y.
template <typename T>
__device__ inline void cta_back_transform(const T* A, int n, int lda, const T* tau, T* Y, int k, int ldy,
                                          T* cvec) {
  const int tid = threadIdx.x, nt = blockDim.x;
  int g = nt / (k > 0 ? k : 1);
  if (g > 32) g = 32;
  int gp = 1;
  while (gp * 2 <= g) gp *= 2;
  g = gp;
  const int ngroups = nt / g;
  const int grp = tid / g, lig = tid % g;
  const unsigned gmask = (g == 32) ? 0xffffffffu : (((1u << g) - 1u) << ((tid & 31) & ~(g - 1)));
  int gx = 1;
  while (gx * 2 <= k && gx * 2 <= nt) gx *= 2;
  const int gy = nt / gx;
  const int ux = tid % gx, uy = tid / gx;
  T* cv2 = cvec + k;
  int j = n - 3;
  // pairs: Y <- H_{j-1} H_j Y in one reduction and one update.  With
  // a = v_j^T Y, b = v_{j-1}^T Y and sg = v_{j-1}^T v_j:
  //   c_j = tau_j a,  c_{j-1} = tau_{j-1} (b - sg c_j),
  //   Y -= v_j c_j^T + v_{j-1} c_{j-1}^T.
  // Rows are indexed from j (v_{j-1}[j] = 1, v_j[j] = 0, v_j[j+1] = 1).
  for (; j >= 1; j -= 2) {
    const T t1 = tau[j], t0 = tau[j - 1];
    if (t1 == T(0.) && t0 == T(0.)) continue;
    const int m = n - j;
    for (int t = grp; t < k; t += ngroups) {
      T a = T(0.), b = T(0.), sg = T(0.);
      for (int i = lig; i < m; i += g) {
        const int row = j + i;
        const T y = Y[(size_t)row * ldy + t];
        const T vb = (i == 0) ? T(1.) : A[(size_t)row * lda + (j - 1)];
        const T va = (i == 0) ? T(0.) : ((i == 1) ? T(1.) : A[(size_t)row * lda + j]);
        if constexpr (std::is_same<T, df64>::value) {
          acc_mac(a, va, y);
          acc_mac(b, vb, y);
          acc_mac(sg, va, vb);
        } else {
          a = vfma(va, y, a);
          b = vfma(vb, y, b);
          sg = vfma(va, vb, sg);
        }
      }
      if constexpr (std::is_same<T, df64>::value) {
        a = df_norm(a);
        b = df_norm(b);
        sg = df_norm(sg);
      }
#ifndef VMC_HOST_EMULATION
      for (int o = g / 2; o > 0; o >>= 1) {
        a += shfl_xor_t(gmask, a, o, g);
        b += shfl_xor_t(gmask, b, o, g);
        sg += shfl_xor_t(gmask, sg, o, g);
      }
#endif
      if (lig == 0) {
        const T cj = t1 * a;
        cvec[t] = cj;
        cv2[t] = t0 * (b - sg * cj);
      }
    }
    __syncthreads();
    for (int i = uy; i < m; i += gy) {
      const int row = j + i;
      const T vb = (i == 0) ? T(1.) : A[(size_t)row * lda + (j - 1)];
      const T va = (i == 0) ? T(0.) : ((i == 1) ? T(1.) : A[(size_t)row * lda + j]);
      T* yrow = Y + (size_t)row * ldy;
      if constexpr (std::is_same<T, df64>::value) {
        for (int t = ux; t < k; t += gx) yrow[t] = df_sub2(yrow[t], va, cvec[t], vb, cv2[t]);
      } else {
        for (int t = ux; t < k; t += gx) yrow[t] -= va * cvec[t] + vb * cv2[t];
      }
    }
    __syncthreads();
  }
  // a last unpaired reflector (j == 0)
  for (; j >= 0; --j) {
    const T tj = tau[j];
    if (tj == T(0.)) continue;
    const int m = n - j - 1;
    for (int t = grp; t < k; t += ngroups) {
      T s = T(0.);
      for (int i = lig; i < m; i += g)
        s = vfma(i == 0 ? T(1.) : A[(size_t)(j + 1 + i) * lda + j], Y[(size_t)(j + 1 + i) * ldy + t], s);
#ifndef VMC_HOST_EMULATION
      for (int o = g / 2; o > 0; o >>= 1) s += shfl_xor_t(gmask, s, o, g);
#endif
      if (lig == 0) cvec[t] = tj * s;
    }
    __syncthreads();
    for (int i = uy; i < m; i += gy) {
      const T vi = (i == 0) ? T(1.) : A[(size_t)(j + 1 + i) * lda + j];
      T* yrow = Y + (size_t)(j + 1 + i) * ldy;
      for (int t = ux; t < k; t += gx) yrow[t] -= vi * cvec[t];
    }
    __syncthreads();
  }
  (void)gmask;
}

// Scratch for cta_sym_topk (all pointers into shared or global memory).
template <typename T>
struct EigScratchT {
  T *d, *e, *e2, *tau, *v, *p, *lam, *cvec, *part;
  T* yr;               // complex solves: real n*k eigenvectors of T before the back-transform
  T* S;                // k*k
  T* lu;               // k * 4 * n
  unsigned char* sw;       // k * n
  int* flag;
};
using EigScratch = EigScratchT<float>;

// The kk largest eigenvalues of the tridiagonal in w (descending, into w.lam);
// returns the Gershgorin scale |T|.
__device__ inline float top_eigenvalues(const EigScratchT<float>& w, int n, int kk) {
  return cta_top_eigenvalues(w.d, w.e, w.e2, n, kk, w.lam);
}

// High 32 bits of an FP64 value: its sign and exponent, tested with integer
// instructions (FP64 compares also issue to the FP64 pipe).
__device__ __forceinline__ int hi_word(double x) {
#ifdef VMC_HOST_EMULATION
  long long b;
  std::memcpy(&b, &x, 8);
  return (int)(b >> 32);
#else
  return __double2hiint(x);
#endif
}
__device__ __forceinline__ int exp_bits(int hi) { return (hi >> 20) & 0x7ff; }

// Characteristic polynomial of the leading principal submatrices of T at x:
// p_i = det(T_i - x I) = (d_{i-1} - x) p_{i-1} - e2_{i-2} p_{i-2}, with its
// x-derivative when want_deriv.  Returns the number of eigenvalues of T below
// x (sign changes along p_0..p_n); *f and *fp receive p_n and p_n' scaled by
// one common power of two.  A minor within ~2^-930 of its predecessor is
// replaced by -2^-930 times it (the ratio form's pivmin guard), and the pair
// is rescaled by 2^-/+600 to stay in range.  No divisions: FP64 division costs
// many FP64 multiply-adds.
template <bool want_deriv>
__device__ __forceinline__ int char_poly(const double* d, const double* e2, int n, double x, double* f, double* fp) {
  double a = 1.0, b = d[0] - x, ap = 0.0, bp = -1.0;
  if (exp_bits(hi_word(b)) < 1023 - 930) b = -0x1p-930;
  int cnt = hi_word(b) < 0;
  for (int i = 1; i < n; ++i) {
    const double dmx = d[i] - x;
    double c = fma(dmx, b, -e2[i - 1] * a);
    if (want_deriv) {
      const double cp = fma(dmx, bp, -fma(e2[i - 1], ap, b));
      ap = bp;
      bp = cp;
    }
    const int hb = hi_word(b);
    int hc = hi_word(c);
    if (exp_bits(hc) + 930 < exp_bits(hb)) {
      c = -0x1p-930 * b;
      hc = hi_word(c);
    }
    cnt += (hc < 0) != (hb < 0);
    a = b;
    b = c;
    const int eb = exp_bits(hc);
    if (eb > 1023 + 600 || (eb < 1023 - 600 && exp_bits(hi_word(a)) < 1023 - 600)) {
      const double sc = eb > 1023 ? 0x1p-600 : 0x1p600;
      a *= sc;
      b *= sc;
      if (want_deriv) {
        ap *= sc;
        bp *= sc;
      }
    }
  }
  *f = b;
  *fp = bp;
  return cnt;
}

// FP64 eigenvalues for the boundary-MPS chain of mixed-precision plans.  FP32
// multisection on the rounded tridiagonal gives each eigenvalue to a few FP32
// ulps of |T|; from that start a Newton iteration on p_n, guarded by the
// bracket that the same recurrence's Sturm count maintains (a step leaving
// the bracket bisects instead), converges to 1e-13 |T| in a few evaluations.
// The bracket starts at +-4e-6 |T| around the FP32 value and widens to the
// Gershgorin interval if its counts disagree.  w.v and w.p (free between the
// tridiagonalisation and the back-transform) hold the FP32 copies.
__device__ inline double top_eigenvalues(const EigScratchT<double>& w, int n, int kk) {
  const int tid = threadIdx.x, nt = blockDim.x;
  float* d32 = reinterpret_cast<float*>(w.v);
  float* e32 = d32 + n;
  float* e2_32 = reinterpret_cast<float*>(w.p);
  float* lam32 = e2_32 + n;
  for (int i = tid; i < n; i += nt) {
    d32[i] = (float)w.d[i];
    if (i < n - 1) {
      e32[i] = (float)w.e[i];
      w.e2[i] = w.e[i] * w.e[i];
    }
  }
  __syncthreads();
  cta_top_eigenvalues(d32, e32, e2_32, n, kk, lam32);
  // FP64 Gershgorin interval, warp-strided as in cta_top_eigenvalues (FP64 operations issue at a
  // fraction of the FP32 rate, so no thread walks all n rows)
  double lo = 1.7e308, hi = -1.7e308;
  for (int i = tid & 31; i < n; i += (nt < 32 ? nt : 32)) {
    const double r = (i > 0 ? fabs(w.e[i - 1]) : 0.0) + (i < n - 1 ? fabs(w.e[i]) : 0.0);
    lo = fmin(lo, w.d[i] - r);
    hi = fmax(hi, w.d[i] + r);
  }
#ifndef VMC_HOST_EMULATION
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
#endif
  const double tnorm = fmax(fabs(lo), fabs(hi));
  // Near a root the evaluated p_n / p_n' carries rounding noise well above
  // 1e-13 |T|, so Newton stops at 1e-11 |T|: two inverse-iteration steps then
  // leave (1e-11 |T| / gap)^2 of a neighbouring eigenvector in the vector, and
  // the eigen-gaps at the cuts stay above ~1e-6 |T|.
  const double span = hi - lo, tol = 1e-11 * tnorm + 1e-280;
  lo -= 1e-12 * span + 1e-280;
  hi += 1e-12 * span + 1e-280;
  for (int t = tid; t < kk; t += nt) {
    const int idx = n - 1 - t;  // the eigenvalue with idx others below it: count(a) <= idx < count(b)
    const double c = (double)lam32[t], delta = 4e-6 * tnorm;
    double a = c - delta, b = c + delta, f, fp;
    if (!(a > lo) || char_poly<false>(w.d, w.e2, n, a, &f, &fp) > idx) a = lo;
    if (!(b < hi) || char_poly<false>(w.d, w.e2, n, b, &f, &fp) <= idx) b = hi;
    double x = fmin(fmax(c, a), b);
    for (int it = 0; it < 64; ++it) {
      const int cx = char_poly<true>(w.d, w.e2, n, x, &f, &fp);
      if (cx <= idx)
        a = x;
      else
        b = x;
      double xn = (fp != 0.0) ? x - f / fp : 0.5 * (a + b);
      if (!(xn > a && xn < b)) xn = 0.5 * (a + b);
      const bool done = fabs(xn - x) <= tol || b - a <= tol;
      x = xn;
      if (done) break;
    }
    w.lam[t] = x;
  }
  __syncthreads();
  return tnorm;
}

template <typename T>
__device__ inline void tri_topk_vectors(int n, int k, T* Y, int ldy, const EigScratchT<T>& w, double* red) {
  VMC_TSTART(t1);
  const int kk = k + 1 <= n ? k + 1 : n;
  const T tnorm = top_eigenvalues(w, n, kk);
  VMC_TSTOP(t1, PH_BISECT);
  VMC_TSTART(t2);
  for (int t = threadIdx.x; t < k; t += blockDim.x) {
    T* lu = w.lu + (size_t)t * 4 * n;
    tri_inverse_iteration(w.d, w.e, n, w.lam[t], tnorm, Y + t, ldy, lu, lu + n, lu + 2 * n, lu + 3 * n,
                          w.sw + (size_t)t * n, 977u * (unsigned)t + 1u);
  }
  __syncthreads();
  // clusters of nearly equal eigenvalues: re-iterate serially, keeping each
  // vector orthogonal to the earlier members of its cluster
  if (threadIdx.x == 0) {
    int start = 0;
    for (int t = 1; t < k; ++t) {
      if (w.lam[t - 1] - w.lam[t] < Tol<T>::cluster * tnorm) {
        T* lu = w.lu + (size_t)t * 4 * n;
        tri_inverse_iteration(w.d, w.e, n, w.lam[t], tnorm, Y + t, ldy, lu, lu + n, lu + 2 * n, lu + 3 * n,
                              w.sw + (size_t)t * n, 977u * (unsigned)t + 1u, Y + start, t - start);
      } else {
        start = t;
      }
    }
  }
  __syncthreads();
  VMC_TSTOP(t2, PH_INVIT);
  VMC_TSTART(t3);
  // the vectors belong to distinct (or cluster-orthogonalised) eigenvalues and
  // are already orthogonal to O(1e-4); one CholQR pass restores eps level
  const bool ok = cta_cholqr(Y, n, k, ldy, w.S, w.flag);
  if (!ok) cta_mgs(Y, n, k, ldy, red);
  VMC_TSTOP(t3, PH_CHOLQR);
}

// Householder tridiagonalisation of an FP64 matrix carried out in df64 on the
// FP32 units (df64.cuh): the matrix, the reflectors and T are converted in
// place (a df64 takes the 8 bytes of a double), reduced, and converted back.
__device__ inline void cta_tridiagonalize_df(double* G, int n, int ldg, const EigScratchT<double>& w) {
  df64* A = reinterpret_cast<df64*>(G);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const size_t o = (size_t)(e / n) * ldg + e % n;
    A[o] = df64(G[o]);
  }
  __syncthreads();
  cta_tridiagonalize(A, n, ldg, reinterpret_cast<df64*>(w.d), reinterpret_cast<df64*>(w.e),
                     reinterpret_cast<df64*>(w.tau), reinterpret_cast<df64*>(w.v), reinterpret_cast<df64*>(w.p),
                     reinterpret_cast<df64*>(w.part));
  // T and tau, then the reflectors (strictly below the diagonal), back to FP64
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    w.d[i] = reinterpret_cast<df64*>(w.d)[i].to_double();
    w.e[i] = reinterpret_cast<df64*>(w.e)[i].to_double();
    w.tau[i] = reinterpret_cast<df64*>(w.tau)[i].to_double();
  }
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int r = e / n, c = e % n;
    if (r > c) {
      const size_t o = (size_t)r * ldg + c;
      G[o] = A[o].to_double();
    }
  }
  __syncthreads();
}

// Top-k eigenvectors of a symmetric n x n matrix held in df64: the Householder tridiagonalisation and
// the back-transform run in df64 on the FP32 units; the eigenvalues (FP32 brackets refined by Newton's
// method) and inverse iteration run in FP64 on T, whose d and e are converted in place.  The reflectors
// stay in A and tau in df64; Y (n x k, row stride ldy) is computed as FP64 by the tridiagonal solver and
// converted to df64 in place (a df64 takes the 8 bytes of a double).
__device__ inline void cta_sym_topk_df(df64* A, int n, int lda, int k, df64* Y, int ldy,
                                       const EigScratchT<double>& w, double* red) {
  VMC_TSTART(t0);
  df64* d = reinterpret_cast<df64*>(w.d);
  df64* e = reinterpret_cast<df64*>(w.e);
  df64* tau = reinterpret_cast<df64*>(w.tau);
  cta_tridiagonalize(A, n, lda, d, e, tau, reinterpret_cast<df64*>(w.v), reinterpret_cast<df64*>(w.p),
                     reinterpret_cast<df64*>(w.part));
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    w.d[i] = d[i].to_double();
    w.e[i] = e[i].to_double();
  }
  __syncthreads();
  VMC_TSTOP(t0, PH_TRIDIAG);
  double* Yd = reinterpret_cast<double*>(Y);
  tri_topk_vectors(n, k, Yd, ldy, w, red);
  for (int el = threadIdx.x; el < n * k; el += blockDim.x) {
    const size_t o = (size_t)(el / k) * ldy + el % k;
    Y[o] = df64(Yd[o]);
  }
  __syncthreads();
  VMC_TSTART(t4);
  cta_back_transform(static_cast<const df64*>(A), n, lda, static_cast<const df64*>(tau), Y, k, ldy,
                     reinterpret_cast<df64*>(w.cvec));
  VMC_TSTOP(t4, PH_BACK);
}

template <typename T>
__device__ inline void cta_sym_topk(T* G, int n, int ldg, int k, T* Y, int ldy, const EigScratchT<T>& w,
                                    double* red) {
  VMC_TSTART(t0);
  if constexpr (std::is_same<T, double>::value)
    cta_tridiagonalize_df(G, n, ldg, w);
  else
    cta_tridiagonalize(G, n, ldg, w.d, w.e, w.tau, w.v, w.p, w.part);
  VMC_TSTOP(t0, PH_TRIDIAG);
  tri_topk_vectors(n, k, Y, ldy, w, red);
  VMC_TSTART(t4);
  cta_back_transform(G, n, ldg, w.tau, Y, k, ldy, w.cvec);
  VMC_TSTOP(t4, PH_BACK);
}

// ---------------------------------------------------------------------------
// Complex Hermitian variants.  Complex elements are interleaved (re, im)
// floats; leading dimensions count elements.
// ---------------------------------------------------------------------------

// Householder tridiagonalisation of the Hermitian n x n matrix A (full storage,
// both triangles kept current), as LAPACK's zhetd2 does it: each reflector
// H_j = I - tau_j v_j v_j^H has a real beta, so T = Q^H A Q is real symmetric
// tridiagonal (d, e) with Q = H_0 ... H_{n-2}; the last step only rotates a
// phase.  tau (complex) and A[j+1+i][j] (i >= 1; v_j[0] = 1 implicit) hold the
// reflectors.  v, p: n complex scratch; part: >= 64 floats.  For one column:
//   p = tau A v,   w = p - (tau/2) (p^H v) v,   A -= v w^H + w v^H.
__device__ inline void cta_tridiagonalize_c(float* A, int n, int lda, float* d, float* e, float* tau, float* v,
                                            float* p, float* part) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int nl = nt < 32 ? nt : 32;
  const int lane = tid % nl, warp = tid / nl, nwarps = nt / nl;
  auto re = [&](int i, int j) -> float& { return A[2 * ((size_t)i * lda + j)]; };
  auto im = [&](int i, int j) -> float& { return A[2 * ((size_t)i * lda + j) + 1]; };
  if (n == 1) {
    if (tid == 0) d[0] = A[0];
    __syncthreads();
    return;
  }
  for (int j = 0; j < n - 1; ++j) {
    const int m = n - j - 1;  // length of the reflected vector (rows j+1..n-1)
    // |x|^2 of A[j+2.., j], one warp
    if (warp == 0) {
      float s = 0.f;
      for (int i = j + 2 + lane; i < n; i += nl) s = fmaf(re(i, j), re(i, j), fmaf(im(i, j), im(i, j), s));
      s = warp_sum_f(s);
      if (lane == 0) part[0] = s;
    }
    __syncthreads();
    const float xn2 = part[0];
    const float ar = re(j + 1, j), ai = im(j + 1, j);
    float tr = 0.f, ti = 0.f, beta = ar, sr = 0.f, si = 0.f;
    if (xn2 > 0.f || ai != 0.f) {
      beta = -copysignf(sqrtf(ar * ar + ai * ai + xn2), ar);
      tr = (beta - ar) / beta;
      ti = -ai / beta;
      // scal = 1 / (alpha - beta)
      const float dr = ar - beta, di = ai, den = dr * dr + di * di;
      sr = dr / den;
      si = -di / den;
    }
    // v (rows j+1..): v_0 = 1, v_i = x_i * scal; column j keeps x until barrier (2)
    for (int i = tid; i < m; i += nt) {
      if (i == 0) {
        v[0] = 1.f;
        v[1] = 0.f;
      } else {
        const float xr = re(j + 1 + i, j), xi = im(j + 1 + i, j);
        v[2 * i] = xr * sr - xi * si;
        v[2 * i + 1] = xr * si + xi * sr;
      }
    }
    if (tid == 0) {
      d[j] = re(j, j);
      e[j] = beta;
      tau[2 * j] = tr;
      tau[2 * j + 1] = ti;
    }
    __syncthreads();  // (1) v visible
    if (tr == 0.f && ti == 0.f) continue;
    // p = tau * A_sub v (one thread per row)
    for (int i = tid; i < m; i += nt) {
      float yr = 0.f, yi = 0.f;
      for (int l = 0; l < m; ++l) {
        const float a_r = re(j + 1 + i, j + 1 + l), a_i = im(j + 1 + i, j + 1 + l);
        const float vr = v[2 * l], vi = v[2 * l + 1];
        yr = fmaf(a_r, vr, fmaf(-a_i, vi, yr));
        yi = fmaf(a_r, vi, fmaf(a_i, vr, yi));
      }
      p[2 * i] = tr * yr - ti * yi;
      p[2 * i + 1] = tr * yi + ti * yr;
    }
    __syncthreads();  // (2) p visible
    // c = p^H v; K = (tau / 2) c
    float cr = 0.f, ci = 0.f;
    for (int i = 0; i < m; ++i) {
      const float pr = p[2 * i], pi = -p[2 * i + 1], vr = v[2 * i], vi = v[2 * i + 1];
      cr = fmaf(pr, vr, fmaf(-pi, vi, cr));
      ci = fmaf(pr, vi, fmaf(pi, vr, ci));
    }
    const float kr = 0.5f * (tr * cr - ti * ci), ki = 0.5f * (tr * ci + ti * cr);
    // reflector into column j, rank-2 update of the trailing matrix:
    // A[i][l] -= v_i conj(w_l) + w_i conj(v_l),  w = p - K v
    for (int i = 1 + tid; i < m; i += nt) {
      re(j + 1 + i, j) = v[2 * i];
      im(j + 1 + i, j) = v[2 * i + 1];
    }
    for (int e2 = tid; e2 < m * m; e2 += nt) {
      const int i = e2 / m, l = e2 - i * m;
      const float vir = v[2 * i], vii = v[2 * i + 1], vlr = v[2 * l], vli = v[2 * l + 1];
      const float wir = p[2 * i] - (kr * vir - ki * vii), wii = p[2 * i + 1] - (kr * vii + ki * vir);
      const float wlr = p[2 * l] - (kr * vlr - ki * vli), wli = p[2 * l + 1] - (kr * vli + ki * vlr);
      // v_i conj(w_l) + w_i conj(v_l)
      const float ur = (vir * wlr + vii * wli) + (wir * vlr + wii * vli);
      const float ui = (vii * wlr - vir * wli) + (wii * vlr - wir * vli);
      re(j + 1 + i, j + 1 + l) -= ur;
      im(j + 1 + i, j + 1 + l) -= ui;
    }
    __syncthreads();  // (3) trailing matrix updated
  }
  if (tid == 0) d[n - 1] = re(n - 1, n - 1);
  __syncthreads();
}

// Y (n x k complex, row stride ldy) <- Q Y with Q = H_0 ... H_{n-2} from
// cta_tridiagonalize_c (H_j = I - tau_j v_j v_j^H applied for j descending).
__device__ inline void cta_back_transform_c(const float* A, int n, int lda, const float* tau, float* Y, int k,
                                            int ldy, float* cvec) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int j = n - 2; j >= 0; --j) {
    const float tr = tau[2 * j], ti = tau[2 * j + 1];
    if (tr == 0.f && ti == 0.f) continue;
    const int m = n - j - 1;
    // c_t = tau * sum_i conj(v_i) Y[j+1+i][t]
    for (int t = tid; t < k; t += nt) {
      float sr = 0.f, si = 0.f;
      for (int i = 0; i < m; ++i) {
        const float vr = i == 0 ? 1.f : A[2 * ((size_t)(j + 1 + i) * lda + j)];
        const float vi = i == 0 ? 0.f : -A[2 * ((size_t)(j + 1 + i) * lda + j) + 1];
        const float yr = Y[2 * ((size_t)(j + 1 + i) * ldy + t)], yi = Y[2 * ((size_t)(j + 1 + i) * ldy + t) + 1];
        sr = fmaf(vr, yr, fmaf(-vi, yi, sr));
        si = fmaf(vr, yi, fmaf(vi, yr, si));
      }
      cvec[2 * t] = tr * sr - ti * si;
      cvec[2 * t + 1] = tr * si + ti * sr;
    }
    __syncthreads();
    for (int e2 = tid; e2 < m * k; e2 += nt) {
      const int i = e2 / k, t = e2 - i * k;
      const float vr = i == 0 ? 1.f : A[2 * ((size_t)(j + 1 + i) * lda + j)];
      const float vi = i == 0 ? 0.f : A[2 * ((size_t)(j + 1 + i) * lda + j) + 1];
      float* y = Y + 2 * ((size_t)(j + 1 + i) * ldy + t);
      y[0] -= vr * cvec[2 * t] - vi * cvec[2 * t + 1];
      y[1] -= vr * cvec[2 * t + 1] + vi * cvec[2 * t];
    }
    __syncthreads();
  }
}

// Y (n x k complex, ldy) <- orthonormal basis of the dominant k-dimensional
// invariant subspace of the Hermitian matrix G (complex, destroyed).
__device__ inline void cta_herm_topk(float* G, int n, int ldg, int k, float* Y, int ldy, const EigScratch& w,
                                     double* red) {
  VMC_TSTART(t0);
  cta_tridiagonalize_c(G, n, ldg, w.d, w.e, w.tau, w.v, w.p, w.part);
  VMC_TSTOP(t0, PH_TRIDIAG);
  tri_topk_vectors(n, k, w.yr, k, w, red);
  for (int e2 = threadIdx.x; e2 < n * k; e2 += blockDim.x) {
    const int i = e2 / k, t = e2 - i * k;
    Y[2 * ((size_t)i * ldy + t)] = w.yr[e2];
    Y[2 * ((size_t)i * ldy + t) + 1] = 0.f;
  }
  __syncthreads();
  VMC_TSTART(t4);
  cta_back_transform_c(G, n, ldg, w.tau, Y, k, ldy, w.cvec);
  VMC_TSTOP(t4, PH_BACK);
}

}  // namespace vmc
