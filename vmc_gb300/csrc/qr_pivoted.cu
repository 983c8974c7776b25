// qr_pivoted.cu -- FP64 / complex128 column-pivoted Householder QR on the GPU,
// the factorisation of the SR QR solve (preconditioners.py:166-214, which calls
// jax.lax.linalg.qr(o_centered, pivoting=True, use_magma=True), i.e. xGEQP3).
//
// The algorithm is LAPACK's unblocked xGEQP3 (xLAQP2), step by step:
//   * pivot: the column of largest partial norm among j..n-1, the first on ties
//     (IxAMAX), swapped with column j over all m rows;
//   * reflector: xLARFG / ZLARFG conventions, H = I - tau v v^H with v[0] = 1,
//     beta = -sign(Re alpha) |(alpha, x)| real, tau = 0 when x = 0 (and, for
//     complex, Im alpha = 0); R's diagonal is beta;
//   * update: the trailing columns get H^H applied (xLARF with conj(tau));
//   * partial norms: downdated by sqrt(1 - (|a_jc| / vn1_c)^2), and recomputed
//     from the column when (vn1_c / vn2_c)^2 times that factor falls to
//     sqrt(eps) or below (xLAQP2's tol3z rule).
// Right-hand sides ride along as extra columns that are updated but never
// pivoted, so they come out as Q^H b.
//
// One kernel picks the pivot, swaps and builds the reflector (one CTA); one
// kernel applies it to the trailing columns (one warp per column, the column
// contiguous in memory).  FP64 arithmetic throughout: it is the precision the
// solve is specified in, and this kernel, at O(m^2 n) work, is bound by the
// part's FP64 rate.
#include <cstdint>

#include "device_common.cuh"
#include "../../include/vmc_gb300.h"

namespace vmc {
namespace qr {

constexpr int kPivotThreads = 1024;
constexpr int kApplyThreads = 256;
// sqrt(LAPACK dlamch('E')) = sqrt(2^-53): xLAQP2's threshold for recomputing a partial norm
constexpr double kTol3z = 1.0536712127723509e-08;

// Element access for real (ES = 1) or interleaved complex (ES = 2) storage;
// column-major, element (i, c) at A[ES * (c * lda + i)].
template <int ES>
struct Mat {
  double* a;
  long long lda;
  __device__ double* at(long long i, long long c) const { return a + ES * (c * lda + i); }
};

template <int ES>
__device__ inline double abs2(const double* x) {
  return ES == 2 ? x[0] * x[0] + x[1] * x[1] : x[0] * x[0];
}

// vn1 = vn2 = ||A[:, c]|| for the n pivotable columns; jpvt = identity.
template <int ES>
__global__ void qr_init_kernel(Mat<ES> A, int m, int n, double* vn1, double* vn2, int32_t* jpvt) {
  const int nl = blockDim.x < 32 ? blockDim.x : 32;
  const int lane = threadIdx.x % nl, wpb = blockDim.x / nl, warp = threadIdx.x / nl;
  for (long long c = (long long)blockIdx.x * wpb + warp; c < n; c += (long long)gridDim.x * wpb) {
    double s = 0.0;
    for (int i = lane; i < m; i += nl) s += abs2<ES>(A.at(i, c));
    s = warp_sum(s);
    if (lane == 0) {
      vn1[c] = vn2[c] = sqrt(s);
      jpvt[c] = (int32_t)c;
    }
  }
}

// Step j: pivot, swap, reflector.  One CTA.
template <int ES>
__global__ void qr_pivot_kernel(Mat<ES> A, int m, int n, int j, double* vn1, double* vn2, int32_t* jpvt,
                                double* tau) {
  VMC_SHARED double red[32];
  VMC_SHARED double best_v[32];
  VMC_SHARED int best_i[32];
  VMC_SHARED int piv;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int nl = nt < 32 ? nt : 32;
  const int lane = tid % nl, warp = tid / nl, nw = nt / nl;
  // argmax of vn1[j..n-1], the smallest index on ties
  double bv = -1.0;
  int bi = n;
  for (int c = j + tid; c < n; c += nt) {
    const double v = vn1[c];
    if (v > bv) { bv = v; bi = c; }  // ascending c per thread: keeps the first maximum
  }
#ifndef VMC_HOST_EMULATION
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
  }
#endif
  if (lane == 0) { best_v[warp] = bv; best_i[warp] = bi; }
  __syncthreads();
  if (tid == 0) {
    double v = best_v[0];
    int i = best_i[0];
    for (int w = 1; w < nw; ++w)
      if (best_v[w] > v || (best_v[w] == v && best_i[w] < i)) { v = best_v[w]; i = best_i[w]; }
    piv = i < n ? i : j;
  }
  __syncthreads();
  const int p = piv;
  if (p != j) {
    for (int i = tid; i < m; i += nt) {
      double* x = A.at(i, p);
      double* y = A.at(i, j);
      for (int e = 0; e < ES; ++e) {
        const double t = x[e];
        x[e] = y[e];
        y[e] = t;
      }
    }
    if (tid == 0) {
      const int32_t t = jpvt[p];
      jpvt[p] = jpvt[j];
      jpvt[j] = t;
      vn1[p] = vn1[j];
      vn2[p] = vn2[j];
    }
  }
  __syncthreads();  // the swapped rows are read by other threads below
  // reflector for A[j:m, j]
  double xs = 0.0;
  for (int i = j + 1 + tid; i < m; i += nt) xs += abs2<ES>(A.at(i, j));
  const double xnorm2 = cta_sum(xs, red);
  double* ajj = A.at(j, j);
  const double ar = ajj[0], ai = ES == 2 ? ajj[1] : 0.0;
  double tr = 0.0, ti = 0.0, beta = ar, sr = 0.0, si = 0.0;
  const bool reflect = xnorm2 > 0.0 || ai != 0.0;
  if (reflect) {
    beta = -copysign(sqrt(ar * ar + ai * ai + xnorm2), ar);
    tr = (beta - ar) / beta;
    ti = -ai / beta;
    // 1 / (alpha - beta)
    const double dr = ar - beta, di = ai, den = dr * dr + di * di;
    sr = dr / den;
    si = -di / den;
  }
  __syncthreads();  // every thread has read A[j][j] before it is overwritten
  if (reflect)
    for (int i = j + 1 + tid; i < m; i += nt) {
      double* x = A.at(i, j);
      if (ES == 2) {
        const double xr = x[0], xi = x[1];
        x[0] = xr * sr - xi * si;
        x[1] = xr * si + xi * sr;
      } else {
        x[0] *= sr;
      }
    }
  if (tid == 0) {
    ajj[0] = beta;
    if (ES == 2) ajj[1] = 0.0;
    tau[ES * j] = tr;
    if (ES == 2) tau[ES * j + 1] = ti;
  }
}

// Step j: A[j:m, c] -= conj(tau) v (v^H A[j:m, c]) for the trailing columns
// c = j+1 .. n_tot-1 (pivotable columns below n, right-hand sides from n),
// then the partial norms of the pivotable ones.  One warp per column.
template <int ES>
__global__ void qr_apply_kernel(Mat<ES> A, int m, int n, int n_tot, int j, double* vn1, double* vn2,
                                const double* tau) {
  const int nl = blockDim.x < 32 ? blockDim.x : 32;
  const int lane = threadIdx.x % nl, wpb = blockDim.x / nl, warp = threadIdx.x / nl;
  const double tr = tau[ES * j], ti = ES == 2 ? tau[ES * j + 1] : 0.0;
  const bool apply = tr != 0.0 || ti != 0.0;
  for (long long c = j + 1 + (long long)blockIdx.x * wpb + warp; c < n_tot; c += (long long)gridDim.x * wpb) {
    if (apply) {
      // s = v^H A[j:m, c], v[j] = 1
      const double* a0 = A.at(j, c);
      double s_re = lane == 0 ? a0[0] : 0.0, s_im = (lane == 0 && ES == 2) ? a0[1] : 0.0;
      for (int i = j + 1 + lane; i < m; i += nl) {
        const double* v = A.at(i, j);
        const double* x = A.at(i, c);
        if (ES == 2) {
          s_re = fma(v[0], x[0], fma(v[1], x[1], s_re));
          s_im = fma(v[0], x[1], fma(-v[1], x[0], s_im));
        } else {
          s_re = fma(v[0], x[0], s_re);
        }
      }
      s_re = warp_sum(s_re);
      if (ES == 2) s_im = warp_sum(s_im);
      // f = conj(tau) s
      const double f_re = tr * s_re + ti * s_im, f_im = tr * s_im - ti * s_re;
      if (lane == 0) {
        double* x = A.at(j, c);
        x[0] -= f_re;
        if (ES == 2) x[1] -= f_im;
      }
      for (int i = j + 1 + lane; i < m; i += nl) {
        const double* v = A.at(i, j);
        double* x = A.at(i, c);
        if (ES == 2) {
          x[0] -= v[0] * f_re - v[1] * f_im;
          x[1] -= v[0] * f_im + v[1] * f_re;
        } else {
          x[0] = fma(-v[0], f_re, x[0]);
        }
      }
      __syncwarp();
    }
    if (c < n && vn1[c] != 0.0) {
      const double a = sqrt(abs2<ES>(A.at(j, c)));
      double t = 1.0 - (a / vn1[c]) * (a / vn1[c]);
      t = t > 0.0 ? t : 0.0;
      const double q = vn1[c] / vn2[c];
      if (t * q * q <= kTol3z) {
        double s = 0.0;
        for (int i = j + 1 + lane; i < m; i += nl) s += abs2<ES>(A.at(i, c));
        s = warp_sum(s);
        if (lane == 0) vn1[c] = vn2[c] = (j + 1 < m) ? sqrt(s) : 0.0;
      } else if (lane == 0) {
        vn1[c] *= sqrt(t);
      }
    }
  }
}

template <int ES>
static vmc_status run(void* stream, double* a, long long lda, int m, int n, int nrhs, double* tau, int32_t* jpvt,
                      double* vn) {
  const Mat<ES> A{a, lda};
  const int k = m < n ? m : n, n_tot = n + nrhs;
  const int wpb = kApplyThreads / 32;
  double* vn1 = vn;
  double* vn2 = vn + n;
  VMC_LAUNCH(qr_init_kernel<ES>, (n + wpb - 1) / wpb, kApplyThreads, 0, stream, A, m, n, vn1, vn2, jpvt);
  for (int j = 0; j < k; ++j) {
    VMC_LAUNCH(qr_pivot_kernel<ES>, 1, kPivotThreads, 0, stream, A, m, n, j, vn1, vn2, jpvt, tau);
    const int cols = n_tot - j - 1;
    if (cols > 0)
      VMC_LAUNCH(qr_apply_kernel<ES>, (cols + wpb - 1) / wpb, kApplyThreads, 0, stream, A, m, n, n_tot, j, vn1,
                 vn2, tau);
  }
  return vmc_last_error() == cudaSuccess ? VMC_OK : VMC_ERR_CUDA;
}

}  // namespace qr
}  // namespace vmc

extern "C" {

size_t vmc_qr_pivoted_workspace_size(int n) { return n > 0 ? (size_t)2 * n * sizeof(double) : 0; }

vmc_status vmc_qr_pivoted(void* stream, int complex_elements, double* a, int64_t lda, int m, int n, int nrhs,
                          double* tau, int32_t* jpvt, void* workspace, size_t workspace_bytes) {
  if (!a || m < 0 || n < 0 || nrhs < 0 || lda < (m > 1 ? m : 1) || (n > 0 && (!tau || !jpvt || !workspace)))
    return VMC_ERR_INVALID;
  if (m == 0 || n == 0) return VMC_OK;
  if (workspace_bytes < vmc_qr_pivoted_workspace_size(n)) return VMC_ERR_WORKSPACE;
  double* vn = static_cast<double*>(workspace);
  return complex_elements ? vmc::qr::run<2>(stream, a, lda, m, n, nrhs, tau, jpvt, vn)
                          : vmc::qr::run<1>(stream, a, lda, m, n, nrhs, tau, jpvt, vn);
}

}  // extern "C"
