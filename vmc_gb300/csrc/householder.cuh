// householder.cuh -- CTA-level Householder QR of a small matrix, for the
// variational boundary-MPS compression (strategy.py:179-427, whose QR is
// geqrf + orgqr through src/vmc/utils/factorizations.py:9-16).
//
// Only the orthogonal factor is formed.  The compression needs an orthonormal
// basis of the span of the leading k columns; where the triangular factor is
// needed the caller recomputes it as Q^T A with a GEMM.  Reflectors follow
// LAPACK's xLARFG conventions: H = I - tau v v^T with v[0] = 1,
// beta = -sign(alpha) * ||(alpha, x)||, and tau = 0 when x is exactly zero, so
// rank-deficient panels give the same unit columns LAPACK gives.  The result
// equals LAPACK's Q up to rounding; the boundary MPS it feeds is invariant
// under the sign of each column.
#pragma once

#include "device_common.cuh"
#include "truncation.cuh"

namespace vmc {

// Q (m x k; element (i, c) at Q[i*qrs + c*qcs]) := the first k columns of the
// orthogonal factor of the QR factorisation of the m x k panel A[:, :k]
// (element (i, j) at A[i*ars + j*acs]); requires k <= m.  H (m x k, leading
// dimension ldh, odd for conflict-free column access) and tau (k floats) are
// scratch; Q must alias neither A nor H.  One warp builds each reflector, the
// warps share the trailing columns; 3 barriers per column.
template <typename T>
__device__ inline void cta_householder_q(const T* A, int m, int k, int ars, int acs, T* Q, int qrs, int qcs,
                                         T* H, int ldh, T* tau) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int nl = nt < 32 ? nt : 32;
  const int lane = tid % nl, warp = tid / nl, nwarps = nt / nl;
  for (int e = tid; e < m * k; e += nt) {
    const int i = e / k, j = e - i * k;
    H[(size_t)i * ldh + j] = A[(size_t)i * ars + (size_t)j * acs];
  }
  __syncthreads();
  for (int j = 0; j < k; ++j) {
    if (warp == 0) {
      T xn = T(0.);
      for (int i = j + 1 + lane; i < m; i += nl) {
        const T x = H[(size_t)i * ldh + j];
        xn = vfma(x, x, xn);
      }
      xn = warp_sum_t(xn);
      const T alpha = H[(size_t)j * ldh + j];
      T t = T(0.), beta = alpha, sc = T(0.);
      if (xn > T(0.)) {
        beta = -vcopysign(vsqrt(vfma(alpha, alpha, xn)), alpha);
        t = (beta - alpha) / beta;
        sc = T(1.) / (alpha - beta);
      }
      warp_sync();
      if (t != T(0.))
        for (int i = j + 1 + lane; i < m; i += nl) H[(size_t)i * ldh + j] *= sc;
      if (lane == 0) {
        H[(size_t)j * ldh + j] = beta;
        tau[j] = t;
      }
    }
    __syncthreads();
    const T t = tau[j];
    if (t != T(0.)) {
      for (int c = j + 1 + warp; c < k; c += nwarps) {
        T w = T(0.);
        for (int i = j + 1 + lane; i < m; i += nl) w = vfma(H[(size_t)i * ldh + j], H[(size_t)i * ldh + c], w);
        w = t * (warp_sum_t(w) + H[(size_t)j * ldh + c]);
        warp_sync();
        if (lane == 0) H[(size_t)j * ldh + c] -= w;
        for (int i = j + 1 + lane; i < m; i += nl)
          H[(size_t)i * ldh + c] = vfma(-w, H[(size_t)i * ldh + j], H[(size_t)i * ldh + c]);
      }
    }
    __syncthreads();
  }
  // Q = H_0 H_1 ... H_{k-1} [I_k; 0]; H_j leaves columns c < j at e_c
  for (int e = tid; e < m * k; e += nt) {
    const int i = e / k, c = e - i * k;
    Q[(size_t)i * qrs + (size_t)c * qcs] = (i == c) ? T(1.) : T(0.);
  }
  __syncthreads();
  for (int j = k - 1; j >= 0; --j) {
    const T t = tau[j];
    if (t != T(0.)) {
      for (int c = j + warp; c < k; c += nwarps) {
        T w = T(0.);
        for (int i = j + 1 + lane; i < m; i += nl)
          w = vfma(H[(size_t)i * ldh + j], Q[(size_t)i * qrs + (size_t)c * qcs], w);
        w = t * (warp_sum_t(w) + Q[(size_t)j * qrs + (size_t)c * qcs]);
        warp_sync();
        if (lane == 0) Q[(size_t)j * qrs + (size_t)c * qcs] -= w;
        for (int i = j + 1 + lane; i < m; i += nl)
          Q[(size_t)i * qrs + (size_t)c * qcs] =
              vfma(-w, H[(size_t)i * ldh + j], Q[(size_t)i * qrs + (size_t)c * qcs]);
      }
    }
    __syncthreads();
  }
}

// Complex variant (interleaved (re, im) elements; strides count elements), as
// zgeqr2 + zung2r: H_j = I - tau_j v_j v_j^H with real beta, A <- H_j^H A for
// the panel, Q = H_0 ... H_{k-1} [I_k; 0].  H: m x k complex scratch (ldh
// elements), tau: k complex.
__device__ inline void cta_householder_q_c(const float* A, int m, int k, int ars, int acs, float* Q, int qrs,
                                           int qcs, float* H, int ldh, float* tau) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int nl = nt < 32 ? nt : 32;
  const int lane = tid % nl, warp = tid / nl, nwarps = nt / nl;
  auto hr = [&](int i, int j) -> float& { return H[2 * ((size_t)i * ldh + j)]; };
  auto hi = [&](int i, int j) -> float& { return H[2 * ((size_t)i * ldh + j) + 1]; };
  for (int e = tid; e < m * k; e += nt) {
    const int i = e / k, j = e - i * k;
    const size_t src = 2 * ((size_t)i * ars + (size_t)j * acs);
    hr(i, j) = A[src];
    hi(i, j) = A[src + 1];
  }
  __syncthreads();
  for (int j = 0; j < k; ++j) {
    if (warp == 0) {
      float xn = 0.f;
      for (int i = j + 1 + lane; i < m; i += nl) xn = fmaf(hr(i, j), hr(i, j), fmaf(hi(i, j), hi(i, j), xn));
      xn = warp_sum_f(xn);
      const float ar = hr(j, j), ai = hi(j, j);
      float tr = 0.f, ti = 0.f, beta = ar, sr = 0.f, si = 0.f;
      if (xn > 0.f || ai != 0.f) {
        beta = -copysignf(sqrtf(ar * ar + ai * ai + xn), ar);
        tr = (beta - ar) / beta;
        ti = -ai / beta;
        const float dr = ar - beta, di = ai, den = dr * dr + di * di;
        sr = dr / den;
        si = -di / den;
      }
      warp_sync();
      if (tr != 0.f || ti != 0.f)
        for (int i = j + 1 + lane; i < m; i += nl) {
          const float xr = hr(i, j), xi = hi(i, j);
          hr(i, j) = xr * sr - xi * si;
          hi(i, j) = xr * si + xi * sr;
        }
      if (lane == 0) {
        hr(j, j) = beta;
        hi(j, j) = 0.f;
        tau[2 * j] = tr;
        tau[2 * j + 1] = ti;
      }
    }
    __syncthreads();
    const float tr = tau[2 * j], ti = tau[2 * j + 1];
    if (tr != 0.f || ti != 0.f) {
      // columns c > j: w = v^H H[:, c];  H[:, c] -= conj(tau) v w
      for (int c = j + 1 + warp; c < k; c += nwarps) {
        float wr = 0.f, wi = 0.f;
        for (int i = j + 1 + lane; i < m; i += nl) {
          const float vr = hr(i, j), vi = -hi(i, j), xr = hr(i, c), xi = hi(i, c);
          wr = fmaf(vr, xr, fmaf(-vi, xi, wr));
          wi = fmaf(vr, xi, fmaf(vi, xr, wi));
        }
        wr = warp_sum_f(wr) + hr(j, c);
        wi = warp_sum_f(wi) + hi(j, c);
        const float fr = tr * wr + ti * wi, fi = tr * wi - ti * wr;  // conj(tau) w
        warp_sync();
        if (lane == 0) {
          hr(j, c) -= fr;
          hi(j, c) -= fi;
        }
        for (int i = j + 1 + lane; i < m; i += nl) {
          const float vr = hr(i, j), vi = hi(i, j);
          hr(i, c) -= vr * fr - vi * fi;
          hi(i, c) -= vr * fi + vi * fr;
        }
      }
    }
    __syncthreads();
  }
  // Q = H_0 ... H_{k-1} [I_k; 0]: apply H_j (not its adjoint) for j descending
  for (int e = tid; e < m * k; e += nt) {
    const int i = e / k, c = e - i * k;
    const size_t q = 2 * ((size_t)i * qrs + (size_t)c * qcs);
    Q[q] = (i == c) ? 1.f : 0.f;
    Q[q + 1] = 0.f;
  }
  __syncthreads();
  for (int j = k - 1; j >= 0; --j) {
    const float tr = tau[2 * j], ti = tau[2 * j + 1];
    if (tr != 0.f || ti != 0.f) {
      for (int c = j + warp; c < k; c += nwarps) {
        float wr = 0.f, wi = 0.f;
        for (int i = j + 1 + lane; i < m; i += nl) {
          const size_t q = 2 * ((size_t)i * qrs + (size_t)c * qcs);
          const float vr = hr(i, j), vi = -hi(i, j);
          wr = fmaf(vr, Q[q], fmaf(-vi, Q[q + 1], wr));
          wi = fmaf(vr, Q[q + 1], fmaf(vi, Q[q], wi));
        }
        const size_t q0 = 2 * ((size_t)j * qrs + (size_t)c * qcs);
        wr = warp_sum_f(wr) + Q[q0];
        wi = warp_sum_f(wi) + Q[q0 + 1];
        const float fr = tr * wr - ti * wi, fi = tr * wi + ti * wr;  // tau w
        warp_sync();
        if (lane == 0) {
          Q[q0] -= fr;
          Q[q0 + 1] -= fi;
        }
        for (int i = j + 1 + lane; i < m; i += nl) {
          const size_t q = 2 * ((size_t)i * qrs + (size_t)c * qcs);
          const float vr = hr(i, j), vi = hi(i, j);
          Q[q] -= vr * fr - vi * fi;
          Q[q + 1] -= vr * fi + vi * fr;
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace vmc
