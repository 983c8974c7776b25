// device_common.cuh -- CTA-cooperative building blocks of the PEPS engine.
//
// Every tensor contraction of the boundary-MPS algorithm is lowered to one
// CTA-wide strided GEMM  C[m,n] (+)= sum_k A[m,k] B[k,n]  whose row / column
// offsets go through up-to-3-level index maps.  A producer writes its output
// directly in the layout its consumer reads with a unit (or uniform) K
// stride, so no separate transposes are needed.
#pragma once

#include <cstdint>

#include "portability.cuh"

namespace vmc {

#if defined(VMC_HOST_EMULATION) && defined(VMC_PHASE_TIMERS)
inline unsigned long long jacobi_sweep_hist[32];
#endif

// offset(i) with i = (i1 * n2 + i2) * n3 + i3  ->  i1*s1 + i2*s2 + i3*s3
struct IMap {
  int n2, n3, s1, s2, s3;
};

__host__ __device__ inline IMap lin(int s) { return IMap{1, 1, s, 0, 0}; }
__host__ __device__ inline IMap two(int n2, int s1, int s2) { return IMap{n2, 1, s1, s2, 0}; }
__host__ __device__ inline IMap three(int n2, int n3, int s1, int s2, int s3) {
  return IMap{n2, n3, s1, s2, s3};
}

__device__ __forceinline__ int imap(const IMap& m, int i) {
  if (m.n2 == 1 && m.n3 == 1) return i * m.s1;
  int i3 = i % m.n3;
  int t = i / m.n3;
  int i2 = t % m.n2;
  int i1 = t / m.n2;
  return i1 * m.s1 + i2 * m.s2 + i3 * m.s3;
}

struct Gemm {
  const float* A;
  const float* B;
  float* C;
  int M, N, K;
  IMap am;   // row offsets of A
  int sak;   // k stride of A
  IMap bn;   // column offsets of B
  int sbk;   // k stride of B
  IMap cm, cn;
  float alpha;
  int accumulate;  // 1: C += alpha*AB, 0: C = alpha*AB
};

// Each thread owns a TM x TN tile whose rows and columns are interleaved
// with stride tiles_m / tiles_n, so consecutive lanes touch consecutive rows
// and columns: unit-stride operands are read without shared-memory bank
// conflicts and with coalesced global loads.
template <int TM, int TN>
__device__ __forceinline__ void gemm_tiles(const Gemm& g) {
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
      int m = tm + i * tiles_m;
      mv[i] = m < g.M;
      aoff[i] = imap(g.am, mv[i] ? m : 0);
    }
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      int n = tn + j * tiles_n;
      nv[j] = n < g.N;
      boff[j] = imap(g.bn, nv[j] ? n : 0);
    }
    float acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = 0.f;
    for (int k = 0; k < g.K; ++k) {
      float a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = g.A[aoff[i] + k * g.sak];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = g.B[boff[j] + k * g.sbk];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      if (!mv[i]) continue;
      const int co = imap(g.cm, tm + i * tiles_m);
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        if (!nv[j]) continue;
        float* dst = g.C + co + imap(g.cn, tn + j * tiles_n);
        float v = g.alpha * acc[i][j];
        *dst = g.accumulate ? (*dst + v) : v;
      }
    }
  }
}

// CTA-wide GEMM; ends with a barrier so C is visible to the whole CTA.
__device__ inline void cta_gemm(const Gemm& g) {
  const int work = g.M * g.N;
  const int nt = blockDim.x;
  if (g.M >= 4 && g.N >= 4 && work >= nt * 16) {
    gemm_tiles<4, 4>(g);
  } else if (g.M >= 2 && g.N >= 2 && work >= nt * 4) {
    gemm_tiles<2, 2>(g);
  } else {
    gemm_tiles<1, 1>(g);
  }
  __syncthreads();
}

__device__ inline Gemm make_gemm(const float* A, IMap am, int sak, const float* B, IMap bn, int sbk,
                                 float* C, IMap cm, IMap cn, int M, int N, int K, float alpha = 1.f,
                                 int accumulate = 0) {
  Gemm g;
  g.A = A; g.B = B; g.C = C; g.M = M; g.N = N; g.K = K;
  g.am = am; g.sak = sak; g.bn = bn; g.sbk = sbk; g.cm = cm; g.cn = cn;
  g.alpha = alpha; g.accumulate = accumulate;
  return g;
}

// ---------------------------------------------------------------------------
// Reductions (result broadcast to all threads).  `red` is >= 32 doubles of
// shared scratch.
// ---------------------------------------------------------------------------
__device__ inline double warp_sum(double v) {
#ifndef VMC_HOST_EMULATION
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
#endif
  return v;
}

__device__ inline double cta_sum(double v, double* red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < nw; ++w) r += red[w];
  __syncthreads();
  return r;
}

// dot(x, y) over n contiguous floats, accumulated in double.
__device__ inline double cta_dot(const float* x, const float* y, int n, double* red) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += (double)x[i] * (double)y[i];
  return cta_sum(s, red);
}

// acc[p*d+q] += <x[p], y[q]> over n floats for all p, q < d, in one pass: each
// thread keeps d*d partial sums, then one CTA reduction (one at a time when
// d*d*warps exceeds the 32 doubles of `red`).
__device__ inline void cta_dots_all(const float* const* x, const float* const* y, int d, int n, double* acc,
                                    double* red) {
  constexpr int kMax = 16;
  double s[kMax];
  const int dd = d * d;
  for (int j = 0; j < dd; ++j) s[j] = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    for (int p = 0; p < d; ++p) {
      const double xp = (double)x[p][i];
      for (int q = 0; q < d; ++q) s[p * d + q] += xp * (double)y[q][i];
    }
  }
  const int nw = (blockDim.x + 31) >> 5;
  if (dd * nw > 32) {
    for (int j = 0; j < dd; ++j) acc[j] += cta_sum(s[j], red);
    return;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j = 0; j < dd; ++j) s[j] = warp_sum(s[j]);
  __syncthreads();
  if (lane == 0)
    for (int j = 0; j < dd; ++j) red[j * nw + wid] = s[j];
  __syncthreads();
  for (int j = 0; j < dd; ++j) {
    double r = 0.0;
    for (int w = 0; w < nw; ++w) r += red[j * nw + w];
    acc[j] += r;
  }
  __syncthreads();
}

__device__ inline void cta_copy(float* dst, const float* src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
  __syncthreads();
}

__device__ inline void cta_fill(float* dst, float v, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = v;
  __syncthreads();
}

__device__ inline void cta_scale(float* dst, float s, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] *= s;
  __syncthreads();
}

// Frobenius-normalise x[0..n) in place; returns the log of the norm taken out
// (0 for a zero vector).  Environments shrink by the contraction at every
// column and would otherwise leave the FP32 range across a wide lattice.
__device__ inline double cta_normalize(float* x, int n, double* red) {
  const double nrm = sqrt(cta_dot(x, x, n, red));
  if (nrm > 0.0) {
    cta_scale(x, (float)(1.0 / nrm), n);
    return log(nrm);
  }
  return 0.0;
}

// ---------------------------------------------------------------------------
// Parallel one-sided (Hestenes) Jacobi: mutually orthogonalise `nv` vectors of
// length `len` stored at V + j*ldv (contiguous elements).  Rotations use the
// circle-method round-robin ordering, so each round's pairs are disjoint and
// processed concurrently by groups of G threads.  If Q != nullptr, the same
// rotations are applied to the `nv` vectors of length `qlen` at Q + j*ldq.
// Stops after a sweep in which every pair satisfied
// |a_p.a_q| <= tol * |a_p| |a_q|, or after max_sweeps sweeps.
// `sflag` is one int of shared scratch.
// ---------------------------------------------------------------------------
__device__ inline void jacobi_orthogonalize(float* V, int nv, int len, int ldv, float* Q, int qlen,
                                            int ldq, float tol, int max_sweeps, int* sflag) {
  if (nv < 2) return;
  const int P = nv + (nv & 1);
  const int npairs = P / 2;
  int G = blockDim.x / npairs;
  if (G > 32) G = 32;
  int gp = 1;
  while (gp * 2 <= G) gp *= 2;
  G = gp < 1 ? 1 : gp;
  const int ngroups = blockDim.x / G;
  const int grp = threadIdx.x / G;
  const int lig = threadIdx.x % G;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));

  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    if (threadIdx.x == 0) *sflag = 0;
    __syncthreads();
    for (int r = 0; r < P - 1; ++r) {
      for (int pi = grp; pi < npairs; pi += ngroups) {
        int p, q;
        if (pi == 0) {
          p = P - 1;
          q = r;
        } else {
          p = (r + pi) % (P - 1);
          q = (r - pi + (P - 1)) % (P - 1);
        }
        const bool active = (p < nv) && (q < nv);
        // every lane of the group takes the same branch (p, q depend on pi only)
        if (active) {
          float* vp = V + (size_t)p * ldv;
          float* vq = V + (size_t)q * ldv;
          float al = 0.f, be = 0.f, ga = 0.f;
          for (int i = lig; i < len; i += G) {
            const float x = vp[i], y = vq[i];
            al = fmaf(x, x, al);
            be = fmaf(y, y, be);
            ga = fmaf(x, y, ga);
          }
          for (int o = G / 2; o > 0; o >>= 1) {
            al += __shfl_xor_sync(gmask, al, o, G);
            be += __shfl_xor_sync(gmask, be, o, G);
            ga += __shfl_xor_sync(gmask, ga, o, G);
          }
          const float denom = sqrtf(al) * sqrtf(be);
          if (denom > 0.f && fabsf(ga) > tol * denom) {
            if (lig == 0) atomicOr(sflag, 1);
            const float zeta = (be - al) / (2.f * ga);
            const float t = copysignf(1.f, zeta) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
            const float c = 1.f / sqrtf(1.f + t * t);
            const float s = c * t;
            for (int i = lig; i < len; i += G) {
              const float x = vp[i], y = vq[i];
              vp[i] = c * x - s * y;
              vq[i] = s * x + c * y;
            }
            if (Q != nullptr) {
              float* qp = Q + (size_t)p * ldq;
              float* qq = Q + (size_t)q * ldq;
              for (int i = lig; i < qlen; i += G) {
                const float x = qp[i], y = qq[i];
                qp[i] = c * x - s * y;
                qq[i] = s * x + c * y;
              }
            }
          }
        }
      }
      __syncthreads();
    }
    const int any = *sflag;
    __syncthreads();
#if defined(VMC_HOST_EMULATION) && defined(VMC_PHASE_TIMERS)
    jacobi_sweep_hist[sweep < 31 ? sweep : 31] += !any;
    if (any && sweep == max_sweeps - 1) jacobi_sweep_hist[31]++;
#endif
    if (!any) break;
  }
}

}  // namespace vmc
