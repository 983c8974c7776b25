// sliced_gram.cu -- the Gram matrices of a sliced Jacobian in FP64: the
// sample-space T the SampleSpace SR solve factorises (qgt.py:173-223 builds it
// from the expanded blocks, sum_k (O o [p == k]) (O o [p == k])^H;
// jacobian.py:56-93), and the parameter-space O_exp^T O_exp of the
// ParameterSpace solve (second kernel below).
//
// For real FP32 log-derivatives o (n samples x ncols sliced columns) and the
// active slice p of every (sample, column):
//
//     T[i, j] = sum_c [p[i, c] == p[j, c]] o[i, c] o[j, c]
//
// which is the expanded product without its zero half (each expanded column is
// o masked to one slice, and the masks of two samples overlap exactly where
// their slices agree).  FP32 inputs make every product exact as the pair
// (p, e) = (o_i o_j rounded, fmaf(o_i, o_j, -p)); the pairs are summed in
// double-float on the FP32 units (Knuth's two-sum), renormalised every 32
// columns and flushed into FP64 accumulators every 256 columns, so the sum
// keeps ~2^-44 relative accuracy per flush block while issuing one FP64
// operation per 64 products: this GPU's FP64 rate is 1/64 of its FP32 rate.
//
// One CTA of 256 threads owns a 64 x 64 tile of T and each thread a 4 x 4
// sub-tile; only tiles on or below the diagonal are computed and each is also
// written transposed.  32-column slabs of both row blocks (values and slice
// indices) are staged in shared memory, column-major, so a thread reads its
// four rows as one float4 / char4.
#include <cstdint>

#include "portability.cuh"
#include "../../include/vmc_gb300.h"

namespace vmc {
namespace gram {

constexpr int kTile = 64, kSlab = 32, kThreads = 256;
constexpr int kRenormSlabs = 1, kFlushSlabs = 8;
constexpr int kPad = 4;  // row pitch 68 floats: the transposed stores hit distinct banks

#ifndef VMC_HOST_EMULATION
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& t) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  t = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void tile_of(int b, int& I, int& J) {
  // b = I (I + 1) / 2 + J with 0 <= J <= I
  int i = (int)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
  while ((long long)(i + 1) * (i + 2) / 2 <= b) ++i;
  while ((long long)i * (i + 1) / 2 > b) --i;
  I = i;
  J = b - i * (i + 1) / 2;
}

__global__ void __launch_bounds__(kThreads) sliced_gram_kernel(const float* __restrict__ o,
                                                                const int8_t* __restrict__ p, int n, int ncols,
                                                                long long ld, double* __restrict__ out) {
  __shared__ __align__(16) float sa[kSlab][kTile + kPad];
  __shared__ __align__(16) float sb[kSlab][kTile + kPad];
  __shared__ __align__(16) int8_t qa[kSlab][kTile];
  __shared__ __align__(16) int8_t qb[kSlab][kTile];
  int I, J;
  tile_of(blockIdx.x, I, J);
  const int r0 = I * kTile, c0 = J * kTile;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  float hi[4][4], lo[4][4];
  double acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) hi[r][c] = lo[r][c] = 0.f, acc[r][c] = 0.0;
  const int n_slabs = (ncols + kSlab - 1) / kSlab;
  for (int s = 0; s < n_slabs; ++s) {
    const int k0 = s * kSlab;
    // stage: consecutive threads read consecutive columns of one row (coalesced), store transposed
    for (int e = tid; e < kTile * kSlab; e += kThreads) {
      const int r = e / kSlab, k = e % kSlab, gk = k0 + k;
      const int ga = r0 + r, gb = c0 + r;
      const bool ka = ga < n && gk < ncols, kb = gb < n && gk < ncols;
      sa[k][r] = ka ? o[(size_t)ga * ld + gk] : 0.f;
      qa[k][r] = ka ? p[(size_t)ga * ld + gk] : (int8_t)-1;
      sb[k][r] = kb ? o[(size_t)gb * ld + gk] : 0.f;
      qb[k][r] = kb ? p[(size_t)gb * ld + gk] : (int8_t)-2;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < kSlab; ++k) {
      const float4 a4 = *reinterpret_cast<const float4*>(&sa[k][ty * 4]);
      const float4 b4 = *reinterpret_cast<const float4*>(&sb[k][tx * 4]);
      const char4 pa4 = *reinterpret_cast<const char4*>(&qa[k][ty * 4]);
      const char4 pb4 = *reinterpret_cast<const char4*>(&qb[k][tx * 4]);
      const float a[4] = {a4.x, a4.y, a4.z, a4.w}, b[4] = {b4.x, b4.y, b4.z, b4.w};
      const int pa[4] = {pa4.x, pa4.y, pa4.z, pa4.w}, pb[4] = {pb4.x, pb4.y, pb4.z, pb4.w};
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const float x = pa[r] == pb[c] ? a[r] : 0.f;
          const float prod = __fmul_rn(x, b[c]);
          const float err = fmaf(x, b[c], -prod);
          float sum, t;
          two_sum(hi[r][c], prod, sum, t);
          hi[r][c] = sum;
          lo[r][c] = __fadd_rn(lo[r][c], __fadd_rn(t, err));
        }
    }
    __syncthreads();
    const bool flush = (s + 1) % kFlushSlabs == 0 || s + 1 == n_slabs;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if (flush) {
          acc[r][c] += (double)hi[r][c] + (double)lo[r][c];
          hi[r][c] = lo[r][c] = 0.f;
        } else if ((s + 1) % kRenormSlabs == 0) {
          const float sum = __fadd_rn(hi[r][c], lo[r][c]);
          lo[r][c] = __fsub_rn(lo[r][c], __fsub_rn(sum, hi[r][c]));
          hi[r][c] = sum;
        }
      }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int i = r0 + ty * 4 + r;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int j = c0 + tx * 4 + c;
      if (i < n && j < n) {
        out[(size_t)i * n + j] = acc[r][c];
        if (I != J) out[(size_t)j * n + i] = acc[r][c];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// ParameterSpace: S[(k, c), (k', c')] = sum_i [p_ic == k][p_ic' == k'] o_ic o_ic', the Gram matrix of
// the expanded Jacobian's columns in slice order (column k * ncols + c), for d == 2 slices.  Each
// sample's product o_ic o_ic' belongs to exactly one of the d^2 = 4 slice pairs, so a thread keeps four
// df64 accumulators per column pair and adds the exact product to the one its slice pair selects
// (selects, one two-sum).  32 x 32 column-pair tiles on and below the diagonal, 256 threads with 2 x 2
// pairs each, 32-sample slabs staged in shared memory; FP64 flushes every 256 samples.
// ---------------------------------------------------------------------------
constexpr int kPTile = 32;

__global__ void __launch_bounds__(kThreads) sliced_gram_params_kernel(const float* __restrict__ o,
                                                                       const int8_t* __restrict__ p, int n,
                                                                       int ncols, long long ld,
                                                                       double* __restrict__ out) {
  __shared__ __align__(16) float sa[kSlab][kPTile];
  __shared__ __align__(16) float sb[kSlab][kPTile];
  __shared__ __align__(16) int8_t qa[kSlab][kPTile];
  __shared__ __align__(16) int8_t qb[kSlab][kPTile];
  int I, J;
  tile_of(blockIdx.x, I, J);
  const int c0 = I * kPTile, d0 = J * kPTile;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  float hi[4][2][2], lo[4][2][2];
  double acc[4][2][2];
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int c = 0; c < 2; ++c) hi[q][r][c] = lo[q][r][c] = 0.f, acc[q][r][c] = 0.0;
  const int n_slabs = (n + kSlab - 1) / kSlab;
  for (int sl = 0; sl < n_slabs; ++sl) {
    const int i0 = sl * kSlab;
    // stage: 32 samples x 32 columns of each block, consecutive threads on consecutive columns
    for (int e = tid; e < kSlab * kPTile; e += kThreads) {
      const int ii = e / kPTile, cc = e % kPTile, gi = i0 + ii;
      const int ga = c0 + cc, gb = d0 + cc;
      const bool ka = gi < n && ga < ncols, kb = gi < n && gb < ncols;
      sa[ii][cc] = ka ? o[(size_t)gi * ld + ga] : 0.f;
      qa[ii][cc] = ka ? p[(size_t)gi * ld + ga] : (int8_t)0;
      sb[ii][cc] = kb ? o[(size_t)gi * ld + gb] : 0.f;
      qb[ii][cc] = kb ? p[(size_t)gi * ld + gb] : (int8_t)0;
    }
    __syncthreads();
#pragma unroll 4
    for (int ii = 0; ii < kSlab; ++ii) {
      const float2 a2 = *reinterpret_cast<const float2*>(&sa[ii][ty * 2]);
      const float2 b2 = *reinterpret_cast<const float2*>(&sb[ii][tx * 2]);
      const float a[2] = {a2.x, a2.y}, b[2] = {b2.x, b2.y};
      const int pa[2] = {qa[ii][ty * 2] & 1, qa[ii][ty * 2 + 1] & 1};
      const int pb[2] = {qb[ii][tx * 2] & 1, qb[ii][tx * 2 + 1] & 1};
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const float prod = __fmul_rn(a[r], b[c]);
          const float err = fmaf(a[r], b[c], -prod);
          const int q = 2 * pa[r] + pb[c];
          const float th = q == 0 ? hi[0][r][c] : q == 1 ? hi[1][r][c] : q == 2 ? hi[2][r][c] : hi[3][r][c];
          const float tl = q == 0 ? lo[0][r][c] : q == 1 ? lo[1][r][c] : q == 2 ? lo[2][r][c] : lo[3][r][c];
          float sum, t;
          two_sum(th, prod, sum, t);
          const float nl = __fadd_rn(tl, __fadd_rn(t, err));
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            hi[k][r][c] = q == k ? sum : hi[k][r][c];
            lo[k][r][c] = q == k ? nl : lo[k][r][c];
          }
        }
    }
    __syncthreads();
    const bool flush = (sl + 1) % kFlushSlabs == 0 || sl + 1 == n_slabs;
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          if (flush) {
            acc[q][r][c] += (double)hi[q][r][c] + (double)lo[q][r][c];
            hi[q][r][c] = lo[q][r][c] = 0.f;
          } else {
            const float sum = __fadd_rn(hi[q][r][c], lo[q][r][c]);
            lo[q][r][c] = __fsub_rn(lo[q][r][c], __fsub_rn(sum, hi[q][r][c]));
            hi[q][r][c] = sum;
          }
        }
  }
  const size_t W = 2 * (size_t)ncols;
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int cc = c0 + ty * 2 + r;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int dd = d0 + tx * 2 + c;
      if (cc < ncols && dd < ncols) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const size_t row = (size_t)(q >> 1) * ncols + cc, col = (size_t)(q & 1) * ncols + dd;
          out[row * W + col] = acc[q][r][c];
          if (I != J) out[col * W + row] = acc[q][r][c];
        }
      }
    }
  }
}
#endif

}  // namespace gram
}  // namespace vmc

extern "C" {

vmc_status vmc_sliced_gram(void* stream, const float* o, const int8_t* p, int n, int ncols, int64_t ld,
                           double* out) {
  if (n < 0 || ncols < 0 || ld < (ncols > 1 ? ncols : 1) || (n > 0 && (!o || !p || !out))) return VMC_ERR_INVALID;
  if (n == 0) return VMC_OK;
  using namespace vmc::gram;
#ifdef VMC_HOST_EMULATION
  // plain FP64 sums (the host build checks the interface and the index arithmetic)
  (void)stream;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = 0.0;
      for (int c = 0; c < ncols; ++c)
        if (p[(size_t)i * ld + c] == p[(size_t)j * ld + c]) s += (double)o[(size_t)i * ld + c] * o[(size_t)j * ld + c];
      out[(size_t)i * n + j] = out[(size_t)j * n + i] = s;
    }
  return VMC_OK;
#else
  const long long tiles = (n + kTile - 1) / kTile;
  const long long blocks = tiles * (tiles + 1) / 2;
  if (blocks > 0x7fffffffLL) return VMC_ERR_UNSUPPORTED;
  VMC_LAUNCH(sliced_gram_kernel, (unsigned)blocks, kThreads, 0, stream, o, p, n, ncols, (long long)ld, out);
  return vmc_last_error() == cudaSuccess ? VMC_OK : VMC_ERR_CUDA;
#endif
}

vmc_status vmc_sliced_gram_params(void* stream, const float* o, const int8_t* p, int n, int ncols, int64_t ld,
                                  int d, double* out) {
  if (n < 0 || ncols < 0 || ld < (ncols > 1 ? ncols : 1) || ((long long)n * ncols > 0 && (!o || !p)) ||
      (ncols > 0 && !out))
    return VMC_ERR_INVALID;
  if (d != 2) return VMC_ERR_UNSUPPORTED;
  if (ncols == 0) return VMC_OK;
  using namespace vmc::gram;
#ifdef VMC_HOST_EMULATION
  (void)stream;
  const size_t W = (size_t)d * ncols;
  for (size_t e = 0; e < W * W; ++e) out[e] = 0.0;
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < ncols; ++c) {
      const double a = o[(size_t)i * ld + c];
      const size_t row = (size_t)p[(size_t)i * ld + c] * ncols + c;
      for (int c2 = 0; c2 < ncols; ++c2)
        out[row * W + (size_t)p[(size_t)i * ld + c2] * ncols + c2] += a * o[(size_t)i * ld + c2];
    }
  return VMC_OK;
#else
  const long long tiles = (ncols + kPTile - 1) / kPTile;
  const long long blocks = tiles * (tiles + 1) / 2;
  if (blocks > 0x7fffffffLL) return VMC_ERR_UNSUPPORTED;
  if (n == 0) return vmc_memset(out, 0, (size_t)4 * ncols * ncols * sizeof(double), (cudaStream_t)stream) ==
                             cudaSuccess ? VMC_OK : VMC_ERR_CUDA;
  VMC_LAUNCH(sliced_gram_params_kernel, (unsigned)blocks, kThreads, 0, stream, o, p, n, ncols, (long long)ld, out);
  return vmc_last_error() == cudaSuccess ? VMC_OK : VMC_ERR_CUDA;
#endif
}

}  // extern "C"
