// sliced_gram.cu -- the sample-space Gram matrix of a sliced Jacobian, the FP64
// matrix the SampleSpace SR solve factorises (qgt.py:173-223 builds it from the
// expanded blocks, sum_k (O o [p == k]) (O o [p == k])^H; jacobian.py:56-93).
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

}  // extern "C"
