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
#ifndef VMC_GEMM_TENSOR_CORES
#define VMC_GEMM_TENSOR_CORES 0
#endif
// CTA GEMMs of at least 16 x 8 x 8 run on the tensor cores (3xTF32)
constexpr bool kGemmTensorCores = VMC_GEMM_TENSOR_CORES != 0;

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
  // complex elements: every index map and stride counts elements of two
  // floats (re, im); conja / conjb conjugate the operand, alpha_im is the
  // imaginary part of alpha
  int cplx;
  int conja, conjb;
  float alpha_im;
};

// Complex variant of gemm_tiles: interleaved (re, im) elements.
template <int TM, int TN>
__device__ __forceinline__ void gemm_tiles_c(const Gemm& g) {
  const int tiles_m = (g.M + TM - 1) / TM;
  const int tiles_n = (g.N + TN - 1) / TN;
  const int n_tiles = tiles_m * tiles_n;
  const float sa = g.conja ? -1.f : 1.f, sb = g.conjb ? -1.f : 1.f;
  for (int t = threadIdx.x; t < n_tiles; t += blockDim.x) {
    const int tn = t % tiles_n;
    const int tm = t / tiles_n;
    int aoff[TM], boff[TN];
    bool mv[TM], nv[TN];
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      int m = tm + i * tiles_m;
      mv[i] = m < g.M;
      aoff[i] = 2 * imap(g.am, mv[i] ? m : 0);
    }
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      int n = tn + j * tiles_n;
      nv[j] = n < g.N;
      boff[j] = 2 * imap(g.bn, nv[j] ? n : 0);
    }
    float cr[TM][TN], ci[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) cr[i][j] = ci[i][j] = 0.f;
    const int ska = 2 * g.sak, skb = 2 * g.sbk;
    for (int k = 0; k < g.K; ++k) {
      float ar[TM], ai[TM], br[TN], bi[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) {
        const float* pa = g.A + aoff[i] + k * ska;
        ar[i] = pa[0];
        ai[i] = sa * pa[1];
      }
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const float* pb = g.B + boff[j] + k * skb;
        br[j] = pb[0];
        bi[j] = sb * pb[1];
      }
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) {
          cr[i][j] = fmaf(ar[i], br[j], fmaf(-ai[i], bi[j], cr[i][j]));
          ci[i][j] = fmaf(ar[i], bi[j], fmaf(ai[i], br[j], ci[i][j]));
        }
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      if (!mv[i]) continue;
      const int co = imap(g.cm, tm + i * tiles_m);
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        if (!nv[j]) continue;
        float* dst = g.C + 2 * (co + imap(g.cn, tn + j * tiles_n));
        const float vr = g.alpha * cr[i][j] - g.alpha_im * ci[i][j];
        const float vi = g.alpha * ci[i][j] + g.alpha_im * cr[i][j];
        if (g.accumulate) {
          dst[0] += vr;
          dst[1] += vi;
        } else {
          dst[0] = vr;
          dst[1] = vi;
        }
      }
    }
  }
}

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

#ifndef VMC_HOST_EMULATION
// ---------------------------------------------------------------------------
// Tensor-core path: warp-level mma.sync m16n8k8 with TF32 operands and FP32
// accumulation.  Each operand is split x = hi + lo (hi = x rounded to TF32,
// lo = the TF32 rounding of the remainder) and hi*hi + hi*lo + lo*hi is
// accumulated, which keeps products to about 2^-22 relative: FP32 accuracy
// for these contractions.  Operands are read in place through the index maps,
// with rows, columns and k beyond the matrix read as zero.
// Fragment layout (PTX ISA, m16n8k8 .tf32): lane = 4*g + t;
//   A: a0 (g, t), a1 (g+8, t), a2 (g, t+4), a3 (g+8, t+4)
//   B: b0 (k=t, n=g), b1 (k=t+4, n=g)
//   D: d0 (g, 2t), d1 (g, 2t+1), d2 (g+8, 2t), d3 (g+8, 2t+1)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t tf32_bits(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_m16n8k8_tf32(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  hi = tf32_bits(x);
  lo = tf32_bits(x - __uint_as_float(hi));
}

__device__ inline void gemm_mma(const Gemm& g) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int gr = lane >> 2, tg = lane & 3;
  const int tiles_m = (g.M + 15) >> 4, tiles_n = (g.N + 7) >> 3;
  for (int t = warp; t < tiles_m * tiles_n; t += nwarps) {
    const int m0 = (t / tiles_n) << 4, n0 = (t % tiles_n) << 3;
    const int r0 = m0 + gr, r1 = r0 + 8, c0 = n0 + gr;
    const bool v0 = r0 < g.M, v1 = r1 < g.M, vc = c0 < g.N;
    const float* a0p = g.A + imap(g.am, v0 ? r0 : 0);
    const float* a1p = g.A + imap(g.am, v1 ? r1 : 0);
    const float* bp = g.B + imap(g.bn, vc ? c0 : 0);
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    for (int k0 = 0; k0 < g.K; k0 += 8) {
      const int ka = k0 + tg, kb = ka + 4;
      const bool ka_ok = ka < g.K, kb_ok = kb < g.K;
      const float x0 = (v0 && ka_ok) ? a0p[(size_t)ka * g.sak] : 0.f;
      const float x1 = (v1 && ka_ok) ? a1p[(size_t)ka * g.sak] : 0.f;
      const float x2 = (v0 && kb_ok) ? a0p[(size_t)kb * g.sak] : 0.f;
      const float x3 = (v1 && kb_ok) ? a1p[(size_t)kb * g.sak] : 0.f;
      const float y0 = (vc && ka_ok) ? bp[(size_t)ka * g.sbk] : 0.f;
      const float y1 = (vc && kb_ok) ? bp[(size_t)kb * g.sbk] : 0.f;
      uint32_t ah[4], al[4], bh[2], bl[2];
      split_tf32(x0, ah[0], al[0]);
      split_tf32(x1, ah[1], al[1]);
      split_tf32(x2, ah[2], al[2]);
      split_tf32(x3, ah[3], al[3]);
      split_tf32(y0, bh[0], bl[0]);
      split_tf32(y1, bh[1], bl[1]);
      mma_m16n8k8_tf32(d, al, bh);
      mma_m16n8k8_tf32(d, ah, bl);
      mma_m16n8k8_tf32(d, ah, bh);
    }
    const int cc0 = n0 + 2 * tg, cc1 = cc0 + 1;
    const bool w00 = v0 && cc0 < g.N, w01 = v0 && cc1 < g.N, w10 = v1 && cc0 < g.N, w11 = v1 && cc1 < g.N;
    const int o0 = w00 || w01 ? imap(g.cm, r0) : 0, o1 = w10 || w11 ? imap(g.cm, r1) : 0;
    const int q0 = cc0 < g.N ? imap(g.cn, cc0) : 0, q1 = cc1 < g.N ? imap(g.cn, cc1) : 0;
    if (w00) { float* p = g.C + o0 + q0; const float v = g.alpha * d[0]; *p = g.accumulate ? (*p + v) : v; }
    if (w01) { float* p = g.C + o0 + q1; const float v = g.alpha * d[1]; *p = g.accumulate ? (*p + v) : v; }
    if (w10) { float* p = g.C + o1 + q0; const float v = g.alpha * d[2]; *p = g.accumulate ? (*p + v) : v; }
    if (w11) { float* p = g.C + o1 + q1; const float v = g.alpha * d[3]; *p = g.accumulate ? (*p + v) : v; }
  }
}
#endif

#ifndef VMC_GEMM_TCGEN05
#define VMC_GEMM_TCGEN05 0
#endif
// CTA GEMMs large enough for a 128-row tensor-core tile run on tcgen05 (tile policy 4)
constexpr bool kGemmTcgen05 = VMC_GEMM_TCGEN05 != 0;
// shared-memory staging of one K chunk of a tcgen05 GEMM: A (128 x 32) and B (128 x 32), TF32 hi and lo
constexpr int kTcRows = 128, kTcK = 32;
constexpr long long kTcStageBytes = 4LL * kTcRows * kTcK * 4;  // 64 KB
constexpr int kTcTmemCols = 128;

#if VMC_GEMM_TCGEN05 && !defined(VMC_HOST_EMULATION)
// ---------------------------------------------------------------------------
// tcgen05 path (sm_100 family): C = alpha * A B on the 5th-generation tensor cores with the accumulator
// in tensor memory.  Per 128-row x (<= 128)-column tile of C and 32-deep K chunk, the CTA stages A and B
// from their index maps into shared memory in the no-swizzle K-major canonical layout (8-row x 16-byte
// core matrices; LBO = byte stride between core matrices along K, SBO = 128 between 8-row groups), split
// into TF32 hi and lo parts; one thread issues hi*hi + hi*lo + lo*hi (12 kind::tf32 MMAs of K = 8),
// commits them to an mbarrier and the CTA waits (bounded: a timeout sets VMC_DEV_TIMEOUT in the status
// word and the GEMM carries on with whatever the accumulator holds).  The products keep ~2^-22 relative
// accuracy, FP32 level.  Warps read the accumulator back with tcgen05.ld (warp w: TMEM lanes
// 32 (w % 4) .. +31 = tile rows; warp groups split the columns) and write C through its index maps.
// ---------------------------------------------------------------------------
VMC_SHARED uint32_t g_tc_tmem;          // TMEM base address (column 0, lane 0) of this CTA
VMC_SHARED __align__(8) uint64_t g_tc_mbar;
VMC_SHARED uint32_t g_tc_phase;         // parity of the mbarrier phase the next commit completes
VMC_SHARED int32_t* g_tc_status;        // the launch's status word

__device__ __forceinline__ uint32_t smem_addr_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Kernel start, all threads: TMEM columns for the accumulator (warp 0), the mbarrier (thread 0).
__device__ inline void tc_setup(int32_t* status) {
  if ((threadIdx.x >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr_u32(&g_tc_tmem)),
                 "r"((uint32_t)kTcTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr_u32(&g_tc_mbar)));
    g_tc_phase = 0;
    g_tc_status = status;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
}

// Kernel end, all threads: return the TMEM columns (every MMA was waited for).
__device__ inline void tc_teardown() {
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if ((threadIdx.x >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(g_tc_tmem), "r"((uint32_t)kTcTmemCols));
}

// Stage rows [r0, r0 + 128) x k [k0, k0 + 32) of an operand (row offsets `rm`, k stride `sk`) as TF32 hi
// and lo in the canonical layout; rows >= nrows and k >= K are zero.
__device__ __forceinline__ void tc_stage(const float* X, const IMap& rm, int sk, int nrows, int K, int r0, int k0,
                                         unsigned char* hi, unsigned char* lo) {
  constexpr uint32_t lbo = (kTcRows / 8) * 128;
  for (int e = threadIdx.x; e < kTcRows * kTcK; e += blockDim.x) {
    const int r = e / kTcK, k = e % kTcK;
    const int gr = r0 + r, gk = k0 + k;
    float x = 0.f;
    if (gr < nrows && gk < K) x = X[imap(rm, gr) + (size_t)gk * sk];
    uint32_t h, l;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(x - __uint_as_float(h)));
    const uint32_t off = (k >> 2) * lbo + (r >> 3) * 128 + (r & 7) * 16 + (k & 3) * 4;
    *reinterpret_cast<uint32_t*>(hi + off) = h;
    *reinterpret_cast<uint32_t*>(lo + off) = l;
  }
}

// Bounded wait for the mbarrier phase the last commit completes; flips the CTA's phase.  Once any CTA of
// the launch has timed out, no further wait spins: the launch runs to its end and the host reads
// VMC_DEV_TIMEOUT from the status word.
__device__ __forceinline__ void tc_wait() {
  const uint32_t bar = smem_addr_u32(&g_tc_mbar), parity = g_tc_phase;
  uint32_t done = (*reinterpret_cast<volatile int32_t*>(g_tc_status) & 2) ? 1u : 0u;
  for (int it = 0; it < (1 << 22) && !done; ++it) {
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity));
  }
  if (!done && threadIdx.x == 0) atomicOr(g_tc_status, 2);  // VMC_DEV_TIMEOUT
  __syncthreads();
  if (threadIdx.x == 0) g_tc_phase = parity ^ 1u;
  asm volatile("tcgen05.fence::after_thread_sync;");
}

__device__ inline void gemm_tc5(const Gemm& g) {
  extern __shared__ __align__(16) float dyn_smem[];
  unsigned char* stage = reinterpret_cast<unsigned char*>(dyn_smem);
  unsigned char* a_hi = stage;
  unsigned char* a_lo = stage + kTcRows * kTcK * 4;
  unsigned char* b_hi = stage + 2 * kTcRows * kTcK * 4;
  unsigned char* b_lo = stage + 3 * kTcRows * kTcK * 4;
  constexpr uint32_t lbo = (kTcRows / 8) * 128;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const int quad = warp & 3, group = warp >> 2, ngroups = nwarps >= 8 ? 2 : 1;
  const uint32_t tmem = g_tc_tmem;
  for (int m0 = 0; m0 < g.M; m0 += kTcRows) {
    for (int n0 = 0; n0 < g.N; n0 += kTcTmemCols) {
      const int nt = min(kTcTmemCols, g.N - n0);
      const int ntp = (nt + 15) & ~15;  // MMA N: a multiple of 16 (zero rows of B beyond N)
      const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(ntp >> 3) << 17) |
                             ((uint32_t)(kTcRows >> 4) << 24);
      for (int k0 = 0; k0 < g.K; k0 += kTcK) {
        tc_stage(g.A, g.am, g.sak, g.M, g.K, m0, k0, a_hi, a_lo);
        // B as rows n (N x K, K-major): element (n, k) at B[bn(n) + k sbk]
        tc_stage(g.B, g.bn, g.sbk, g.N, g.K, n0, k0, b_hi, b_lo);
        asm volatile("fence.proxy.async.shared::cta;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        if (threadIdx.x == 0) {
          asm volatile("tcgen05.fence::after_thread_sync;");
          const int ksteps = min(kTcK, g.K - k0 + 7) / 8;
          for (int s = 0; s < ksteps; ++s) {
            const uint32_t ao = s * 2 * lbo;
            const uint64_t dah = tc_smem_desc(smem_addr_u32(a_hi) + ao, lbo, 128);
            const uint64_t dal = tc_smem_desc(smem_addr_u32(a_lo) + ao, lbo, 128);
            const uint64_t dbh = tc_smem_desc(smem_addr_u32(b_hi) + ao, lbo, 128);
            const uint64_t dbl = tc_smem_desc(smem_addr_u32(b_lo) + ao, lbo, 128);
            const uint32_t first = (k0 == 0 && s == 0) ? 0u : 1u;
            asm volatile(
                "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                "l"(dal), "l"(dbh), "r"(idesc), "r"(first));
            asm volatile("tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, 1;" ::"r"(tmem), "l"(dah), "l"(dbl),
                         "r"(idesc));
            asm volatile("tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, 1;" ::"r"(tmem), "l"(dah), "l"(dbh),
                         "r"(idesc));
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_addr_u32(&g_tc_mbar)));
        }
        tc_wait();  // the staging buffers are rewritten by the next chunk
      }
      // accumulator -> C: warp quad q holds rows 32 q .. +31 of the tile; column groups split by warp group
      if (warp < 4 * ngroups) {
        const int row = m0 + quad * 32 + lane;
        const int cols_per = ((ntp / ngroups) + 7) & ~7;
        const int c_begin = group * cols_per, c_end = min(ntp, c_begin + cols_per);
        const int co = row < g.M ? imap(g.cm, row) : 0;
        for (int c0 = c_begin; c0 < c_end; c0 += 8) {
          uint32_t v[8];
          const uint32_t addr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0;
          asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                       : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                         "=r"(v[7])
                       : "r"(addr));
          asm volatile("tcgen05.wait::ld.sync.aligned;");
          if (row < g.M) {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const int n = n0 + c0 + j;
              if (c0 + j < nt) {
                float* dst = g.C + co + imap(g.cn, n);
                const float val = g.alpha * __uint_as_float(v[j]);
                *dst = g.accumulate ? (*dst + val) : val;
              }
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncthreads();  // the next tile's MMAs overwrite the accumulator
      asm volatile("tcgen05.fence::after_thread_sync;");
    }
  }
}
#endif

// CTA-wide GEMM; ends with a barrier so C is visible to the whole CTA.
// Register-tile policy of the CTA's GEMMs, set per chain from its plan (an
// autotuned choice per (D, chi)): 0 the default thresholds below; 1 smaller
// tiles (more threads busy on small products); 2 larger tiles (fewer loads
// per multiply-add on large ones).
VMC_SHARED int g_tile_policy;

// VMC_GEMM_NOINLINE=1 compiles one out-of-line copy of the GEMM instead of one
// per call site (smaller code, one call per GEMM).
#if defined(VMC_GEMM_NOINLINE) && VMC_GEMM_NOINLINE
#define VMC_GEMM_LINKAGE static __device__ __noinline__
#else
#define VMC_GEMM_LINKAGE __device__ inline
#endif

VMC_GEMM_LINKAGE void cta_gemm(const Gemm& g) {
  const int work = g.M * g.N;
  const int pol = g_tile_policy;
  const int nt = pol == 1 ? 2 * blockDim.x : pol == 2 ? blockDim.x / 2 : blockDim.x;
  if (g.cplx) {
    if (g.M >= 4 && g.N >= 2 && work >= nt * 8) {
      gemm_tiles_c<4, 2>(g);
    } else if (g.M >= 2 && g.N >= 2 && work >= nt * 4) {
      gemm_tiles_c<2, 2>(g);
    } else {
      gemm_tiles_c<1, 1>(g);
    }
    __syncthreads();
    return;
  }
#if VMC_GEMM_TCGEN05 && !defined(VMC_HOST_EMULATION)
  if (g.M >= 64 && g.N >= 16 && g.K >= 16 && (long long)g.M * g.N * g.K >= (1LL << 17)) {
    gemm_tc5(g);
    __syncthreads();
    return;
  }
#endif
#ifndef VMC_HOST_EMULATION
  if (kGemmTensorCores && g.M >= 16 && g.N >= 8 && g.K >= 8 && work >= nt * 32) {
    gemm_mma(g);
    __syncthreads();
    return;
  }
#endif
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
  g.cplx = 0; g.conja = 0; g.conjb = 0; g.alpha_im = 0.f;
  return g;
}

// ---------------------------------------------------------------------------
// FP64-accumulating CTA GEMM for the boundary-MPS chain of mixed-precision
// plans: A is FP64, B is FP64 or FP32 (the site tensors), C is FP64.  Same
// index maps and thread-tile interleaving as the FP32 GEMM above.
// ---------------------------------------------------------------------------
template <typename TA, typename TB>
struct GemmX {
  const TA* A;
  const TB* B;
  double* C;
  int M, N, K;
  IMap am;
  int sak;
  IMap bn;
  int sbk;
  IMap cm, cn;
  double alpha;
  int accumulate;
};

template <typename TA, typename TB>
__device__ inline GemmX<TA, TB> make_gemm_x(const TA* A, IMap am, int sak, const TB* B, IMap bn, int sbk,
                                             double* C, IMap cm, IMap cn, int M, int N, int K, double alpha = 1.0,
                                             int accumulate = 0) {
  GemmX<TA, TB> g;
  g.A = A; g.B = B; g.C = C; g.M = M; g.N = N; g.K = K;
  g.am = am; g.sak = sak; g.bn = bn; g.sbk = sbk; g.cm = cm; g.cn = cn;
  g.alpha = alpha; g.accumulate = accumulate;
  return g;
}

template <typename TA, typename TB, int TM, int TN>
__device__ __forceinline__ void gemm_tiles_x(const GemmX<TA, TB>& g) {
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
    double acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = 0.0;
    for (int k = 0; k < g.K; ++k) {
      double a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = (double)g.A[aoff[i] + k * g.sak];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = (double)g.B[boff[j] + k * g.sbk];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      if (!mv[i]) continue;
      const int co = imap(g.cm, tm + i * tiles_m);
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        if (!nv[j]) continue;
        double* dst = g.C + co + imap(g.cn, tn + j * tiles_n);
        const double v = g.alpha * acc[i][j];
        *dst = g.accumulate ? (*dst + v) : v;
      }
    }
  }
}

// CTA-wide FP64 GEMM; ends with a barrier.
template <typename TA, typename TB>
__device__ inline void cta_gemm_x(const GemmX<TA, TB>& g) {
  const int work = g.M * g.N;
  const int nt = blockDim.x;
  if (g.M >= 4 && g.N >= 4 && work >= nt * 16) {
    gemm_tiles_x<TA, TB, 4, 4>(g);
  } else if (g.M >= 2 && g.N >= 2 && work >= nt * 4) {
    gemm_tiles_x<TA, TB, 2, 2>(g);
  } else {
    gemm_tiles_x<TA, TB, 1, 1>(g);
  }
  __syncthreads();
}

// S (k x k) = Y^T Y for the n x k matrix Y (row stride ldy), in Y's precision.
__device__ inline void cta_gram_t(float* Y, int n, int k, int ldy, float* S) {
  cta_gemm(make_gemm(Y, lin(1), ldy, Y, lin(1), ldy, S, lin(k), lin(1), k, k, n));
}
__device__ inline void cta_gram_t(double* Y, int n, int k, int ldy, double* S) {
  cta_gemm_x(make_gemm_x(static_cast<const double*>(Y), lin(1), ldy, static_cast<const double*>(Y), lin(1), ldy, S,
                         lin(k), lin(1), k, k, n));
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

// dot(x, y) over n contiguous floats: FP32 partial sums per thread (two
// chains), combined across the CTA in double.  FP64 arithmetic runs at a
// small fraction of the FP32 rate on this part, so it is kept out of the loop.
__device__ inline double cta_dot(const float* x, const float* y, int n, double* red) {
  float s0 = 0.f, s1 = 0.f;
  int i = threadIdx.x;
  const int st = blockDim.x;
  for (; i + st < n; i += 2 * st) {
    s0 = fmaf(x[i], y[i], s0);
    s1 = fmaf(x[i + st], y[i + st], s1);
  }
  if (i < n) s0 = fmaf(x[i], y[i], s0);
  return cta_sum((double)s0 + (double)s1, red);
}

// acc[p*d+q] += <x[p], y[q]> over n floats for all p, q < d.  For d = 2 the
// four products share one pass and one CTA reduction (register accumulators,
// FP32 per thread, double across threads); other d fall back to one cta_dot
// per pair.
__device__ inline void cta_dots_all(const float* const* x, const float* const* y, int d, int n, double* acc,
                                    double* red) {
  const int nw = (blockDim.x + 31) >> 5;
  if (d != 2 || 4 * nw > 32) {
    for (int p = 0; p < d; ++p)
      for (int q = 0; q < d; ++q) acc[p * d + q] += cta_dot(x[p], y[q], n, red);
    return;
  }
  const float* x0 = x[0];
  const float* x1 = x[1];
  const float* y0 = y[0];
  const float* y1 = y[1];
  float f00 = 0.f, f01 = 0.f, f10 = 0.f, f11 = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float a = x0[i], b = x1[i], u = y0[i], v = y1[i];
    f00 = fmaf(a, u, f00);
    f01 = fmaf(a, v, f01);
    f10 = fmaf(b, u, f10);
    f11 = fmaf(b, v, f11);
  }
  double s[4] = {(double)f00, (double)f01, (double)f10, (double)f11};
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < 4; ++j) s[j] = warp_sum(s[j]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < 4; ++j) red[j * nw + wid] = s[j];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    double r = 0.0;
    for (int w = 0; w < nw; ++w) r += red[j * nw + w];
    acc[j] += r;
  }
  __syncthreads();
}

// Bilinear complex dot sum_i x_i y_i over n interleaved (re, im) elements;
// returns the real part, *im the imaginary part.  FP32 partials per thread,
// double across the CTA.
__device__ inline double cta_cdot(const float* x, const float* y, int n, double* red, double* im) {
  float sr = 0.f, si = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float xr = x[2 * i], xi = x[2 * i + 1], yr = y[2 * i], yi = y[2 * i + 1];
    sr = fmaf(xr, yr, fmaf(-xi, yi, sr));
    si = fmaf(xr, yi, fmaf(xi, yr, si));
  }
  const double re = cta_sum((double)sr, red);
  *im = cta_sum((double)si, red);
  return re;
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

// Rescale x[0..n) in place by the power of two that brings max|x| into
// [0.5, 1); returns the log of the factor taken out (0 for a zero or
// non-finite vector).  Power-of-two scaling is exact, so the returned log
// matches the applied scale bit for bit.  Environments shrink by the
// contraction at every column and would otherwise leave the FP32 range across
// a wide lattice.
__device__ inline double cta_normalize(float* x, int n, double* red) {
  float m = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, fabsf(x[i]));
#ifndef VMC_HOST_EMULATION
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
#endif
  float* fred = reinterpret_cast<float*>(red);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) fred[wid] = m;
  __syncthreads();
  m = 0.f;
  for (int w = 0; w < nw; ++w) m = fmaxf(m, fred[w]);
  __syncthreads();
  if (!(m > 0.f) || !isfinite(m)) return 0.0;
  int e = 0;
  frexpf(m, &e);  // m = f * 2^e, f in [0.5, 1)
  e = e < -120 ? -120 : (e > 120 ? 120 : e);  // keep 2^-e a normal float
  if (e == 0) return 0.0;
  const float sc = ldexpf(1.f, -e);
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] *= sc;
  __syncthreads();
  return (double)e * 0.69314718055994530942;
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
