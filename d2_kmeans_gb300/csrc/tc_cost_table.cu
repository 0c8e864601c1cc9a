// Word-embedding cost table on the 5th-generation tensor cores (tcgen05).
//
// T[l][v][k] = |c_{l,k}|^2 + |v|^2 - 2 <c_{l,k}, v> needs the inner products
// G = Cs * Vocab^T  ((k*m) x V, contraction over d).  They are computed with
// tcgen05.mma kind::tf32 in the 3xTF32 scheme: every FP32 operand x is split
// into hi = tf32(x) and lo = tf32(x - hi), and G accumulates
// hi*hi + hi*lo + lo*hi in FP32 in tensor memory.  The dropped lo*lo term and
// the TF32 rounding of lo leave an error near 2^-22 of |c||v| per product,
// which keeps the |c|^2 + |v|^2 - 2 c.v cancellation at FP32 accuracy.
//
// One CTA = one warpgroup = one 128 x 256 output tile (M x N).  Per K block of
// 32 TF32 values, the warpgroup loads the A (128 x 32) and B (256 x 32) slices,
// splits them and stores hi / lo in the no-swizzle K-major core-matrix layout
// (8 rows x 16 bytes per core matrix, core matrices adjacent along K 128 bytes
// apart, 8-row groups 1024 bytes apart); one thread issues the 4 k-steps x 3
// MMAs and a tcgen05.commit that arrives on an mbarrier.  The epilogue reads
// the accumulator with tcgen05.ld (each warp its 32 lanes = 32 rows) and writes
// T, one coalesced 128-byte row segment per vocabulary column and warp.
#include <cstdint>

#include "d2g_internal.cuh"

namespace d2g {

namespace tc {

constexpr int TM = 128;   // rows of the tile (MMA M)
constexpr int TN = 256;   // columns of the tile (MMA N)
constexpr int TKB = 32;   // TF32 values per K block
constexpr int KC = TKB / 4;             // 16-byte chunks along K per block
constexpr int CORE = 32;                // floats per core matrix (8 rows x 4)
constexpr uint32_t kLBO = 128;          // bytes between core matrices along K
constexpr uint32_t kSBO = KC * 128;     // bytes between 8-row groups
constexpr int kTmemCols = 256;
constexpr size_t kSmemBytes = (size_t)(2 * TM + 2 * TN) * TKB * 4;  // A hi/lo, B hi/lo

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// tcgen05 shared-memory descriptor: start, leading (K) and stride (M/N) byte
// offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(const void *p) {
  const uint64_t a = (smem_addr(p) & 0x3FFFF) >> 4;
  return a | ((uint64_t)(kLBO >> 4) << 16) | ((uint64_t)(kSBO >> 4) << 32) | (1ull << 46);
}

// instruction descriptor: D = F32, A = B = TF32, both K-major, N = TN, M = TM
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TN >> 3) << 17) |
                            ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mbar_init1(uint64_t *b) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(b)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// bounded wait (about one second), then give up and report
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *b, uint32_t parity) {
  if (mbar_test(b, parity)) return true;
  const unsigned long long t0 = now_ns();
  for (;;) {
    for (int i = 0; i < 64; ++i)
      if (mbar_test(b, parity)) return true;
    if (now_ns() - t0 > 1000000000ull) return false;
  }
}

// Load rows [r0, r0+R) x K block [t0, t0+TKB) of a row-major FP32 matrix
// (nr x d), split into TF32 hi / lo and store both in the core-matrix layout.
// Out-of-range entries are zero.  128 threads.
__device__ __forceinline__ void stage_split(const float *__restrict__ a, int nr, int d, int r0,
                                            int t0, int R, bool vec, float *hi, float *lo) {
  const int tid = threadIdx.x;
  for (int q = tid; q < R * KC; q += 128) {
    // q -> (row & 7) fastest, then chunk, then row group
    const int r8 = q & 7, c = (q >> 3) % KC, g = (q >> 3) / KC;
    const int row = g * 8 + r8, r = r0 + row, t = t0 + c * 4;
    float x[4];
    if (vec) {
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r < nr && t < d) v = __ldg(reinterpret_cast<const float4 *>(a + (size_t)r * d + t));
      x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) x[j] = (r < nr && t + j < d) ? __ldg(a + (size_t)r * d + t + j) : 0.f;
    }
    float h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      h[j] = tf32_round(x[j]);
      l[j] = tf32_round(x[j] - h[j]);
    }
    const int o = (g * KC + c) * CORE + r8 * 4;
    *reinterpret_cast<float4 *>(hi + o) = make_float4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<float4 *>(lo + o) = make_float4(l[0], l[1], l[2], l[3]);
  }
}

}  // namespace tc

__global__ void __launch_bounds__(128, 1)
    cost_table_tc_kernel(const float *__restrict__ cs, int nrows, const float *__restrict__ vocab,
                         int V, int d, const float *__restrict__ cnorm,
                         const float *__restrict__ vnorm, int m, int MP, float *__restrict__ T,
                         int *__restrict__ err) {
  using namespace tc;
  extern __shared__ __align__(1024) float sm[];
  float *Ahi = sm, *Alo = Ahi + TM * TKB, *Bhi = Alo + TM * TKB, *Blo = Bhi + TN * TKB;
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r0 = blockIdx.y * TM, v0 = blockIdx.x * TN;

  if (warp == 0) {  // tensor-memory accumulator: 128 lanes x 256 FP32 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(&tmem_base)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init1(&mbar);
    fail = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  const int nkb = (d + TKB - 1) / TKB;
  const bool vec = (d & 3) == 0;
  for (int kb = 0; kb < nkb; ++kb) {
    const int t0 = kb * TKB;
    // Staging: lanes 8j..8j+7 of a warp take the 8 rows of one core matrix at
    // K chunk c+j, so each 8-lane phase stores 128 contiguous bytes and a warp
    // reads 64 contiguous bytes from each of 8 rows.
    stage_split(cs, nrows, d, r0, t0, TM, vec, Ahi, Alo);
    stage_split(vocab, V, d, v0, t0, TN, vec, Bhi, Blo);
    // generic-proxy stores must be visible to the tensor core's async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int s = 0; s < TKB / 8; ++s) {  // one MMA k-step = 8 TF32 = two 16-byte chunks
        const int off = s * 2 * CORE;
        const uint64_t ah = smem_desc(Ahi + off), al = smem_desc(Alo + off);
        const uint64_t bh = smem_desc(Bhi + off), bl = smem_desc(Blo + off);
        mma_tf32(tmem, ah, bh, (kb > 0 || s > 0) ? 1u : 0u);
        mma_tf32(tmem, ah, bl, 1u);
        mma_tf32(tmem, al, bh, 1u);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_addr(&mbar))
          : "memory");
    }
    // the MMAs have read the block once the commit arrives
    if (!tc::mbar_wait_bounded(&mbar, kb & 1)) fail = 1;
    __syncthreads();
    if (fail) break;
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  if (!fail) {
    // epilogue: warp w owns accumulator lanes (rows) 32w .. 32w+31
    const int row = r0 + warp * 32 + lane;
    const bool rok = row < nrows;
    const int l = rok ? row / m : 0, k = rok ? row - l * m : 0;
    const float cn = rok ? cnorm[row] : 0.f;
    for (int c0 = 0; c0 < TN; c0 += 16) {
      uint32_t g[16];
      const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(g[0]), "=r"(g[1]), "=r"(g[2]), "=r"(g[3]), "=r"(g[4]), "=r"(g[5]), "=r"(g[6]),
            "=r"(g[7]), "=r"(g[8]), "=r"(g[9]), "=r"(g[10]), "=r"(g[11]), "=r"(g[12]),
            "=r"(g[13]), "=r"(g[14]), "=r"(g[15])
          : "r"(ta));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int v = v0 + c0 + j;
        if (rok && v < V) {
          const float c = cn + __ldg(vnorm + v) - 2.f * __uint_as_float(g[j]);
          T[((size_t)l * V + v) * MP + k] = fmaxf(c, 0.f);
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(err, kErrTcTimeout);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols)
                 : "memory");
}

cudaError_t launch_cost_table_tc(const float *cs, int nrows, const float *vocab, int V, int d,
                                 const float *cnorm, const float *vnorm, int m, int MP, float *T,
                                 int *err, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  // per device; the first call for a device comes before any graph capture
  static bool configured[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 64) return cudaErrorInvalidDevice;
  if (!configured[dev]) {
    e = cudaFuncSetAttribute(cost_table_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tc::kSmemBytes);
    if (e != cudaSuccess) return e;
    configured[dev] = true;
  }
  dim3 grid((V + tc::TN - 1) / tc::TN, (nrows + tc::TM - 1) / tc::TM);
  cost_table_tc_kernel<<<grid, 128, tc::kSmemBytes, st>>>(cs, nrows, vocab, V, d, cnorm, vnorm, m,
                                                          MP, T, err);
  return cudaGetLastError();
}

}  // namespace d2g
