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
// Operands are split once into a blocked layout that is the shared-memory
// image of one (row tile, K block): for each tile of BR rows and each K block
// of 32 values, hi then lo, each in the no-swizzle K-major core-matrix order
// (8 rows x 16 bytes per core matrix, core matrices adjacent along K 128 bytes
// apart, 8-row groups 1024 bytes apart).  The vocabulary is split once per
// phase (it never changes), the centroids once per table.
//
// One CTA of 128 threads computes one 128 x 256 output tile.  Thread 0 runs a
// two-stage pipeline: a K block of A (hi + lo, 32 KB) and B (hi + lo, 64 KB)
// arrives by two bulk copies on the stage's "full" mbarrier; four k-steps x
// three MMAs accumulate into a 256-column TMEM accumulator; tcgen05.commit
// arrives on the stage's "empty" mbarrier, after which the stage is refilled
// with the block two ahead.  The epilogue reads TMEM with tcgen05.ld (each
// warp its 32 lanes = 32 rows) and writes T, one coalesced 128-byte row
// segment per vocabulary column and warp.  Every wait is bounded.
#include <cstdint>
#include <mutex>

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
constexpr int SA = TM * TKB, SB = TN * TKB;   // floats of one hi (or lo) block of A / B
constexpr int STAGE = 2 * SA + 2 * SB;        // A hi, A lo, B hi, B lo
constexpr size_t kSmemBytes = (size_t)2 * STAGE * 4;  // two stages, 192 KB

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
}

__device__ __forceinline__ void mbar_expect(uint64_t *b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *b) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(b))
      : "memory");
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

}  // namespace tc

// Split a row-major FP32 matrix (R x d) into the blocked TF32 hi / lo layout:
// dst[((rt * nkb + kb) * 2 + hl) * BR * 32 + core-matrix offset], rows padded to
// a multiple of BR and K to nkb * 32 with zeros.  One thread per 16-byte chunk.
__global__ void tf32_split_kernel(const float *__restrict__ src, int R, int d, int BR, int nrt,
                                  int nkb, float *__restrict__ dst) {
  using namespace tc;
  const size_t n = (size_t)nrt * BR * nkb * KC;
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int per_row = nkb * KC;
  const int row = (int)(i / per_row), ci = (int)(i - (size_t)row * per_row);
  const int kb = ci / KC, ch = ci - kb * KC;
  const int rt = row / BR, r = row - rt * BR;
  const int t0 = kb * TKB + ch * 4;
  float x[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) x[j] = (row < R && t0 + j < d) ? __ldg(src + (size_t)row * d + t0 + j) : 0.f;
  float h[4], l[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    h[j] = tf32_round(x[j]);
    l[j] = tf32_round(x[j] - h[j]);
  }
  const size_t blk = ((size_t)rt * nkb + kb) * 2 * (size_t)BR * TKB;
  const int off = ((r >> 3) * KC + ch) * CORE + (r & 7) * 4;
  *reinterpret_cast<float4 *>(dst + blk + off) = make_float4(h[0], h[1], h[2], h[3]);
  *reinterpret_cast<float4 *>(dst + blk + (size_t)BR * TKB + off) = make_float4(l[0], l[1], l[2], l[3]);
}

__global__ void __launch_bounds__(128, 1)
    cost_table_tc_kernel(const float *__restrict__ asplit, int nrows, const float *__restrict__ bsplit,
                         int V, int nkb, const float *__restrict__ cnorm,
                         const float *__restrict__ vnorm, int m, int MP, float *__restrict__ T,
                         int *__restrict__ err) {
  using namespace tc;
  extern __shared__ __align__(1024) float sm[];
  __shared__ __align__(8) uint64_t full[2], empty[2];
  __shared__ uint32_t tmem_base;
  __shared__ int fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r0 = blockIdx.y * TM, v0 = blockIdx.x * TN;
  const float *ablk = asplit + (size_t)blockIdx.y * nkb * 2 * SA;  // [kb][hi, lo][SA]
  const float *bblk = bsplit + (size_t)blockIdx.x * nkb * 2 * SB;  // [kb][hi, lo][SB]

  if (warp == 0) {  // tensor-memory accumulator: 128 lanes x 256 FP32 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(&tmem_base)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init1(&full[0]);
    mbar_init1(&full[1]);
    mbar_init1(&empty[0]);
    mbar_init1(&empty[1]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fail = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (tid == 0) {
    auto load = [&](int kb, int s) {
      float *st = sm + s * STAGE;
      mbar_expect(&full[s], (uint32_t)STAGE * 4u);
      bulk_load(st, ablk + (size_t)kb * 2 * SA, 2u * SA * 4u, &full[s]);
      bulk_load(st + 2 * SA, bblk + (size_t)kb * 2 * SB, 2u * SB * 4u, &full[s]);
    };
    load(0, 0);
    if (nkb > 1) load(1, 1);
    int issued = nkb > 1 ? 2 : 1;  // K blocks whose copies were issued
    bool ok = true;
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb & 1;
      const uint32_t par = (uint32_t)(kb >> 1) & 1u;
      if (!mbar_wait_bounded(&full[s], par)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const float *Ah = sm + s * STAGE, *Al = Ah + SA, *Bh = Al + SA, *Bl = Bh + SB;
#pragma unroll
      for (int ks = 0; ks < TKB / 8; ++ks) {  // one MMA k-step = 8 TF32 = two 16-byte chunks
        const int off = ks * 2 * CORE;
        const uint64_t ah = smem_desc(Ah + off), al = smem_desc(Al + off);
        const uint64_t bh = smem_desc(Bh + off), bl = smem_desc(Bl + off);
        mma_tf32(tmem, ah, bh, (kb > 0 || ks > 0) ? 1u : 0u);
        mma_tf32(tmem, ah, bl, 1u);
        mma_tf32(tmem, al, bh, 1u);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_addr(&empty[s]))
          : "memory");
      if (kb + 2 < nkb) {  // refill this stage once its MMAs have read it
        if (!mbar_wait_bounded(&empty[s], par)) {
          ok = false;
          break;
        }
        load(kb + 2, s);
        ++issued;
      }
    }
    if (!ok) {
      fail = 1;
      // let the copies in flight land (bounded) before the CTA leaves
      for (int kb = 0; kb < issued; ++kb) mbar_wait_bounded(&full[kb & 1], (uint32_t)(kb >> 1) & 1u);
    }
  }
  // the last commit completes after every MMA of the tile
  {
    const int last = nkb - 1;
    if (!mbar_wait_bounded(&empty[last & 1], (uint32_t)(last >> 1) & 1u)) fail = 1;
  }
  __syncthreads();
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
    atomicCAS(err, 0, kErrTcTimeout);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols)
                 : "memory");
}

size_t tf32_split_floats(int R, int d, int BR) {
  const size_t nrt = (size_t)(R + BR - 1) / BR, nkb = (size_t)(d + tc::TKB - 1) / tc::TKB;
  return nrt * nkb * 2 * (size_t)BR * tc::TKB;
}

cudaError_t launch_tf32_split(const float *src, int R, int d, int BR, float *dst, cudaStream_t st) {
  const int nrt = (R + BR - 1) / BR, nkb = (d + tc::TKB - 1) / tc::TKB;
  const size_t n = (size_t)nrt * BR * nkb * tc::KC;
  if (n == 0) return cudaSuccess;
  tf32_split_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, R, d, BR, nrt, nkb, dst);
  return cudaGetLastError();
}

// csplit: the centroids' split buffer (tf32_split_floats(nrows, d, 128) floats);
// vsplit: the vocabulary split once with launch_tf32_split(vocab, V, d, 256, ...)
cudaError_t launch_cost_table_tc(const float *cs, int nrows, const float *vsplit, int V, int d,
                                 const float *cnorm, const float *vnorm, int m, int MP, float *T,
                                 float *csplit, int *err, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  // per device; the first call for a device comes before any graph capture
  static bool configured[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = launch_device(&dev);
  if (e != cudaSuccess) return e;
  {
    static std::mutex mu;  // phases on other host threads
    std::lock_guard<std::mutex> lk(mu);
    if (!configured[dev]) {
      e = cudaFuncSetAttribute(cost_table_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)tc::kSmemBytes);
      if (e != cudaSuccess) return e;
      configured[dev] = true;
    }
  }
  e = launch_tf32_split(cs, nrows, d, tc::TM, csplit, st);
  if (e != cudaSuccess) return e;
  const int nkb = (d + tc::TKB - 1) / tc::TKB;
  dim3 grid((V + tc::TN - 1) / tc::TN, (nrows + tc::TM - 1) / tc::TM);
  cost_table_tc_kernel<<<grid, 128, tc::kSmemBytes, st>>>(csplit, nrows, vsplit, V, nkb, cnorm, vnorm,
                                                          m, MP, T, err);
  return cudaGetLastError();
}

}  // namespace d2g
