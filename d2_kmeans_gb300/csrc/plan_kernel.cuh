// Fused B-ADMM plan update (batched FP32 form).
//
// One pass over every transport plan per iteration, steps 1-3 of
// src/d2/centroid_Bregman.c:155-175 plus the per-plan reductions that feed
// steps 4-6:
//
//   T = Z * exp(-(C + Y)) + 1e-9              C computed in registers (Euclidean)
//                                              or read from an L2-resident table
//   X = T / colsum(T) * w_j                    column sums: in-thread + shuffles
//   Z' = X * exp(Y) + 1e-9
//   Z  = Z' * (c_w[label] / rowsum(Z'))        row sums: smem (+ DSMEM in a cluster)
//   Y += X - Z
//
// Z and Y are read once and written once (16 B per plan entry, the HBM
// roofline), with 128-bit streaming loads/stores.  X is never stored unless a
// later pass needs it.  Per plan the kernel emits the row sums of Z' (step 4's
// Zr), on support-update iterations the X moments sum_j X[k,j]*(1, s_j)
// (step 5), and on check iterations per-CTA partials of <C,X>, |X-Z|, |Z-Z0|
// (step 6).
//
// Thread mapping: a CTA of NT threads owns JC = G*S columns; TPC
// threads share one column (RPT rows each, MP = TPC*RPT), each thread holds S
// consecutive columns.  Plans start on S-column group boundaries, so a thread
// never straddles two plans.
#pragma once

#include <cooperative_groups.h>

#include <algorithm>
#include <mutex>

#include "d2g_internal.cuh"

namespace cg = cooperative_groups;

namespace d2g {

template <int MP>
struct GeoT {
  static constexpr int RPT = MP >= 256 ? 8 : 4;
  static constexpr int TPC = MP / RPT;
  static constexpr int NT = plan_threads(MP);        // threads per CTA
  static constexpr int S = plan_cols_per_thread(MP); // columns per thread
  static constexpr int G = NT / TPC;
  static constexpr int JC = G * S;
  static_assert(TPC >= 1 && TPC <= 32 && (32 % TPC) == 0, "TPC must divide a warp");
  // a unit's column weights and symbols arrive by untiled bulk copy from
  // col_w + g0 * S (ng * S * 4 bytes): 16-byte alignment needs S * 4 % 16 == 0
  static_assert((S * 4) % 16 == 0, "columns per thread must keep the per-column bulk copies 16-byte aligned");
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// 2^x on the MUFU unit (PTX ex2.approx).  The plan update works in base 2:
// exp(v) = 2^(v*log2(e)), with Y stored pre-multiplied by log2(e) and the
// cost scale 1/rho folded into log2(e)/rho, so each exponential is one FMA and
// one ex2.
__device__ __forceinline__ float ex2f(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// Row pairs through the packed FP32x2 instructions (one issue slot for two
// lanes' arithmetic, each lane rounded exactly as its scalar form).
__device__ __forceinline__ float2 bc2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 ex2f2(float2 x) { return make_float2(ex2f(x.x), ex2f(x.y)); }
__device__ __forceinline__ float2 nex2f2(float2 x) { return make_float2(ex2f(-x.x), ex2f(-x.y)); }
__device__ __forceinline__ float2 pr2(const float *v, int h) { return make_float2(v[2 * h], v[2 * h + 1]); }
__device__ __forceinline__ void st2(float *v, int h, float2 u) {
  v[2 * h] = u.x;
  v[2 * h + 1] = u.y;
}
// The same pair arithmetic as two scalar instructions (P = false), for
// kernels at one CTA per SM where the packed form's longer dependent
// latency costs more than the issue slots it saves.  Results are identical.
template <bool P>
__device__ __forceinline__ float2 fma2x(float2 a, float2 b, float2 c) {
  if constexpr (P) return __ffma2_rn(a, b, c);
  else return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
}
template <bool P>
__device__ __forceinline__ float2 mul2x(float2 a, float2 b) {
  if constexpr (P) return __fmul2_rn(a, b);
  else return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
}
template <bool P>
__device__ __forceinline__ float2 add2x(float2 a, float2 b) {
  if constexpr (P) return __fadd2_rn(a, b);
  else return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
}
constexpr float kLog2e = 1.4426950408889634f;  // log2(e)
constexpr float kLn2 = 0.6931471805599453f;    // ln(2) = 1/log2(e)

template <int TPC>
__device__ __forceinline__ float seg_sum(float v) {
#pragma unroll
  for (int o = TPC / 2; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide fixed-order sum of 3 doubles; thread 0 gets the result.
template <int NT>
__device__ __forceinline__ void block_sum3(double v0, double v1, double v2, double *out) {
  __shared__ double red[NT / 32][3];
  v0 = warp_sum_d(v0);
  v1 = warp_sum_d(v1);
  v2 = warp_sum_d(v2);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    red[w][0] = v0;
    red[w][1] = v1;
    red[w][2] = v2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0, c = 0;
    for (int i = 0; i < NT / 32; ++i) {
      a += red[i][0];
      b += red[i][1];
      c += red[i][2];
    }
    out[0] = a;
    out[1] = b;
    out[2] = c;
  }
}

// Per-thread view of its S columns x RPT rows.
template <int MP, int MODE>
struct Tile {
  using Gm = GeoT<MP>;
  static constexpr int RPT = Gm::RPT, TPC = Gm::TPC, G = Gm::G, S = Gm::S;
  static constexpr bool EUC = MODE != COST_TABLE;
  static constexpr int DS = MODE == COST_EUCLID8 ? 8 : 4;        // stored coordinates
  static constexpr int NDIM = MODE == COST_EUCLID3 ? 3 : DS;     // coordinates summed

  int g, r, k0, rank, cta_g0, cta_ng, p, nvalid, pl_g0, pl_ng, lab;
  int lp;  // staged records: the plan's index among the plans of its item
  bool active;
  size_t colbase;
  float sp[EUC ? S : 1][DS];      // column supports
  float2 cc[EUC ? RPT / 2 : 1][DS];  // centroid supports of this thread's row pairs
  int sym[S];
  const float *tab;

  __device__ __forceinline__ void init(const PlanArgs &a) {
    const int item = blockIdx.x / a.cs;
    init_at(a, item, blockIdx.x - item * a.cs);
  }

  __device__ __forceinline__ void init_at(const PlanArgs &a, int item, int rank_) {
    const int tid = threadIdx.x;
    g = tid / TPC;
    r = tid % TPC;
    k0 = r * RPT;
    rank = rank_;
    const int ig0 = a.item_g0[item], ing = a.item_ng[item];
    cta_g0 = ig0 + rank * G;
    cta_ng = min(G, ing - rank * G);
    active = g < cta_ng;
    const int gg = cta_g0 + g;
    p = 0;
    nvalid = 0;
    pl_g0 = 0;
    pl_ng = 0;
    lab = 0;
    if (active) {
      const int meta = a.grp_meta[gg];
      p = meta >> 4;
      nvalid = meta & 15;
      pl_g0 = a.plan_g0[p];
      pl_ng = a.plan_ng[p];
      lab = a.plan_label[p];
    }
    colbase = (size_t)gg * S;
  }

  // item-local view from a staged group record (persistent TMA kernel)
  __device__ __forceinline__ void init_rec(int4 rec, int item_g0, int item_ng) {
    const int tid = threadIdx.x;
    g = tid / TPC;
    r = tid % TPC;
    k0 = r * RPT;
    rank = 0;
    cta_g0 = item_g0;
    cta_ng = item_ng;
    active = g < cta_ng;
    p = 0;
    nvalid = 0;
    pl_g0 = 0;
    pl_ng = 0;
    lab = 0;
    lp = 0;
    if (active) {
      p = rec.x;
      pl_g0 = rec.y;
      lab = rec.z;
      pl_ng = rec.w >> 12;
      lp = (rec.w >> 4) & 255;
      nvalid = rec.w & 15;
    }
    colbase = (size_t)(item_g0 + g) * S;
  }

  // supports of the centroid rows k0 .. k0 + RPT - 1, as row pairs
  __device__ __forceinline__ void load_centroids(const PlanArgs &a) {
#pragma unroll
    for (int h = 0; h < RPT / 2; ++h) {
#pragma unroll
      for (int t4 = 0; t4 < DS / 4; ++t4) {
        const float4 u = __ldg((const float4 *)(a.cs32 + ((size_t)lab * MP + k0 + 2 * h) * DS) + t4);
        const float4 v = __ldg((const float4 *)(a.cs32 + ((size_t)lab * MP + k0 + 2 * h + 1) * DS) + t4);
        cc[h][4 * t4 + 0] = make_float2(u.x, v.x);
        cc[h][4 * t4 + 1] = make_float2(u.y, v.y);
        cc[h][4 * t4 + 2] = make_float2(u.z, v.z);
        cc[h][4 * t4 + 3] = make_float2(u.w, v.w);
      }
    }
  }

  // costs from staged column data: supports sp_sm [JC][DS] or table rows sym_sm [JC]
  __device__ __forceinline__ void load_costs_staged(const PlanArgs &a, const float *sp_sm,
                                                    const int *sym_sm) {
    const int lc = g * S;
    if constexpr (EUC) {
#pragma unroll
      for (int s = 0; s < S; ++s) {
#pragma unroll
        for (int t4 = 0; t4 < DS / 4; ++t4) {
          float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
          if (s < nvalid) v = *((const float4 *)(sp_sm + (lc + s) * DS) + t4);
          sp[s][4 * t4 + 0] = v.x;
          sp[s][4 * t4 + 1] = v.y;
          sp[s][4 * t4 + 2] = v.z;
          sp[s][4 * t4 + 3] = v.w;
        }
      }
      load_centroids(a);
    } else {
#pragma unroll
      for (int s = 0; s < S; ++s) sym[s] = s < nvalid ? sym_sm[lc + s] : 0;
      tab = a.ctab + (size_t)lab * a.ctab_lstride;
    }
  }

  __device__ __forceinline__ void load_costs(const PlanArgs &a) {
    if constexpr (EUC) {
#pragma unroll
      for (int s = 0; s < S; ++s) {
#pragma unroll
        for (int t4 = 0; t4 < DS / 4; ++t4) {
          float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
          if (s < nvalid) v = __ldg((const float4 *)(a.col_supp + (colbase + s) * DS) + t4);
          sp[s][4 * t4 + 0] = v.x;
          sp[s][4 * t4 + 1] = v.y;
          sp[s][4 * t4 + 2] = v.z;
          sp[s][4 * t4 + 3] = v.w;
        }
      }
      load_centroids(a);
    } else {
#pragma unroll
      for (int s = 0; s < S; ++s) sym[s] = s < nvalid ? __ldg(a.col_sym + colbase + s) : 0;
      tab = a.ctab + (size_t)lab * a.ctab_lstride;
    }
  }

  // ground cost of column s for this thread's RPT rows (not divided by rho)
  __device__ __forceinline__ void costs(int s, float (&c)[RPT]) const {
    if constexpr (EUC) {
      // two rows at a time through the FP32x2 instructions; cc - sp is
      // formed as fma(sp, -1, cc), the same single rounding
#pragma unroll
      for (int h = 0; h < RPT / 2; ++h) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int t = 0; t < NDIM; ++t) {  // (padded coordinates are 0 on both sides)
          const float2 d = __ffma2_rn(make_float2(sp[s][t], sp[s][t]), make_float2(-1.f, -1.f), cc[h][t]);
          acc = __ffma2_rn(d, d, acc);
        }
        c[2 * h] = acc.x;
        c[2 * h + 1] = acc.y;
      }
    } else {
      const float *row = tab + (size_t)sym[s] * MP + k0;
#pragma unroll
      for (int q4 = 0; q4 < RPT / 4; ++q4) {
        const float4 v = __ldg((const float4 *)row + q4);
        c[4 * q4 + 0] = v.x;
        c[4 * q4 + 1] = v.y;
        c[4 * q4 + 2] = v.z;
        c[4 * q4 + 3] = v.w;
      }
    }
  }
};

template <int N>
__device__ __forceinline__ void ld_rows(const float *p, float (&v)[N], bool ok) {
#pragma unroll
  for (int q4 = 0; q4 < N / 4; ++q4) {
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ok) t = __ldcs((const float4 *)p + q4);
    v[4 * q4 + 0] = t.x;
    v[4 * q4 + 1] = t.y;
    v[4 * q4 + 2] = t.z;
    v[4 * q4 + 3] = t.w;
  }
}

// streaming (evict-first) 128-bit stores: global memory only
template <int N>
__device__ __forceinline__ void st_rows(float *p, const float (&v)[N]) {
#pragma unroll
  for (int q4 = 0; q4 < N / 4; ++q4)
    __stcs((float4 *)p + q4, make_float4(v[4 * q4], v[4 * q4 + 1], v[4 * q4 + 2], v[4 * q4 + 3]));
}

// 128-bit stores to shared memory
template <int N>
__device__ __forceinline__ void st_rows_sm(float *p, const float (&v)[N]) {
#pragma unroll
  for (int q4 = 0; q4 < N / 4; ++q4)
    ((float4 *)p)[q4] = make_float4(v[4 * q4], v[4 * q4 + 1], v[4 * q4 + 2], v[4 * q4 + 3]);
}

template <int MP, int MODE>
__global__ void __launch_bounds__(GeoT<MP>::NT) rho_partial_kernel(const PlanArgs a, double *part) {
  using T = Tile<MP, MODE>;
  constexpr int RPT = T::RPT, S = T::S;
  T t;
  t.init(a);
  t.load_costs(a);
  // the thread's S x RPT costs added pairwise in FP32 (a few roundings), the
  // thread totals in FP64 (GB300's FP64 pipe is narrow)
  float v[S * RPT];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    float c[RPT];
    t.costs(s, c);
#pragma unroll
    for (int q = 0; q < RPT; ++q) v[s * RPT + q] = (s < t.nvalid && t.k0 + q < a.m) ? c[q] : 0.f;
  }
#pragma unroll
  for (int w = S * RPT / 2; w >= 1; w >>= 1)
#pragma unroll
    for (int j = 0; j < w; ++j) v[j] += v[j + w];
  const double acc = (double)v[0];
  __shared__ double res[3];
  block_sum3<GeoT<MP>::NT>(acc, 0.0, 0.0, res);
  if (threadIdx.x == 0) part[blockIdx.x] = res[0];
}

// Layout conversion between the packed FP32 plans and the reference layout
// (FP64, column-major str x m_i per instance at str*p_str_cum[i]).
//   dir 0: ref -> packed (a.Z), every plan
//   dir 1: packed (a.Z) -> ref     (used for Z, Y and X by pointing a.Z there)
//   dir 2: re-initialise the plans with reinit set to w_j * c_w[label]
//          (src/d2/centroid_Bregman.c:116-124); other plans are left as they are
//   dir 3: as dir 1, times ln(2) (Y is stored scaled by log2(e))
template <int MP>
__global__ void __launch_bounds__(GeoT<MP>::NT) pack_convert_kernel(const PlanArgs a, int dir,
                                                                double *ref,
                                                                const long long *plan_refcol,
                                                                const char *reinit,
                                                                const double *cw64, int str) {
  using T = Tile<MP, COST_TABLE>;
  constexpr int RPT = T::RPT, S = T::S;
  T t;
  t.init(a);
  if (!t.active) return;
  const long long base = plan_refcol[t.p] * str;  // plan_refcol holds p_str_cum (columns)
  const int jj0 = (t.cta_g0 + t.g - t.pl_g0) * S;
  if (dir == 2 && !reinit[t.p]) return;
  // a re-initialised plan is written whole, its pad columns too (zeros): the
  // plan kernels rely on pad columns holding Z = 0, and a pass that failed
  // part-way may have left anything there
  const int ncols = dir == 2 ? S : t.nvalid;
  for (int s = 0; s < ncols; ++s) {
    const size_t off = (t.colbase + s) * MP + t.k0;
    const long long rc = base + (long long)(jj0 + s) * str;
    float v[RPT];
    if (dir == 2) {  // re-initialised plan Z = w (x) c_w, in FP32 (GB300's FP64 pipe is narrow)
      const float wj = s < t.nvalid ? a.col_w[t.colbase + s] : 0.f;
#pragma unroll
      for (int q = 0; q < RPT; ++q) {
        const int k = t.k0 + q;
        v[q] = k < str ? wj * a.cw32[(size_t)t.lab * MP + k] : 0.f;
      }
      st_rows(a.Z + off, v);
    } else if (dir == 0) {
#pragma unroll
      for (int q = 0; q < RPT; ++q) {
        const int k = t.k0 + q;
        v[q] = k < str ? (float)ref[rc + k] : 0.f;
      }
      st_rows(a.Z + off, v);
    } else {
      ld_rows(a.Z + off, v, true);
      const double sc = dir == 3 ? (double)kLn2 : 1.0;
#pragma unroll
      for (int q = 0; q < RPT; ++q)
        if (t.k0 + q < str) ref[rc + t.k0 + q] = (double)v[q] * sc;
    }
  }
}


// Scatter per-column data from the reference layout into the packed layout:
// weights, Euclidean supports (padded to DS with zeros) and table rows (bin id
// j for dense histograms, the vocabulary / bin id otherwise).  Pad columns get
// zeros.
template <int MP>
__global__ void __launch_bounds__(GeoT<MP>::NT) pack_columns_kernel(
    const PlanArgs a, const long long *plan_cum, const double *w_ref, const double *supp_ref,
    const int *sym_ref, float *col_w, float *col_supp, int *col_sym, int dim, int DS,
    int dense_hist) {
  using T = Tile<MP, COST_TABLE>;
  T t;
  t.init(a);
  // the first min(S, TPC) threads of a group take its columns in turn
  if (!t.active || t.r >= T::S) return;
  const long long cum = plan_cum[t.p];
  const int jj0 = (t.cta_g0 + t.g - t.pl_g0) * T::S;
  for (int s = t.r; s < T::S; s += T::TPC) {
    const size_t pc = t.colbase + s;
    const bool ok = s < t.nvalid;
    const long long rc = cum + jj0 + s;
    col_w[pc] = ok ? (float)w_ref[rc] : 0.f;
    if (col_supp)
      for (int d = 0; d < DS; ++d)
        col_supp[pc * DS + d] = (ok && d < dim) ? (float)supp_ref[rc * dim + d] : 0.f;
    if (col_sym) col_sym[pc] = ok ? (dense_hist ? jj0 + s : sym_ref[rc]) : 0;
  }
}

// <C, X> with the cost of the current centroids over a stored X (packed):
// the residual check of an iteration that also moved the supports (the
// reference evaluates obj after step 5, :301).  Partial per CTA into slot 3.
template <int MP, int MODE>
__global__ void __launch_bounds__(GeoT<MP>::NT) obj_kernel(const PlanArgs a) {
  using T = Tile<MP, MODE>;
  constexpr int RPT = T::RPT, S = T::S;
  if (a.iter >= a.ctl->stop_iter) return;
  T t;
  t.init(a);
  t.load_costs(a);
  const float inv_rho = a.ctl->inv_rho;
  float acc = 0.f;
#pragma unroll
  for (int s = 0; s < S; ++s) {
    float c[RPT], x[RPT];
    t.costs(s, c);
    ld_rows(a.X_out + (t.colbase + s) * MP + t.k0, x, s < t.nvalid);
#pragma unroll
    for (int q = 0; q < RPT; ++q)
      if (s < t.nvalid && t.k0 + q < a.m) acc = fmaf(c[q] * inv_rho, x[q], acc);
  }
  __shared__ double res[3];
  block_sum3<GeoT<MP>::NT>((double)acc, 0.0, 0.0, res);
  if (threadIdx.x == 0) a.resid_part[(size_t)(a.resid_off + blockIdx.x) * 4 + 3] = res[0];
}

// ---------------------------------------------------------------------------
// Persistent, TMA-pipelined form of the plan update (the production kernel).
//
// Each CTA (or each cluster, for plans wider than one CTA exchanged
// synchronously) walks its units blockIdx.x, +gridDim.x, ...  A unit's Z and
// Y tiles (contiguous in the packed layout), group records, weights and
// supports or table rows arrive in shared memory by bulk async copy
// (cp.async.bulk + mbarrier transaction count) into one of two stages; the
// copy of the next unit is issued as soon as the current one has landed, so
// HBM reads overlap the exp / normalisation work of the current unit.  Table
// costs of 16 <= MP <= 128 can be staged too (cp.async of the next unit's
// rows).  Results go back with streaming 128-bit stores from registers.  Z
// and Y are read from shared memory twice (step 1 and the final step 2/3),
// which keeps only X and Z' in registers.

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *b, unsigned cnt) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(cnt) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes,
                                          unsigned long long *b) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(b))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait (limit_ns of device time, one second unless the control block
// sets another), so a lost copy reports an error instead of hanging the GPU.
__device__ __forceinline__ bool mbar_wait(unsigned long long *b, unsigned parity,
                                          unsigned long long limit_ns) {
  if (mbar_try_wait(b, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    for (int i = 0; i < 64; ++i)
      if (mbar_try_wait(b, parity)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}
// the wait limit of a launch: Ctl::wait_ns, or one second
__device__ __forceinline__ unsigned long long wait_limit(const Ctl *c) {
  const unsigned long long w = c->wait_ns;
  return w ? w : 1000000000ull;
}
// the unit whose tile copy this launch withholds (Ctl::fault_iter/fault_unit,
// a test hook that makes one bounded wait run out), or -1
__device__ __forceinline__ int withheld_unit(const Ctl *c, int iter) {
  return c->fault_iter == iter ? c->fault_unit : -1;
}

template <int MP>
__host__ __device__ constexpr int tma_tile_floats() {
  return GeoT<MP>::JC * MP;
}

// table costs staged in shared memory by bulk copies (one table row per column)
__host__ __device__ constexpr bool plan_stages_costs(int MP, int MODE) {
  return MODE == COST_TABLE && MP >= 16 && MP <= 128;
}

// WIDE: the phase has plans wider than one CTA (cluster launches, deferred
// units); without them the exchange machinery compiles out.
template <int MP, int MODE, bool CHECK, bool FULL, bool WIDE>
__global__ void __launch_bounds__(GeoT<MP>::NT, MP >= 256 ? 1 : 2)
    plan_kernel_tma(const PlanArgs a, int nitems) {
  using T = Tile<MP, MODE>;
  constexpr int RPT = T::RPT, TPC = T::TPC, G = T::G, S = T::S;
  constexpr bool PK = MP < 256;  // packed FP32x2 pair arithmetic (scalar at one CTA per SM)
  constexpr int TILE = tma_tile_floats<MP>();
  constexpr int JC = G * S;
  constexpr int CW = T::EUC ? T::DS : 1;  // staged column data: supports or table row
  // table costs of 16 <= MP <= 128 can be staged in shared memory: while a
  // unit computes, every thread copies 16-byte pieces of the next unit's
  // table rows with cp.async (TILE / 4 pieces per unit, PPT per thread)
  constexpr bool SCC = plan_stages_costs(MP, MODE);
  constexpr int CPR = MP / 4;                                  // pieces per table row
  constexpr int NT = GeoT<MP>::NT;
  constexpr int PPT = SCC ? TILE / 4 / NT : 1;
  const bool SC = SCC && a.stage_costs;
  extern __shared__ __align__(128) float smem[];
  float *stZ = smem;                                  // [2][TILE]
  float *stY = smem + 2 * TILE;                       // [2][TILE]
  int4 *stR = (int4 *)(smem + 4 * TILE);              // [2][G] group records
  float *stW = (float *)(stR + 2 * G);                // [2][JC] weights
  float *stC = stW + 2 * JC;                          // [2][JC*CW] supports / table rows
  float *stS = stC + 2 * JC * CW;                     // [2][MP] deferred row scale of the slice's plan
  float *stK = stS + 2 * MP;                          // [2][TILE] staged table costs (SC)
  float *sm_x = stK + (SCC ? 2 * TILE : 0);           // [2][8][MP] cluster: every rank's row totals
  float *sm_momx = sm_x + 2 * 8 * MP;                 // [2][dim+1][MP] cluster: this CTA's moments
  float *sm_rs = sm_momx + 2 * (a.dim + 1) * MP;      // [G][MP] row partials, then plan totals
  float *sm_mom = sm_rs + G * MP;                     // [dim+1][G][MP]
  __shared__ __align__(8) unsigned long long mbar[2];
  __shared__ int sh_fail;
  __shared__ int sh_g0[2], sh_ng[2];

  if (a.iter >= a.ctl->stop_iter) return;
  const int tid = threadIdx.x;
  // A plan wider than one CTA ("wide") is cut into slices (ranks) of G groups.
  // Synchronous exchange (CS > 1): the slices of one wide plan run on a
  // thread-block cluster and trade row sums through DSMEM before step 2
  // finishes.  Deferred exchange (PF_OUT_DEF, CS == 1 unit launches): a unit
  // is a range of at most G groups holding whole small plans and at most one
  // wide slice, at its start; the slice stores Z' (step 2 before the row
  // scaling) and U = Y + X and its row partials go to global memory, where a
  // combine kernel forms the plan's row scale c_w / rowsum(Z').  The next
  // iteration applies that scale on load (PF_IN_DEF): Z = Z' * scale, Y = U - Z.
  const int CS = WIDE ? a.cs : 1;
  const bool clustered = WIDE && CS > 1;
  const bool outdef = WIDE && (a.flags & PF_OUT_DEF) != 0;
  const bool indef = WIDE && (a.flags & PF_IN_DEF) != 0;
  const int crank = clustered ? (int)(blockIdx.x % CS) : 0;
  const int u0 = clustered ? (int)(blockIdx.x / CS) : (int)blockIdx.x;
  const int ustep = clustered ? (int)(gridDim.x / CS) : (int)gridDim.x;
  const int nunits = nitems;
  if (a.iter == 0 && a.resid_off == 0 && blockIdx.x == 0 && tid == 0) a.ctl->t_start_ns = global_ns();
  const unsigned long long wlim = wait_limit(a.ctl);
  const int fault_u = withheld_unit(a.ctl, a.iter);
  // one stage = the slice's Z and Y tiles, group records, weights and supports
  // (+ the deferred row scale of its wide plan, slot >= 0)
  auto issue = [&](int unit, int g0, int ng, int slot, int stg) {
    const size_t off = (size_t)g0 * S * MP;
    const unsigned bytes = (unsigned)ng * S * MP * 4u;
    const unsigned rb = (unsigned)ng * 16u, wb = (unsigned)ng * S * 4u, cb = wb * CW;
    const unsigned sb = slot >= 0 ? (unsigned)MP * 4u : 0u;
    mbar_expect_tx(&mbar[stg], 2u * bytes + rb + wb + cb + sb);
    if (ng <= 0) return;  // an empty slice: the phase completes on the arrival alone
    if (unit == fault_u) return;  // test hook: the stage's transaction never completes
    bulk_load(stZ + stg * TILE, a.Z + off, bytes, &mbar[stg]);
    bulk_load(stY + stg * TILE, a.Y + off, bytes, &mbar[stg]);
    bulk_load(stR + stg * G, a.grp_rec + g0, rb, &mbar[stg]);
    bulk_load(stW + stg * JC, a.col_w + (size_t)g0 * S, wb, &mbar[stg]);
    if constexpr (T::EUC)
      bulk_load(stC + stg * JC * CW, a.col_supp + (size_t)g0 * S * CW, cb, &mbar[stg]);
    else
      bulk_load(stC + stg * JC * CW, a.col_sym + (size_t)g0 * S, cb, &mbar[stg]);
    if (sb) bulk_load(stS + stg * MP, a.rowsc + (size_t)slot * MP, sb, &mbar[stg]);
  };
  // bounds of unit u; slot of its leading wide slice when that arrives deferred, else -1
  // Thread 0 fetches unit bounds ahead of use, in three steps one unit apart:
  // the item's raw bounds, then this rank's slice and its leading group
  // record, then the slot and the copy.  Any arithmetic on a loaded value
  // right after the load would stall warp 0, and with it every warp at the
  // unit's next barrier.
  auto resolve = [&](int ig0, int ing, int &g0, int &ng) {
    g0 = ig0 + crank * G;
    ng = min(G, ing - crank * G);
    if (ng < 0) ng = 0;
  };
  auto lead_rec = [&](int g0, int ng) {
    return (indef && ng > 0) ? a.grp_rec[g0] : make_int4(0, 0, 0, 0);
  };
  auto slot_of = [&](int4 r, int ng) { return (indef && ng > 0 && (r.w >> 12) > G) ? r.x : -1; };
  // staged table costs: the table row of each piece of the next unit (-1: none)
  int crow_p[PPT];
  auto load_rows_idx = [&](int g0, int ng) {
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
      const int c = (tid + NT * j) / CPR;
      crow_p[j] = c < ng * S ? __ldg(a.col_crow + (size_t)g0 * S + c) : -1;
    }
  };
  auto issue_rows = [&](int stg) {
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
      const int i = tid + NT * j, c = i / CPR, part = i - c * CPR;
      // (the row index is checked here, where the loaded value is consumed
      // anyway: a row outside the table is reported, not read)
      if (crow_p[j] >= a.ctab_rows) ctl_fail(a.ctl, 9);
      else if (crow_p[j] >= 0)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                         smem_u32(stK + stg * TILE + c * MP + part * 4)),
                     "l"(a.ctab + (size_t)crow_p[j] * MP + part * 4)
                     : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  // thread 0: the next unit's slice and lead record (n1_*), the unit after's raw bounds (n2_*)
  int n1_g0 = 0, n1_ng = 0, n2_ig0 = 0, n2_ing = 0;
  int4 n1_rec = make_int4(0, 0, 0, 0);
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    sh_fail = 0;
    mbar_fence_init();
    if (u0 < nunits) {
      int g0, ng;
      resolve(a.item_g0[u0], a.item_ng[u0], g0, ng);
      sh_g0[0] = g0;
      sh_ng[0] = ng;
      issue(u0, g0, ng, slot_of(lead_rec(g0, ng), ng), 0);
      if (u0 + ustep < nunits) {
        resolve(a.item_g0[u0 + ustep], a.item_ng[u0 + ustep], n1_g0, n1_ng);
        n1_rec = lead_rec(n1_g0, n1_ng);
      }
      if (u0 + 2 * ustep < nunits) {
        n2_ig0 = a.item_g0[u0 + 2 * ustep];
        n2_ing = a.item_ng[u0 + 2 * ustep];
      }
    }
  }
  if (SC && u0 < nunits) {  // the first unit's rows
    __syncthreads();
    load_rows_idx(sh_g0[0], sh_ng[0]);
    issue_rows(0);
  }
  __syncthreads();

  const int m = a.m;
  const float inv_rho = a.ctl->inv_rho;    // for <C,X> (natural units)
  const float ir2 = a.ctl->inv_rho_l2;     // log2(e)/rho: exponents in base 2
  const bool update = a.flags & PF_UPDATE;
  const bool write_x = a.flags & PF_WRITE_X;
  double s_obj = 0.0, s_pr = 0.0, s_dr = 0.0;  // FP64 across items, FP32 within one item
  int it = 0;
  // A CTA whose wait ran out leaves the loop at once, except in a cluster
  // launch: there it stays "dry" for its remaining units (no waits, no copies,
  // no stores, every group idle) so that it still meets its peers at each
  // unit's cluster barrier, and leaves with them.
  bool dry = false;
  int fail_it = 0;
  for (int u = u0; u < nunits; u += ustep, ++it) {
    const int stg = it & 1;
    if (!dry && !mbar_wait(&mbar[stg], (it >> 1) & 1, wlim)) sh_fail = 1;
    if (SC) asm volatile("cp.async.wait_all;" ::: "memory");  // this unit's table rows
    __syncthreads();
    if (sh_fail && !dry) {
      fail_it = it;
      if (!clustered) break;
      dry = true;
    }
    const int cur_g0 = sh_g0[stg], cur_ng = dry ? 0 : sh_ng[stg];
    const int rank = crank;
    if (tid == 0 && u + ustep < nunits && !dry) {
      issue(u + ustep, n1_g0, n1_ng, slot_of(n1_rec, n1_ng), stg ^ 1);
      sh_g0[stg ^ 1] = n1_g0;
      sh_ng[stg ^ 1] = n1_ng;
      if (u + 2 * ustep < nunits) {
        resolve(n2_ig0, n2_ing, n1_g0, n1_ng);
        n1_rec = lead_rec(n1_g0, n1_ng);
        if (u + 3 * ustep < nunits) {
          n2_ig0 = a.item_g0[u + 3 * ustep];
          n2_ing = a.item_ng[u + 3 * ustep];
        }
      }
    }
    const bool has_next = u + ustep < nunits;

    T t;
    t.init_rec(stR[stg * G + (threadIdx.x / TPC)], cur_g0, cur_ng);
    t.load_costs_staged(a, stC + stg * JC * CW, (const int *)(stC + stg * JC * CW));
    const float *zs = stZ + stg * TILE, *ys = stY + stg * TILE;
    const int lcol0 = t.g * S;  // the thread's first column within the slice
    float x[S][RPT], zp[S][RPT], w[S];
#pragma unroll
    for (int s = 0; s < S; ++s) w[s] = s < t.nvalid ? stW[stg * JC + lcol0 + s] : 0.f;
    // groups of a wide plan: deferred input scaled on load, deferred output
    const bool wp = WIDE && t.active && t.pl_ng > G;
    const bool sc_in = indef && wp, def_out = outdef && wp;
    float scin[RPT];
#pragma unroll
    for (int q = 0; q < RPT; ++q) scin[q] = sc_in ? stS[stg * MP + t.k0 + q] : 1.f;
    // Z and Y of column s from the stage; deferred input holds Z' and U
    auto ld_zy = [&](int s, float (&z)[RPT], float (&y)[RPT]) {
#pragma unroll
      for (int q4 = 0; q4 < RPT / 4; ++q4) {
        const float4 zz = *((const float4 *)(zs + (lcol0 + s) * MP + t.k0) + q4);
        const float4 yy = *((const float4 *)(ys + (lcol0 + s) * MP + t.k0) + q4);
        z[4 * q4] = zz.x; z[4 * q4 + 1] = zz.y; z[4 * q4 + 2] = zz.z; z[4 * q4 + 3] = zz.w;
        y[4 * q4] = yy.x; y[4 * q4 + 1] = yy.y; y[4 * q4 + 2] = yy.z; y[4 * q4 + 3] = yy.w;
      }
      if (sc_in) {
#pragma unroll
        for (int h = 0; h < RPT / 2; ++h) {
          const float2 zz = mul2x<PK>(pr2(z, h), pr2(scin, h));
          st2(z, h, zz);
          st2(y, h, fma2x<PK>(bc2(-kLog2e), zz, pr2(y, h)));
        }
      }
    };

    // ground costs of column s for this thread's rows
    auto costs = [&](int s, float (&c)[RPT]) {
      if (SC) {
#pragma unroll
        for (int q4 = 0; q4 < RPT / 4; ++q4) {
          const float4 v = *((const float4 *)(stK + stg * TILE + (lcol0 + s) * MP + t.k0) + q4);
          c[4 * q4] = v.x; c[4 * q4 + 1] = v.y; c[4 * q4 + 2] = v.z; c[4 * q4 + 3] = v.w;
        }
      } else {
        t.costs(s, c);
      }
    };

    // step 1 and the first half of step 2 (Y is kept scaled by log2(e))
#pragma unroll
    for (int s = 0; s < S; ++s) {
      float c[RPT], z[RPT], y[RPT];
      costs(s, c);
      ld_zy(s, z, y);
      const bool colok = s < t.nvalid;
      // Full height (m == MP): a padded column holds Z = Y = 0 and weight 0,
      // so its X comes out 0 through the column scale and no mask is needed
      // (its column sum is ROUNDOFF-positive); step 2 adds ROUNDOFF to valid
      // columns only.  Rows go in pairs through the FP32x2 instructions.
      float2 vs = bc2(0.f);
#pragma unroll
      for (int h = 0; h < RPT / 2; ++h) {
        float2 v = fma2x<PK>(pr2(z, h), nex2f2(fma2x<PK>(pr2(c, h), bc2(ir2), pr2(y, h))), bc2(kRoundoff));
        if constexpr (!FULL) {
          if (!(colok && t.k0 + 2 * h < m)) v.x = 0.f;
          if (!(colok && t.k0 + 2 * h + 1 < m)) v.y = 0.f;
        }
        st2(x[s], h, v);
        vs = h == 0 ? v : add2x<PK>(vs, v);
      }
      const float csum = seg_sum<TPC>(vs.x + vs.y);
      const float f = (FULL || colok) ? __fdividef(w[s], csum) : 0.f;  // (column sum > 0)
      const float eps2 = colok ? kRoundoff : 0.f;
#pragma unroll
      for (int h = 0; h < RPT / 2; ++h) {
        const float2 xv = mul2x<PK>(pr2(x[s], h), bc2(f));
        float2 zz = fma2x<PK>(xv, ex2f2(pr2(y, h)), bc2(eps2));
        if constexpr (!FULL) {
          if (!(t.k0 + 2 * h < m)) zz.x = 0.f;
          if (!(t.k0 + 2 * h + 1 < m)) zz.y = 0.f;
        }
        st2(x[s], h, xv);
        st2(zp[s], h, zz);
      }
    }
    {
      float rp[RPT];
#pragma unroll
      for (int h = 0; h < RPT / 2; ++h) {
        float2 u = pr2(zp[0], h);
#pragma unroll
        for (int s = 1; s < S; ++s) u = add2x<PK>(u, pr2(zp[s], h));
        st2(rp, h, u);
      }
      st_rows_sm(sm_rs + t.g * MP + t.k0, rp);
    }
    if constexpr (T::EUC) {
      if (update) {
        for (int d = 0; d <= a.dim; ++d) {
          float mv[RPT];
#pragma unroll
          for (int q = 0; q < RPT; ++q) {
            float acc = 0.f;
#pragma unroll
            for (int s = 0; s < S; ++s) {
              float sv = 1.f;
              if (d < a.dim) {
#pragma unroll
                for (int tt = 0; tt < T::DS; ++tt)
                  if (tt == d) sv = t.sp[s][tt];
              }
              acc = fmaf(x[s][q], sv, acc);
            }
            mv[q] = acc;
          }
          st_rows_sm(sm_mom + (d * G + t.g) * MP + t.k0, mv);
        }
      }
    }
    __syncthreads();
    // the next unit's bounds are visible now: fetch its table-row indices
    if (SC && has_next && !dry) load_rows_idx(sh_g0[stg ^ 1], sh_ng[stg ^ 1]);

    float tot[RPT];
    bool writer = false;
    const bool upd_euc = T::EUC && update;
    if (CS == 1) {
      // the first group of each plan (or wide slice) in the unit sums its
      // partials once: a small plan's total is published in shared memory, a
      // wide slice's partial leaves for the combine kernel
      const int lo = t.active ? max(t.pl_g0 - t.cta_g0, 0) : 0;
      const int hi = t.active ? min(t.pl_g0 + t.pl_ng - t.cta_g0, t.cta_ng) : 0;
      // a unit that is one deferred wide slice publishes nothing in shared memory
      bool one_slice = false;
      if (outdef) {
        const int4 r0 = stR[stg * G];
        one_slice = (r0.w >> 12) > G && r0.y + (r0.w >> 12) >= cur_g0 + cur_ng;
      }
      writer = t.active && t.g == lo;
      if (writer) {
#pragma unroll
        for (int q = 0; q < RPT; ++q) tot[q] = 0.f;
        for (int j = lo; j < hi; ++j) {
#pragma unroll
          for (int q4 = 0; q4 < RPT / 4; ++q4) {
            const float4 u4 = *((const float4 *)(sm_rs + j * MP + t.k0) + q4);
            tot[4 * q4] += u4.x;
            tot[4 * q4 + 1] += u4.y;
            tot[4 * q4 + 2] += u4.z;
            tot[4 * q4 + 3] += u4.w;
          }
        }
        if (def_out) {
          const int rk = (t.cta_g0 + lo - t.pl_g0) / G;
          st_rows(a.rowpart + ((size_t)t.p * kMaxCluster + rk) * MP + t.k0, tot);
        } else {
          st_rows_sm(sm_rs + lo * MP + t.k0, tot);
        }
        if (upd_euc) {  // (support updates never run deferred)
          float *xo = a.xmom_out + (size_t)t.p * (a.dim + 1) * MP;
          for (int d = 0; d <= a.dim; ++d) {
            float mv[RPT];
#pragma unroll
            for (int q = 0; q < RPT; ++q) mv[q] = 0.f;
            for (int j = lo; j < hi; ++j)
#pragma unroll
              for (int q = 0; q < RPT; ++q) mv[q] += sm_mom[(d * G + j) * MP + t.k0 + q];
            st_rows(xo + d * MP + t.k0, mv);
          }
        }
      }
      if (one_slice) {
#pragma unroll
        for (int q = 0; q < RPT; ++q) tot[q] = 1.f;
      } else {
        __syncthreads();
#pragma unroll
        for (int q4 = 0; q4 < RPT / 4; ++q4) {
          const float4 u4 = *((const float4 *)(sm_rs + lo * MP + t.k0) + q4);
          tot[4 * q4] = def_out ? 1.f : u4.x;
          tot[4 * q4 + 1] = def_out ? 1.f : u4.y;
          tot[4 * q4 + 2] = def_out ? 1.f : u4.z;
          tot[4 * q4 + 3] = def_out ? 1.f : u4.w;
        }
      }
    } else if constexpr (WIDE) {
      // one plan across the cluster: this CTA's partial is pushed into every
      // rank's shared memory (double-buffered by stage), one cluster barrier,
      // then every rank adds the CS partials from its own shared memory
      cg::cluster_group cl = cg::this_cluster();
      writer = rank == 0 && t.g == 0 && t.active;
      if (t.g == 0) {
        float pt[RPT];
#pragma unroll
        for (int q = 0; q < RPT; ++q) pt[q] = 0.f;
        for (int j = 0; j < cur_ng; ++j) {
#pragma unroll
          for (int q4 = 0; q4 < RPT / 4; ++q4) {
            const float4 u = *((const float4 *)(sm_rs + j * MP + t.k0) + q4);
            pt[4 * q4] += u.x;
            pt[4 * q4 + 1] += u.y;
            pt[4 * q4 + 2] += u.z;
            pt[4 * q4 + 3] += u.w;
          }
        }
        for (int rk = 0; rk < CS; ++rk) {
          float *dst = cl.map_shared_rank(sm_x + (stg * 8 + rank) * MP, rk) + t.k0;
#pragma unroll
          for (int q4 = 0; q4 < RPT / 4; ++q4)
            ((float4 *)dst)[q4] = make_float4(pt[4 * q4], pt[4 * q4 + 1], pt[4 * q4 + 2], pt[4 * q4 + 3]);
        }
        if (upd_euc) {
          for (int d = 0; d <= a.dim; ++d) {
            float mv[RPT];
#pragma unroll
            for (int q = 0; q < RPT; ++q) mv[q] = 0.f;
            for (int j = 0; j < cur_ng; ++j)
#pragma unroll
              for (int q = 0; q < RPT; ++q) mv[q] += sm_mom[(d * G + j) * MP + t.k0 + q];
            st_rows_sm(sm_momx + (stg * (a.dim + 1) + d) * MP + t.k0, mv);
          }
        }
      }
      cl.sync();
#pragma unroll
      for (int q = 0; q < RPT; ++q) tot[q] = 0.f;
      for (int rk = 0; rk < CS; ++rk) {
#pragma unroll
        for (int q4 = 0; q4 < RPT / 4; ++q4) {
          const float4 u = *((const float4 *)(sm_x + (stg * 8 + rk) * MP + t.k0) + q4);
          tot[4 * q4] += u.x;
          tot[4 * q4 + 1] += u.y;
          tot[4 * q4 + 2] += u.z;
          tot[4 * q4 + 3] += u.w;
        }
      }
      if (writer && upd_euc) {  // moments: pulled from the ranks on update iterations only
        float *xo = a.xmom_out + (size_t)t.p * (a.dim + 1) * MP;
        for (int d = 0; d <= a.dim; ++d) {
          float mv[RPT];
#pragma unroll
          for (int q = 0; q < RPT; ++q) mv[q] = 0.f;
          for (int rk = 0; rk < CS; ++rk) {
            const float *rem = cl.map_shared_rank(sm_momx + (stg * (a.dim + 1) + d) * MP, rk);
#pragma unroll
            for (int q = 0; q < RPT; ++q) mv[q] += rem[t.k0 + q];
          }
          st_rows(xo + d * MP + t.k0, mv);
        }
      }
    }
    float rsum = 0.f;  // step 4's per-instance normalisation of Zr (:180); t.p is the slot here
#pragma unroll
    for (int q = 0; q < RPT; ++q) rsum += (FULL || t.k0 + q < m) ? tot[q] : 0.f;
    rsum = seg_sum<TPC>(rsum);
    if (writer && !def_out) {
      float zr[RPT];
      const float inv = 1.f / rsum;
#pragma unroll
      for (int q = 0; q < RPT; ++q) zr[q] = tot[q] * inv;
      st_rows(a.rowsum_out + (size_t)t.p * MP + t.k0, zr);
    }

    // second half of step 2, and step 3
    float sc[RPT];
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      const bool ok = t.active && (FULL || t.k0 + q < m) && !def_out;
      sc[q] = ok ? __fdividef(__ldg(a.cw32 + (size_t)t.lab * MP + t.k0 + q), tot[q]) : 0.f;
    }
    float i_obj = 0.f, i_pr = 0.f, i_dr = 0.f;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      if (s < t.nvalid) {
        float y[RPT], z0[RPT], zn[RPT], yn[RPT];
        if (CHECK || sc_in) {
          ld_zy(s, z0, y);
        } else {
#pragma unroll
          for (int q4 = 0; q4 < RPT / 4; ++q4) {
            const float4 yy = *((const float4 *)(ys + (lcol0 + s) * MP + t.k0) + q4);
            y[4 * q4] = yy.x; y[4 * q4 + 1] = yy.y; y[4 * q4 + 2] = yy.z; y[4 * q4 + 3] = yy.w;
          }
        }
        if (def_out) {  // Z' and U = Y + X
#pragma unroll
          for (int h = 0; h < RPT / 2; ++h) {
            st2(zn, h, pr2(zp[s], h));
            st2(yn, h, fma2x<PK>(bc2(kLog2e), pr2(x[s], h), pr2(y, h)));
          }
        } else {
#pragma unroll
          for (int h = 0; h < RPT / 2; ++h) {
            const float2 zz = mul2x<PK>(pr2(zp[s], h), pr2(sc, h));
            // (x - zn as fma(zn, -1, x): the same single rounding)
            st2(zn, h, zz);
            st2(yn, h, fma2x<PK>(bc2(kLog2e), fma2x<PK>(zz, bc2(-1.f), pr2(x[s], h)), pr2(y, h)));
          }
        }
        if constexpr (CHECK) {
          float c[RPT];
          costs(s, c);
#pragma unroll
          for (int q = 0; q < RPT; ++q) {
            i_obj = fmaf(c[q] * inv_rho, x[s][q], i_obj);
            i_pr += fabsf(x[s][q] - zn[q]);
            i_dr += fabsf(zn[q] - z0[q]);
          }
        }
        const size_t off = (t.colbase + s) * MP + t.k0;
        st_rows(a.Z + off, zn);
        st_rows(a.Y + off, yn);
        if (write_x) st_rows(a.X_out + off, x[s]);
      }
    }
    if constexpr (CHECK) {
      s_obj += i_obj;
      s_pr += i_pr;
      s_dr += i_dr;
    }
    if (SC && has_next && !dry) issue_rows(stg ^ 1);  // lands during the next unit's wait
    // No barrier here: every reader of this unit's stage, row partials and
    // staged rows passes the next unit's opening barrier before thread 0
    // reissues the stage (two units later) or anyone writes partials again.
  }
  // rank 0 may still be reading a peer's shared memory (the moments of the
  // last item): no CTA of a cluster leaves before all of them are done
  if (clustered) cg::this_cluster().sync();
  if (SC) asm volatile("cp.async.wait_all;" ::: "memory");  // no table-row copy outlives the CTA
  if (sh_fail) {
    if (tid == 0) {
      ctl_fail(a.ctl, 7);
      // A bulk copy did not complete.  The only copy that can be in flight is
      // the one of the unit that failed (fail_it), on stage fail_it & 1 at
      // phase parity (fail_it >> 1) & 1: the next stage is issued only after
      // a successful wait.  Wait for it once more, again bounded, so that no
      // copy lands in the shared memory of a CTA that has left.
      mbar_wait(&mbar[fail_it & 1], (fail_it >> 1) & 1, wlim);
    }
    return;
  }
  if constexpr (CHECK) {
    // one partial per CTA in the slot of its first (item, rank); its other slots get zeros
    __shared__ double res[3];
    block_sum3<GeoT<MP>::NT>(s_obj, s_pr, s_dr, res);
    // (check iterations never run deferred: a unit is an item, the rank is crank)
    if (tid == 0 && u0 < nitems) {
      double *pp = a.resid_part + (size_t)(a.resid_off + u0 * CS + crank) * 4;
      pp[0] = res[0];
      pp[1] = res[1];
      pp[2] = res[2];
      for (int item = u0 + ustep; item < nitems; item += ustep) {
        double *qq = a.resid_part + (size_t)(a.resid_off + item * CS + crank) * 4;
        qq[0] = qq[1] = qq[2] = 0.0;
      }
    }
  }
}

static inline cudaLaunchConfig_t plan_cfg(int nblocks, int threads, size_t smem, cudaStream_t st,
                                          cudaLaunchAttribute *attr, int cs) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nblocks, 1, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  if (cs > 1) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  return cfg;
}

template <int MP, int MODE, bool CHECK, bool FULL, bool WIDE>
cudaError_t launch_plan_tma_t(const PlanArgs &a, int nitems, size_t smem, cudaStream_t st) {
  // persistent grid: as many clusters of a.cs CTAs as are resident at once
  // (cached per instantiation; phases on other host threads share the cache)
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  struct Shape {
    int grid[kMaxCluster + 1] = {0};  // resident CTAs for cluster size c (0: plain launches)
    int nsm = 0;
    size_t configured_smem = 0;
  };
  static Shape shapes[kMaxDevices];
  int dev = 0;
  if (cudaError_t e = launch_device(&dev); e != cudaSuccess) return e;
  Shape &sh = shapes[dev];
  int *grid = sh.grid;
  constexpr int JC = GeoT<MP>::JC;
  constexpr int CW = MODE == COST_TABLE ? 1 : (MODE == COST_EUCLID8 ? 8 : 4);
  const size_t sm = smem + (size_t)4 * tma_tile_floats<MP>() * sizeof(float) +
                    2 * (size_t)GeoT<MP>::G * 16 + 2 * (size_t)JC * 4 * (1 + CW) + (size_t)2 * MP * 4 +
                    (plan_stages_costs(MP, MODE) ? (size_t)2 * tma_tile_floats<MP>() * 4 : 0) +
                    (size_t)2 * 8 * MP * 4 + (size_t)2 * (a.dim + 1) * MP * 4;
  auto kern = plan_kernel_tma<MP, MODE, CHECK, FULL, WIDE>;
  if (sh.configured_smem < sm) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    for (int c = 0; c <= kMaxCluster; ++c) grid[c] = 0;
    sh.configured_smem = sm;
  }
  const int cs = a.cs;
  if (grid[cs] == 0) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs * 1024, 1, 1);
    cfg.blockDim = dim3(GeoT<MP>::NT, 1, 1);
    cfg.dynamicSmemBytes = sm;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int ncl = 0;
    cudaError_t e = cudaOccupancyMaxActiveClusters(&ncl, kern, &cfg);
    if (e != cudaSuccess) return e;
    grid[cs] = (ncl > 0 ? ncl : 1) * cs;
  }
  if (grid[0] == 0) {  // plain launches: resident CTAs per SM x SMs
    int per = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sh.nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, GeoT<MP>::NT, sm);
    if (e != cudaSuccess) return e;
    grid[0] = (per > 0 ? per : 1) * sh.nsm;
  }
  if (nitems <= 0) return cudaSuccess;
  const bool plain = cs == 1;
  const long long units = (long long)nitems * cs;
  int cap = plain ? grid[0] : grid[cs];
  if (plain && a.ctas_per_sm > 0) cap = std::min(cap, a.ctas_per_sm * sh.nsm);
  const int g = units < cap ? (int)units : cap;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = plan_cfg(g, GeoT<MP>::NT, sm, st, attr, plain ? 1 : cs);
  return cudaLaunchKernelEx(&cfg, kern, a, nitems);
}

template <int MP, int MODE, bool CHECK>
cudaError_t launch_plan_t(const PlanArgs &a, int nitems, size_t smem, cudaStream_t st) {
  if (a.wide) {
    if (a.m == MP) return launch_plan_tma_t<MP, MODE, CHECK, true, true>(a, nitems, smem, st);
    return launch_plan_tma_t<MP, MODE, CHECK, false, true>(a, nitems, smem, st);
  }
  if (a.m == MP) return launch_plan_tma_t<MP, MODE, CHECK, true, false>(a, nitems, smem, st);
  return launch_plan_tma_t<MP, MODE, CHECK, false, false>(a, nitems, smem, st);
}

template <int MP>
cudaError_t launch_plan_mp(int mode, bool check, const PlanArgs &a, int nitems, size_t smem,
                           cudaStream_t st) {
  if (mode == COST_EUCLID3)
    return check ? launch_plan_t<MP, COST_EUCLID3, true>(a, nitems, smem, st)
                 : launch_plan_t<MP, COST_EUCLID3, false>(a, nitems, smem, st);
  if (mode == COST_EUCLID4)
    return check ? launch_plan_t<MP, COST_EUCLID4, true>(a, nitems, smem, st)
                 : launch_plan_t<MP, COST_EUCLID4, false>(a, nitems, smem, st);
  if (mode == COST_EUCLID8)
    return check ? launch_plan_t<MP, COST_EUCLID8, true>(a, nitems, smem, st)
                 : launch_plan_t<MP, COST_EUCLID8, false>(a, nitems, smem, st);
  return check ? launch_plan_t<MP, COST_TABLE, true>(a, nitems, smem, st)
               : launch_plan_t<MP, COST_TABLE, false>(a, nitems, smem, st);
}

template <int MP>
cudaError_t launch_rho_mp(int mode, const PlanArgs &a, int nitems, double *part, cudaStream_t st) {
  const dim3 grid(nitems * a.cs), block(GeoT<MP>::NT);
  if (mode == COST_EUCLID4 || mode == COST_EUCLID3)  // (d = 3: the same costs, bit for bit)
    rho_partial_kernel<MP, COST_EUCLID4><<<grid, block, 0, st>>>(a, part);
  else if (mode == COST_EUCLID8)
    rho_partial_kernel<MP, COST_EUCLID8><<<grid, block, 0, st>>>(a, part);
  else
    rho_partial_kernel<MP, COST_TABLE><<<grid, block, 0, st>>>(a, part);
  return cudaGetLastError();
}

template <int MP>
cudaError_t launch_convert_mp(int dir, const PlanArgs &a, int nitems, double *ref,
                              const long long *plan_refcol, const char *reinit,
                              const double *cw64, int str, cudaStream_t st) {
  pack_convert_kernel<MP><<<nitems * a.cs, GeoT<MP>::NT, 0, st>>>(a, dir, ref, plan_refcol, reinit,
                                                              cw64, str);
  return cudaGetLastError();
}

template <int MP>
cudaError_t launch_pack_columns_mp(const PlanArgs &a, int nitems, const long long *plan_cum,
                                   const double *w_ref, const double *supp_ref, const int *sym_ref,
                                   float *col_w, float *col_supp, int *col_sym, int dim, int DS,
                                   int dense_hist, cudaStream_t st) {
  pack_columns_kernel<MP><<<nitems * a.cs, GeoT<MP>::NT, 0, st>>>(a, plan_cum, w_ref, supp_ref, sym_ref,
                                                              col_w, col_supp, col_sym, dim, DS,
                                                              dense_hist);
  return cudaGetLastError();
}

template <int MP>
cudaError_t launch_obj_mp(int mode, const PlanArgs &a, int nitems, cudaStream_t st) {
  if (mode == COST_EUCLID4 || mode == COST_EUCLID3)
    obj_kernel<MP, COST_EUCLID4><<<nitems * a.cs, GeoT<MP>::NT, 0, st>>>(a);
  else if (mode == COST_EUCLID8)
    obj_kernel<MP, COST_EUCLID8><<<nitems * a.cs, GeoT<MP>::NT, 0, st>>>(a);
  else
    obj_kernel<MP, COST_TABLE><<<nitems * a.cs, GeoT<MP>::NT, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace d2g

#include "plan_pair.cuh"

namespace d2g {

#define D2G_INSTANTIATE_MP(MPV)                                                                \
  template cudaError_t launch_plan_mp<MPV>(int, bool, const PlanArgs &, int, size_t,           \
                                           cudaStream_t);                                      \
  template cudaError_t launch_rho_mp<MPV>(int, const PlanArgs &, int, double *, cudaStream_t); \
  template cudaError_t launch_convert_mp<MPV>(int, const PlanArgs &, int, double *,            \
                                              const long long *, const char *, const double *, \
                                              int, cudaStream_t);                          \
  template cudaError_t launch_pack_columns_mp<MPV>(const PlanArgs &, int, const long long *,   \
                                                   const double *, const double *, const int *, \
                                                   float *, float *, int *, int, int, int,      \
                                                   cudaStream_t);                               \
  template cudaError_t launch_obj_mp<MPV>(int, const PlanArgs &, int, cudaStream_t);          \
  template cudaError_t launch_pair_mp<MPV>(int, bool, const PlanArgs &, int, cudaStream_t);

}  // namespace d2g
