// Fixed-centroid transport solves for the serving loop.
//
// A request is one query distribution (m_q supports in R^d, weights w_q); it
// is solved against all K resident centroids (str = m supports each, fixed
// weights c_w[l]) with B-ADMM steps 1-3 of src/d2/centroid_Bregman.c:155-175
// for `iters` iterations, from Z = w_q (x) c_w[l] and Y = 0, with
// rho = rhoCoeff * mean(C) over the request's K plans; the answer is
// cost_l = <C_l, X_l> for every centroid and its argmin.
//
// With the centroid weights fixed there is no coupling between plans, so a
// plan's whole iteration loop runs on chip: Z and Y stay in registers (row
// pairs, for the packed FP32x2 instructions), C in shared memory, column sums
// use shuffles, row sums go through shared memory (and DSMEM when a plan spans
// a thread-block cluster).  Nothing touches HBM inside the loop; the kernel is
// bound by issue and latency (MUFU ex2, FP32, the per-iteration row-sum
// exchange).  64 registers: four CTAs of 256 threads per SM.
//
// Work items come from compact descriptors, not per-group tables:
//   item = {request, first centroid l0, plans in the item, groups per plan}
// Plans of one item are consecutive centroids of one request, each ng = ceil(m_q/4)
// groups of 4 columns; an item either packs several plans into one CTA or
// spreads one plan over a cluster of cs CTAs.
#include <cooperative_groups.h>

#include <type_traits>

#include "d2g_internal.cuh"

namespace cg = cooperative_groups;

namespace d2g {



__device__ __forceinline__ float sv_ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ unsigned sv_smem(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long sv_now() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// mbarrier in this CTA's shared memory, one arrival per phase
__device__ __forceinline__ void sv_mbar_init(unsigned long long *b) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sv_smem(b)) : "memory");
}

__device__ __forceinline__ void sv_mbar_expect(unsigned long long *b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sv_smem(b)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool sv_mbar_test(unsigned long long *b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(sv_smem(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait (about one second), then report
__device__ __forceinline__ bool sv_mbar_wait(unsigned long long *b, unsigned parity) {
  if (sv_mbar_test(b, parity)) return true;
  const unsigned long long t0 = sv_now();
  for (;;) {
    for (int i = 0; i < 32; ++i)
      if (sv_mbar_test(b, parity)) return true;
    if (sv_now() - t0 > 1000000000ull) return false;
  }
}

// 16 bytes into the shared memory of cluster rank `rank` at the same offset as
// `local`, completing `bytes` on that rank's mbarrier at the offset of `bar`
__device__ __forceinline__ void sv_push4(const float *local, const unsigned long long *bar,
                                         unsigned rank, float4 v) {
  unsigned ra, rb;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(sv_smem(local)), "r"(rank));
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(rb) : "r"(sv_smem(bar)), "r"(rank));
  asm volatile(
      "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(ra),
      "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "r"(rb)
      : "memory");
}

// Pairs of rows go through the packed FP32x2 instructions (one issue slot
// for two lanes' worth of arithmetic, each lane rounded as its scalar form).
__device__ __forceinline__ float2 sv_bc(float v) { return make_float2(v, v); }

__device__ __forceinline__ float2 sv_ex2x2(float2 x) { return make_float2(sv_ex2(x.x), sv_ex2(x.y)); }

__device__ __forceinline__ float2 sv_nex2x2(float2 x) { return make_float2(sv_ex2(-x.x), sv_ex2(-x.y)); }

template <int TPC>
__device__ __forceinline__ float sv_seg_sum(float v) {
#pragma unroll
  for (int o = TPC / 2; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int MP, bool FULL>
__global__ void __launch_bounds__(256, 4) serve_kernel(const ServeArgs a) {
  constexpr int RPT = 4, TPC = MP / RPT, G = 256 / TPC, S = 4;
  constexpr float kL2e = 1.4426950408889634f;  // log2(e)
  __shared__ __align__(16) float sm_c[G * S * MP];       // ground costs of the CTA's entries
  __shared__ __align__(16) float sm_rs[2][G * MP];       // per-group row partials, by parity
  __shared__ __align__(16) float sm_x[2][8][MP];         // cluster: every rank's partial, by parity
  __shared__ double sm_cost[G];
  __shared__ __align__(8) unsigned long long sm_bar[2];  // cluster: partials of all ranks landed, by parity
  __shared__ int sm_fail;
  __shared__ float4 sm_w4[256], sm_cw4[256];  // per thread: its columns' weights, its rows' c_w

  const int tid = threadIdx.x, g = tid / TPC, r = tid % TPC, k0 = r * RPT;
  const int lane = tid & 31, warp = tid >> 5;
  const int cs = a.cs;
  const int item_i = blockIdx.x / cs, rank = blockIdx.x - item_i * cs;
  const int4 it = a.items[item_i];
  const int req = it.x, l0 = it.y, nplans = it.z, ng = it.w;
  const float4 rq = a.reqs[req];
  const int qcol0 = __float_as_int(rq.x), mq = __float_as_int(rq.y);
  const float ir2 = rq.z;

  // this thread's plan, group within the plan, and columns
  int plan, gq;
  if (cs == 1) {
    plan = g / ng;
    gq = g - plan * ng;
  } else {
    plan = 0;
    gq = rank * G + g;
  }
  const bool active = cs == 1 ? plan < nplans : gq < ng;
  const int l = l0 + (active ? plan : 0);
  const int c0 = gq * S;  // first column of the group within the query
  const int nvalid = active ? min(S, mq - c0) : 0;
  // groups of this thread's plan inside this CTA (for the row sums)
  // (threads past the CTA's plans read no partials)
  const int lo = cs == 1 ? (active ? plan * ng : 0) : 0;
  const int hi = cs == 1 ? (active ? lo + ng : 0) : min(G, ng - rank * G);
  float *cme = sm_c + (g * S) * MP + k0;  // this thread's costs: column s at cme[s*MP + q]

  // costs (to shared memory), weights, start point
  // Z and Y of row pairs (k0, k0 + 1) and (k0 + 2, k0 + 3): z[s][h] = rows 2h, 2h + 1
  float2 z[S][2], y[S][2];
  float w[S], cw[RPT];
#pragma unroll
  for (int q = 0; q < RPT; ++q) cw[q] = __ldg(a.c_w32 + (size_t)l * MP + k0 + q);
  {
    float c[S][RPT];
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const bool ok = s < nvalid;
      w[s] = ok ? __ldg(a.q_w + qcol0 + c0 + s) : 0.f;
#pragma unroll
      for (int q = 0; q < RPT; ++q) c[s][q] = 0.f;
    }
    for (int t = 0; t < a.dim; ++t) {
      float cv[RPT], qv[S];
#pragma unroll
      for (int q = 0; q < RPT; ++q) cv[q] = __ldg(a.c_supp32 + ((size_t)l * MP + k0 + q) * a.dim + t);
#pragma unroll
      for (int s = 0; s < S; ++s)
        qv[s] = s < nvalid ? __ldg(a.q_supp + (size_t)(qcol0 + c0 + s) * a.dim + t) : 0.f;
#pragma unroll
      for (int s = 0; s < S; ++s)
#pragma unroll
        for (int h = 0; h < 2; ++h) {  // row pairs: cv - qv as fma(qv, -1, cv), one rounding
          const float2 d = __ffma2_rn(sv_bc(qv[s]), sv_bc(-1.f), make_float2(cv[2 * h], cv[2 * h + 1]));
          const float2 acc = __ffma2_rn(d, d, make_float2(c[s][2 * h], c[s][2 * h + 1]));
          c[s][2 * h] = acc.x;
          c[s][2 * h + 1] = acc.y;
        }
    }
#pragma unroll
    for (int s = 0; s < S; ++s)
      *((float4 *)(cme + s * MP)) = make_float4(c[s][0], c[s][1], c[s][2], c[s][3]);
    sm_w4[tid] = make_float4(w[0], w[1], w[2], w[3]);
    sm_cw4[tid] = make_float4(cw[0], cw[1], cw[2], cw[3]);
#pragma unroll
    for (int s = 0; s < S; ++s)  // start point, after the costs (fewer live registers there)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        z[s][h] = s < nvalid ? make_float2(w[s] * cw[2 * h], w[s] * cw[2 * h + 1]) : sv_bc(0.f);
        y[s][h] = sv_bc(0.f);
      }
  }
  const int m = a.m;
  const unsigned xbytes = (unsigned)cs * MP * 4u;  // one partial from every rank per iteration
  if (cs > 1) {
    // Row partials travel by st.async into every rank's shared memory and
    // complete on that rank's mbarrier (one per iteration parity), so an
    // iteration waits only for the bytes it needs, not for a cluster barrier.
    if (tid == 0) {
      sv_mbar_init(&sm_bar[0]);
      sv_mbar_init(&sm_bar[1]);
      sm_fail = 0;
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      sv_mbar_expect(&sm_bar[0], xbytes);
      sv_mbar_expect(&sm_bar[1], xbytes);
    }
    cg::this_cluster().sync();  // every rank's barriers exist before the first push
  }
  // Without padded rows (FULL) the padded columns of a query's last group
  // need no masks: their weight, Z and Y are 0, so step 1 gives X = 0 (its
  // column sum is ROUNDOFF-positive), and step 2's ROUNDOFF is added only to
  // valid columns, which keeps their Z' and row sums at 0.
  //
  // X lives only while its column is processed: step 3 is applied as
  // Y += X right after step 2 and Y -= Z once the row scale is known, and
  // <C, X> of the last iteration is accumulated on the way.
  // A warp whose groups are all past the plans (the tail of a plan's last
  // slice, or unused groups of a packed CTA) skips the arithmetic and only
  // takes part in the row-sum exchange with zeros.
  const bool wact = __any_sync(0xffffffffu, active);
  float2 pc2 = sv_bc(0.f);
  // one iteration (the last one also accumulates <C, X>)
  auto iteration = [&](const int iter, auto last_tag) {
    constexpr bool last = decltype(last_tag)::value;
    const int buf = iter & 1;
    float2 rp2[2] = {sv_bc(0.f), sv_bc(0.f)};
    if (wact) {
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const bool colok = s < nvalid;
      const float4 cc = *((const float4 *)(cme + s * MP));
      const float2 c[2] = {make_float2(cc.x, cc.y), make_float2(cc.z, cc.w)};
      float2 v[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        v[h] = __ffma2_rn(z[s][h], sv_nex2x2(__ffma2_rn(c[h], sv_bc(ir2), y[s][h])), sv_bc(kRoundoff));
        if constexpr (!FULL) {
          if (!(colok && k0 + 2 * h < m)) v[h].x = 0.f;
          if (!(colok && k0 + 2 * h + 1 < m)) v[h].y = 0.f;
        }
      }
      const float2 vs = __fadd2_rn(v[0], v[1]);
      const float csum = sv_seg_sum<TPC>(vs.x + vs.y);
      const float ws = s == 0 ? sm_w4[tid].x : s == 1 ? sm_w4[tid].y : s == 2 ? sm_w4[tid].z : sm_w4[tid].w;
      const float f = (FULL || colok) ? __fdividef(ws, csum) : 0.f;
      const float eps2 = colok ? kRoundoff : 0.f;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float2 xv = __fmul2_rn(v[h], sv_bc(f));
        float2 zp = __ffma2_rn(xv, sv_ex2x2(y[s][h]), sv_bc(eps2));
        if constexpr (!FULL) {
          if (!(k0 + 2 * h < m)) zp.x = 0.f;
          if (!(k0 + 2 * h + 1 < m)) zp.y = 0.f;
        }
        y[s][h] = __ffma2_rn(sv_bc(kL2e), xv, y[s][h]);  // step 3, first half
        z[s][h] = zp;
        rp2[h] = __fadd2_rn(rp2[h], zp);
        if constexpr (last) pc2 = __ffma2_rn(c[h], xv, pc2);
      }
    }
    }
    float rp[RPT] = {rp2[0].x, rp2[0].y, rp2[1].x, rp2[1].y};
    float tot[RPT] = {0.f, 0.f, 0.f, 0.f};
    if (cs == 1) {
      *((float4 *)(sm_rs[buf] + g * MP + k0)) = make_float4(rp[0], rp[1], rp[2], rp[3]);
      __syncthreads();
      // every thread sums its own plan's partials (no second barrier: the
      // partials are double-buffered by iteration parity)
#pragma unroll 4
      for (int j = lo; j < hi; ++j) {
        const float4 u = *((const float4 *)(sm_rs[buf] + j * MP + k0));
        tot[0] += u.x; tot[1] += u.y; tot[2] += u.z; tot[3] += u.w;
      }
    } else {
      // one plan over the cluster: the warp's groups are pre-added with
      // shuffles; warp w < cs adds the warps' partials and pushes the CTA's
      // partial into rank w; each rank then adds the cs partials in rank order
#pragma unroll
      for (int o = TPC; o < 32; o <<= 1)
#pragma unroll
        for (int q = 0; q < RPT; ++q) rp[q] += __shfl_xor_sync(0xffffffffu, rp[q], o);
      if (lane < TPC) *((float4 *)(sm_rs[buf] + warp * MP + k0)) = make_float4(rp[0], rp[1], rp[2], rp[3]);
      __syncthreads();
      if (warp < cs && lane < TPC) {  // warp w pushes to rank w
        float4 pt = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int w8 = 0; w8 < 8; ++w8) {
          const float4 u = *((const float4 *)(sm_rs[buf] + w8 * MP + k0));
          pt.x += u.x; pt.y += u.y; pt.z += u.z; pt.w += u.w;
        }
        sv_push4(&sm_x[buf][rank][k0], &sm_bar[buf], (unsigned)warp, pt);
      }
      if (!sv_mbar_wait(&sm_bar[buf], (unsigned)(iter >> 1) & 1u)) sm_fail = 1;
#pragma unroll 4
      for (int rk = 0; rk < cs; ++rk) {
        const float4 u = *((const float4 *)(&sm_x[buf][rk][0] + k0));
        tot[0] += u.x; tot[1] += u.y; tot[2] += u.z; tot[3] += u.w;
      }
      // re-arm this parity's barrier for iteration iter + 2 (every thread of
      // this CTA has passed this iteration's wait before any rank can push
      // iteration iter + 2's partials)
      if (tid == 0) sv_mbar_expect(&sm_bar[buf], xbytes);
    }
    // second half of step 2 with the fixed centroid weights, and step 3
    float sc[RPT];
    const float4 cw4 = sm_cw4[tid];
    const float cwq[RPT] = {cw4.x, cw4.y, cw4.z, cw4.w};
#pragma unroll
    for (int q = 0; q < RPT; ++q) sc[q] = tot[q] > 0.f ? __fdividef(cwq[q], tot[q]) : 0.f;
    // (padded rows have tot = 0, so sc = 0 zeroes their Z; padded columns
    // stay at Z = Y = 0 by themselves)
    const float2 sc2[2] = {make_float2(sc[0], sc[1]), make_float2(sc[2], sc[3])};
    if (wact)
#pragma unroll
    for (int s = 0; s < S; ++s)
#pragma unroll
      for (int h = 0; h < 2; ++h) {  // second half of step 3: Y -= Z
        const float2 zn = __fmul2_rn(z[s][h], sc2[h]);
        y[s][h] = __ffma2_rn(sv_bc(-kL2e), zn, y[s][h]);
        z[s][h] = zn;
      }
  };
  for (int iter = 0; iter + 1 < a.iters; ++iter) iteration(iter, std::false_type{});
  if (a.iters > 0) iteration(a.iters - 1, std::true_type{});
  // cost_l = <C, X> of the last iteration, per plan
  float pc = sv_seg_sum<TPC>(pc2.x + pc2.y);
  if (r == 0) sm_cost[g] = (double)pc;
  if (cs == 1) {
    __syncthreads();
    if (active && g == lo && r == 0) {
      double t = 0.0;
      for (int j = lo; j < hi; ++j) t += sm_cost[j];
      a.cost_out[(size_t)req * a.K + l] = (float)t;
    }
  } else {
    cg::cluster_group cl = cg::this_cluster();
    __syncthreads();
    if (tid == 0 && sm_fail) atomicExch(a.err, 1);
    if (tid == 0) {
      double t = 0.0;
      for (int j = 0; j < hi; ++j) t += sm_cost[j];
      sm_cost[0] = t;
    }
    cl.sync();
    if (rank == 0 && tid == 0) {
      double t = 0.0;
      for (int rk = 0; rk < cs; ++rk) t += *cl.map_shared_rank(&sm_cost[0], rk);
      a.cost_out[(size_t)req * a.K + l] = (float)t;
    }
    cl.sync();
  }
}

template <int MP, bool FULL>
static cudaError_t launch_serve_mp(const ServeArgs &a, int nitems, cudaStream_t st) {
  if (nitems <= 0) return cudaSuccess;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nitems * a.cs);
  cfg.blockDim = dim3(256);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  if (a.cs > 1) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = a.cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, serve_kernel<MP, FULL>, a);
}

cudaError_t launch_serve(int MP, const ServeArgs &a, int nitems, cudaStream_t st) {
  const bool full = a.m == MP;
  switch (MP) {
    case 16: return full ? launch_serve_mp<16, true>(a, nitems, st) : launch_serve_mp<16, false>(a, nitems, st);
    case 32: return full ? launch_serve_mp<32, true>(a, nitems, st) : launch_serve_mp<32, false>(a, nitems, st);
    case 64: return full ? launch_serve_mp<64, true>(a, nitems, st) : launch_serve_mp<64, false>(a, nitems, st);
    default: return cudaErrorInvalidValue;  // (the server takes str <= 64: a 512-support query fits 8 CTAs)
  }
}

}  // namespace d2g
