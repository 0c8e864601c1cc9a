// Cross-plan FP64 reductions: cluster weights (step 4), cluster supports
// (step 5), rho (src/d2/centroid_Bregman.c:109) and residuals (step 6).
//
// Every sum here runs in a fixed order (per-warp strided loops, warps
// combined in index order, chunks combined in index order), so results are
// bit-reproducible run to run; there are no floating-point atomics.  These
// sums replace the reference's MPI_Allreduce sites (:188, :215-217, :308-310)
// on one GPU.
#include <algorithm>

#include "d2g_internal.cuh"

namespace d2g {

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

constexpr int kRedThreads = 256;
constexpr int kRedWarps = kRedThreads / 32;
constexpr int kMaxM = 256;  // cluster reductions handle str <= 256 per pass

// planes: 0..dim-1 moment numerators, dim = X row sums, dim+1 = weights
__device__ __forceinline__ int plane_of(const ClusterArgs &a, int z) {
  if (!a.do_moments) return a.dim + 1;
  return z;  // z in [0, dim+1] when both, [0, dim] when moments only
}

template <typename T>
__device__ __forceinline__ double ld_val(const T *p) {
  return (double)p[0];
}

// grid (nchunk, K, nplanes): per (cluster, chunk, plane) partial sums over the
// cluster's plans, plans in ascending instance order.  NK = ceil(str/32)
// 32-wide slices of the support axis per lane.  GB300's FP64 rate is low, so
// the per-plan normalisation is one FP64 reciprocal per plan, not a division
// per entry.
template <int NK>
__global__ void __launch_bounds__(kRedThreads) cluster_partial_kernel(const ClusterArgs a) {
  if (a.iter >= a.ctl->stop_iter) return;
  const int c = blockIdx.x, l = blockIdx.y, plane = plane_of(a, blockIdx.z);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = a.cl_ptr[l], e = a.cl_ptr[l + 1];
  const int pb = b + c * a.chunk, pe = min(e, pb + a.chunk);
  const int m = a.m;
  double acc[NK];
#pragma unroll
  for (int i = 0; i < NK; ++i) acc[i] = 0.0;
  const bool weights = plane == a.dim + 1;
  const bool slotted = a.cl_plans == nullptr;  // batched form: already normalised, in slot order
  if (weights && slotted) {
    // Each warp takes GP consecutive plans at a time: their FP32 row sums are
    // added pairwise in FP32 (at most log2(GP) roundings of terms <= 1), the
    // group total in FP64.  GB300's FP64 pipe is narrow; this keeps the long
    // accumulation (up to 10^5-10^6 plans per cluster) in FP64 with GP times
    // fewer FP64 operations.
    constexpr int GP = NK <= 2 ? 16 : (NK == 4 ? 8 : 4);
    for (int i0 = pb + warp * GP; i0 < pe; i0 += kRedWarps * GP) {
#pragma unroll
      for (int i = 0; i < NK; ++i) {
        const int k = lane + 32 * i;
        float v[GP];
#pragma unroll
        for (int j = 0; j < GP; ++j)
          v[j] = (i0 + j < pe && k < m) ? a.rowsum32[(size_t)(i0 + j) * a.rstride + k] : 0.f;
#pragma unroll
        for (int w = GP / 2; w >= 1; w >>= 1)
#pragma unroll
          for (int j = 0; j < w; ++j) v[j] += v[j + w];
        acc[i] += (double)v[0];
      }
    }
  }
  if (!weights) {
    // moment planes: each warp adds its plans pb + warp, pb + warp + 8, ... in
    // that order, U of them loaded before any is added (the loads overlap;
    // the sums are those of the one-plan-at-a-time loop, bit for bit)
    constexpr int U = NK <= 2 ? 8 : (NK == 4 ? 4 : 2);
    for (int ii0 = pb + warp; ii0 < pe; ii0 += kRedWarps * U) {
      double v[U][NK];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int ii = ii0 + u * kRedWarps;
        const int p = ii < pe ? (slotted ? ii : a.cl_plans[ii]) : -1;
        const size_t base = ((size_t)(p < 0 ? 0 : p) * (a.dim + 1) + plane) * a.rstride;
#pragma unroll
        for (int i = 0; i < NK; ++i) {
          const int k = lane + 32 * i;
          v[u][i] = 0.0;
          if (p >= 0 && k < m) v[u][i] = a.xmom32 ? (double)a.xmom32[base + k] : a.xmom64[base + k];
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (ii0 + u * kRedWarps < pe)
#pragma unroll
          for (int i = 0; i < NK; ++i)
            if (lane + 32 * i < m) acc[i] += v[u][i];
    }
  }
  // weights of the FP64 form: plans through the cluster's list, each one's
  // row sums normalised here
  for (int ii = pb + warp; ii < pe && weights && !slotted; ii += kRedWarps) {
    const int p = a.cl_plans[ii];
    double v[NK], s = 0.0;
#pragma unroll
    for (int i = 0; i < NK; ++i) {
      const int k = lane + 32 * i;
      v[i] = 0.0;
      if (k < m)
        v[i] = a.rowsum32 ? (double)a.rowsum32[(size_t)p * a.rstride + k] : a.rowsum64[(size_t)p * a.rstride + k];
      s += v[i];
    }
    const double inv = 1.0 / wsum(s);  // step 4: the instance's Zr column normalised (:180)
#pragma unroll
    for (int i = 0; i < NK; ++i) acc[i] = fma(v[i], inv, acc[i]);
  }
  __shared__ double sm[kRedWarps][kMaxM];
#pragma unroll
  for (int i = 0; i < NK; ++i) {
    const int k = lane + 32 * i;
    if (k < m) sm[warp][k] = acc[i];
  }
  __syncthreads();
  const int nplanes = a.dim + 2;
  for (int k = threadIdx.x; k < m; k += kRedThreads) {
    double s = 0.0;
    for (int w = 0; w < kRedWarps; ++w) s += sm[w][k];
    a.part[(((size_t)l * nplanes + plane) * a.nchunk + c) * m + k] = s;
  }
}

// grid (K, nplanes_out): finalise cluster weights / supports from the partials.
__global__ void __launch_bounds__(kRedThreads) cluster_final_kernel(const ClusterArgs a) {
  if (a.iter >= a.ctl->stop_iter) return;
  const int l = blockIdx.x;
  const int m = a.m, nplanes = a.dim + 2;
  int plane;
  if (a.do_weights && a.do_moments)
    plane = blockIdx.y == 0 ? a.dim + 1 : (int)blockIdx.y - 1;
  else if (a.do_weights)
    plane = a.dim + 1;
  else
    plane = blockIdx.y;
  // the cluster's sum over its chunks; a sharded update reads instead the
  // sums over all shards that the exchange left in xsum
  const int p0 = a.do_moments ? 0 : a.dim + 1, npu = a.do_moments ? a.dim + 2 : 1;
  auto chunk_sum = [&](int pl, int k) {
    if (a.xsum) return a.xsum[((size_t)l * npu + (pl - p0)) * m + k];
    double s = 0.0;
    const double *pp = a.part + (((size_t)l * nplanes + pl) * a.nchunk) * m + k;
    for (int c = 0; c < a.nchunk; ++c) s += pp[(size_t)c * m];
    return s;
  };
  if (plane == a.dim + 1) {
    __shared__ double sv[kMaxM];
    __shared__ double tot_sh;
    for (int k = threadIdx.x; k < m; k += kRedThreads) sv[k] = chunk_sum(plane, k);
    __syncthreads();
    if (threadIdx.x == 0) {  // step 4's per-cluster normalisation (:190)
      double t = 0.0;
      for (int k = 0; k < m; ++k) t += sv[k];
      tot_sh = t;
      if (!(t > 0.0) || !isfinite(t)) ctl_fail(a.ctl, 1);
    }
    __syncthreads();
    const double t = tot_sh;
    for (int k = threadIdx.x; k < a.MP; k += kRedThreads) {
      if (k < m) {
        const double v = sv[k] / t;
        a.cw64[(size_t)l * m + k] = v;
        if (a.cw32) a.cw32[(size_t)l * a.MP + k] = (float)v;
      } else if (a.cw32) {
        a.cw32[(size_t)l * a.MP + k] = 0.f;
      }
    }
    if (l == 0 && threadIdx.x == 0) {  // end of iteration: time budget (:318)
      Ctl *ctl = a.ctl;
      ctl->iters_done = a.iter + 1;
      if (gtimer() - ctl->t_start_ns > ctl->budget_ns) ctl->stop_iter = a.iter + 1;
    }
  } else if (plane < a.dim) {  // support numerator plane t = plane (:219-221)
    for (int k = threadIdx.x; k < m; k += kRedThreads) {
      const double num = chunk_sum(plane, k), den = chunk_sum(a.dim, k);
      if (!(den > 0.0)) ctl_fail(a.ctl, 2);
      const double v = num / den;
      a.cs64[((size_t)l * m + k) * a.dim + plane] = v;
      if (a.cs32) a.cs32[((size_t)l * a.MP + k) * a.DS + plane] = (float)v;
    }
  }
}

// grid (K, planes used): a shard's sums over its chunks, in chunk order, into
// xsum [K][planes used][m] for the exchange between shards (the planes used:
// the weights alone, or the moments 0..dim and the weights)
__global__ void __launch_bounds__(kRedThreads) cluster_local_kernel(const ClusterArgs a, double *xsum) {
  if (a.iter >= a.ctl->stop_iter) return;
  const int l = blockIdx.x, m = a.m, nplanes = a.dim + 2;
  const int p0 = a.do_moments ? 0 : a.dim + 1, npu = a.do_moments ? a.dim + 2 : 1;
  const int pl = p0 + (int)blockIdx.y;
  for (int k = threadIdx.x; k < m; k += kRedThreads) {
    double s = 0.0;
    const double *pp = a.part + (((size_t)l * nplanes + pl) * a.nchunk) * m + k;
    for (int c = 0; c < a.nchunk; ++c) s += pp[(size_t)c * m];
    xsum[((size_t)l * npu + (pl - p0)) * m + k] = s;
  }
}

size_t cluster_xsum_count(const ClusterArgs &a) {
  return (size_t)a.K * (a.do_moments ? a.dim + 2 : 1) * a.m;
}

cudaError_t launch_cluster_partial(const ClusterArgs &a, cudaStream_t st) {
  const int np_in = (a.do_moments ? a.dim + 1 : 0) + (a.do_weights ? 1 : 0);
  dim3 g1(a.nchunk, a.K, np_in);
  if (a.do_moments && !a.do_weights) g1.z = a.dim + 1;
  const int nk = (a.m + 31) / 32;
  if (nk <= 1)
    cluster_partial_kernel<1><<<g1, kRedThreads, 0, st>>>(a);
  else if (nk <= 2)
    cluster_partial_kernel<2><<<g1, kRedThreads, 0, st>>>(a);
  else if (nk <= 4)
    cluster_partial_kernel<4><<<g1, kRedThreads, 0, st>>>(a);
  else
    cluster_partial_kernel<8><<<g1, kRedThreads, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_cluster_local(const ClusterArgs &a, double *xsum, cudaStream_t st) {
  cluster_local_kernel<<<dim3(a.K, a.do_moments ? a.dim + 2 : 1), kRedThreads, 0, st>>>(a, xsum);
  return cudaGetLastError();
}

cudaError_t launch_cluster_final(const ClusterArgs &a, cudaStream_t st) {
  const int np_out = (a.do_weights ? 1 : 0) + (a.do_moments ? a.dim : 0);
  cluster_final_kernel<<<dim3(a.K, np_out), kRedThreads, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_cluster_reduce(const ClusterArgs &a, cudaStream_t st) {
  const int np_in = (a.do_moments ? a.dim + 1 : 0) + (a.do_weights ? 1 : 0);
  // partial planes: moments 0..dim then weights (dim+1)
  dim3 g1(a.nchunk, a.K, np_in);
  if (a.do_moments && !a.do_weights) g1.z = a.dim + 1;
  const int nk = (a.m + 31) / 32;
  if (nk <= 1)
    cluster_partial_kernel<1><<<g1, kRedThreads, 0, st>>>(a);
  else if (nk <= 2)
    cluster_partial_kernel<2><<<g1, kRedThreads, 0, st>>>(a);
  else if (nk <= 4)
    cluster_partial_kernel<4><<<g1, kRedThreads, 0, st>>>(a);
  else
    cluster_partial_kernel<8><<<g1, kRedThreads, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int np_out = (a.do_weights ? 1 : 0) + (a.do_moments ? a.dim : 0);
  cluster_final_kernel<<<dim3(a.K, np_out), kRedThreads, 0, st>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- rho
__global__ void rho_final_kernel(const double *part, int n, Ctl *ctl, double nent) {
  __shared__ double sm[1024 / 32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  s = wsum(s);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
    const double rho = ctl->rho_coeff * t / nent;  // :109
    ctl->rho = rho;
    ctl->inv_rho = (float)(1.0 / rho);
    ctl->inv_rho_l2 = (float)(1.4426950408889634 / rho);  // log2(e)/rho
    if (!(rho > 0.0) || !isfinite(rho)) ctl_fail(ctl, 3);
  }
}

cudaError_t launch_rho_final(const double *part, int n, Ctl *ctl, double nent, cudaStream_t st) {
  rho_final_kernel<<<1, 1024, 0, st>>>(part, n, ctl, nent);
  return cudaGetLastError();
}

// sharded update, rho over all shards: this shard's {sum |C|, entries} into
// xbuf for the exchange, then rho from the exchanged totals
__global__ void rho_local_kernel(const double *part, int n, double nent, double *xbuf) {
  __shared__ double sm[1024 / 32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  s = wsum(s);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
    xbuf[0] = t;
    xbuf[1] = nent;
  }
}

__global__ void rho_set_kernel(const double *xbuf, Ctl *ctl) {
  const double rho = ctl->rho_coeff * xbuf[0] / xbuf[1];
  ctl->rho = rho;
  ctl->inv_rho = (float)(1.0 / rho);
  ctl->inv_rho_l2 = (float)(1.4426950408889634 / rho);
  if (!(rho > 0.0) || !isfinite(rho)) ctl_fail(ctl, 3);
}

cudaError_t launch_rho_local(const double *part, int n, double nent, double *xbuf, cudaStream_t st) {
  rho_local_kernel<<<1, 1024, 0, st>>>(part, n, nent, xbuf);
  return cudaGetLastError();
}

cudaError_t launch_rho_set(const double *xbuf, Ctl *ctl, cudaStream_t st) {
  rho_set_kernel<<<1, 1, 0, st>>>(xbuf, ctl);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- residuals
// part: 4 doubles per CTA (obj, primres, dualres, obj-after-support-update)
// xmode 0: finalise; 1: this shard's three sums into xbuf (for the exchange
// between shards); 2: finalise from the exchanged totals in xbuf
__global__ void resid_final_kernel(const double *part, int n, Ctl *ctl, double *slot, int iter,
                                   int obj_from_slot3, int xmode, double *xbuf) {
  if (iter >= ctl->stop_iter) return;
  if (xmode == 2) {
    if (threadIdx.x == 0) {
      const double N = ctl->global_size;
      slot[0] = iter + 1;
      slot[1] = xbuf[0] * (ctl->rho / N);  // :312-314, this shard's rho as in the reference
      slot[2] = xbuf[1] / N;
      slot[3] = xbuf[2] / N;
    }
    return;
  }
  __shared__ double sm[3][1024 / 32];
  double o = 0.0, p = 0.0, d = 0.0;
  const int oi = obj_from_slot3 ? 3 : 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    o += part[(size_t)i * 4 + oi];
    p += part[(size_t)i * 4 + 1];
    d += part[(size_t)i * 4 + 2];
  }
  o = wsum(o);
  p = wsum(p);
  d = wsum(d);
  if ((threadIdx.x & 31) == 0) {
    sm[0][threadIdx.x >> 5] = o;
    sm[1][threadIdx.x >> 5] = p;
    sm[2][threadIdx.x >> 5] = d;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double to = 0.0, tp = 0.0, td = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      to += sm[0][w];
      tp += sm[1][w];
      td += sm[2][w];
    }
    if (xmode == 1) {
      xbuf[0] = to;
      xbuf[1] = tp;
      xbuf[2] = td;
      return;
    }
    const double N = ctl->global_size;
    slot[0] = iter + 1;
    slot[1] = to * (ctl->rho / N);  // :312-314
    slot[2] = tp / N;
    slot[3] = td / N;
  }
}

cudaError_t launch_resid_final(const double *part, int n, Ctl *ctl, double *trace_slot, int iter,
                               bool obj_from_slot3, cudaStream_t st, int xmode, double *xbuf) {
  resid_final_kernel<<<1, 1024, 0, st>>>(part, n, ctl, trace_slot, iter, obj_from_slot3 ? 1 : 0, xmode,
                                         xbuf);
  return cudaGetLastError();
}

// sharded update: out[i] = sum over the shards' buffers in shard order
__global__ void shard_sum_kernel(ShardBufs b, size_t n, double *out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int r = 0; r < b.n; ++r) s += b.p[r][i];
    out[i] = s;
  }
}

cudaError_t launch_shard_sum(const ShardBufs &b, size_t n, double *out, cudaStream_t st) {
  const unsigned nb = (unsigned)std::min<size_t>((n + 255) / 256, 1024);
  shard_sum_kernel<<<nb ? nb : 1, 256, 0, st>>>(b, n, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- centroids
__global__ void centroid_to_f32_kernel(const double *cw64, const double *cs64, float *cw32,
                                       float *cs32, int K, int m, int dim, int MP, int DS) {
  const int l = blockIdx.x;
  for (int k = threadIdx.x; k < MP; k += blockDim.x) {
    cw32[(size_t)l * MP + k] = k < m ? (float)cw64[(size_t)l * m + k] : 0.f;
    if (cs32)
      for (int t = 0; t < DS; ++t)
        cs32[((size_t)l * MP + k) * DS + t] =
            (k < m && t < dim) ? (float)cs64[((size_t)l * m + k) * dim + t] : 0.f;
  }
}

cudaError_t launch_centroid_to_f32(const double *cw64, const double *cs64, float *cw32,
                                   float *cs32, int K, int m, int dim, int MP, int DS,
                                   cudaStream_t st) {
  centroid_to_f32_kernel<<<K, 256, 0, st>>>(cw64, cs64, cw32, cs32, K, m, dim, MP, DS);
  return cudaGetLastError();
}

}  // namespace d2g
