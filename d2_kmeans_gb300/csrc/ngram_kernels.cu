// N-gram phases (D2_N_GRAM): supports are tuples of `dim` symbols over an
// alphabet of V symbols with a V x V symbol cost.
//
// Ground cost (src/d2/centroid_util.c:31-33 -> _dpdist_symbolic,
// src/utils/blas_like64.c:232-242): centroid support k of cluster l against an
// instance support with symbols x_0..x_{dim-1},
//   C = sum_t dist[c_{l,k,t} * V + x_t].
// The batched form numbers the distinct instance tuples u = 0..U-1 and keeps
// one table per cluster, T[l][u][k] (FP32 of the FP64 sum), which the plan
// kernel reads row by row exactly as it reads a word-embedding phase's table.
//
// Support update (src/d2/centroid_Bregman.c:269-294, every updatePerLoops
// iterations after the first): with the plans Z of that iteration,
//   cnt[l][k][t][v] = sum over the columns of cluster l whose symbol at
//                     position t is v of Z[k, col]   (entries above 1e-10;
//                     accumulate_symbolic, include/d2/centroid_util.h:15-23)
//   c_{l,k,t}       = the first v minimising sum_u dist[v + u*V] * cnt[l][k][t][u]
//                     (minimize_symbolic, centroid_util.h:25-37: a column-major
//                     GEMM dist * cnt, then an argmin per column)
// The counts run per occurrence list (cluster, position, symbol) in a fixed
// column order: FP64 one column after the other in the FP64 form; FP32 over
// chunks of 32 columns and FP64 across chunks in the batched form.  The cost
// sums run over u in order with separately rounded products and sums, as the
// reference's BLAS computes them.  When the update iteration is the second of
// a pair pass, the batched plans are still deferred (Z' with one row scale
// per plan): the counts form Z = Z' * scale as they read, the product the
// pass that follows would store.
#include <cmath>
#include <map>
#include <unordered_map>

#include "d2g_internal.cuh"

namespace d2g {

int number_tuples(const int *sym, size_t count, int dim, int V, std::vector<int> &key,
                  std::vector<int> &tup) {
  key.resize(count);
  tup.clear();
  for (size_t e = 0; e < count * dim; ++e)
    if (sym[e] < 0 || sym[e] >= V) return -1;
  if (dim * std::log2((double)V) < 62.0) {  // a tuple as a base-V integer
    std::unordered_map<unsigned long long, int> id;
    id.reserve(1024);
    for (size_t e = 0; e < count; ++e) {
      unsigned long long code = 0;
      for (int t = 0; t < dim; ++t) code = code * (unsigned long long)V + (unsigned long long)sym[e * dim + t];
      auto it = id.emplace(code, (int)id.size());
      if (it.second) tup.insert(tup.end(), sym + e * dim, sym + (e + 1) * dim);
      key[e] = it.first->second;
    }
    return (int)id.size();
  }
  std::map<std::vector<int>, int> id;
  for (size_t e = 0; e < count; ++e) {
    std::vector<int> t(sym + e * dim, sym + (e + 1) * dim);
    auto it = id.emplace(t, (int)id.size());
    if (it.second) tup.insert(tup.end(), t.begin(), t.end());
    key[e] = it.first->second;
  }
  return (int)id.size();
}

// FP64 form: cnt[(l*m + k)*dim + t][v] from the list of key (l*dim + t)*V + v,
// one warp per list, lanes over the centroid supports k, the columns added
// one by one in list (reference) order.
__global__ void ngram_count64_kernel(const int *__restrict__ key, const int *__restrict__ ptr,
                                     const int *__restrict__ occ, int nlists, const double *__restrict__ Z,
                                     long long zstride, int m, int dim, int V, double *__restrict__ cnt,
                                     const Ctl *ctl, int iter) {
  if (iter >= ctl->stop_iter) return;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= nlists) return;
  const int kk = key[w];
  const int v = kk % V, lt = kk / V, t = lt % dim, l = lt / dim;
  const int b = ptr[w], e = ptr[w + 1];
  for (int k = lane; k < m; k += 32) {
    double s = 0.0;
    for (int o = b; o < e; ++o) {
      const double z = Z[(size_t)occ[o] * zstride + k];
      if (z > 1E-10) s += z;
    }
    cnt[(((size_t)l * m + k) * dim + t) * V + v] = s;
  }
}

// Batched form: one CTA per list.  Warp w takes the chunks w, w + 8, ... of
// kChunk columns; a chunk is summed in FP32 (its loads independent, so they
// overlap), the chunk sums in FP64; the 8 warps' sums are added in warp
// order.  The order is fixed, so the counts repeat bit for bit.
constexpr int kCountWarps = 8, kChunk = 32;
__global__ void __launch_bounds__(kCountWarps * 32) ngram_count32_kernel(
    const int *__restrict__ key, const int *__restrict__ ptr, const int *__restrict__ occ,
    const float *__restrict__ Z, long long zstride, int m, int dim, int V, double *__restrict__ cnt,
    const Ctl *ctl, int iter, const float *__restrict__ rowsc, const int *__restrict__ grp_meta, int S,
    int nplans) {
  if (iter >= ctl->stop_iter) return;
  __shared__ double part[kCountWarps][32];
  __shared__ int cols[kCountWarps][kChunk];
  __shared__ int plans[kCountWarps][kChunk];
  const int lst = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int kk = key[lst];
  const int v = kk % V, lt = kk / V, t = lt % dim, l = lt / dim;
  const int b = ptr[lst], e = ptr[lst + 1];
  const bool deferred = rowsc != nullptr;
  for (int k0 = 0; k0 < m; k0 += 32) {
    const int k = k0 + lane;
    double acc = 0.0;
    for (int c0 = b + warp * kChunk; c0 < e; c0 += kCountWarps * kChunk) {
      const int nc = min(kChunk, e - c0);
      __syncwarp();
      if (lane < nc) {
        const int c = occ[c0 + lane];
        cols[warp][lane] = c;
        if (deferred) {
          int p = __ldg(grp_meta + c / S) >> 4;
          if (p < 0 || p >= nplans) {  // self-check: a plan outside the phase
            ctl_fail((Ctl *)ctl, 9);
            p = 0;
          }
          plans[warp][lane] = p;
        }
      }
      __syncwarp();
      float s = 0.f;
      if (k < m) {
#pragma unroll 8
        for (int j = 0; j < nc; ++j) {
          float z = __ldg(Z + (size_t)cols[warp][j] * zstride + k);
          if (deferred) z *= __ldg(rowsc + (size_t)plans[warp][j] * zstride + k);
          s += z > 1E-10f ? z : 0.f;
        }
      }
      acc += (double)s;
    }
    part[warp][lane] = acc;
    __syncthreads();
    if (warp == 0 && k < m) {
      double tot = 0.0;
#pragma unroll
      for (int w = 0; w < kCountWarps; ++w) tot += part[w][lane];
      cnt[(((size_t)l * m + k) * dim + t) * V + v] = tot;
    }
    __syncthreads();
  }
}

// one warp per (cluster, support, position) column q = (l*m + k)*dim + t;
// lanes over candidate symbols r; the first minimum wins, as in the reference
__global__ void ngram_min_kernel(const double *__restrict__ cnt, int ncols, int V,
                                 const double *__restrict__ dist, int *__restrict__ csym,
                                 const Ctl *ctl, int iter) {
  if (iter >= ctl->stop_iter) return;
  const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (q >= ncols) return;
  const double *z = cnt + (size_t)q * V;
  double best = 0.0;
  int arg = -1;
  for (int r = lane; r < V; r += 32) {
    double s = 0.0;
    for (int u = 0; u < V; ++u) s = __dadd_rn(s, __dmul_rn(z[u], dist[(size_t)r + (size_t)u * V]));
    if (arg < 0 || s < best) {
      best = s;
      arg = r;
    }
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
    if (oa >= 0 && (arg < 0 || ob < best || (ob == best && oa < arg))) {
      best = ob;
      arg = oa;
    }
  }
  if (lane == 0) csym[q] = arg;
}

// T[l][u][k] = sum_t dist[csym[(l*m + k)*dim + t] * V + tup[u*dim + t]] for
// k < m, 0 in the padded rows k < MP
__global__ void ngram_table_kernel(const int *__restrict__ csym, const int *__restrict__ tup, int U,
                                   int K, int m, int MP, int dim, int V,
                                   const double *__restrict__ dist, float *__restrict__ T,
                                   const Ctl *ctl, int iter) {
  if (iter >= ctl->stop_iter) return;
  const long long n = (long long)K * U * MP;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i % MP);
    const long long lu = i / MP;
    const int u = (int)(lu % U), l = (int)(lu / U);
    float c = 0.f;
    if (k < m) {
      const int *cs = csym + ((size_t)l * m + k) * dim;
      const int *x = tup + (size_t)u * dim;
      double s = 0.0;
      for (int t = 0; t < dim; ++t) s += dist[(size_t)cs[t] * V + x[t]];
      c = (float)s;
    }
    T[i] = c;
  }
}

// Exact-transport costs of n-gram supports for the assignment step
// (src/d2/clustering.c:102-115): rows are the distinct centroid tuples, columns
// the distinct instance tuples, cost = sum_t dist[row symbol * V + column symbol]
// in FP64 and its FP32 rounding.
__global__ void ngram_pair_table_kernel(const int *__restrict__ rt, int Ur, const int *__restrict__ ct,
                                        int Uc, int dim, int V, const double *__restrict__ dist,
                                        double *__restrict__ T64, float *__restrict__ T32) {
  const long long n = (long long)Ur * Uc;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / Uc), c = (int)(i - (long long)r * Uc);
    double s = 0.0;
    for (int t = 0; t < dim; ++t) s += dist[(size_t)rt[(size_t)r * dim + t] * V + ct[(size_t)c * dim + t]];
    T64[i] = s;
    T32[i] = (float)s;
  }
}

cudaError_t launch_ngram_pair_table(const int *rt, int Ur, const int *ct, int Uc, int dim, int V,
                                    const double *dist, double *T64, float *T32, cudaStream_t st) {
  const long long n = (long long)Ur * Uc;
  long long nb = (n + 255) / 256;
  if (nb > 152LL * 32) nb = 152LL * 32;
  ngram_pair_table_kernel<<<(unsigned)(nb < 1 ? 1 : nb), 256, 0, st>>>(rt, Ur, ct, Uc, dim, V, dist,
                                                                       T64, T32);
  return cudaGetLastError();
}

cudaError_t launch_ngram_support(const NgramArgs &g, cudaStream_t st) {
  const size_t ncnt = (size_t)g.K * g.m * g.dim * g.V;
  cudaError_t e = cudaMemsetAsync(g.cnt, 0, ncnt * sizeof(double), st);
  if (e != cudaSuccess) return e;
  if (g.nlists > 0) {
    if (g.Z32)
      ngram_count32_kernel<<<g.nlists, kCountWarps * 32, 0, st>>>(g.key, g.ptr, g.occ, g.Z32, g.zstride, g.m,
                                                                  g.dim, g.V, g.cnt, g.ctl, g.iter, g.rowsc,
                                                                  g.grp_meta, g.S, g.nplans);
    else
      ngram_count64_kernel<<<(unsigned)(((long long)g.nlists * 32 + 255) / 256), 256, 0, st>>>(
          g.key, g.ptr, g.occ, g.nlists, g.Z64, g.zstride, g.m, g.dim, g.V, g.cnt, g.ctl, g.iter);
  }
  const int ncols = g.K * g.m * g.dim;
  ngram_min_kernel<<<(unsigned)(((long long)ncols * 32 + 255) / 256), 256, 0, st>>>(
      g.cnt, ncols, g.V, g.dist, g.csym, g.ctl, g.iter);
  return cudaGetLastError();
}

cudaError_t launch_ngram_table(const NgramArgs &g, cudaStream_t st) {
  const long long n = (long long)g.K * g.U * g.MP;
  long long nb = (n + 255) / 256;
  if (nb > 152LL * 32) nb = 152LL * 32;
  ngram_table_kernel<<<(unsigned)(nb < 1 ? 1 : nb), 256, 0, st>>>(g.csym, g.tup, g.U, g.K, g.m, g.MP,
                                                                   g.dim, g.V, g.dist, g.T, g.ctl,
                                                                   g.iter);
  return cudaGetLastError();
}

}  // namespace d2g
