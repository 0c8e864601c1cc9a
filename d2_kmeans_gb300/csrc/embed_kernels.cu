// Word-embedding phase (D2_WORD_EMBED) of the batched form.
//
// Ground costs (src/d2/centroid_util.c:22-24 -> blas_like64.c:210-220):
// C[k, j] = |c_{l,k} - v_{s_j}|^2 for the token id s_j of column j.  All
// costs of cluster l come from one table over the vocabulary,
//   T[l][v][k] = |c_{l,k}|^2 + |v|^2 - 2 <c_{l,k}, v>      (clamped at 0),
// a (k*m) x V x d contraction; the plan kernel reads C as T[l][s_j][0..m).
//
// Support update (centroid_Bregman.c:229-263): with the X of the update
// iteration stored by the plan kernel,
//   W[l][v][k]   = sum over columns of cluster l with token v of X[k, col]
//   num[l][k][t] = sum_v W[l][v][k] * vocab[v][t],   den[l][k] = sum_v W[l][v][k]
//   c_supp[l][k] = num / den
// W is gathered in a fixed order from per-(cluster, token) occurrence lists;
// the vocabulary sum runs in FP32 over chunks of the vocabulary and the
// chunks are combined in FP64.
#include "d2g_internal.cuh"

namespace d2g {

constexpr int kTile = 64;   // output tile (rows x columns)
constexpr int kTK = 16;     // contraction slice staged in shared memory

// T[l][v][k] for rows r = l*m + k of the centroid matrix (K*m x d) and
// vocabulary rows v (V x d); 256 threads, 4 x 4 outputs each.
__global__ void __launch_bounds__(256) cost_table_kernel(const float *__restrict__ cs, int nrows,
                                                         const float *__restrict__ vocab, int V,
                                                         int d, const float *__restrict__ cnorm,
                                                         const float *__restrict__ vnorm, int m,
                                                         int MP, float *__restrict__ T) {
  __shared__ float As[kTK][kTile + 4];  // [t][row]
  __shared__ float Bs[kTK][kTile + 4];  // [t][v]
  const int r0 = blockIdx.y * kTile, v0 = blockIdx.x * kTile;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[4][4] = {};
  for (int t0 = 0; t0 < d; t0 += kTK) {
    for (int i = threadIdx.x; i < kTK * kTile; i += 256) {
      const int rr = i / kTK, tt = i % kTK;
      const int row = r0 + rr, vv = v0 + rr, t = t0 + tt;
      As[tt][rr] = (row < nrows && t < d) ? cs[(size_t)row * d + t] : 0.f;
      Bs[tt][rr] = (vv < V && t < d) ? vocab[(size_t)vv * d + t] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int tt = 0; tt < kTK; ++tt) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        a[i] = As[tt][ty * 4 + i];
        b[i] = Bs[tt][tx * 4 + i];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int row = r0 + ty * 4 + i;
    if (row >= nrows) continue;
    const int l = row / m, k = row - l * m;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int v = v0 + tx * 4 + j;
      if (v >= V) continue;
      const float c = cnorm[row] + vnorm[v] - 2.f * acc[i][j];
      T[((size_t)l * V + v) * MP + k] = fmaxf(c, 0.f);
    }
  }
}

// |row|^2 of a row-major matrix, FP32 from FP64 accumulation
__global__ void row_norms_kernel(const float *__restrict__ a, int n, int d, float *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int t = 0; t < d; ++t) {
    const double v = a[(size_t)i * d + t];
    s += v * v;
  }
  out[i] = (float)s;
}

// W[l][v][k]: one warp per occupied (cluster, token) pair, lanes over k.
__global__ void w_gather_kernel(const int *__restrict__ pair_key, const int *__restrict__ pair_ptr,
                                const int *__restrict__ occ_col, int npairs,
                                const float *__restrict__ X, int MP, int m, int V,
                                float *__restrict__ W) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= npairs) return;
  const int key = pair_key[warp];  // l * V + v
  const int b = pair_ptr[warp], e = pair_ptr[warp + 1];
  for (int k = lane; k < m; k += 32) {
    float s = 0.f;
    for (int o = b; o < e; ++o) s += X[(size_t)occ_col[o] * MP + k];
    W[(size_t)key * MP + k] = s;
  }
}

// Partial numerators / denominators over one vocabulary chunk:
// part[chunk][l][k][t] = sum_{v in chunk} W[l][v][k] * vocab1[v][t], t <= d
// (vocab1 has a trailing column of ones, so t = d is the denominator).
// grid (ceil((d+1)/64), K, nchunk); 256 threads; rows k (MP <= 64 per tile).
__global__ void __launch_bounds__(256) support_num_kernel(const float *__restrict__ W,
                                                          const float *__restrict__ vocab, int V,
                                                          int d, int MP, int chunk, int m,
                                                          float *__restrict__ part) {
  __shared__ float As[kTK][kTile + 4];  // [v][k]
  __shared__ float Bs[kTK][kTile + 4];  // [v][t]
  const int t0 = blockIdx.x * kTile, l = blockIdx.y, c = blockIdx.z;
  const int vb = c * chunk, ve = min(V, vb + chunk);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int d1 = d + 1;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < MP; k0 += kTile) {
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int v0 = vb; v0 < ve; v0 += kTK) {
      for (int i = threadIdx.x; i < kTK * kTile; i += 256) {
        const int vv = i / kTile, q = i % kTile;
        const int v = v0 + vv;
        As[vv][q] = (v < ve && k0 + q < MP) ? W[((size_t)l * V + v) * MP + k0 + q] : 0.f;
        const int t = t0 + q;
        Bs[vv][q] = (v < ve && t < d1) ? (t < d ? vocab[(size_t)v * d + t] : 1.f) : 0.f;
      }
      __syncthreads();
#pragma unroll
      for (int vv = 0; vv < kTK; ++vv) {
        float a[4], bb[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          a[i] = As[vv][ty * 4 + i];
          bb[i] = Bs[vv][tx * 4 + i];
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], bb[j], acc[i][j]);
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int k = k0 + ty * 4 + i;
      if (k >= m) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int t = t0 + tx * 4 + j;
        if (t < d1) part[(((size_t)c * gridDim.y + l) * MP + k) * d1 + t] = acc[i][j];
      }
    }
  }
}

// c_supp[l][k][t] = sum_chunks num / sum_chunks den, chunks in order, FP64.
// grid (K, ceil(m*d / 256)): one thread per (cluster, support, coordinate).
__global__ void support_final_kernel(const float *__restrict__ part, int nchunk, int K, int MP,
                                     int m, int d, double *__restrict__ cs64,
                                     float *__restrict__ cs32f, Ctl *ctl, int iter) {
  if (iter >= ctl->stop_iter) return;
  const int l = blockIdx.x;
  const int d1 = d + 1;
  const int i = blockIdx.y * blockDim.x + threadIdx.x;
  if (i < m * d) {
    const int k = i / d, t = i - k * d;
    double num = 0.0, den = 0.0;
    for (int c = 0; c < nchunk; ++c) {
      const float *p = part + (((size_t)c * K + l) * MP + k) * d1;
      num += (double)p[t];
      den += (double)p[d];
    }
    if (!(den > 0.0)) ctl_fail(ctl, 2);
    const double v = num / den;
    cs64[((size_t)l * m + k) * d + t] = v;
    cs32f[((size_t)l * m + k) * d + t] = (float)v;  // row-major (K*m) x d for the table GEMM
  }
}

// FP64 -> FP32 copy
__global__ void to_f32_kernel(const double *__restrict__ a, size_t n, float *__restrict__ b) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

cudaError_t launch_cost_table(const float *cs, int K, int m, const float *vocab, int V, int d,
                              float *cnorm, const float *vnorm, int MP, float *T, int gemm,
                              const float *vsplit, float *csplit, int *err, cudaStream_t st) {
  const int nrows = K * m;
  row_norms_kernel<<<(nrows + 255) / 256, 256, 0, st>>>(cs, nrows, d, cnorm);
  if (gemm == 0)
    return launch_cost_table_tc(cs, nrows, vsplit, V, d, cnorm, vnorm, m, MP, T, csplit, err, st);
  dim3 grid((V + kTile - 1) / kTile, (nrows + kTile - 1) / kTile);
  cost_table_kernel<<<grid, 256, 0, st>>>(cs, nrows, vocab, V, d, cnorm, vnorm, m, MP, T);
  return cudaGetLastError();
}

cudaError_t launch_vocab_norms(const float *vocab, int V, int d, float *vnorm, cudaStream_t st) {
  row_norms_kernel<<<(V + 255) / 256, 256, 0, st>>>(vocab, V, d, vnorm);
  return cudaGetLastError();
}

cudaError_t launch_to_f32(const double *a, size_t n, float *b, cudaStream_t st) {
  to_f32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a, n, b);
  return cudaGetLastError();
}

cudaError_t launch_embed_table(const EmbedArgs &e, cudaStream_t st) {
  return launch_cost_table(e.cs32f, e.K, e.m, e.vocab, e.V, e.d, e.cnorm, e.vnorm, e.MP, e.T, e.gemm,
                           e.vsplit, e.csplit, &e.ctl->err, st);
}

cudaError_t launch_embed_support(const EmbedArgs &e, cudaStream_t st) {
  cudaError_t err = cudaMemsetAsync(e.W, 0, (size_t)e.K * e.V * e.MP * sizeof(float), st);
  if (err != cudaSuccess) return err;
  if (e.npairs > 0)
    w_gather_kernel<<<(e.npairs * 32 + 255) / 256, 256, 0, st>>>(e.pair_key, e.pair_ptr, e.occ_col,
                                                                 e.npairs, e.X, e.MP, e.m, e.V, e.W);
  dim3 g2((e.d + 1 + kTile - 1) / kTile, e.K, e.nchunk);
  support_num_kernel<<<g2, 256, 0, st>>>(e.W, e.vocab, e.V, e.d, e.MP, e.chunk, e.m, e.part);
  support_final_kernel<<<dim3(e.K, (e.m * e.d + 255) / 256), 256, 0, st>>>(
      e.part, e.nchunk, e.K, e.MP, e.m, e.d, e.cs64, e.cs32f, e.ctl, e.iter);
  return cudaGetLastError();
}

}  // namespace d2g
