// Plain FP64 form of the B-ADMM centroid update.
//
// The reference's loop structure (src/d2/centroid_Bregman.c:95-318) moved to
// the GPU as it stands: FP64 throughout, the reference layout (column-major
// str x m_i blocks at str*p_str_cum[i]), C, X, Y, Z and Z0 all materialised
// in HBM, and one grid-wide kernel per reference step.  It is the FP64
// parity path and the "plain per-step GPU" denominator of the batched form's
// speed-up; per iteration it moves ~136 B per plan entry against the fused
// kernel's 16 B and runs its exp() in FP64.
#include <math.h>

#include "d2g_internal.cuh"

namespace d2g {

constexpr int kPT = 256;

static inline unsigned grid_for(long long n) {
  long long b = (n + kPT - 1) / kPT;
  if (b > 152LL * 64) b = 152LL * 64;  // grid-stride beyond 64 blocks per SM
  return (unsigned)(b < 1 ? 1 : b);
}

#define GRID_STRIDE(i, n) \
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n); i += (long long)gridDim.x * blockDim.x)

__device__ __forceinline__ double dwsum(double v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ground cost, centroid_util.c:8-36 / blas_like64.c:199-230 (histograms: the
// phase's own cost matrix, dense = flat copy, sparse = row by bin id)
__device__ __forceinline__ double plain_cost_at(const PlainArgs &a, long long c, int k) {
  const int i = a.col_inst[c];
  const int l = a.label[i];
  if (a.metric == D2_EUCLIDEAN_L2) {
    const double *A = a.cs64 + ((size_t)l * a.str + k) * a.dim;
    const double *B = a.supp + (size_t)c * a.dim;
    double s = 0.0;
    for (int t = 0; t < a.dim; ++t) s += (A[t] - B[t]) * (A[t] - B[t]);
    return s;
  }
  if (a.metric == D2_WORD_EMBED) {
    const double *A = a.cs64 + ((size_t)l * a.str + k) * a.dim;
    const int sym = a.sym[c];
    double s = 0.0;
    if (sym < 0) {
      for (int t = 0; t < a.dim; ++t) s += A[t] * A[t];
    } else {
      const double *v = a.vocab + (size_t)sym * a.dim;
      for (int t = 0; t < a.dim; ++t) s += (A[t] - v[t]) * (A[t] - v[t]);
    }
    return s;
  }
  if (a.metric == D2_N_GRAM) {  // blas_like64.c:232-242
    const int *A = a.csym + ((size_t)l * a.str + k) * a.dim;
    const int *B = a.sym + (size_t)c * a.dim;
    double s = 0.0;
    for (int t = 0; t < a.dim; ++t) s += a.dist[(size_t)A[t] * a.vocab_size + B[t]];
    return s;
  }
  if (a.metric == D2_HISTOGRAM) {
    const long long j = c - a.cum[i];
    return a.dist[(size_t)j * a.str + k];
  }
  return a.dist[(size_t)a.sym[c] * a.vocab_size + k];  // D2_SPARSE_HISTOGRAM
}

__global__ void plain_cost_kernel(const PlainArgs a, int scale) {
  const double rho = scale ? a.ctl->rho : 1.0;
  GRID_STRIDE(e, a.nent) {
    const long long c = e / a.str;
    const int k = (int)(e - c * a.str);
    const double v = plain_cost_at(a, c, k);
    a.C[e] = scale ? v / rho : v;
  }
}

__global__ void plain_abs_partial(const PlainArgs a) {
  __shared__ double sm[kPT / 32];
  double s = 0.0;
  GRID_STRIDE(e, a.nent) s += fabs(a.C[e]);
  s = dwsum(s);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kPT / 32; ++w) t += sm[w];
    a.part[blockIdx.x] = t;
  }
}

__global__ void plain_div_rho(const PlainArgs a) {
  const double rho = a.ctl->rho;
  GRID_STRIDE(e, a.nent) a.C[e] /= rho;  // :110
}

__global__ void plain_init_kernel(const PlainArgs a) {  // :116-128
  GRID_STRIDE(e, a.nent) {
    const long long c = e / a.str;
    const int k = (int)(e - c * a.str);
    const int i = a.col_inst[c];
    if (a.reinit[i] == 1) a.Z[e] = a.w[c] * a.cw64[(size_t)a.label[i] * a.str + k];
    a.Y[e] = 0.0;
  }
}

__global__ void plain_step1a(const PlainArgs a) {  // :155-157
  if (a.iter >= a.ctl->stop_iter) return;
  GRID_STRIDE(e, a.nent) a.X[e] = a.Z[e] * exp(-(a.C[e] + a.Y[e])) + 1e-9;
}

__global__ void plain_step1b(const PlainArgs a) {  // cnorm + grms, :158-159
  if (a.iter >= a.ctl->stop_iter) return;
  GRID_STRIDE(c, a.col) {
    double *x = a.X + (size_t)c * a.str;
    double s = 0.0;
    for (int k = 0; k < a.str; ++k) s += x[k];
    if (!(s > 0.0)) ctl_fail(a.ctl, 4);
    const double w = a.w[c];
    for (int k = 0; k < a.str; ++k) {
      x[k] /= s;
      x[k] *= w;
    }
  }
}

__global__ void plain_step2a(const PlainArgs a) {  // :164-167
  if (a.iter >= a.ctl->stop_iter) return;
  GRID_STRIDE(e, a.nent) {
    a.Z0[e] = a.Z[e];
    a.Z[e] = a.X[e] * exp(a.Y[e]) + 1e-9;
  }
}

__global__ void plain_step2b(const PlainArgs a) {  // rnorm + gcms per instance, :168-171
  if (a.iter >= a.ctl->stop_iter) return;
  GRID_STRIDE(t, (long long)a.size * a.str) {
    const int i = (int)(t / a.str), k = (int)(t - (long long)i * a.str);
    double *z = a.Z + (size_t)a.cum[i] * a.str + k;
    const int mi = a.p_str[i];
    double s = 0.0;
    for (int j = 0; j < mi; ++j) s += z[(size_t)j * a.str];
    if (!(s > 0.0)) ctl_fail(a.ctl, 5);
    const double cw = a.cw64[(size_t)a.label[i] * a.str + k];
    for (int j = 0; j < mi; ++j) {
      z[(size_t)j * a.str] /= s;
      z[(size_t)j * a.str] *= cw;
    }
    a.zr[t] = s;
  }
}

__global__ void plain_step3(const PlainArgs a) {  // :175
  if (a.iter >= a.ctl->stop_iter) return;
  GRID_STRIDE(e, a.nent) a.Y[e] += a.X[e] - a.Z[e];
}

// step 5 per-instance moments: sum_j X[k,j] * (support_j[t]) and sum_j X[k,j]
__global__ void plain_moments(const PlainArgs a) {  // :201-212, :233-247
  if (a.iter >= a.ctl->stop_iter) return;
  GRID_STRIDE(t, (long long)a.size * a.str) {
    const int i = (int)(t / a.str), k = (int)(t - (long long)i * a.str);
    const long long c0 = a.cum[i];
    const double *x = a.X + (size_t)c0 * a.str + k;
    const int mi = a.p_str[i];
    double *out = a.xmom + (size_t)i * (a.dim + 1) * a.str + k;
    double rs = 0.0;
    for (int j = 0; j < mi; ++j) rs += x[(size_t)j * a.str];
    out[(size_t)a.dim * a.str] = rs;
    for (int d = 0; d < a.dim; ++d) {
      double s = 0.0;
      for (int j = 0; j < mi; ++j) {
        const double sv = a.metric == D2_WORD_EMBED ? a.vocab[(size_t)a.sym[c0 + j] * a.dim + d]
                                                    : a.supp[(size_t)(c0 + j) * a.dim + d];
        s += x[(size_t)j * a.str] * sv;
      }
      out[(size_t)d * a.str] = s;
    }
  }
}

__global__ void plain_check_partial(const PlainArgs a) {  // :300-305
  if (a.iter >= a.ctl->stop_iter) return;
  __shared__ double sm[3][kPT / 32];
  double o = 0.0, p = 0.0, d = 0.0;
  GRID_STRIDE(e, a.nent) {
    o += a.C[e] * a.X[e];
    const double xd = a.X[e] - a.Z[e];
    const double zd = a.Z0[e] - a.Z[e];
    a.X[e] = xd;
    a.Z0[e] = zd;
    p += fabs(xd);
    d += fabs(zd);
  }
  o = dwsum(o);
  p = dwsum(p);
  d = dwsum(d);
  if ((threadIdx.x & 31) == 0) {
    sm[0][threadIdx.x >> 5] = o;
    sm[1][threadIdx.x >> 5] = p;
    sm[2][threadIdx.x >> 5] = d;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double to = 0.0, tp = 0.0, td = 0.0;
    for (int w = 0; w < kPT / 32; ++w) {
      to += sm[0][w];
      tp += sm[1][w];
      td += sm[2][w];
    }
    a.part[(size_t)blockIdx.x * 4 + 0] = to;
    a.part[(size_t)blockIdx.x * 4 + 1] = tp;
    a.part[(size_t)blockIdx.x * 4 + 2] = td;
  }
}

cudaError_t plain_cost(const PlainArgs &a, cudaStream_t st) {
  if (a.metric == D2_EUCLIDEAN_L2 || a.metric == D2_WORD_EMBED || a.metric == D2_N_GRAM || a.iter < 0) {
    plain_cost_kernel<<<grid_for(a.nent), kPT, 0, st>>>(a, a.iter >= 0 ? 1 : 0);
  }
  return cudaGetLastError();
}

// a.iter < 0: initial cost (histograms included), then rho; C /= rho
cudaError_t plain_rho(const PlainArgs &a, cudaStream_t st) {
  const unsigned nb = grid_for(a.nent);
  plain_abs_partial<<<nb, kPT, 0, st>>>(a);
  cudaError_t e = launch_rho_final(a.part, (int)nb, a.ctl, (double)a.nent, st);
  if (e != cudaSuccess) return e;
  plain_div_rho<<<grid_for(a.nent), kPT, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t plain_init(const PlainArgs &a, cudaStream_t st) {
  plain_init_kernel<<<grid_for(a.nent), kPT, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t plain_iter_steps(const PlainArgs &a, bool update, cudaStream_t st) {
  const unsigned ne = grid_for(a.nent);
  plain_step1a<<<ne, kPT, 0, st>>>(a);
  plain_step1b<<<grid_for(a.col), kPT, 0, st>>>(a);
  plain_step2a<<<ne, kPT, 0, st>>>(a);
  plain_step2b<<<grid_for((long long)a.size * a.str), kPT, 0, st>>>(a);
  plain_step3<<<ne, kPT, 0, st>>>(a);
  if (update) plain_moments<<<grid_for((long long)a.size * a.str), kPT, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t plain_check(const PlainArgs &a, cudaStream_t st) {
  plain_check_partial<<<grid_for(a.nent), kPT, 0, st>>>(a);
  return cudaGetLastError();
}

unsigned plain_check_blocks(long long nent) { return grid_for(nent); }

int plain_launches_per_iter(bool update, bool check) {
  return 5 + 2 + (update ? 1 + 2 + 1 : 0) + (check ? 2 : 0);
}

}  // namespace d2g
