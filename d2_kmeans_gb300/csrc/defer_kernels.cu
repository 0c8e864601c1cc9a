// Deferred row normalisation of plans wider than one CTA (the plan kernel's
// PF_OUT_DEF / PF_IN_DEF modes).
//
// Step 2 of src/d2/centroid_Bregman.c:164-171 scales row k of a plan by
// c_w[label, k] / rowsum_k(Z'), Z' = X * exp(Y) + 1e-9.  A plan split over CS
// CTA slices needs every slice's row sums for that scale.  Instead of trading
// them inside the iteration (a cluster barrier per plan), each slice writes
// its partial row sums and stores Z' and U = Y + X; rowsum_combine_kernel adds
// the partials in rank order, writes the plan's normalised row sums (step 4's
// Zr, by slot) and the row scale; the next iteration's plan kernel applies the
// scale as it loads the plan: Z = Z' * scale, Y = U - Z.  The arithmetic per
// entry is that of the synchronous form: Z is the same product Z' * scale, Y
// gets X and -Z in two roundings instead of one.  plan_finalize_kernel
// applies the scale of the last iteration when the loop ends deferred.
//
// The pair passes of plan_pair.cuh leave every plan deferred the same way:
// pair_scale_kernel forms the scale of every plan from its raw row sums, and
// pair_finalize_kernel applies it where a single pass or the end follows.
#include "d2g_internal.cuh"

namespace d2g {

constexpr float kLog2eF = 1.4426950408889634f;  // Y is stored multiplied by log2(e)

// one block per wide plan {slot, slices holding columns, label, -}; MP <= 256
__global__ void __launch_bounds__(256) rowsum_combine_kernel(const int4 *__restrict__ wide,
                                                             const float *__restrict__ rowpart,
                                                             const float *__restrict__ cw32, int MP,
                                                             int m, float *__restrict__ rowsum_out,
                                                             float *__restrict__ rowsc,
                                                             const Ctl *ctl, int iter) {
  if (iter >= ctl->stop_iter) return;
  const int4 d = __ldg(wide + blockIdx.x);
  const int k = threadIdx.x, lane = k & 31, warp = k >> 5;
  float tot = 0.f;
  if (k < MP)
    for (int r = 0; r < d.y; ++r) tot += rowpart[((size_t)d.x * kMaxCluster + r) * MP + k];
  // the plan's total over its m rows: warps in index order
  __shared__ float ws[8];
  float v = k < m ? tot : 0.f;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) ws[warp] = v;
  __syncthreads();
  float rsum = 0.f;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) rsum += ws[i];
  if (k < MP) {
    rowsum_out[(size_t)d.x * MP + k] = tot * (1.f / rsum);
    rowsc[(size_t)d.x * MP + k] = k < m ? __ldg(cw32 + (size_t)d.z * MP + k) / tot : 0.f;
  }
}

// one block per (item, rank) slice of a bucket of wide plans
__global__ void __launch_bounds__(256) plan_finalize_kernel(float *__restrict__ Z,
                                                            float *__restrict__ Y,
                                                            const int *__restrict__ item_g0,
                                                            const int *__restrict__ item_ng, int cs,
                                                            int G, int S, int MP,
                                                            const int4 *__restrict__ grp_rec,
                                                            const float *__restrict__ rowsc,
                                                            const unsigned char *__restrict__ def_iter,
                                                            const Ctl *ctl) {
  const int last = ctl->iters_done - 1;
  if (last < 0 || !def_iter[last]) return;
  const int item = blockIdx.x / cs, rk = blockIdx.x - item * cs;
  const int g0 = item_g0[item] + rk * G;
  const int ng = min(G, item_ng[item] - rk * G);
  if (ng <= 0) return;
  const int slot = grp_rec[g0].x;
  const float *sc = rowsc + (size_t)slot * MP;
  const size_t base = (size_t)g0 * S * MP;
  const int n = ng * S * MP;
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const float z = Z[base + e] * sc[e & (MP - 1)];
    Z[base + e] = z;
    Y[base + e] = fmaf(-kLog2eF, z, Y[base + e]);
  }
}

// pair passes: one thread per (plan in packed order, 4 rows)
__global__ void pair_scale_kernel(const float *__restrict__ rawsum, const int *__restrict__ plan_slot,
                                  const int *__restrict__ plan_label, const float *__restrict__ cw32,
                                  long long n4, int MP, int m, float4 *__restrict__ rowsc, const Ctl *ctl,
                                  int iter, int nplans, int nlab) {
  if (iter >= ctl->stop_iter) return;
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n4) return;
  const long long e = i * 4;
  const int p = (int)(e / MP), k = (int)(e - (long long)p * MP);
  const int slot = __ldg(plan_slot + p), lab = __ldg(plan_label + p);
  // self-check: a slot outside the plans or a label outside the clusters
  if (slot < 0 || slot >= nplans || lab < 0 || lab >= nlab || (k & 3)) {
    ctl_fail((Ctl *)ctl, 9);
    return;
  }
  const float4 cw = __ldg((const float4 *)(cw32 + (size_t)lab * MP + k));
  const float4 r = *(const float4 *)(rawsum + (size_t)slot * MP + k);
  rowsc[i] = make_float4(k + 0 < m ? cw.x / r.x : 0.f, k + 1 < m ? cw.y / r.y : 0.f,
                         k + 2 < m ? cw.z / r.z : 0.f, k + 3 < m ? cw.w / r.w : 0.f);
}

// Z = Z' * scale, Y = U - Z over every packed column: one float4 (4 rows of a
// column) per thread; the plan of a group is grp_meta >> 4
__global__ void __launch_bounds__(256) pair_finalize_kernel(float4 *__restrict__ Z, float4 *__restrict__ Y,
                                                            const int *__restrict__ grp_meta, long long n4,
                                                            int S, int MP, const float *__restrict__ rowsc,
                                                            int nplans, int *err) {
  const long long per4 = (long long)S * MP / 4;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4;
       i += (long long)gridDim.x * blockDim.x) {
    const int p = __ldg(&grp_meta[i / per4]) >> 4;
    const int k0 = (int)((i * 4) % MP);
    if (p < 0 || p >= nplans) {  // self-check: a plan outside the phase
      atomicCAS(err, 0, 9);
      continue;
    }
    const float4 sc = __ldg((const float4 *)(rowsc + (size_t)p * MP + k0));
    float4 z = Z[i], y = Y[i];
    z.x *= sc.x;
    z.y *= sc.y;
    z.z *= sc.z;
    z.w *= sc.w;
    y.x = fmaf(-kLog2eF, z.x, y.x);
    y.y = fmaf(-kLog2eF, z.y, y.y);
    y.z = fmaf(-kLog2eF, z.z, y.z);
    y.w = fmaf(-kLog2eF, z.w, y.w);
    Z[i] = z;
    Y[i] = y;
  }
}

cudaError_t launch_pair_scale(const float *rawsum, const int *plan_slot, const int *plan_label,
                              const float *cw32, int nplans, int MP, int m, float *rowsc, const Ctl *ctl,
                              int iter, int nlab, cudaStream_t st) {
  const long long n4 = (long long)nplans * MP / 4;
  if (n4 <= 0) return cudaSuccess;
  pair_scale_kernel<<<(unsigned)((n4 + 255) / 256), 256, 0, st>>>(rawsum, plan_slot, plan_label, cw32, n4, MP,
                                                                  m, (float4 *)rowsc, ctl, iter, nplans, nlab);
  return cudaGetLastError();
}

cudaError_t launch_pair_finalize(float *Z, float *Y, const int *grp_meta, int ngroups, int S, int MP,
                                 const float *rowsc, int nplans, int *err, cudaStream_t st) {
  const long long n4 = (long long)ngroups * S * MP / 4;
  if (n4 <= 0) return cudaSuccess;
  long long blocks = (n4 + 255) / 256;
  if (blocks > 152LL * 32) blocks = 152LL * 32;
  pair_finalize_kernel<<<(unsigned)blocks, 256, 0, st>>>((float4 *)Z, (float4 *)Y, grp_meta, n4, S, MP, rowsc,
                                                         nplans, err);
  return cudaGetLastError();
}

cudaError_t launch_rowsum_combine(const int4 *wide, int nwide, const float *rowpart,
                                  const float *cw32, int MP, int m, float *rowsum_out,
                                  float *rowsc, const Ctl *ctl, int iter, cudaStream_t st) {
  if (nwide <= 0) return cudaSuccess;
  const int threads = MP < 32 ? 32 : MP;
  rowsum_combine_kernel<<<nwide, threads, 0, st>>>(wide, rowpart, cw32, MP, m, rowsum_out, rowsc,
                                                   ctl, iter);
  return cudaGetLastError();
}

cudaError_t launch_plan_finalize(float *Z, float *Y, const int *item_g0, const int *item_ng,
                                 int nitems, int cs, int G, int S, int MP, const int4 *grp_rec,
                                 const float *rowsc, const unsigned char *def_iter, const Ctl *ctl,
                                 cudaStream_t st) {
  if (nitems <= 0) return cudaSuccess;
  plan_finalize_kernel<<<nitems * cs, 256, 0, st>>>(Z, Y, item_g0, item_ng, cs, G, S, MP, grp_rec,
                                                    rowsc, def_iter, ctl);
  return cudaGetLastError();
}

}  // namespace d2g
