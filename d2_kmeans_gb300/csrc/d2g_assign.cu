// Exact transport costs for the assignment step: the host side of
// emd_kernel.cu.
//
// d2g_emd_pairs is the batched form of the reference's d2_match_by_distmat
// (src/d2/solver_mosek.cc:61-226) as d2_compute_distance calls it
// (src/d2/clustering.c:33-122): for each requested (row object, column
// object) pair, the exact optimal transport cost between the two discrete
// distributions, with the ground cost built the way the reference builds it
// for the phase's metric: squared Euclidean distances of the supports
// (_dpdist2, src/utils/blas_like64.c:199-208) or the phase's bin-to-bin
// cost matrix (histograms, sparse histograms).
#include <float.h>
#include <math.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "d2g_internal.cuh"

namespace d2g {
d2g_config cfg_snapshot();
namespace {

// a device allocation released on scope exit
struct DevMem {
  void *p = nullptr;
  ~DevMem() {
    if (p) cudaFree(p);
  }
  template <class T>
  T *get() const {
    return (T *)p;
  }
};

template <class T>
int upload(DevMem &d, const T *h, size_t n, cudaStream_t st) {
  if (!h || n == 0) return D2G_OK;
  D2G_CUDA(cudaMalloc(&d.p, n * sizeof(T)));
  D2G_CUDA(cudaMemcpyAsync(d.p, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
  return D2G_OK;
}

struct SideHost {
  std::vector<size_t> cum;
  size_t col = 0;
  int max_str = 0;
};

int side_layout(const d2g_dists *s, SideHost &h) {
  if (!s || (!s->p_str && s->str <= 0 && s->size > 0) || (s->size > 0 && !s->p_w)) return D2G_E_INVAL;
  h.cum.resize(s->size);
  size_t c = 0;
  int mx = 0;
  for (size_t i = 0; i < s->size; ++i) {
    const int k = s->p_str ? s->p_str[i] : s->str;
    if (k < 0) return D2G_E_INVAL;
    h.cum[i] = c;
    c += (size_t)k;
    mx = std::max(mx, k);
  }
  h.col = c;
  h.max_str = mx;
  return D2G_OK;
}

}  // namespace
}  // namespace d2g

using namespace d2g;

extern "C" int d2g_emd_pairs(int metric_type, int dim, const d2g_dists *rows, const d2g_dists *cols,
                             const double *dist_mat, int vocab_size, size_t npairs,
                             const int *pair_row, const int *pair_col, double *cost, int *pivots) {
  const bool euclid = metric_type == D2_EUCLIDEAN_L2;
  const bool table = metric_type == D2_HISTOGRAM || metric_type == D2_SPARSE_HISTOGRAM;
  if (!euclid && !table) {
    set_error("d2g_emd_pairs: metric type without an exact-transport path");
    return D2G_E_UNSUPPORTED;
  }
  if (npairs == 0) return D2G_OK;
  if (!pair_row || !pair_col || !cost) return D2G_E_INVAL;
  if (euclid && (dim < 1 || dim > 7)) {
    set_error("d2g_emd_pairs: Euclidean supports of dimension 1..7");
    return D2G_E_UNSUPPORTED;
  }
  if (table && (!dist_mat || vocab_size <= 0)) return D2G_E_INVAL;
  SideHost R, Cc;
  int rc = side_layout(rows, R);
  if (rc) return rc;
  rc = side_layout(cols, Cc);
  if (rc) return rc;
  if (euclid && ((R.col && !rows->p_supp) || (Cc.col && !cols->p_supp))) return D2G_E_INVAL;
  for (size_t p = 0; p < npairs; ++p)
    if (pair_row[p] < 0 || (size_t)pair_row[p] >= rows->size || pair_col[p] < 0 ||
        (size_t)pair_col[p] >= cols->size)
      return D2G_E_INVAL;
  if (table) {  // every key inside the cost matrix
    auto keys_ok = [&](const d2g_dists *s, const SideHost &h) {
      if (s->p_supp_sym) {
        for (size_t e = 0; e < h.col; ++e)
          if (s->p_supp_sym[e] < 0 || s->p_supp_sym[e] >= vocab_size) return false;
        return true;
      }
      return h.max_str <= vocab_size;
    };
    if (!keys_ok(rows, R) || !keys_ok(cols, Cc)) {
      set_error("d2g_emd_pairs: a bin id outside the cost matrix");
      return D2G_E_INVAL;
    }
  }
  const int nmax = ((R.max_str + Cc.max_str + 31) / 32) * 32;
  if (nmax > 8192) {
    set_error("d2g_emd_pairs: more than 8192 supports in one pair");
    return D2G_E_UNSUPPORTED;
  }
  if (emd_slice(nmax, euclid ? EMD_EUCLID : EMD_TABLE, dim) > 220 * 1024) {
    set_error("d2g_emd_pairs: a pair too large for one warp's shared memory");
    return D2G_E_UNSUPPORTED;
  }

  cudaStream_t st = 0;
  float tscale = 0.f;
  DevMem rw, rcum, rstr, rsupp, rsym, cw, ccum, cstr, csupp, csym, T64, T32, pr, pc, out, piv;
  rc = upload(rw, rows->p_w, R.col, st);
  if (!rc) rc = upload(rcum, R.cum.data(), R.cum.size(), st);
  if (!rc && rows->p_str) rc = upload(rstr, rows->p_str, rows->size, st);
  if (!rc && euclid) rc = upload(rsupp, rows->p_supp, R.col * dim, st);
  if (!rc && table && rows->p_supp_sym) rc = upload(rsym, rows->p_supp_sym, R.col, st);
  if (!rc) rc = upload(cw, cols->p_w, Cc.col, st);
  if (!rc) rc = upload(ccum, Cc.cum.data(), Cc.cum.size(), st);
  if (!rc && cols->p_str) rc = upload(cstr, cols->p_str, cols->size, st);
  if (!rc && euclid) rc = upload(csupp, cols->p_supp, Cc.col * dim, st);
  if (!rc && table && cols->p_supp_sym) rc = upload(csym, cols->p_supp_sym, Cc.col, st);
  if (!rc && table) {
    const size_t vv = (size_t)vocab_size * vocab_size;
    std::vector<float> t32(vv);
    double mx = 0.0;
    for (size_t e = 0; e < vv; ++e) {
      t32[e] = (float)dist_mat[e];
      mx = std::max(mx, fabs(dist_mat[e]));
    }
    tscale = (float)mx;
    rc = upload(T64, dist_mat, vv, st);
    if (!rc) rc = upload(T32, t32.data(), vv, st);
    if (!rc) D2G_CUDA(cudaStreamSynchronize(st));  // t32 leaves scope
  }
  if (!rc) rc = upload(pr, pair_row, npairs, st);
  if (!rc) rc = upload(pc, pair_col, npairs, st);
  if (rc) return rc;
  D2G_CUDA(cudaMalloc(&out.p, npairs * sizeof(double)));
  D2G_CUDA(cudaMalloc(&piv.p, npairs * sizeof(int)));

  EmdArgs a{};
  a.mode = euclid ? EMD_EUCLID : EMD_TABLE;
  a.dim = dim;
  a.rw = rw.get<double>();
  a.rcum = rcum.get<size_t>();
  a.rstr = rstr.get<int>();
  a.rfix = rows->str;
  a.rsupp = rsupp.get<double>();
  a.rsym = rsym.get<int>();
  a.cw = cw.get<double>();
  a.ccum = ccum.get<size_t>();
  a.cstr = cstr.get<int>();
  a.cfix = cols->str;
  a.csupp = csupp.get<double>();
  a.csym = csym.get<int>();
  a.T32 = T32.get<float>();
  a.T64 = T64.get<double>();
  a.V = vocab_size;
  a.tscale = tscale;
  a.prow = pr.get<int>();
  a.pcol = pc.get<int>();
  a.npairs = (long long)npairs;
  a.out = out.get<double>();
  a.piv = piv.get<int>();
  a.nmax = nmax;
  a.max_piv = 64 * nmax + 1024;
  D2G_CUDA(launch_emd(a, st));
  std::vector<int> hp(npairs);
  D2G_CUDA(cudaMemcpyAsync(cost, out.p, npairs * sizeof(double), cudaMemcpyDeviceToHost, st));
  D2G_CUDA(cudaMemcpyAsync(hp.data(), piv.p, npairs * sizeof(int), cudaMemcpyDeviceToHost, st));
  D2G_CUDA(cudaStreamSynchronize(st));
  if (pivots) memcpy(pivots, hp.data(), npairs * sizeof(int));
  for (size_t p = 0; p < npairs; ++p)
    if (hp[p] < 0) {
      set_error("d2g_emd_pairs: a pair did not reach an optimal basis");
      return D2G_E_NUMERIC;
    }
  return D2G_OK;
}

// ------------------------------------------------------------------------
// The assignment step on the reference's structures: d2_compute_distance,
// d2_labeling, d2_labeling_prep (Elkan's triangle-inequality pruning) and
// d2_labeling_post (src/d2/clustering.c:33-376), every distance an exact
// transport cost from emd_kernel.cu.  Distances are batched: d2_labeling
// sends all size x k pairs at once; the pruned labeling keeps the
// reference's per-instance order of decisions (which distances it computes,
// the bounds it writes) and runs it in waves - each instance advances
// through its centroid loop until it needs a distance, the wave's pairs go
// to the GPU together, and the results let every instance continue.

namespace d2g {
namespace {

// one phase of one mph, on the device (weights, prefix sums, counts,
// supports or bin ids)
struct DevPhase {
  DevMem w, cum, str, supp, sym;
  DevMem tup;     // n-gram phases: the distinct tuples [ntup * dim]; sym holds each support's tuple
  int ntup = 0;
  // what the copy was made from
  const void *kw = nullptr, *ks = nullptr, *ky = nullptr;
  size_t size = 0, col = 0;
  int max_str = 0, dim = 0, metric = -1;
  std::vector<int> h_str;
  std::vector<size_t> h_cum;
};

int upload_phase(const sph *s, size_t size, DevPhase &d, cudaStream_t st) {
  d = DevPhase();
  std::vector<size_t> cum(size);
  d.h_str.resize(size);
  size_t c = 0;
  int mx = 0;
  for (size_t i = 0; i < size; ++i) {
    const int k = s->p_str ? s->p_str[i] : s->str;
    if (k < 0) return D2G_E_INVAL;
    cum[i] = s->p_str_cum ? s->p_str_cum[i] : c;
    d.h_str[i] = k;
    c = cum[i] + (size_t)k;
    mx = std::max(mx, k);
  }
  d.size = size;
  d.col = c;
  d.max_str = mx;
  d.h_cum = cum;
  d.dim = s->dim;
  d.metric = s->metric_type;
  int rc = upload(d.w, s->p_w, c, st);
  if (!rc) rc = upload(d.cum, cum.data(), size, st);
  if (!rc) rc = upload(d.str, d.h_str.data(), size, st);
  if (!rc && s->metric_type == D2_EUCLIDEAN_L2) rc = upload(d.supp, s->p_supp, c * (size_t)s->dim, st);
  const bool symbolic = s->metric_type == D2_SPARSE_HISTOGRAM || s->metric_type == D2_WORD_EMBED;
  if (!rc && s->metric_type == D2_N_GRAM) {
    // number the distinct symbol tuples; every support keyed by its tuple
    const int dim = s->dim, V = s->vocab_size;
    if (!s->p_supp_sym || V <= 0 || dim < 1) return D2G_E_INVAL;
    std::vector<int> key, tup;
    d.ntup = number_tuples(s->p_supp_sym, c, dim, V, key, tup);
    if (d.ntup < 0) {
      set_error("labeling: an n-gram symbol outside the alphabet");
      return D2G_E_INVAL;
    }
    rc = upload(d.sym, key.data(), c, st);
    if (!rc) rc = upload(d.tup, tup.data(), tup.size(), st);
  }
  if (!rc && symbolic) {
    if (!s->p_supp_sym || s->vocab_size <= 0) return D2G_E_INVAL;
    for (size_t e = 0; e < c; ++e)
      if (s->p_supp_sym[e] < 0 || s->p_supp_sym[e] >= s->vocab_size) {
        set_error("labeling: a word or bin id outside the vocabulary");
        return D2G_E_INVAL;
      }
    rc = upload(d.sym, s->p_supp_sym, c, st);
  }
  if (!rc) D2G_CUDA(cudaStreamSynchronize(st));
  d.kw = s->p_w;
  d.ks = s->p_supp;
  d.ky = s->p_supp_sym;
  return rc;
}

bool same_source(const DevPhase &d, const sph *s, size_t size) {
  if (d.kw != s->p_w || d.ks != s->p_supp || d.ky != s->p_supp_sym || d.size != size ||
      d.metric != s->metric_type || d.dim != s->dim)
    return false;
  for (size_t i = 0; i < size; ++i)
    if (d.h_str[i] != (s->p_str ? s->p_str[i] : s->str)) return false;
  return true;
}

// the ground-cost table of a histogram phase: cost(row bin r, column bin c)
// = dist_mat[c * V + r], the reference's column-major use of dist_mat
// (clustering.c:88-95, blas_like64.c:222-230)
struct DevTable {
  DevMem T32, T64;
  const double *src = nullptr;
  int V = 0;
  float scale = 0.f;
};

int upload_table(const double *dm, int V, DevTable &t, cudaStream_t st) {
  if (t.src == dm && t.V == V) return D2G_OK;
  t = DevTable();
  const size_t vv = (size_t)V * V;
  std::vector<double> t64(vv);
  std::vector<float> t32(vv);
  double mx = 0.0;
  for (int r = 0; r < V; ++r)
    for (int c = 0; c < V; ++c) {
      t64[(size_t)r * V + c] = dm[(size_t)c * V + r];
      t32[(size_t)r * V + c] = (float)dm[(size_t)c * V + r];
      mx = std::max(mx, fabs(dm[(size_t)c * V + r]));
    }
  t.scale = (float)mx;
  int rc = upload(t.T64, t64.data(), vv, st);
  if (!rc) rc = upload(t.T32, t32.data(), vv, st);
  if (!rc) D2G_CUDA(cudaStreamSynchronize(st));
  if (rc) return rc;
  t.src = dm;
  t.V = V;
  return D2G_OK;
}

// the FP64 vocabulary of a word-embedding phase on the device, and the FP32
// cost table of the centroids of the current call (built once per call:
// the centroids do not change between the waves of one labeling)
struct DevVocab {
  DevMem v;
  const double *src = nullptr;
  int V = 0, d = 0;
  DevMem T;
  unsigned long long tgen = 0;
  const double *tsrc = nullptr;
  float tscale = 0.f;
};

// T[(l * V + v) * m + k] = |c_{l,k} - vocab_v|^2 in FP32, difference form:
// the FP32 costs the simplex prices with for word-embedding phases (the FP64
// check recomputes the cells near zero from the FP64 data).  64 x 64 tiles
// of (support, word), 32 dimensions per step.
__global__ void __launch_bounds__(256) embed_label_table(const double *__restrict__ c, int m,
                                                         const double *__restrict__ vocab, int V,
                                                         int d, float *__restrict__ T) {
  __shared__ float cs[64][33], vs[64][33];
  const int l = blockIdx.z, k0 = blockIdx.y * 64, v0 = blockIdx.x * 64;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  for (int t0 = 0; t0 < d; t0 += 32) {
    for (int e = threadIdx.x; e < 64 * 32; e += 256) {
      const int r = e >> 5, t = e & 31, tt = t0 + t;
      const int k = k0 + r, v = v0 + r;
      cs[r][t] = (k < m && tt < d) ? (float)c[((size_t)l * m + k) * d + tt] : 0.f;
      vs[r][t] = (v < V && tt < d) ? (float)vocab[(size_t)v * d + tt] : 0.f;
    }
    __syncthreads();
#pragma unroll 4
    for (int t = 0; t < 32; ++t) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        a[i] = cs[ty + 16 * i][t];
        b[i] = vs[tx + 16 * i][t];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float df = a[i] - b[j];
          acc[i][j] = fmaf(df, df, acc[i][j]);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k = k0 + ty + 16 * i, v = v0 + tx + 16 * j;
      if (k < m && v < V) T[((size_t)l * V + v) * m + k] = acc[i][j];
    }
}

struct AssignCache {
  std::mutex mu;
  std::vector<DevPhase> data;  // per phase of the instance mph
  std::vector<DevTable> tables;
  std::vector<DevVocab> vocab;
  unsigned long long gen = 0;  // advanced by every public call
};
AssignCache g_assign;

// launch the pairs sel[] (indices into pa / pb) with the arguments a and add
// their costs to d[]; an n-gram phase (ngram_dim > 0) adds 2 * cost / dim,
// its cost per symbol counted twice (src/d2/clustering.c:112-115)
int run_pairs(EmdArgs a, const std::vector<int> &pa, const std::vector<int> &pb,
              const std::vector<size_t> &sel, std::vector<double> &d, cudaStream_t st,
              int ngram_dim = 0) {
  const size_t np = sel.size();
  if (np == 0) return D2G_OK;
  std::vector<int> qa(np), qb(np);
  for (size_t p = 0; p < np; ++p) {
    qa[p] = pa[sel[p]];
    qb[p] = pb[sel[p]];
  }
  DevMem dpa, dpb, out, piv;
  int rc = upload(dpa, qa.data(), np, st);
  if (!rc) rc = upload(dpb, qb.data(), np, st);
  if (rc) return rc;
  D2G_CUDA(cudaMalloc(&out.p, np * sizeof(double)));
  D2G_CUDA(cudaMalloc(&piv.p, np * sizeof(int)));
  a.prow = dpb.get<int>();
  a.pcol = dpa.get<int>();
  a.npairs = (long long)np;
  a.out = out.get<double>();
  a.piv = piv.get<int>();
  D2G_CUDA(launch_emd(a, st));
  std::vector<double> h(np);
  std::vector<int> hp(np);
  D2G_CUDA(cudaMemcpyAsync(h.data(), out.p, np * sizeof(double), cudaMemcpyDeviceToHost, st));
  D2G_CUDA(cudaMemcpyAsync(hp.data(), piv.p, np * sizeof(int), cudaMemcpyDeviceToHost, st));
  D2G_CUDA(cudaStreamSynchronize(st));
  for (size_t p = 0; p < np; ++p) {
    if (hp[p] < 0) {
      set_error("labeling: a transport problem did not reach an optimal basis");
      return D2G_E_NUMERIC;
    }
    d[sel[p]] += ngram_dim ? 2 * (h[p] / ngram_dim) : h[p];
  }
  return D2G_OK;
}

double max_sq_norm(const double *x, size_t count, int dim) {
  double mx = 0.0;
  for (size_t e = 0; e < count; ++e) {
    double s = 0.0;
    for (int t = 0; t < dim; ++t) s += x[e * dim + t] * x[e * dim + t];
    mx = std::max(mx, s);
  }
  return mx;
}

constexpr size_t kTableBytes = (size_t)2 << 30;  // FP32 cost table per launch, at most

// exact transport of (rows: B object pb[p], columns: A object pa[p]) for
// phase n, added to d[p]
int phase_pairs(const sph *sa, const DevPhase &A, const sph *sb, const DevPhase &B, DevTable *tab,
                DevVocab *voc, const std::vector<int> &pa, const std::vector<int> &pb,
                std::vector<double> &d, cudaStream_t st) {
  const size_t np = pa.size();
  if (np == 0) return D2G_OK;
  const int metric = sa->metric_type;
  EmdArgs a{};
  a.dim = sa->dim;
  a.rw = B.w.get<double>();
  a.rcum = B.cum.get<size_t>();
  a.rstr = B.str.get<int>();
  a.rsupp = B.supp.get<double>();
  a.rsym = nullptr;  // centroids of histogram phases are dense
  a.cw = A.w.get<double>();
  a.ccum = A.cum.get<size_t>();
  a.cstr = A.str.get<int>();
  a.csupp = A.supp.get<double>();
  a.nmax = ((A.max_str + B.max_str + 31) / 32) * 32;
  std::vector<size_t> all(np);
  for (size_t p = 0; p < np; ++p) all[p] = p;
  const bool big_euclid = metric == D2_EUCLIDEAN_L2 && sa->dim > 7;
  if (metric == D2_EUCLIDEAN_L2 && !big_euclid) {
    if (sa->dim < 1 || sb->dim != sa->dim) return D2G_E_INVAL;
    a.mode = EMD_EUCLID;
  } else if (metric == D2_HISTOGRAM || metric == D2_SPARSE_HISTOGRAM) {
    if (!sa->dist_mat || sa->vocab_size <= 0) return D2G_E_INVAL;
    int rc = upload_table(sa->dist_mat, sa->vocab_size, *tab, st);
    if (rc) return rc;
    a.mode = EMD_TABLE;
    a.T32 = tab->T32.get<float>();
    a.T64 = tab->T64.get<double>();
    a.V = sa->vocab_size;
    a.tscale = tab->scale;
    a.csym = metric == D2_SPARSE_HISTOGRAM ? A.sym.get<int>() : nullptr;
    if (B.max_str > a.V || (metric == D2_HISTOGRAM && A.max_str > a.V)) {
      set_error("labeling: a histogram with more bins than the cost matrix");
      return D2G_E_INVAL;
    }
  } else if (metric == D2_WORD_EMBED || big_euclid) {
    // rows: R^d supports; columns: word ids into vocab_vec (_dpdist2_sym,
    // blas_like64.c:210-220) or, for Euclidean supports of d > 7, the column
    // supports themselves taken as the vocabulary
    const int dim = sa->dim, m = B.max_str;
    if (dim < 1 || sb->dim != dim || sb->metric_type != D2_EUCLIDEAN_L2 || !sb->p_supp) return D2G_E_INVAL;
    if (metric == D2_WORD_EMBED && (!sa->vocab_vec || sa->vocab_size <= 0)) return D2G_E_INVAL;
    for (size_t i = 0; i < B.size; ++i)
      if (B.h_str[i] != m) {
        set_error("labeling: row objects of unequal support sizes in a table-cost phase");
        return D2G_E_UNSUPPORTED;
      }
    a.mode = EMD_EMBED;
    a.tm = m;
    const double cn = max_sq_norm(sb->p_supp, B.col, dim);
    if (metric == D2_WORD_EMBED) {
      const int V = sa->vocab_size;
      if (voc->src != sa->vocab_vec || voc->V != V || voc->d != dim) {
        *voc = DevVocab();
        int rc = upload(voc->v, sa->vocab_vec, (size_t)V * dim, st);
        if (rc) return rc;
        voc->src = sa->vocab_vec;
        voc->V = V;
        voc->d = dim;
      }
      if (voc->tgen != g_assign.gen || voc->tsrc != sb->p_supp) {
        voc->T = DevMem();
        D2G_CUDA(cudaMalloc(&voc->T.p, B.size * (size_t)V * m * sizeof(float)));
        dim3 grid((V + 63) / 64, (m + 63) / 64, (unsigned)B.size);
        embed_label_table<<<grid, 256, 0, st>>>(B.supp.get<double>(), m, voc->v.get<double>(), V, dim,
                                                voc->T.get<float>());
        D2G_CUDA(cudaGetLastError());
        const double vn = max_sq_norm(sa->vocab_vec, V, dim);
        voc->tscale = (float)((sqrt(cn) + sqrt(vn)) * (sqrt(cn) + sqrt(vn)));
        voc->tgen = g_assign.gen;
        voc->tsrc = sb->p_supp;
      }
      a.T32 = voc->T.get<float>();
      a.V = V;
      a.vocab = voc->v.get<double>();
      a.tscale = voc->tscale;
      a.csym = A.sym.get<int>();
    } else {
      // chunks of instances whose supports' table fits kTableBytes
      const double vn = max_sq_norm(sa->p_supp, A.col, dim);
      a.tscale = (float)((sqrt(cn) + sqrt(vn)) * (sqrt(cn) + sqrt(vn)));
      a.csym = nullptr;
      const std::vector<size_t> &cum = A.h_cum;
      std::vector<size_t> order(all);
      std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return pa[x] < pa[y]; });
      const size_t vmax = std::max<size_t>(kTableBytes / (B.size * (size_t)m * sizeof(float)), (size_t)A.max_str);
      size_t i = 0;
      while (i < order.size()) {
        const size_t base = cum[pa[order[i]]];
        size_t j = i;
        while (j < order.size() && cum[pa[order[j]]] + A.h_str[pa[order[j]]] - base <= vmax) ++j;
        const size_t last = pa[order[j - 1]];
        const int V = (int)(cum[last] + A.h_str[last] - base);
        DevMem T;
        D2G_CUDA(cudaMalloc(&T.p, B.size * (size_t)V * m * sizeof(float)));
        dim3 grid((V + 63) / 64, (m + 63) / 64, (unsigned)B.size);
        embed_label_table<<<grid, 256, 0, st>>>(B.supp.get<double>(), m, A.supp.get<double>() + base * dim,
                                                V, dim, T.get<float>());
        D2G_CUDA(cudaGetLastError());
        EmdArgs c = a;
        c.T32 = T.get<float>();
        c.V = V;
        c.vocab = A.supp.get<double>() + base * dim;
        c.key_off = base;
        if (c.nmax > 8192 || emd_slice(c.nmax, c.mode, c.dim) > 220 * 1024) {
          set_error("labeling: a pair too large for one warp's shared memory");
          return D2G_E_UNSUPPORTED;
        }
        c.max_piv = 64 * c.nmax + 1024;
        std::vector<size_t> sel(order.begin() + i, order.begin() + j);
        int rc = run_pairs(c, pa, pb, sel, d, st);
        if (rc) return rc;
        i = j;
      }
      return D2G_OK;
    }
  } else if (metric == D2_N_GRAM) {
    // costs between the distinct centroid tuples (rows) and the distinct
    // instance tuples (columns), _dpdist_symbolic (blas_like64.c:232-242) with
    // the instance phase's alphabet and symbol cost
    const int dim = sa->dim, V = sa->vocab_size;
    if (dim < 1 || sb->dim != dim || !sa->dist_mat || V <= 0 || !sb->p_supp_sym) return D2G_E_INVAL;
    const size_t cells = (size_t)B.ntup * A.ntup;
    if (cells * 12 > ((size_t)4 << 30)) {
      set_error("labeling: n-gram tuple cost table above 4 GiB");
      return D2G_E_UNSUPPORTED;
    }
    DevMem dist, T64, T32;
    int rc = upload(dist, sa->dist_mat, (size_t)V * V, st);
    if (rc) return rc;
    D2G_CUDA(cudaMalloc(&T64.p, cells * sizeof(double)));
    D2G_CUDA(cudaMalloc(&T32.p, cells * sizeof(float)));
    D2G_CUDA(launch_ngram_pair_table(B.tup.get<int>(), B.ntup, A.tup.get<int>(), A.ntup, dim, V,
                                     dist.get<double>(), T64.get<double>(), T32.get<float>(), st));
    double mx = 0.0;
    for (size_t e = 0; e < (size_t)V * V; ++e) mx = std::max(mx, fabs(sa->dist_mat[e]));
    a.mode = EMD_TABLE;
    a.T32 = T32.get<float>();
    a.T64 = T64.get<double>();
    a.V = A.ntup;
    a.tscale = (float)(dim * mx);  // bounds every tuple cost
    a.rsym = B.sym.get<int>();
    a.csym = A.sym.get<int>();
    if (a.nmax > 8192 || emd_slice(a.nmax, a.mode, a.dim) > 220 * 1024) {
      set_error("labeling: a pair too large for one warp's shared memory");
      return D2G_E_UNSUPPORTED;
    }
    a.max_piv = 64 * a.nmax + 1024;
    return run_pairs(a, pa, pb, all, d, st, dim);
  } else {
    set_error("labeling: metric type without an exact-transport path");
    return D2G_E_UNSUPPORTED;
  }
  if (a.nmax > 8192 || emd_slice(a.nmax, a.mode, a.dim) > 220 * 1024) {
    set_error("labeling: a pair too large for one warp's shared memory");
    return D2G_E_UNSUPPORTED;
  }
  a.max_piv = 64 * a.nmax + 1024;
  return run_pairs(a, pa, pb, all, d, st);
}

// distances of pairs (A object pa[p], B object pb[p]) as d2_compute_distance
// returns them: sqrt of the phase costs' sum (phases in order), 0 if <= 0.
// A = the instances when cache_a (their device copy is kept across calls).
int pair_distances(mph *A, mph *B, int selected_phase, const std::vector<int> &pa,
                   const std::vector<int> &pb, std::vector<double> &out, bool cache_a) {
  const size_t np = pa.size();
  out.assign(np, 0.0);
  if (np == 0) return D2G_OK;
  if (A->s_ph != B->s_ph) return D2G_E_INVAL;
  cudaStream_t st = 0;
  std::lock_guard<std::mutex> lk(g_assign.mu);
  if (cache_a && g_assign.data.size() < (size_t)A->s_ph) g_assign.data.resize(A->s_ph);
  if (g_assign.tables.size() < (size_t)A->s_ph) g_assign.tables.resize(A->s_ph);
  if (g_assign.vocab.size() < (size_t)A->s_ph) g_assign.vocab.resize(A->s_ph);
  for (int n = 0; n < A->s_ph; ++n) {
    if (selected_phase >= 0 && n != selected_phase) continue;
    const sph *sa = A->ph + n, *sb = B->ph + n;
    DevPhase localA, devB;
    DevPhase *dA = &localA;
    int rc;
    if (cache_a) {
      dA = &g_assign.data[n];
      rc = same_source(*dA, sa, A->size) ? D2G_OK : upload_phase(sa, A->size, *dA, st);
    } else {
      rc = upload_phase(sa, A->size, localA, st);
    }
    if (!rc) rc = upload_phase(sb, B->size, devB, st);
    if (!rc) rc = phase_pairs(sa, *dA, sb, devB, &g_assign.tables[n], &g_assign.vocab[n], pa, pb, out, st);
    if (rc) return rc;
  }
  for (size_t p = 0; p < np; ++p) out[p] = out[p] <= 0.0 ? 0.0 : sqrt(out[p]);
  return D2G_OK;
}

// a public call starts: tables built for earlier centroids are stale
void new_call() {
  std::lock_guard<std::mutex> lk(g_assign.mu);
  ++g_assign.gen;
}

double wall_seconds() {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

// Elkan's per-instance loop (clustering.c:177-224) as a resumable state:
// advance() runs the reference's decisions until the next distance it needs
struct ElkanInst {
  int i, init_label, jj, j, stage;  // stage 0: test j; 1: 3a pending; 2: 3b test; 3: 3b pending
  double minv;
  int need;
};

}  // namespace
}  // namespace d2g

extern "C" {
// The reference's driver owns these (src/d2/clustering.c:21-24); the weak
// definitions let libd2g.so load without it.
__attribute__((weak)) int d2_alg_type = 0;  // D2_CENTROID_BADMM
}

namespace d2g {
namespace {
constexpr double kTimeBudgetRatio = 2000.0;  // clustering.c:20

bool elkan_advance(ElkanInst &s, int k, const double *L, const double *U, const double *c,
                   const char *r) {
  while (s.j < k) {
    if (s.stage == 0) {
      const int j = s.j;
      if (!((j != s.jj || s.init_label < 0) && *U > L[j] && *U > c[(size_t)j * k + s.jj] / 2.)) {
        ++s.j;
        continue;
      }
      if (*r == 1) {  // 3a: the bound is stale, compute d(i, jj)
        s.need = s.jj;
        s.stage = 1;
        return true;
      }
      s.minv = *U;
      s.stage = 2;
    }
    if (s.stage == 2) {  // 3b
      const int j = s.j;
      if ((s.minv > L[j] || s.minv > c[(size_t)j * k + s.jj] / 2.) && j != s.jj) {
        s.need = j;
        s.stage = 3;
        return true;
      }
      s.stage = 0;
      ++s.j;
      continue;
    }
    return false;  // stages 1 and 3 are resolved by elkan_apply
  }
  return false;
}

void elkan_apply(ElkanInst &s, double d, double *L, double *U, char *r) {
  if (s.stage == 1) {
    L[s.jj] = d;
    *U = d;
    s.minv = d;
    *r = 0;
    s.stage = 2;
  } else {  // stage 3
    L[s.j] = d;
    if (d < s.minv) {
      s.jj = s.j;
      s.minv = d;
      *U = d;
    }
    s.stage = 0;
    ++s.j;
  }
}

}  // namespace
}  // namespace d2g

extern "C" int d2g_compute_distances(mph *a, mph *b, int selected_phase, size_t npairs,
                                     const int *ia, const int *jb, double *out) {
  new_call();
  if (!a || !b || (npairs && (!ia || !jb || !out))) return D2G_E_INVAL;
  std::vector<int> pa(ia, ia + npairs), pb(jb, jb + npairs);
  for (size_t p = 0; p < npairs; ++p)
    if (pa[p] < 0 || (size_t)pa[p] >= a->size || pb[p] < 0 || (size_t)pb[p] >= b->size)
      return D2G_E_INVAL;
  std::vector<double> d;
  int rc = pair_distances(a, b, selected_phase, pa, pb, d, false);
  if (rc) return rc;
  memcpy(out, d.data(), npairs * sizeof(double));
  return D2G_OK;
}

extern "C" int d2g_labeling(mph *p_data, mph *centroids, var_mph *var_work, int selected_phase,
                            size_t *count_out, double *cost_out) {
  new_call();
  if (!p_data || !centroids || !var_work || !p_data->label) return D2G_E_INVAL;
  const size_t size = p_data->size, k = centroids->size;
  if (k == 0) return D2G_E_INVAL;
  std::vector<int> pa(size * k), pb(size * k);
  for (size_t i = 0; i < size; ++i)
    for (size_t j = 0; j < k; ++j) {
      pa[i * k + j] = (int)i;
      pb[i * k + j] = (int)j;
    }
  std::vector<double> d;
  int rc = pair_distances(p_data, centroids, selected_phase, pa, pb, d, true);
  if (rc) return rc;
  size_t count = 0;
  double cost = 0.0;
  int *label = p_data->label;
  for (size_t i = 0; i < size; ++i) {  // clustering.c:341-365
    double mind = -1;
    int jj = label[i] >= 0 ? label[i] : 0;
    for (size_t j = 0; j < k; ++j) {
      const double v = d[i * k + j];
      if (mind < 0 || v < mind) {
        mind = v;
        jj = (int)j;
      }
    }
    cost += mind * mind;
    if (label[i] == jj) {
      if (d2_alg_type == 0 && var_work->label_switch) var_work->label_switch[i] = 0;
    } else {
      label[i] = jj;
      if (d2_alg_type == 0 && var_work->label_switch) var_work->label_switch[i] = 1;
      ++count;
    }
  }
  if (count_out) *count_out = count;
  if (cost_out) *cost_out = cost;
  return D2G_OK;
}

extern "C" int d2g_labeling_prep(mph *p_data, mph *centroids, var_mph *var_work, int selected_phase,
                                 size_t *count_out, size_t *dist_count_out) {
  new_call();
  if (!p_data || !centroids || !var_work || !p_data->label) return D2G_E_INVAL;
  trieq *tr = &var_work->tr;
  if (!tr->l || !tr->u || !tr->s || !tr->c || !tr->r) return D2G_E_INVAL;
  const size_t size = p_data->size;
  const int k = (int)centroids->size;
  if (k <= 0) return D2G_E_INVAL;
  size_t count = 0, dist_count = 0;
  // step 1 (clustering.c:148-172): pairwise centroid distances, s = half the nearest
  for (int i = 0; i < k; ++i) tr->s[i] = DBL_MAX;
  for (size_t e = 0; e < (size_t)k * k; ++e) tr->c[e] = 0;
  {
    std::vector<int> pa, pb;
    for (int i = 0; i < k; ++i)
      for (int j = i + 1; j < k; ++j) {
        pa.push_back(i);
        pb.push_back(j);
      }
    std::vector<double> d;
    int rc = pair_distances(centroids, centroids, selected_phase, pa, pb, d, false);
    if (rc) return rc;
    for (size_t p = 0; p < pa.size(); ++p) {  // in the reference's (i, j) order
      const int i = pa[p], j = pb[p];
      const double v = d[p];
      ++dist_count;
      tr->c[(size_t)i * k + j] = v;
      tr->c[i + (size_t)j * k] = v;
      if (tr->s[i] > v / 2.f) tr->s[i] = v / 2.f;
      if (tr->s[j] > v / 2.f) tr->s[j] = v / 2.f;
    }
  }
  if (d2_alg_type == 0 && var_work->label_switch)
    for (size_t i = 0; i < size; ++i) var_work->label_switch[i] = 0;
  // steps 2-3 in waves
  int *label = p_data->label;
  std::vector<ElkanInst> act;
  for (size_t i = 0; i < size; ++i)
    if (label[i] < 0 || tr->u[i] > tr->s[label[i]]) {
      ElkanInst s{};
      s.i = (int)i;
      s.init_label = label[i];
      s.jj = label[i] >= 0 ? label[i] : 0;
      s.j = 0;
      s.stage = 0;
      act.push_back(s);
    }
  std::vector<ElkanInst> next;
  std::vector<int> pa, pb;
  std::vector<double> d;
  while (!act.empty()) {
    next.clear();
    pa.clear();
    pb.clear();
    for (ElkanInst &s : act) {
      double *L = tr->l + (size_t)s.i * k;
      if (elkan_advance(s, k, L, tr->u + s.i, tr->c, tr->r + s.i)) {
        pa.push_back(s.i);
        pb.push_back(s.need);
        next.push_back(s);
      } else if (s.jj != s.init_label) {  // clustering.c:226-231
        label[s.i] = s.jj;
        if (d2_alg_type == 0 && var_work->label_switch) var_work->label_switch[s.i] = 1;
        ++count;
      }
    }
    if (next.empty()) break;
    int rc = pair_distances(p_data, centroids, selected_phase, pa, pb, d, true);
    if (rc) return rc;
    dist_count += pa.size();
    for (size_t p = 0; p < next.size(); ++p) {
      ElkanInst &s = next[p];
      elkan_apply(s, d[p], tr->l + (size_t)s.i * k, tr->u + s.i, tr->r + s.i);
    }
    act.swap(next);
  }
  if (count_out) *count_out = count;
  if (dist_count_out) *dist_count_out = dist_count;
  return D2G_OK;
}

extern "C" int d2g_labeling_post(mph *p_data, mph *c_old, mph *c_new, var_mph *var_work,
                                 int selected_phase) {
  new_call();
  if (!p_data || !c_old || !c_new || !var_work || !p_data->label) return D2G_E_INVAL;
  trieq *tr = &var_work->tr;
  if (!tr->l || !tr->u || !tr->r) return D2G_E_INVAL;
  const int k = (int)c_old->size;
  std::vector<int> idx(k);
  for (int i = 0; i < k; ++i) idx[i] = i;
  std::vector<double> dc;
  // d_changes[i] = d2_compute_distance(c_new, i, c_old, i) (clustering.c:300-303)
  int rc = pair_distances(c_new, c_old, selected_phase, idx, idx, dc, false);
  if (rc) return rc;
  for (size_t j = 0; j < p_data->size; ++j) {  // :305-310
    double *L = tr->l + j * k;
    for (int i = 0; i < k; ++i) L[i] = std::max(L[i] - dc[i], 0.0);
    tr->u[j] += dc[p_data->label[j]];
    tr->r[j] = 1;
  }
  return D2G_OK;
}

// The reference's own entry points (include/d2/clustering.h), same
// signatures; a failure is reported through d2g_last_error and, for the
// counting functions, a return of (size_t)-1.  Like the reference, the
// labelings set the global time_budget for the next centroid update from
// their own wall time (clustering.c:245, :372).
extern "C" double d2_compute_distance(mph *a, size_t i, mph *b, size_t j, int selected_phase,
                                      var_mph *var_work, size_t index_task) {
  (void)var_work;
  (void)index_task;
  const int ia = (int)i, jb = (int)j;
  double out = 0.0;
  return d2g_compute_distances(a, b, selected_phase, 1, &ia, &jb, &out) ? NAN : out;
}

extern "C" size_t d2_labeling(mph *p_data, mph *centroids, var_mph *var_work, int selected_phase) {
  size_t count = 0;
  const double t0 = wall_seconds();
  if (d2g_labeling(p_data, centroids, var_work, selected_phase, &count, nullptr)) return (size_t)-1;
  if (!cfg_snapshot().keep_time_budget)
    time_budget = kTimeBudgetRatio * (wall_seconds() - t0) / p_data->num_of_labels;
  return count;
}

extern "C" size_t d2_labeling_prep(mph *p_data, mph *centroids, var_mph *var_work,
                                   int selected_phase) {
  size_t count = 0;
  const double t0 = wall_seconds();
  if (d2g_labeling_prep(p_data, centroids, var_work, selected_phase, &count, nullptr))
    return (size_t)-1;
  if (!cfg_snapshot().keep_time_budget) time_budget = kTimeBudgetRatio * (wall_seconds() - t0);
  return count;
}

extern "C" size_t d2_labeling_post(mph *p_data, mph *c_old, mph *c_new, var_mph *var_work,
                                   int selected_phase) {
  return d2g_labeling_post(p_data, c_old, c_new, var_work, selected_phase) ? (size_t)-1 : 0;
}
