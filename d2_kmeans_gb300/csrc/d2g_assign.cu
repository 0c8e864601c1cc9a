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
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "d2g_internal.cuh"

namespace d2g {
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
    for (size_t e = 0; e < vv; ++e) t32[e] = (float)dist_mat[e];
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
