// The reference-facing drop-in: d2_centroid_sphBregman and its companions
// with the signatures, globals and data layout of bobye/d2_kmeans
// (include/d2/clustering.h:223-230, src/d2/centroid_Bregman.c:17-325,
// src/d2/centroid_util.c:8-36), implemented on the resident d2g_phase API.
//
// Device state is kept per var_sphBregman work object (one per phase, as the
// reference's d2_allocate_work creates them) and reused across calls while
// the phase's shape and support sizes stay the same; weights, supports,
// labels and the warm-start plans are re-sent on every call, so a caller
// that edits its host arrays in place sees the same results as the reference.
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "d2g_internal.cuh"

namespace d2g {
d2g_config cfg_snapshot();
}

extern "C" {
// centroid_Bregman.c:17-22: the clustering and the k=1 "centroid" defaults
BADMM_options badmm_clu_options = {100, 2.0, 10};
BADMM_options badmm_cen_options = {2000, 1.0, 10};
BADMM_options *p_badmm_options = &badmm_clu_options;

// The reference's driver owns this global (src/d2/clustering.c:21); the weak
// definition lets libd2g.so load without that driver.
__attribute__((weak)) double time_budget = 1e300;
}

namespace {

struct DropinState {
  d2g_phase *ph = nullptr;
  int metric = -1, dim = -1, str = -1, K = -1, precision = -1;
  size_t size = 0, col = 0;
  std::vector<int> p_str;
  const void *p_w = nullptr, *p_supp = nullptr, *p_sym = nullptr, *dist = nullptr, *vocab = nullptr;
};

std::mutex g_mu;
std::unordered_map<const var_sphBregman *, DropinState> g_states;
// host work arrays allocated page-locked (cudaMallocHost), freed accordingly
std::unordered_set<void *> g_pinned;

// Z is copied back after every call: page-locked, the copy runs at the
// host link's full rate.  Falls back to malloc where pinning is refused.
void *alloc_pinned(size_t bytes) {
  void *p = nullptr;
  if (cudaMallocHost(&p, bytes) == cudaSuccess) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_pinned.insert(p);
    return p;
  }
  cudaGetLastError();
  return malloc(bytes);
}

void free_host(void *p) {
  if (!p) return;
  bool pinned = false;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    pinned = g_pinned.erase(p) > 0;
  }
  if (pinned)
    cudaFreeHost(p);
  else
    free(p);
}

int err(int code, const char *msg) {
  d2g::set_error(msg);
  return code;
}

}  // namespace

// The implementations live in namespace d2g so that this library's own outer
// loop (d2g_cluster.cu) reaches them directly, not through the exported
// names a program may define for itself.
namespace d2g {

int work_alloc_bregman(sph *ph, size_t size, var_sphBregman *w) {
  // centroid_Bregman.c:26-35: same host buffers and sizes
  if (!ph || !w || ph->str <= 0 || ph->col == 0 || size == 0) return err(D2G_E_INVAL, "bad work shape");
  const size_t nent = (size_t)ph->str * ph->col;
  w->X = (double *)malloc(nent * sizeof(double));
  w->Z = (double *)alloc_pinned(nent * sizeof(double));
  w->Xc = (double *)malloc(ph->col * sizeof(double));
  w->Zr = (double *)malloc((size_t)ph->str * size * sizeof(double));
  w->Y = (double *)malloc(nent * sizeof(double));
  if (!w->X || !w->Z || !w->Xc || !w->Zr || !w->Y) return err(D2G_E_NOMEM, "host work allocation");
  return D2G_OK;
}

int work_free_bregman(var_sphBregman *w) {
  if (!w) return D2G_E_INVAL;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_states.find(w);
    if (it != g_states.end()) {
      if (it->second.ph) d2g_phase_destroy(it->second.ph);
      g_states.erase(it);
    }
  }
  free(w->X);
  free_host(w->Z);
  free(w->Y);
  free(w->Xc);
  free(w->Zr);
  w->X = w->Z = w->Y = w->Xc = w->Zr = nullptr;
  return D2G_OK;
}

int centroid_update(mph *p_data, var_mph *var_work, int idx_ph, sph *c0, sph *c) {
  if (!p_data || !var_work || !c || idx_ph < 0 || idx_ph >= p_data->s_ph || !var_work->l_var_sphBregman)
    return err(D2G_E_INVAL, "bad arguments");
  if (!c0) {
    // :95-98 initialises c at random with d2_centroid_rands
    // (src/d2/centroid_rand.c:161-295): the program's own where it links one
    // (a program that links this library in place of centroid_Bregman.c keeps
    // centroid_rand.c), else this library's d2g_centroid_rands, which gives
    // the same result.  One process: there is no broadcast_centroids step.
    if (c->str != p_data->ph[idx_ph].str) return err(D2G_E_INVAL, "c->str differs from the phase's str");
    const int rc0 = d2g::centroid_rands(p_data, idx_ph, c);
    if (rc0) return rc0;
  } else {
    *c = *c0;  // :100 warm start
  }
  sph *dp = p_data->ph + idx_ph;
  var_sphBregman *bw = var_work->l_var_sphBregman + idx_ph;
  const BADMM_options *o = p_badmm_options;
  if (!o) return err(D2G_E_INVAL, "p_badmm_options is NULL");

  d2g_phase_desc d{};
  d.metric_type = dp->metric_type;
  d.dim = dp->dim;
  d.str = c->str;  // the centroid's support size (:102)
  d.size = p_data->size;
  d.p_str = dp->p_str;
  d.p_w = dp->p_w;
  d.p_supp = dp->p_supp;
  d.p_supp_sym = dp->p_supp_sym;
  d.vocab_vec = dp->vocab_vec;
  d.dist_mat = dp->dist_mat;
  d.vocab_size = dp->vocab_size;
  d.label = p_data->label;
  d.num_of_labels = p_data->num_of_labels;
  d.global_size = p_data->global_size;
  const d2g_config cfg = d2g::cfg_snapshot();

  std::lock_guard<std::mutex> lk(g_mu);
  DropinState &s = g_states[bw];
  const bool same = s.ph && s.metric == d.metric_type && s.dim == d.dim && s.str == d.str &&
                    s.K == d.num_of_labels && s.size == d.size && s.col == dp->col &&
                    s.precision == cfg.precision && s.p_w == d.p_w && s.p_supp == d.p_supp &&
                    s.p_sym == d.p_supp_sym && s.dist == d.dist_mat && s.vocab == d.vocab_vec &&
                    s.p_str.size() == d.size &&
                    memcmp(s.p_str.data(), d.p_str, d.size * sizeof(int)) == 0;
  int rc;
  if (!same) {
    if (s.ph) d2g_phase_destroy(s.ph);
    s = DropinState();
    rc = d2g_phase_create(&d, cfg.precision, &s.ph);
    if (rc) {
      g_states.erase(bw);
      return rc;
    }
    s.metric = d.metric_type;
    s.dim = d.dim;
    s.str = d.str;
    s.K = d.num_of_labels;
    s.size = d.size;
    s.col = dp->col;
    s.precision = cfg.precision;
    s.p_str.assign(d.p_str, d.p_str + d.size);
    s.p_w = d.p_w;
    s.p_supp = d.p_supp;
    s.p_sym = d.p_supp_sym;
    s.dist = d.dist_mat;
    s.vocab = d.vocab_vec;
  } else {
    rc = d2g_phase_refresh(s.ph, &d);
    if (rc) return rc;
  }

  const char *ls = var_work->label_switch;
  bool warm = false;
  if (ls)
    for (size_t i = 0; i < d.size && !warm; ++i) warm = ls[i] != 1;
  if (warm) {  // plans of unswitched instances carry over (:116-124)
    rc = d2g_phase_set_plans(s.ph, bw->Z);
    if (rc) return rc;
  }
  d2g_badmm_opts bo;
  bo.maxIters = o->maxIters;
  bo.rhoCoeff = o->rhoCoeff;
  bo.updatePerLoops = o->updatePerLoops;
  bo.time_budget = time_budget;
  rc = dp->metric_type == D2_N_GRAM ? d2g_badmm_run_sym(s.ph, &bo, c->p_w, c->p_supp_sym, ls)
                                    : d2g_badmm_run(s.ph, &bo, c->p_w, c->p_supp, ls);
  if (rc) return rc;
  rc = d2g_phase_get_plans(s.ph, bw->Z);
  if (rc) return rc;
  if (cfg.sync_scratch) {
    d2g_run_stats st;
    d2g_phase_stats(s.ph, &st);
    double *C = var_work->g_var ? var_work->g_var[idx_ph].C : nullptr;
    if (st.path == 1)
      rc = d2g_phase_get_scratch(s.ph, bw->X, bw->Y, C);
    else
      rc = d2g_phase_get_scratch(s.ph, nullptr, bw->Y, nullptr);
    if (rc) return rc;
  }
  if (cfg.verbose) {  // the reference's VPRINTF lines (:144, :147-148, :315)
    std::vector<size_t> cnt(d.num_of_labels, 0);
    for (size_t i = 0; i < d.size; ++i) ++cnt[d.label[i]];
    printf("\tlabel counts:");
    for (int l = 0; l < d.num_of_labels; ++l) printf("%zu ", cnt[l]);
    printf("\n\titer\tobj\t\tprimres\t\tdualres\t\tseconds\n");
    printf("\t----------------------------------------------------------------\n");
    d2g_run_stats st;
    d2g_phase_stats(s.ph, &st);
    int n = 0;
    d2g_phase_trace(s.ph, nullptr, 0, &n);
    std::vector<double> tr((size_t)4 * n);
    d2g_phase_trace(s.ph, tr.data(), n, &n);
    for (int i = 0; i < n; ++i) {
      const double secs = st.iterations ? st.total_ms * 1e-3 * tr[4 * i] / st.iterations : 0.0;
      printf("\t%d\t%f\t%f\t%f\t%f\n", (int)tr[4 * i], tr[4 * i + 1], tr[4 * i + 2], tr[4 * i + 3], secs);
    }
    fflush(stdout);
  }
  return D2G_OK;
}

}  // namespace d2g

extern "C" int d2_allocate_work_sphBregman(sph *ph, size_t size, var_sphBregman *w) {
  return d2g::work_alloc_bregman(ph, size, w);
}

extern "C" int d2_free_work_sphBregman(var_sphBregman *w) { return d2g::work_free_bregman(w); }

extern "C" int d2_centroid_sphBregman(mph *p_data, var_mph *var_work, int idx_ph, sph *c0, sph *c) {
  return d2g::centroid_update(p_data, var_work, idx_ph, c0, c);
}

extern "C" void calculate_distmat(sph *data_ph, int *label, size_t size, sph *c, double *C) {
  // centroid_util.c:8-36: histogram costs are fixed (nothing to do)
  if (!data_ph || !label || !c || !C || size == 0) {
    d2g::set_error("calculate_distmat: bad arguments");
    return;
  }
  const int mt = data_ph->metric_type;
  if (mt == D2_HISTOGRAM || mt == D2_SPARSE_HISTOGRAM) return;
  if (mt != D2_EUCLIDEAN_L2 && mt != D2_WORD_EMBED && mt != D2_N_GRAM) {
    d2g::set_error("calculate_distmat: unsupported metric type");
    return;
  }
  size_t K = 0;  // clusters referenced by the labels
  for (size_t i = 0; i < size; ++i) K = std::max(K, (size_t)(label[i] + 1));
  d2g::distmat_fp64(data_ph->dim, c->str, size, data_ph->p_str, mt, data_ph->p_supp,
                    data_ph->p_supp_sym, data_ph->vocab_vec, data_ph->vocab_size, label, c->p_supp,
                    K, C, data_ph->dist_mat, c->p_supp_sym);
}
