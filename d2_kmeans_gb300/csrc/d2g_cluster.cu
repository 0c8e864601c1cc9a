// The outer loop of AD2-clustering on this library: d2_clustering
// (src/d2/clustering.c:409-525) and d2_assignment (:528-548) with the GPU
// assignment step (d2g_assign.cu) and the GPU centroid update
// (d2g_dropin.cu).
//
// Same rounds as the reference: label (Elkan's pruned labeling when
// use_triangle), write the log files every tenth round, stop when fewer than
// 0.1 % of the instances changed label, copy the centroids (pruned form),
// update every selected phase's centroids, update the bounds; after the
// loop the pruned form labels once more without pruning.  The labelings set
// time_budget for the next update as the reference's do (clustering.c:245,
// :372) unless d2g_config.keep_time_budget is set; that rule makes the
// update depend on the labeling's wall time, so runs that must repeat bit
// for bit keep the budget fixed.
//
// Work arrays are this library's own: label_switch, the triangle bounds and
// one var_sphBregman per phase (the reference's d2_allocate_work also
// allocates str * (col + k * str) host doubles of cost scratch per phase,
// which nothing here reads).  Centroids not given (centroids->ph == NULL)
// are initialised by the program's own d2_centroid_rands
// (src/d2/centroid_rand.c:161-295, looked up with dlsym) into arrays laid
// out as d2_allocate_sph lays them out (src/d2/clustering_util.c:18-73).
#include <dlfcn.h>
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <vector>

#include "d2g_internal.cuh"

namespace d2g {
d2g_config cfg_snapshot();
int work_alloc_bregman(sph *ph, size_t size, var_sphBregman *w);
int work_free_bregman(var_sphBregman *w);
int centroid_update(mph *p_data, var_mph *var_work, int idx_ph, sph *c0, sph *c);
}

namespace {

constexpr double kTimeBudgetRatio = 2000.0;  // clustering.c:20

double now_s() {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

bool selected(int n, int sel) { return sel < 0 || n == sel; }

struct LoopWork {
  var_mph vw{};
  std::vector<var_sph> gv;
  std::vector<var_sphBregman> bw;
  std::vector<char> alloc;  // which phases hold a var_sphBregman
  std::vector<char> label_switch, r;
  std::vector<double> l, u, s, c;
};

int work_alloc(mph *p, LoopWork &w, bool tri, int sel) {
  const size_t size = p->size, k = p->num_of_labels;
  w.gv.assign(p->s_ph, var_sph{});
  w.bw.assign(p->s_ph, var_sphBregman{});
  w.alloc.assign(p->s_ph, 0);
  w.label_switch.assign(size, 0);
  w.vw.s_ph = p->s_ph;
  w.vw.g_var = w.gv.data();
  w.vw.l_var_sphBregman = w.bw.data();
  w.vw.label_switch = w.label_switch.data();
  if (tri) {  // clustering_util.c:218-228
    w.l.assign(size * k, 0.0);
    w.u.assign(size, DBL_MAX);
    w.s.assign(k, 0.0);
    w.c.assign(k * k, 0.0);
    w.r.assign(size, 1);
    w.vw.tr.l = w.l.data();
    w.vw.tr.u = w.u.data();
    w.vw.tr.s = w.s.data();
    w.vw.tr.c = w.c.data();
    w.vw.tr.r = w.r.data();
  }
  for (int n = 0; n < p->s_ph; ++n) {
    if (!selected(n, sel)) continue;
    const size_t cap = size > k ? size : k;
    int rc = d2g::work_alloc_bregman(p->ph + n, cap, &w.bw[n]);
    if (rc) return rc;
    w.alloc[n] = 1;
  }
  return D2G_OK;
}

void work_free(LoopWork &w) {
  for (size_t n = 0; n < w.bw.size(); ++n)
    if (w.alloc[n]) d2g::work_free_bregman(&w.bw[n]);
}

// d2_copy (clustering.c:253-285) of the centroids into arrays owned here
struct CentroidCopy {
  mph m{};
  std::vector<sph> ph;
  std::vector<std::vector<int>> p_str;
  std::vector<std::vector<size_t>> cum;
  std::vector<std::vector<double>> w, supp;
  std::vector<std::vector<int>> sym;
};

void copy_centroids(const mph *a, CentroidCopy &b) {
  b.ph.assign(a->s_ph, sph{});
  b.p_str.resize(a->s_ph);
  b.cum.resize(a->s_ph);
  b.w.resize(a->s_ph);
  b.supp.resize(a->s_ph);
  b.sym.resize(a->s_ph);
  for (int n = 0; n < a->s_ph; ++n) {
    const sph &s = a->ph[n];
    sph &d = b.ph[n];
    d = s;
    if (s.col == 0) continue;
    b.p_str[n].assign(s.p_str, s.p_str + a->size);
    b.cum[n].assign(s.p_str_cum, s.p_str_cum + a->size);
    b.w[n].assign(s.p_w, s.p_w + s.col);
    d.p_str = b.p_str[n].data();
    d.p_str_cum = b.cum[n].data();
    d.p_w = b.w[n].data();
    if (s.metric_type == D2_EUCLIDEAN_L2 && s.p_supp) {
      b.supp[n].assign(s.p_supp, s.p_supp + s.col * (size_t)s.dim);
      d.p_supp = b.supp[n].data();
    }
    if (s.metric_type == D2_N_GRAM && s.p_supp_sym) {  // the symbols; dist_mat is shared
      b.sym[n].assign(s.p_supp_sym, s.p_supp_sym + s.col * (size_t)s.dim);
      d.p_supp_sym = b.sym[n].data();
    }
  }
  b.m = *a;
  b.m.ph = b.ph.data();
}

// the log files of clustering.c:464-471, in d2_write's and d2_write_labels'
// formats (clustering_io.c:204-275)
void write_log(const char *log_file, const mph *c, const mph *p) {
  char name[1024];
  snprintf(name, sizeof name, "%s_c.d2", log_file);
  if (FILE *f = fopen(name, "w+")) {
    for (size_t i = 0; i < c->size; ++i)
      for (int j = 0; j < c->s_ph; ++j) {
        const sph &s = c->ph[j];
        if (s.col == 0) {
          fprintf(f, "%d\n0\n\n", s.dim);
          continue;
        }
        const int str = s.p_str[i];
        const size_t pos = s.p_str_cum[i];
        fprintf(f, "%d\n%d\n", s.dim, str);
        for (int k = 0; k < str; ++k) fprintf(f, "%lf ", s.p_w[pos + k]);
        fprintf(f, "\n");
        if (s.metric_type == D2_EUCLIDEAN_L2) {
          for (int k = 0; k < str; ++k) {
            for (int d = 0; d < s.dim; ++d) fprintf(f, "%lf ", s.p_supp[(pos + k) * s.dim + d]);
            fprintf(f, "\n");
          }
        } else if (s.metric_type == D2_WORD_EMBED || s.metric_type == D2_SPARSE_HISTOGRAM) {
          for (int k = 0; k < str; ++k) fprintf(f, "%d ", s.p_supp_sym[pos + k] + 1);
          fprintf(f, "\n");
        }
      }
    fclose(f);
  }
  snprintf(name, sizeof name, "%s.label", log_file);
  if (FILE *f = fopen(name, "w")) {
    for (size_t i = 0; i < p->size; ++i) fprintf(f, "%d\n", p->label[i]);
    fclose(f);
  }
}

// centroids->ph == NULL: arrays as d2_allocate_sph lays them out, filled by
// d2_centroid_rands (clustering.c:383-404): the program's own, else this
// library's d2g_centroid_rands
int init_centroids(mph *p, mph *c, int sel) {
  const int k = p->num_of_labels;
  c->s_ph = p->s_ph;
  c->size = k;
  c->ph = (sph *)calloc(p->s_ph, sizeof(sph));
  if (!c->ph) return D2G_E_NOMEM;
  for (int n = 0; n < p->s_ph; ++n) {
    const sph &s = p->ph[n];
    sph &d = c->ph[n];
    d.dim = s.dim;
    d.metric_type = s.metric_type % 7;  // D2_GROUP_SIZE: embeddings get Euclidean centroids
    if (!selected(n, sel)) continue;
    const size_t m = (size_t)k * s.str;
    d.str = d.max_str = s.str;
    d.max_col = m;
    d.p_str = (int *)calloc(k, sizeof(int));
    d.p_str_cum = (size_t *)calloc(k, sizeof(size_t));
    d.p_w = (double *)malloc(m * sizeof(double));
    if (d.metric_type == D2_EUCLIDEAN_L2) d.p_supp = (double *)malloc(m * (size_t)s.dim * sizeof(double));
    if (d.metric_type == D2_N_GRAM) d.p_supp_sym = (int *)malloc(m * (size_t)s.dim * sizeof(int));
    if (!d.p_str || !d.p_str_cum || !d.p_w || (d.metric_type == D2_EUCLIDEAN_L2 && !d.p_supp) ||
        (d.metric_type == D2_N_GRAM && !d.p_supp_sym))
      return D2G_E_NOMEM;
    const int rc = d2g::centroid_rands(p, n, &d);
    if (rc) return rc;
  }
  return D2G_OK;
}

}  // namespace

extern "C" int d2g_clustering(int num_of_clusters, int max_iter, mph *p_data, mph *centroids,
                              int selected_phase, int use_triangle, const char *log_file,
                              int *rounds) {
  if (!p_data || !centroids || num_of_clusters <= 0 || max_iter <= 0 || selected_phase >= p_data->s_ph)
    return D2G_E_INVAL;
  if (d2_alg_type != 0) {
    d2g::set_error("d2_clustering: only the B-ADMM centroid update (d2_alg_type 0) is built");
    return D2G_E_UNSUPPORTED;
  }
  p_data->num_of_labels = num_of_clusters;
  int rc = D2G_OK;
  if (!centroids->ph) rc = init_centroids(p_data, centroids, selected_phase);
  if (rc) return rc;
  if (centroids->s_ph != p_data->s_ph || centroids->size != (size_t)num_of_clusters) return D2G_E_INVAL;
  const bool tri = use_triangle != 0;
  const bool set_budget = !d2g::cfg_snapshot().keep_time_budget;
  LoopWork w;
  rc = work_alloc(p_data, w, tri, selected_phase);
  CentroidCopy copy;
  int iter = 0;
  for (; !rc && iter < max_iter; ++iter) {
    size_t changed = 0;
    const double t0 = now_s();
    if (tri) {
      rc = d2g_labeling_prep(p_data, centroids, &w.vw, selected_phase, &changed, nullptr);
      if (!rc && set_budget) time_budget = kTimeBudgetRatio * (now_s() - t0);
    } else {
      rc = d2g_labeling(p_data, centroids, &w.vw, selected_phase, &changed, nullptr);
      if (!rc && set_budget) time_budget = kTimeBudgetRatio * (now_s() - t0) / num_of_clusters;
    }
    if (rc) break;
    if (log_file && (iter + 1) % 10 == 0) write_log(log_file, centroids, p_data);
    if (changed < 0.001 * p_data->global_size) break;  // clustering.c:478
    if (tri) copy_centroids(centroids, copy);
    for (int n = 0; n < p_data->s_ph && !rc; ++n)
      if (selected(n, selected_phase))
        rc = d2g::centroid_update(p_data, &w.vw, n, centroids->ph + n, centroids->ph + n);
    if (!rc && tri) rc = d2g_labeling_post(p_data, &copy.m, centroids, &w.vw, selected_phase);
  }
  if (!rc && tri) {  // clustering.c:509
    const double t0 = now_s();
    rc = d2g_labeling(p_data, centroids, &w.vw, selected_phase, nullptr, nullptr);
    if (!rc && set_budget) time_budget = kTimeBudgetRatio * (now_s() - t0) / num_of_clusters;
  }
  work_free(w);
  if (rounds) *rounds = iter;
  return rc;
}

extern "C" int d2g_assignment(int num_of_clusters, mph *p_data, mph *centroids, int selected_phase,
                              size_t *count) {
  if (!p_data || !centroids || num_of_clusters <= 0) return D2G_E_INVAL;
  p_data->num_of_labels = num_of_clusters;
  std::vector<char> ls(p_data->size, 0);
  var_mph vw{};
  vw.s_ph = p_data->s_ph;
  vw.label_switch = ls.data();
  return d2g_labeling(p_data, centroids, &vw, selected_phase, count, nullptr);
}

// The reference's entry point (clustering.h), same signature; it returns 0
// like the reference, or this library's negative error code.
extern "C" int d2_clustering(int num_of_clusters, int max_iter, mph *p_data, mph *centroids,
                             int selected_phase, char use_triangle, const char *log_file) {
  return d2g_clustering(num_of_clusters, max_iter, p_data, centroids, selected_phase, use_triangle,
                        log_file, nullptr);
}
