/*
 * TEST INFRASTRUCTURE ONLY: the CPU oracle for the assignment step.
 *
 * A restatement of the reference's d2_compute_distance, d2_labeling_prep,
 * d2_labeling_post and d2_labeling (src/d2/clustering.c:33-376) on the
 * reference's structures (the layout-identical copies in include/d2g.h),
 * with every transport cost from d2o_emd (emd_oracle.c) where the reference
 * calls MOSEK through d2_match_by_distmat.  Same loops, same order, same
 * comparisons; the printing and the time_budget side effect are left out.
 * Metric types: Euclidean, histogram, sparse histogram, word embeddings,
 * n-grams.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>

#include "d2_oracle.h"
#include "d2g.h"

/* clustering.c:33-122: rows are b's object j, columns a's object i */
static double distance(const mph *a, size_t i, const mph *b, size_t j, int selected_phase) {
  double d = 0.0;
  for (int n = 0; n < a->s_ph; ++n) {
    if (selected_phase >= 0 && n != selected_phase) continue;
    const sph *as = a->ph + n, *bs = b->ph + n;
    const int dim = as->dim;
    const int nr = bs->p_str[j], nc = as->p_str[i];
    const size_t rb = bs->p_str_cum[j], ca = as->p_str_cum[i];
    double *C = (double *)malloc(sizeof(double) * (size_t)nr * nc);
    switch (as->metric_type) {
      case D2_EUCLIDEAN_L2: /* _dpdist2 (blas_like64.c:199-208): C[c*nr + r] */
        for (int c = 0; c < nc; ++c)
          for (int r = 0; r < nr; ++r) {
            double s = 0.0;
            for (int t = 0; t < dim; ++t) {
              const double v = bs->p_supp[(rb + r) * dim + t] - as->p_supp[(ca + c) * dim + t];
              s += v * v;
            }
            C[(size_t)c * nr + r] = s;
          }
        break;
      case D2_HISTOGRAM: /* the phase's dist_mat, as is (:88-95) */
        for (size_t e = 0; e < (size_t)nr * nc; ++e) C[e] = as->dist_mat[e];
        break;
      case D2_WORD_EMBED: /* _dpdist2_sym (blas_like64.c:210-220) */
        for (int c = 0; c < nc; ++c) {
          const int sym = as->p_supp_sym[ca + c];
          for (int r = 0; r < nr; ++r) {
            double s = 0.0;
            for (int t = 0; t < dim; ++t) {
              const double b = bs->p_supp[(rb + r) * dim + t];
              if (sym < 0)
                s += b * b;
              else
                s += (b - as->vocab_vec[(size_t)sym * dim + t]) * (b - as->vocab_vec[(size_t)sym * dim + t]);
            }
            C[(size_t)c * nr + r] = s;
          }
        }
        break;
      case D2_SPARSE_HISTOGRAM: /* _dpdist2_submat (blas_like64.c:222-230) */
        for (int c = 0; c < nc; ++c)
          for (int r = 0; r < nr; ++r)
            C[(size_t)c * nr + r] =
                as->dist_mat[(size_t)as->p_supp_sym[ca + c] * as->vocab_size + r];
        break;
      case D2_N_GRAM: /* _dpdist_symbolic (blas_like64.c:232-242), rows b's symbols */
        for (int c = 0; c < nc; ++c)
          for (int r = 0; r < nr; ++r) {
            double s = 0.0;
            for (int t = 0; t < dim; ++t)
              s += as->dist_mat[(size_t)bs->p_supp_sym[(rb + r) * dim + t] * as->vocab_size +
                                as->p_supp_sym[(ca + c) * dim + t]];
            C[(size_t)c * nr + r] = s;
          }
        break;
      default:
        free(C);
        return NAN;
    }
    const double val = d2o_emd(nr, nc, C, bs->p_w + rb, as->p_w + ca, NULL);
    if (as->metric_type == D2_N_GRAM)
      d += 2 * (val / dim); /* :112-115: the cost per symbol, counted twice */
    else
      d += val;
    free(C);
  }
  if (d <= 0) return 0.;
  return sqrt(d);
}

double d2o_compute_distance(const void *a, size_t i, const void *b, size_t j, int selected_phase) {
  return distance((const mph *)a, i, (const mph *)b, j, selected_phase);
}

/* clustering.c:134-248 */
size_t d2o_labeling_prep(void *p_data_, const void *centroids_, void *var_work_, int selected_phase,
                         size_t *dist_count_out) {
  mph *p_data = (mph *)p_data_;
  const mph *centroids = (const mph *)centroids_;
  var_mph *var_work = (var_mph *)var_work_;
  size_t i, count = 0, dist_count = 0;
  const size_t size = p_data->size;
  const size_t k = centroids->size;
  int *label = p_data->label;
  trieq *tr = &var_work->tr;
  for (i = 0; i < k; ++i) tr->s[i] = DBL_MAX;
  for (i = 0; i < k * k; ++i) tr->c[i] = 0;
  for (i = 0; i < k; ++i)
    for (size_t j = i + 1; j < k; ++j) {
      const double d = distance(centroids, i, centroids, j, selected_phase);
      dist_count += 1;
      tr->c[i * k + j] = d;
      tr->c[i + j * k] = d;
      if (tr->s[i] > d / 2.f) tr->s[i] = d / 2.f;
      if (tr->s[j] > d / 2.f) tr->s[j] = d / 2.f;
    }
  for (i = 0; i < size; ++i) var_work->label_switch[i] = 0;
  for (i = 0; i < size; ++i) {
    if (label[i] < 0 || tr->u[i] > tr->s[label[i]]) {
      const int init_label = label[i];
      int jj = init_label >= 0 ? init_label : 0;
      double min_distance = 0.0;
      double *U = tr->u + i;
      double *L = tr->l + i * k;
      for (size_t j = 0; j < k; ++j)
        if (((int)j != jj || init_label < 0) && *U > L[j] && *U > tr->c[j * k + jj] / 2.) {
          if (tr->r[i] == 1) {
            const double d = distance(p_data, i, centroids, jj, selected_phase);
            dist_count += 1;
            L[jj] = d;
            *U = d;
            min_distance = d;
            tr->r[i] = 0;
          } else {
            min_distance = *U;
          }
          if ((min_distance > L[j] || min_distance > tr->c[j * k + jj] / 2.) && (int)j != jj) {
            const double d = distance(p_data, i, centroids, j, selected_phase);
            dist_count += 1;
            L[j] = d;
            if (d < min_distance) {
              jj = (int)j;
              min_distance = d;
              *U = d;
            }
          }
        }
      if (jj != init_label) {
        label[i] = jj;
        var_work->label_switch[i] = 1;
        count += 1;
      }
    }
  }
  if (dist_count_out) *dist_count_out = dist_count;
  return count;
}

/* clustering.c:287-318 */
void d2o_labeling_post(void *p_data_, const void *c_old_, const void *c_new_, void *var_work_,
                       int selected_phase) {
  mph *p_data = (mph *)p_data_;
  const mph *c_old = (const mph *)c_old_, *c_new = (const mph *)c_new_;
  var_mph *var_work = (var_mph *)var_work_;
  const size_t k = c_old->size;
  double *d_changes = (double *)malloc(sizeof(double) * k);
  for (size_t i = 0; i < k; ++i) d_changes[i] = distance(c_new, i, c_old, i, selected_phase);
  for (size_t j = 0; j < p_data->size; ++j) {
    double *L = var_work->tr.l + j * k;
    for (size_t i = 0; i < k; ++i) L[i] = fmax(L[i] - d_changes[i], 0);
    var_work->tr.u[j] += d_changes[p_data->label[j]];
    var_work->tr.r[j] = 1;
  }
  free(d_changes);
}

/* clustering.c:327-376 */
size_t d2o_labeling(void *p_data_, const void *centroids_, void *var_work_, int selected_phase,
                    double *cost_out) {
  mph *p_data = (mph *)p_data_;
  const mph *centroids = (const mph *)centroids_;
  var_mph *var_work = (var_mph *)var_work_;
  size_t count = 0;
  double cost = 0.0;
  for (size_t i = 0; i < p_data->size; ++i) {
    double min_distance = -1;
    int jj = p_data->label[i] >= 0 ? p_data->label[i] : 0;
    for (size_t j = 0; j < centroids->size; ++j) {
      const double d = distance(p_data, i, centroids, j, selected_phase);
      if (min_distance < 0 || d < min_distance) {
        min_distance = d;
        jj = (int)j;
      }
    }
    cost += min_distance * min_distance;
    if (p_data->label[i] == jj) {
      var_work->label_switch[i] = 0;
    } else {
      p_data->label[i] = jj;
      var_work->label_switch[i] = 1;
      count++;
    }
  }
  if (cost_out) *cost_out = cost;
  return count;
}
