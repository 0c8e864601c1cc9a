/*
 * TEST INFRASTRUCTURE ONLY: drives the reference's own compiled
 * d2_centroid_sphBregman (src/d2/centroid_Bregman.c:51-325, built unmodified
 * from the reference tree by oracle/Makefile into oracle/_ref/) through the
 * plain-array interface of d2_oracle.h.
 *
 * It fills the reference's sph / mph / var_mph structures
 * (include/d2/clustering.h:14-95,117-124,176-200) the way d2_read and
 * d2_allocate_work do (src/d2/clustering_io.c:14-202,
 * src/d2/clustering_util.c:152-230), with two harness choices:
 *   - time_budget is the caller's (the reference reads the global, :24,:318);
 *   - histogram costs are filled from the phase's own dist_mat, which is what
 *     clustering_util.c:183-188 intends (it indexes ph[k] by instance).
 * The obj / primres / dualres trace is only printed by the reference
 * (VPRINTF, :315), so stdout is captured around the call and parsed.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "d2/clustering.h"
#include "d2/param.h"
#include "d2_oracle.h"

/* time_budget, world_rank, nprocs and d2_alg_type come from the reference's
 * own src/d2/clustering.c:21-26, compiled into the same library */
extern double time_budget;

extern BADMM_options *p_badmm_options;

int d2r_badmm(const d2o_phase *ph, const d2o_opts *opt, double *c_w, double *c_supp,
              double *Z, double *Xout, double *Yout, double *Cout, double *trace, int *ntrace,
              double *rho_out, int *iters_out) {
  const int str = ph->str, K = ph->num_of_labels;
  const size_t size = ph->size, col = ph->col, nent = (size_t)str * col;
  sph data;
  mph p;
  var_mph work;
  var_sph gv;
  var_sphBregman bv;
  sph c;
  BADMM_options o;
  memset(&data, 0, sizeof data);
  memset(&p, 0, sizeof p);
  memset(&work, 0, sizeof work);
  memset(&c, 0, sizeof c);

  data.dim = ph->dim;
  data.str = str;
  data.max_str = str;
  data.col = col;
  data.max_col = col;
  data.p_str = (int *)ph->p_str;
  data.p_str_cum = malloc(size * sizeof(size_t));
  data.p_str_cum[0] = 0;
  for (size_t i = 1; i < size; ++i) data.p_str_cum[i] = data.p_str_cum[i - 1] + ph->p_str[i - 1];
  data.p_w = (double *)ph->p_w;
  data.metric_type = ph->metric;
  data.p_supp = (double *)ph->p_supp;
  data.p_supp_sym = (int *)ph->p_supp_sym;
  data.dist_mat = (double *)ph->dist_mat;
  data.vocab_size = ph->vocab_size;
  data.vocab_vec = (double *)ph->vocab_vec;

  p.s_ph = 1;
  p.size = size;
  p.global_size = ph->global_size;
  p.label = (int *)ph->label;
  p.num_of_labels = K;
  p.ph = &data;

  gv.C = malloc(str * (col + (size_t)K * str) * sizeof(double)); /* clustering_util.c:179 */
  gv.X = gv.L = NULL;
  if (ph->metric == D2O_HISTOGRAM) {
    for (size_t i = 0; i < size; ++i)
      memcpy(gv.C + str * data.p_str_cum[i], ph->dist_mat, (size_t)str * ph->p_str[i] * sizeof(double));
  } else if (ph->metric == D2O_SPARSE_HISTOGRAM) {
    for (size_t i = 0; i < size; ++i)
      for (int j = 0; j < ph->p_str[i]; ++j)
        for (int k = 0; k < str; ++k)
          gv.C[str * (data.p_str_cum[i] + j) + k] =
              ph->dist_mat[(size_t)ph->p_supp_sym[data.p_str_cum[i] + j] * ph->vocab_size + k];
  }
  d2_allocate_work_sphBregman(&data, size > (size_t)K ? size : (size_t)K, &bv);
  memcpy(bv.Z, Z, nent * sizeof(double));
  work.s_ph = 1;
  work.g_var = &gv;
  work.l_var_sphBregman = &bv;
  work.label_switch = (char *)ph->label_switch;

  c.dim = ph->dim;
  c.str = str;
  c.max_str = str;
  c.col = (size_t)K * str;
  c.p_w = c_w;
  c.p_supp = c_supp;
  c.p_supp_sym = ph->c_sym; /* n-gram centroids: symbols, updated in place */
  c.metric_type = ph->metric % D2_GROUP_SIZE; /* clustering.c:390 */
  c.vocab_size = ph->vocab_size;
  c.vocab_vec = (double *)ph->vocab_vec;
  c.dist_mat = (double *)ph->dist_mat;

  o.maxIters = opt->maxIters;
  o.rhoCoeff = opt->rhoCoeff;
  o.updatePerLoops = opt->updatePerLoops;
  BADMM_options *saved_opts = p_badmm_options;
  p_badmm_options = &o;
  time_budget = opt->time_budget;

  /* capture the printed trace */
  fflush(stdout);
  int saved_fd = dup(1);
  FILE *tmp = tmpfile();
  dup2(fileno(tmp), 1);
  int rc = d2_centroid_sphBregman(&p, &work, 0, &c, &c);
  fflush(stdout);
  dup2(saved_fd, 1);
  close(saved_fd);
  p_badmm_options = saved_opts;

  int nt = 0;
  char line[512];
  rewind(tmp);
  while (fgets(line, sizeof line, tmp)) {
    int it;
    double a, b, d, s;
    if (sscanf(line, " %d %lf %lf %lf %lf", &it, &a, &b, &d, &s) == 5) {
      if (trace) {
        trace[4 * nt + 0] = it;
        trace[4 * nt + 1] = a;
        trace[4 * nt + 2] = b;
        trace[4 * nt + 3] = d;
      }
      ++nt;
    }
  }
  fclose(tmp);
  if (ntrace) *ntrace = nt;
  if (rho_out) *rho_out = NAN;
  if (iters_out) *iters_out = opt->maxIters + 1;

  memcpy(Z, bv.Z, nent * sizeof(double));
  if (Xout) memcpy(Xout, bv.X, nent * sizeof(double));
  if (Yout) memcpy(Yout, bv.Y, nent * sizeof(double));
  if (Cout) memcpy(Cout, gv.C, nent * sizeof(double));
  d2_free_work_sphBregman(&bv);
  free(gv.C);
  free(data.p_str_cum);
  return rc;
}

/* the reference's own d2_allocate + d2_read (src/d2/clustering_util.c:93-130,
 * src/d2/clustering_io.c:14-201) into a heap mph */

int d2r_read(const char *filename, const char *meta_filename, int s_ph, size_t size,
             const int *avg_strides, const int *dims, const int *types, void **out) {
  mph *p = (mph *)calloc(1, sizeof(mph));
  if (d2_allocate(p, s_ph, size, avg_strides, dims, types)) return -1;
  *out = p;
  return d2_read(filename, meta_filename, p);
}

int d2r_mph_free(void *pv) {
  /* d2_allocate leaves the pointers a metric does not use unset: free by type */
  mph *p = (mph *)pv;
  for (int n = 0; n < p->s_ph; ++n) {
    sph *ph = p->ph + n;
    const int mt = ph->metric_type;
    free(ph->p_str);
    free(ph->p_str_cum);
    free(ph->p_w);
    if (mt == D2_EUCLIDEAN_L2) free(ph->p_supp);
    if (mt == D2_WORD_EMBED || mt == D2_SPARSE_HISTOGRAM) free(ph->p_supp_sym);
    if (ph->is_meta_allocated) {
      if (mt == D2_HISTOGRAM || mt == D2_SPARSE_HISTOGRAM) free(ph->dist_mat);
      if (mt == D2_WORD_EMBED) free(ph->vocab_vec);
    }
  }
  free(p->ph);
  free(p->label);
  free(p);
  return 0;
}

