/*
 * TEST INFRASTRUCTURE ONLY: C restatement of the reference B-ADMM centroid
 * update, used as the parity oracle and as the timed CPU baseline ("port").
 * Nothing in the product links this file.
 *
 * It restates src/d2/centroid_Bregman.c:95-318 (bobye/d2_kmeans) and the
 * helpers it calls, step by step and in the same floating-point order, in
 * FP64, single-threaded, so that with oracle/cblas_shim.c's fixed BLAS order
 * it reproduces the compiled reference bit for bit:
 *   pdist2 / pdist2_sym            src/utils/blas_like64.c:199-220
 *   cnorm / rnorm / grms / gcms    src/utils/blas_like64.c:41-56,122-154
 *   irms / rsum2                   src/utils/blas_like64.c:69-77,113-119
 *   calculate_distmat              src/d2/centroid_util.c:8-36
 *   pdist_symbolic (n-gram costs)  src/utils/blas_like64.c:232-242
 *   n-gram support update          src/d2/centroid_Bregman.c:269-294 with
 *                                  accumulate_symbolic / minimize_symbolic,
 *                                  include/d2/centroid_util.h:15-37
 *   histogram cost layout         src/d2/clustering_util.c:183-198 (as intended:
 *                                  the reference indexes ph[k] with an instance
 *                                  index there; this oracle uses the phase's own
 *                                  dist_mat)
 * Deviations, all on error paths: an empty cluster returns -5 and a
 * non-positive normaliser returns -6 where the reference assert()s.
 */
#include "d2_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <float.h>
#include <string.h>
#include <time.h>

#define ROUNDOFF (1E-9) /* centroid_Bregman.c:20 */

static double now_seconds(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + (double)ts.tv_nsec / 1e9;
}

/* ground cost of one instance against its centroid, column-major str x m_i,
 * entry (k, j) at [j*str + k]: centroid_util.c:17-33 -> blas_like64.c:199-220 */
static void cost_block(const d2o_phase *ph, size_t i, size_t cum, const double *c_supp,
                       double *Ci) {
  const int str = ph->str, d = ph->dim, mi = ph->p_str[i];
  const int l = ph->label[i];
  if (ph->metric == D2O_EUCLIDEAN_L2) {
    const double *A = c_supp + (size_t)l * str * d; /* centroid supports */
    const double *B = ph->p_supp + cum * d;         /* instance supports */
    for (int j = 0; j < mi; ++j)
      for (int k = 0; k < str; ++k) {
        double s = 0;
        for (int t = 0; t < d; ++t) s += (A[k * d + t] - B[j * d + t]) * (A[k * d + t] - B[j * d + t]);
        Ci[(size_t)j * str + k] = s;
      }
  } else if (ph->metric == D2O_WORD_EMBED) {
    const double *A = c_supp + (size_t)l * str * d;
    for (int j = 0; j < mi; ++j) {
      int sym = ph->p_supp_sym[cum + j];
      for (int k = 0; k < str; ++k) {
        double s = 0;
        for (int t = 0; t < d; ++t) {
          if (sym < 0)
            s += A[k * d + t] * A[k * d + t];
          else {
            double v = ph->vocab_vec[(size_t)sym * d + t];
            s += (A[k * d + t] - v) * (A[k * d + t] - v);
          }
        }
        Ci[(size_t)j * str + k] = s;
      }
    }
  } else if (ph->metric == D2O_N_GRAM) {
    /* centroid_util.c:31-33 -> _dpdist_symbolic, blas_like64.c:232-242: the
     * cost of centroid support k against instance support j sums the symbol
     * costs position by position, dist_mat[centroid symbol * V + instance symbol] */
    const int *A = ph->c_sym + (size_t)l * str * d;
    const int *B = ph->p_supp_sym + cum * d;
    const int V = ph->vocab_size;
    for (int j = 0; j < mi; ++j)
      for (int k = 0; k < str; ++k) {
        double s = 0;
        for (int t = 0; t < d; ++t) s += ph->dist_mat[(size_t)A[k * d + t] * V + B[j * d + t]];
        Ci[(size_t)j * str + k] = s;
      }
  } else if (ph->metric == D2O_HISTOGRAM) {
    /* dense histogram: the plan's cost is the bin-to-bin matrix itself */
    for (size_t e = 0; e < (size_t)str * mi; ++e) Ci[e] = ph->dist_mat[e];
  } else { /* D2O_SPARSE_HISTOGRAM: blas_like64.c:222-230, str == vocab_size */
    for (int j = 0; j < mi; ++j) {
      int sym = ph->p_supp_sym[cum + j];
      for (int k = 0; k < str; ++k)
        Ci[(size_t)j * str + k] = ph->dist_mat[(size_t)sym * ph->vocab_size + k];
    }
  }
}

static void calc_distmat(const d2o_phase *ph, const size_t *cum, const double *c_supp, double *C) {
  if (ph->metric == D2O_HISTOGRAM || ph->metric == D2O_SPARSE_HISTOGRAM) return; /* fixed */
  for (size_t i = 0; i < ph->size; ++i) cost_block(ph, i, cum[i], c_supp, C + ph->str * cum[i]);
}

void d2o_cost_blocks(const d2o_phase *ph, const double *c_supp, double *C) {
  size_t cum = 0;
  for (size_t i = 0; i < ph->size; ++i) {
    cost_block(ph, i, cum, c_supp, C + ph->str * cum);
    cum += (size_t)ph->p_str[i];
  }
}

/* column-normalise an m x n column-major block; sums into sa (blas_like64.c:122-136) */
static int cnorm(size_t m, size_t n, double *a, double *sa) {
  for (size_t i = 0; i < n; ++i) {
    double s = 0;
    for (size_t j = 0; j < m; ++j) s += a[i * m + j];
    sa[i] = s;
  }
  for (size_t i = 0; i < n; ++i)
    if (!(sa[i] > 0)) return -6;
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < m; ++j) a[i * m + j] /= sa[i];
  return 0;
}

/* The update, with the reference's MPI exchanges (`#ifdef __USE_MPI__` in
 * src/d2/centroid_Bregman.c) made through `xr` when it is given: an in-place
 * SUM of n doubles over all ranks (label counts :142, cluster weights :188,
 * support numerators and X row sums :215-217 / :250-252, n-gram symbol counts
 * :282, obj / primres / dualres :308-310).  Like the reference, each rank
 * takes rho from its own instances (:109); global_rho != 0 sums |C| and the
 * entry count over the ranks first instead (not in the reference). */
static int badmm_impl(const d2o_phase *ph, const d2o_opts *opt, double *c_w, double *c_supp,
                      double *Z, double *Xout, double *Yout, double *Cout, double *trace, int *ntrace,
                      double *rho_out, int *iters_out, d2o_allreduce_fn xr, void *xctx, int global_rho) {
  const int str = ph->str, dim = ph->dim, K = ph->num_of_labels;
  const size_t size = ph->size, col = ph->col, nent = (size_t)str * col;
  const int euclid = ph->metric == D2O_EUCLIDEAN_L2, embed = ph->metric == D2O_WORD_EMBED;
  const int ngram = ph->metric == D2O_N_GRAM;
  int rc = 0, nt = 0, iter;
  if (str <= 0 || size == 0 || col == 0 || K <= 0) return -1;
  if (ngram && (!ph->c_sym || !ph->dist_mat || ph->vocab_size < 1 || dim < 1)) return -1;

  size_t *cum = malloc(size * sizeof(size_t));
  double *C = malloc(nent * sizeof(double)), *X = malloc(nent * sizeof(double));
  double *Y = malloc(nent * sizeof(double)), *Z0 = malloc(nent * sizeof(double));
  double *Xc = malloc((col > (size_t)K ? col : (size_t)K) * sizeof(double) + sizeof(double));
  size_t zr_n = (size > (size_t)K ? size : (size_t)K) * str;
  double *Zr = malloc(zr_n * sizeof(double));
  size_t *count = calloc(K, sizeof(size_t));
  /* n-gram support update scratch (the reference's Zr2, :127-130) */
  double *zsym = ngram ? malloc((size_t)K * str * dim * ph->vocab_size * sizeof(double)) : NULL;
  double *zbuf = ngram ? malloc((size_t)ph->vocab_size * sizeof(double)) : NULL;
  if (!cum || !C || !X || !Y || !Z0 || !Xc || !Zr || !count || (ngram && (!zsym || !zbuf))) {
    rc = -1;
    goto done;
  }

  cum[0] = 0; /* p_str_cum as built by d2_read, clustering_io.c:176-181 */
  for (size_t i = 1; i < size; ++i) cum[i] = cum[i - 1] + ph->p_str[i - 1];

  /* histograms: C is the cost filled by the caller at allocation (clustering_util.c:183-198) */
  if (!euclid && !embed && !ngram)
    for (size_t i = 0; i < size; ++i) cost_block(ph, i, cum[i], c_supp, C + str * cum[i]);
  calc_distmat(ph, cum, c_supp, C); /* :106 */

  /* rho from the initial cost, then C /= rho: :109-110 */
  double asum = 0;
  for (size_t e = 0; e < nent; ++e) asum += fabs(C[e]);
  double rho = opt->rhoCoeff * asum / (double)nent;
  if (xr && global_rho) {
    double g[2] = {asum, (double)nent};
    if (xr(g, 2, xctx)) { rc = -2; goto done; }
    rho = opt->rhoCoeff * g[0] / g[1];
  }
  for (size_t e = 0; e < nent; ++e) C[e] /= rho;

  /* warm start: re-initialise only switched instances, :116-124 */
  for (size_t i = 0; i < size; ++i)
    if (ph->label_switch[i] == 1) {
      double *zi = Z + str * cum[i];
      const double *wi = ph->p_w + cum[i], *cwi = c_w + (size_t)ph->label[i] * str;
      for (size_t j = 0; j < (size_t)str * ph->p_str[i]; ++j) zi[j] = wi[j / str] * cwi[j % str];
    }
  for (size_t e = 0; e < nent; ++e) Y[e] = 0; /* :128 */

  for (size_t i = 0; i < size; ++i) ++count[ph->label[i]]; /* :138-144 */
  if (xr) { /* :142 */
    for (int l = 0; l < K; ++l) Xc[l] = (double)count[l];
    if (xr(Xc, (size_t)K, xctx)) { rc = -2; goto done; }
    for (int l = 0; l < K; ++l) count[l] = (size_t)Xc[l];
  }
  for (int l = 0; l < K; ++l)
    if (count[l] == 0) { rc = -5; goto done; }

  double t0 = now_seconds();
  for (iter = 0; iter <= opt->maxIters; ++iter) { /* :150, maxIters+1 iterations */
    /* step 1, :155-159 */
    for (size_t e = 0; e < nent; ++e) X[e] = Z[e] * exp(-(C[e] + Y[e])) + ROUNDOFF;
    if ((rc = cnorm(str, col, X, Xc))) goto done;
    for (size_t c = 0; c < col; ++c)
      for (int k = 0; k < str; ++k) X[c * str + k] *= ph->p_w[c];

    /* step 2, :164-171 */
    for (size_t e = 0; e < nent; ++e) {
      Z0[e] = Z[e];
      Z[e] = X[e] * exp(Y[e]) + ROUNDOFF;
    }
    for (size_t i = 0; i < size; ++i) {
      double *zi = Z + str * cum[i], *zri = Zr + str * i;
      const double *cwi = c_w + (size_t)ph->label[i] * str;
      const int mi = ph->p_str[i];
      for (int k = 0; k < str; ++k) zri[k] = 0;
      for (int j = 0; j < mi; ++j)
        for (int k = 0; k < str; ++k) zri[k] += zi[(size_t)j * str + k];
      for (int k = 0; k < str; ++k)
        if (!(zri[k] > 0)) { rc = -6; goto done; }
      for (int j = 0; j < mi; ++j)
        for (int k = 0; k < str; ++k) zi[(size_t)j * str + k] /= zri[k];
      for (int j = 0; j < mi; ++j)
        for (int k = 0; k < str; ++k) zi[(size_t)j * str + k] *= cwi[k];
    }

    /* step 3, :175 */
    for (size_t e = 0; e < nent; ++e) Y[e] += X[e] - Z[e];

    /* step 4, :179-190 */
    for (size_t e = 0; e < (size_t)str * K; ++e) c_w[e] = 0;
    if ((rc = cnorm(str, size, Zr, Xc))) goto done;
    for (size_t i = 0; i < size; ++i) {
      double *cwl = c_w + (size_t)ph->label[i] * str;
      for (int k = 0; k < str; ++k) cwl[k] += Zr[str * i + k];
    }
    if (xr && xr(c_w, (size_t)str * K, xctx)) { rc = -2; goto done; } /* :188 */
    if ((rc = cnorm(str, K, c_w, Xc))) goto done;

    /* step 5, :194-267 */
    if (iter % opt->updatePerLoops == 0 && (euclid || embed)) {
      const size_t sxd = (size_t)str * dim;
      for (size_t e = 0; e < sxd * K; ++e) c_supp[e] = 0;
      for (size_t e = 0; e < (size_t)str * K; ++e) Zr[e] = 0;
      for (size_t i = 0; i < size; ++i) {
        const int l = ph->label[i], mi = ph->p_str[i];
        const double *xi = X + str * cum[i];
        double *cs = c_supp + l * sxd, *zr = Zr + (size_t)l * str;
        if (euclid) {
          /* dgemm (col-major, N, T): cs(t,k) += sum_j supp(t,j) X(k,j), netlib order, :206-208 */
          const double *si = ph->p_supp + cum[i] * dim;
          for (int k = 0; k < str; ++k)
            for (int j = 0; j < mi; ++j) {
              double xv = xi[(size_t)j * str + k];
              for (int t = 0; t < dim; ++t) cs[(size_t)k * dim + t] += xv * si[(size_t)j * dim + t];
            }
          for (int j = 0; j < mi; ++j) /* rsum2, :211 */
            for (int k = 0; k < str; ++k) zr[k] += xi[(size_t)j * str + k];
        } else { /* :233-247 */
          for (int j = 0; j < mi; ++j) {
            const double *v = ph->vocab_vec + (size_t)ph->p_supp_sym[cum[i] + j] * dim;
            for (int k = 0; k < str; ++k) {
              double xv = xi[(size_t)j * str + k];
              for (int t = 0; t < dim; ++t) cs[(size_t)k * dim + t] += xv * v[t];
              zr[k] += xv;
            }
          }
        }
      }
      if (xr && (xr(c_supp, sxd * K, xctx) || xr(Zr, (size_t)str * K, xctx))) { /* :215-217 */
        rc = -2;
        goto done;
      }
      for (int l = 0; l < K; ++l) { /* irms, :219-221 */
        double *cs = c_supp + l * sxd, *zr = Zr + (size_t)l * str;
        for (int k = 0; k < str; ++k)
          if (!(zr[k] > 0)) { rc = -6; goto done; }
        for (int k = 0; k < str; ++k)
          for (int t = 0; t < dim; ++t) cs[(size_t)k * dim + t] /= zr[k];
      }
      calc_distmat(ph, cum, c_supp, C); /* :225-227 */
      for (size_t e = 0; e < nent; ++e) C[e] /= rho;
    }
    if (iter % opt->updatePerLoops == 0 && ngram && iter > 0) { /* :269-294 */
      /* weighted symbol counts per (cluster, support, position): the plan Z of
       * this iteration, entries above 1e-10 only (accumulate_symbolic,
       * include/d2/centroid_util.h:15-23), instances and supports in order */
      const int V = ph->vocab_size;
      const size_t sxdv = (size_t)str * dim * V;
      for (size_t e = 0; e < sxdv * K; ++e) zsym[e] = 0;
      for (size_t i = 0; i < size; ++i) {
        const int mi = ph->p_str[i];
        const int *si = ph->p_supp_sym + cum[i] * dim;
        const double *zi = Z + str * cum[i];
        double *z = zsym + (size_t)ph->label[i] * sxdv;
        for (int j = 0; j < mi; ++j)
          for (int k = 0; k < str; ++k) {
            const double val = zi[(size_t)j * str + k];
            if (val > 1E-10)
              for (int t = 0; t < dim; ++t) z[(size_t)V * (dim * k + t) + si[j * dim + t]] += val;
          }
      }
      if (xr && xr(zsym, sxdv * K, xctx)) { rc = -2; goto done; } /* :282 */
      /* each centroid symbol moves to the symbol of least expected cost
       * (minimize_symbolic, centroid_util.h:25-37): zbuf = dist_mat * z as the
       * column-major dgemm computes it (a running sum over u), first minimum */
      for (int l = 0; l < K; ++l) {
        const double *z = zsym + (size_t)l * sxdv;
        for (int q = 0; q < str * dim; ++q) {
          const double *zq = z + (size_t)q * V;
          for (int r = 0; r < V; ++r) zbuf[r] = 0.0;
          for (int u = 0; u < V; ++u) {
            const double t = 1.0 * zq[u];
            for (int r = 0; r < V; ++r) zbuf[r] += t * ph->dist_mat[(size_t)r + (size_t)u * V];
          }
          double mn = DBL_MAX;
          int arg = 0;
          for (int r = 0; r < V; ++r)
            if (zbuf[r] < mn) { mn = zbuf[r]; arg = r; }
          ph->c_sym[(size_t)l * str * dim + q] = arg;
        }
      }
      calc_distmat(ph, cum, c_supp, C); /* :289-291 */
      for (size_t e = 0; e < nent; ++e) C[e] /= rho;
    }

    /* step 6, :300-316 */
    if ((iter % 100 == 99) || (iter < 100 && iter % 20 == 19)) {
      double obj = 0, pr = 0, dr = 0;
      for (size_t e = 0; e < nent; ++e) obj += C[e] * X[e];
      for (size_t e = 0; e < nent; ++e) X[e] += -1 * Z[e];
      for (size_t e = 0; e < nent; ++e) Z0[e] += -1 * Z[e];
      for (size_t e = 0; e < nent; ++e) pr += fabs(X[e]);
      for (size_t e = 0; e < nent; ++e) dr += fabs(Z0[e]);
      if (xr) { /* :308-310 */
        double g[3] = {obj, pr, dr};
        if (xr(g, 3, xctx)) { rc = -2; goto done; }
        obj = g[0];
        pr = g[1];
        dr = g[2];
      }
      obj *= rho / ph->global_size;
      pr /= ph->global_size;
      dr /= ph->global_size;
      if (trace) {
        trace[4 * nt + 0] = iter + 1;
        trace[4 * nt + 1] = obj;
        trace[4 * nt + 2] = pr;
        trace[4 * nt + 3] = dr;
      }
      ++nt;
    }
    if (now_seconds() - t0 > opt->time_budget) { ++iter; break; } /* :318 */
  }
  if (iters_out) *iters_out = iter > opt->maxIters + 1 ? opt->maxIters + 1 : iter;
  if (rho_out) *rho_out = rho;
  if (Xout) memcpy(Xout, X, nent * sizeof(double));
  if (Yout) memcpy(Yout, Y, nent * sizeof(double));
  if (Cout) memcpy(Cout, C, nent * sizeof(double));
done:
  if (ntrace) *ntrace = nt;
  free(cum); free(C); free(X); free(Y); free(Z0); free(Xc); free(Zr); free(count);
  free(zsym); free(zbuf);
  return rc;
}

int d2o_badmm(const d2o_phase *ph, const d2o_opts *opt, double *c_w, double *c_supp,
              double *Z, double *Xout, double *Yout, double *Cout, double *trace, int *ntrace,
              double *rho_out, int *iters_out) {
  return badmm_impl(ph, opt, c_w, c_supp, Z, Xout, Yout, Cout, trace, ntrace, rho_out, iters_out,
                    NULL, NULL, 0);
}

int d2o_badmm_mpi(const d2o_phase *ph, const d2o_opts *opt, double *c_w, double *c_supp,
                  double *Z, double *trace, int *ntrace, double *rho_out, int *iters_out,
                  d2o_allreduce_fn xr, void *xctx, int global_rho) {
  return badmm_impl(ph, opt, c_w, c_supp, Z, NULL, NULL, NULL, trace, ntrace, rho_out, iters_out,
                    xr, xctx, global_rho);
}

int d2o_serve_query(int dim, int str, int k, const double *c_w, const double *c_supp,
                    int m_q, const double *w_q, const double *supp_q, int iters,
                    double rhoCoeff, double *cost_out) {
  const size_t pe = (size_t)str * m_q, nent = pe * k;
  double *C = malloc(nent * sizeof(double)), *X = malloc(nent * sizeof(double));
  double *Y = calloc(nent, sizeof(double)), *Z = malloc(nent * sizeof(double));
  double *rs = malloc((size_t)str * sizeof(double));
  int best = -1;
  if (!C || !X || !Y || !Z || !rs) goto out;
  double asum = 0;
  for (int l = 0; l < k; ++l) {
    const double *A = c_supp + (size_t)l * str * dim;
    double *Cl = C + l * pe;
    for (int j = 0; j < m_q; ++j)
      for (int kk = 0; kk < str; ++kk) {
        double s = 0;
        for (int t = 0; t < dim; ++t)
          s += (A[kk * dim + t] - supp_q[j * dim + t]) * (A[kk * dim + t] - supp_q[j * dim + t]);
        Cl[(size_t)j * str + kk] = s;
        asum += s;
      }
  }
  double rho = rhoCoeff * asum / (double)nent;
  for (size_t e = 0; e < nent; ++e) C[e] /= rho;
  for (int l = 0; l < k; ++l)
    for (int j = 0; j < m_q; ++j)
      for (int kk = 0; kk < str; ++kk) Z[l * pe + (size_t)j * str + kk] = w_q[j] * c_w[l * str + kk];
  for (int it = 0; it < iters; ++it) {
    for (int l = 0; l < k; ++l) {
      double *Xl = X + l * pe, *Yl = Y + l * pe, *Zl = Z + l * pe;
      const double *Cl = C + l * pe, *cwl = c_w + (size_t)l * str;
      for (size_t e = 0; e < pe; ++e) Xl[e] = Zl[e] * exp(-(Cl[e] + Yl[e])) + ROUNDOFF;
      for (int j = 0; j < m_q; ++j) {
        double s = 0;
        for (int kk = 0; kk < str; ++kk) s += Xl[(size_t)j * str + kk];
        for (int kk = 0; kk < str; ++kk) Xl[(size_t)j * str + kk] /= s;
        for (int kk = 0; kk < str; ++kk) Xl[(size_t)j * str + kk] *= w_q[j];
      }
      for (size_t e = 0; e < pe; ++e) Zl[e] = Xl[e] * exp(Yl[e]) + ROUNDOFF;
      for (int kk = 0; kk < str; ++kk) rs[kk] = 0;
      for (int j = 0; j < m_q; ++j)
        for (int kk = 0; kk < str; ++kk) rs[kk] += Zl[(size_t)j * str + kk];
      for (int j = 0; j < m_q; ++j)
        for (int kk = 0; kk < str; ++kk) {
          Zl[(size_t)j * str + kk] /= rs[kk];
          Zl[(size_t)j * str + kk] *= cwl[kk];
        }
      for (size_t e = 0; e < pe; ++e) Yl[e] += Xl[e] - Zl[e];
    }
  }
  double bestc = 0;
  for (int l = 0; l < k; ++l) {
    double s = 0;
    for (size_t e = 0; e < pe; ++e) s += C[l * pe + e] * X[l * pe + e];
    cost_out[l] = s * rho;
    if (best < 0 || cost_out[l] < bestc) { best = l; bestc = cost_out[l]; }
  }
out:
  free(C); free(X); free(Y); free(Z); free(rs);
  return best;
}

/* ------------------------------------------------------------ d2 input files
 * Restatement of d2_allocate's data part (src/d2/clustering_util.c:18-59,
 * 93-130) and of d2_read (src/d2/clustering_io.c:14-201): the same fscanf
 * token reads, weight checks and renormalisation, id shift and array growth.
 * Deviation: where the reference assert()s (missing file, dimension mismatch,
 * weight <= 1e-9) this returns -1. */
#include <stdio.h>

#include "d2g.h"

static int o_alloc_sph(sph *ph, int d, int stride, size_t num, double semicol, int type) {
  const size_t m = (size_t)(num * (stride + semicol));
  ph->max_col = m;
  ph->dim = d;
  ph->str = stride;
  ph->max_str = stride;
  ph->p_str = (int *)calloc(num, sizeof(int));
  ph->p_str_cum = (size_t *)calloc(num, sizeof(size_t));
  ph->p_w = (double *)malloc((m ? m : 1) * sizeof(double));
  ph->metric_type = type;
  ph->p_supp = NULL;
  ph->p_supp_sym = NULL;
  if (type == D2O_EUCLIDEAN_L2) ph->p_supp = (double *)malloc((m * d > 0 ? m * d : 1) * sizeof(double));
  if (type == D2O_WORD_EMBED || type == D2O_SPARSE_HISTOGRAM) ph->p_supp_sym = (int *)malloc((m ? m : 1) * sizeof(int));
  ph->is_meta_allocated = 0;
  return 0;
}

int d2o_mph_free(void *pv) {
  mph *p = (mph *)pv;
  if (!p) return -1;
  for (int n = 0; n < p->s_ph; ++n) {
    sph *ph = p->ph + n;
    free(ph->p_str);
    free(ph->p_str_cum);
    free(ph->p_w);
    free(ph->p_supp);
    free(ph->p_supp_sym);
    if (ph->is_meta_allocated) {
      free(ph->dist_mat);
      free(ph->vocab_vec);
    }
  }
  free(p->ph);
  free(p->label);
  free(p);
  return 0;
}

int d2o_read(const char *filename, const char *meta_filename, int s_ph, size_t size,
             const int *avg_strides, const int *dims, const int *types, void **out) {
  mph *p = (mph *)calloc(1, sizeof(mph));
  p->s_ph = s_ph;
  p->size = size;
  p->ph = (sph *)calloc((size_t)s_ph, sizeof(sph));
  p->label = (int *)malloc(size * sizeof(int));
  for (size_t i = 0; i < size; ++i) p->label[i] = -1;
  for (int n = 0; n < s_ph; ++n) o_alloc_sph(p->ph + n, dims[n], avg_strides[n], size, 0.6, types[n]);
  *out = p;

  int **p_str = (int **)malloc(s_ph * sizeof(int *));
  int **p_sym = (int **)malloc(s_ph * sizeof(int *));
  double **p_supp = (double **)malloc(s_ph * sizeof(double *));
  double **p_w = (double **)malloc(s_ph * sizeof(double *));
  for (int n = 0; n < s_ph; ++n) {
    p_str[n] = p->ph[n].p_str;
    p_sym[n] = p->ph[n].p_supp_sym;
    p_supp[n] = p->ph[n].p_supp;
    p_w[n] = p->ph[n].p_w;
    p->ph[n].col = 0;
  }
  int rc = 0;
  /* meta files (:55-89) */
  for (int n = 0; n < s_ph && !rc; ++n) {
    sph *ph = p->ph + n;
    char extra[1024];
    const int hist = ph->metric_type == D2O_HISTOGRAM || ph->metric_type == D2O_SPARSE_HISTOGRAM;
    if (!hist && ph->metric_type != D2O_WORD_EMBED) continue;
    if (meta_filename && s_ph == 1)
      snprintf(extra, sizeof extra, "%s", meta_filename);
    else
      snprintf(extra, sizeof extra, "%s.%s%d", filename, hist ? "hist" : "vocab", n);
    FILE *fm = fopen(extra, "r");
    if (!fm) { rc = -1; break; }
    if (hist) {
      int str = 0;
      if (fscanf(fm, "%d", &str) != 1 || str <= 0) { fclose(fm); rc = -1; break; }
      ph->dist_mat = (double *)malloc((size_t)str * str * sizeof(double));
      for (size_t i = 0; i < (size_t)str * str; ++i)
        if (fscanf(fm, "%lf", &ph->dist_mat[i]) != 1) rc = -1;
      ph->vocab_size = str;
    } else {
      int dim = 0;
      if (fscanf(fm, "%d", &dim) != 1 || dim != ph->dim) { fclose(fm); rc = -1; break; }
      if (fscanf(fm, "%d", &ph->vocab_size) != 1) { fclose(fm); rc = -1; break; }
      ph->vocab_vec = (double *)malloc((size_t)dim * ph->vocab_size * sizeof(double));
      for (size_t i = 0; i < (size_t)ph->vocab_size * dim; ++i)
        if (fscanf(fm, "%lf", &ph->vocab_vec[i]) != 1) rc = -1;
    }
    ph->is_meta_allocated = 1;
    fclose(fm);
  }
  FILE *fp = rc ? NULL : fopen(filename, "r");
  if (!fp) rc = -1;
  /* main file (:91-176) */
  for (size_t i = 0; !rc && i < size; ++i) {
    for (int n = 0; n < s_ph; ++n) {
      sph *ph = p->ph + n;
      int dim, str;
      if (fscanf(fp, "%d", &dim) != 1) {
        fprintf(stderr, "rank 0 warning: only read %zd d2!\n", i);
        p->size = i;
        size = i;
        break;
      }
      if (dim != ph->dim) { rc = -1; break; }
      if (fscanf(fp, "%d", &str) != 1 || str < 0) { rc = -1; break; }
      if (str == 0) continue;
      *p_str[n] = str;
      if (str > ph->max_str) ph->max_str = str;
      if (ph->col + str > ph->max_col) { /* grow as the reference does (:110-135) */
        const size_t cap = 2 * ph->max_col > ph->col + str ? 2 * ph->max_col : ph->col + str;
        ph->p_w = (double *)realloc(ph->p_w, cap * sizeof(double));
        p_w[n] = ph->p_w + ph->col;
        if (ph->metric_type == D2O_EUCLIDEAN_L2) {
          ph->p_supp = (double *)realloc(ph->p_supp, cap * dim * sizeof(double));
          p_supp[n] = ph->p_supp + ph->col * dim;
        } else if (ph->metric_type == D2O_WORD_EMBED || ph->metric_type == D2O_SPARSE_HISTOGRAM) {
          ph->p_supp_sym = (int *)realloc(ph->p_supp_sym, cap * sizeof(int));
          p_sym[n] = ph->p_supp_sym + ph->col;
        }
        ph->max_col = cap;
      }
      ph->col += str;
      double *w = p_w[n], wsum = 0.;
      for (int j = 0; j < str; ++j) {
        if (fscanf(fp, "%lf", &w[j]) != 1) { rc = -1; break; }
        if (ph->metric_type != D2O_HISTOGRAM && !(w[j] > 1E-9)) { rc = -1; break; }
        wsum += w[j];
      }
      if (rc) break;
      for (int j = 0; j < str; ++j) w[j] /= wsum;
      p_w[n] += str;
      if (ph->metric_type == D2O_EUCLIDEAN_L2) {
        for (int j = 0; j < str * dim; ++j)
          if (fscanf(fp, "%lf", &p_supp[n][j]) != 1) rc = -1;
        p_supp[n] += str * dim;
      } else if (ph->metric_type == D2O_WORD_EMBED || ph->metric_type == D2O_SPARSE_HISTOGRAM) {
        for (int j = 0; j < str; ++j) {
          if (fscanf(fp, "%d", &p_sym[n][j]) != 1) rc = -1;
          p_sym[n][j]--; /* ids start at one */
          if (p_sym[n][j] < 0) p_sym[n][j] = ph->vocab_size - 1;
        }
        p_sym[n] += str;
      }
      p_str[n]++;
    }
  }
  if (fp) fclose(fp);
  /* cumulative sizes (:178-190) */
  for (int n = 0; !rc && n < s_ph; ++n) {
    sph *ph = p->ph + n;
    if (ph->col > 0) {
      ph->p_str_cum[0] = 0;
      for (size_t i = 1; i < size; ++i) ph->p_str_cum[i] = ph->p_str_cum[i - 1] + ph->p_str[i - 1];
      if (ph->metric_type == D2O_SPARSE_HISTOGRAM) ph->str = ph->vocab_size;
    }
  }
  p->global_size = p->size;
  free(p_w);
  free(p_supp);
  free(p_str);
  free(p_sym);
  return rc;
}

