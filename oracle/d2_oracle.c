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
 *   histogram cost layout          src/d2/clustering_util.c:183-198 (as intended:
 *                                  the reference indexes ph[k] with an instance
 *                                  index there; this oracle uses the phase's own
 *                                  dist_mat)
 * Deviations, all on error paths: an empty cluster returns -5 and a
 * non-positive normaliser returns -6 where the reference assert()s.
 */
#include "d2_oracle.h"

#include <math.h>
#include <stdlib.h>
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

int d2o_badmm(const d2o_phase *ph, const d2o_opts *opt, double *c_w, double *c_supp,
              double *Z, double *Xout, double *Yout, double *Cout, double *trace, int *ntrace,
              double *rho_out, int *iters_out) {
  const int str = ph->str, dim = ph->dim, K = ph->num_of_labels;
  const size_t size = ph->size, col = ph->col, nent = (size_t)str * col;
  const int euclid = ph->metric == D2O_EUCLIDEAN_L2, embed = ph->metric == D2O_WORD_EMBED;
  int rc = 0, nt = 0, iter;
  if (str <= 0 || size == 0 || col == 0 || K <= 0) return -1;

  size_t *cum = malloc(size * sizeof(size_t));
  double *C = malloc(nent * sizeof(double)), *X = malloc(nent * sizeof(double));
  double *Y = malloc(nent * sizeof(double)), *Z0 = malloc(nent * sizeof(double));
  double *Xc = malloc((col > (size_t)K ? col : (size_t)K) * sizeof(double) + sizeof(double));
  size_t zr_n = (size > (size_t)K ? size : (size_t)K) * str;
  double *Zr = malloc(zr_n * sizeof(double));
  size_t *count = calloc(K, sizeof(size_t));
  if (!cum || !C || !X || !Y || !Z0 || !Xc || !Zr || !count) { rc = -1; goto done; }

  cum[0] = 0; /* p_str_cum as built by d2_read, clustering_io.c:176-181 */
  for (size_t i = 1; i < size; ++i) cum[i] = cum[i - 1] + ph->p_str[i - 1];

  /* histograms: C is the cost filled by the caller at allocation (clustering_util.c:183-198) */
  if (!euclid && !embed)
    for (size_t i = 0; i < size; ++i) cost_block(ph, i, cum[i], c_supp, C + str * cum[i]);
  calc_distmat(ph, cum, c_supp, C); /* :106 */

  /* rho from the initial cost, then C /= rho: :109-110 */
  double asum = 0;
  for (size_t e = 0; e < nent; ++e) asum += fabs(C[e]);
  double rho = opt->rhoCoeff * asum / (double)nent;
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

    /* step 6, :300-316 */
    if ((iter % 100 == 99) || (iter < 100 && iter % 20 == 19)) {
      double obj = 0, pr = 0, dr = 0;
      for (size_t e = 0; e < nent; ++e) obj += C[e] * X[e];
      for (size_t e = 0; e < nent; ++e) X[e] += -1 * Z[e];
      for (size_t e = 0; e < nent; ++e) Z0[e] += -1 * Z[e];
      for (size_t e = 0; e < nent; ++e) pr += fabs(X[e]);
      for (size_t e = 0; e < nent; ++e) dr += fabs(Z0[e]);
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
  return rc;
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
