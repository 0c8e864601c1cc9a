/*
 * TEST INFRASTRUCTURE ONLY: the CPU oracle for the B-ADMM centroid update.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may
 * load anything built from this directory, and only as the checker or the
 * timed CPU baseline.  The product (d2_kmeans_gb300/libd2g.so) never links
 * or calls it.
 *
 * One plain-array interface, two implementations:
 *   d2o_badmm  - d2_oracle.c, a C restatement of the reference algorithm
 *                (src/d2/centroid_Bregman.c:51-325 and the helpers it calls);
 *                it builds on any host, including the GPU machine.
 *   d2r_badmm  - ref_harness.c, which fills the reference's own sph / mph /
 *                var_mph structures and calls the reference's compiled
 *                d2_centroid_sphBregman (built from the reference sources by
 *                oracle/Makefile into oracle/_ref/, only where the reference
 *                tree is present).
 * Both take the same arguments and produce the same outputs, so a test can
 * check one against the other bit for bit.
 */
#ifndef D2_ORACLE_H_
#define D2_ORACLE_H_
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* metric codes are the reference's (include/d2/param.h:23-28) */
#define D2O_EUCLIDEAN_L2 0
#define D2O_HISTOGRAM 5
#define D2O_N_GRAM 6
#define D2O_WORD_EMBED 7
#define D2O_SPARSE_HISTOGRAM 12

typedef struct {
  int metric;            /* one of the D2O_* codes */
  int dim;               /* support dimension (Euclidean / embedding), 0 for histograms */
  int str;               /* centroid support size m */
  size_t size;           /* number of instances n */
  size_t col;            /* sum of p_str */
  const int *p_str;      /* [size] support size of each instance */
  const double *p_w;     /* [col] instance weights (each instance sums to 1) */
  const double *p_supp;  /* [col*dim] Euclidean supports, row per support point */
  const int *p_supp_sym; /* [col] 0-based vocabulary / bin ids (embedding, sparse histogram);
                            [col*dim] symbols, dim per support point (n-gram) */
  const double *vocab_vec; /* [vocab_size*dim] embedding vectors */
  int vocab_size;        /* vocabulary size, or number of bins for histograms */
  const double *dist_mat;  /* [vocab_size*vocab_size] bin-to-bin cost (histograms) or
                              symbol-to-symbol cost (n-gram) */
  const int *label;      /* [size] cluster of each instance */
  int num_of_labels;     /* k */
  const char *label_switch; /* [size] 1 = re-initialise this instance's plan */
  size_t global_size;    /* N used to normalise obj/primres/dualres */
  int *c_sym;            /* n-gram only: [k*str*dim] centroid symbols, in/out (the
                            reference's c->p_supp_sym); NULL for other metrics */
} d2o_phase;

typedef struct {
  int maxIters;          /* the loop runs maxIters+1 iterations */
  double rhoCoeff;
  int updatePerLoops;
  double time_budget;    /* seconds; the loop stops after an iteration that exceeds it */
} d2o_opts;

/* Outputs.  c_w [k*str] and c_supp [k*str*dim] are in/out (initial centroids
 * in, updated centroids out); Z [str*col] is in/out (warm-start plans for
 * instances whose label_switch is 0).  X, Y and C [str*col] are optional
 * outputs (NULL to skip); C is returned already divided by rho.  trace gets 4
 * doubles (iter+1, obj, primres, dualres) per residual check and *ntrace the
 * number of checks; rho_out (optional) gets rho; iters_out (optional) gets the
 * number of iterations run.  Returns 0, or -5 for an empty cluster, -6 for a
 * non-positive normaliser, -1 for invalid arguments. */
int d2o_badmm(const d2o_phase *ph, const d2o_opts *opt, double *c_w, double *c_supp,
              double *Z, double *X, double *Y, double *C, double *trace, int *ntrace,
              double *rho_out, int *iters_out);

/* The reference's MPI build of the same update (src/d2/centroid_Bregman.c
 * with __USE_MPI__): this process holds one shard of the instances
 * (global_size = all ranks' instances) and every MPI_Allreduce of the
 * reference becomes a call of xr, which must SUM the n doubles of buf in
 * place over all ranks and return 0.  Each rank's rho comes from its own
 * instances, as in the reference; global_rho != 0 takes it over all ranks. */
typedef int (*d2o_allreduce_fn)(double *buf, size_t n, void *ctx);
int d2o_badmm_mpi(const d2o_phase *ph, const d2o_opts *opt, double *c_w, double *c_supp,
                  double *Z, double *trace, int *ntrace, double *rho_out, int *iters_out,
                  d2o_allreduce_fn xr, void *xctx, int global_rho);

int d2r_badmm(const d2o_phase *ph, const d2o_opts *opt, double *c_w, double *c_supp,
              double *Z, double *X, double *Y, double *C, double *trace, int *ntrace,
              double *rho_out, int *iters_out);

/* Fixed-centroid transport solve used by the serving loop: for one query
 * distribution (m_q supports in R^dim, weights w_q) and each of k resident
 * centroids (str supports, weights c_w, supports c_supp), run B-ADMM steps
 * 1-3 of src/d2/centroid_Bregman.c:155-175 with the centroid weights held
 * fixed, for iters iterations starting from Z = c_w (x) w_q, Y = 0, with
 * rho = rhoCoeff * mean(C) over the query's k plans (the reference takes rho
 * over all plans of the phase, :109).  cost_out[l] receives
 * <C_l, X_l> (unnormalised ground cost of the final plan); returns the argmin
 * centroid.  The reference has no such function; this is the oracle of the
 * serving path. */
int d2o_serve_query(int dim, int str, int k, const double *c_w, const double *c_supp,
                    int m_q, const double *w_q, const double *supp_q, int iters,
                    double rhoCoeff, double *cost_out);

/* Ground costs of every instance against its cluster's centroid, C [str*col],
 * instance i's block column-major str x m_i at str*cum[i] (the per-instance
 * blocks of calculate_distmat, src/d2/centroid_util.c:8-36, through
 * _dpdist2 / _dpdist2_sym / _dpdist_symbolic, src/utils/blas_like64.c:199-242;
 * histograms get the copy of their cost matrix that the harness fills in,
 * because the reference's calculate_distmat leaves their C untouched).
 * c_supp: [k*str*dim] Euclidean / embedding centroids; n-gram centroids come
 * from ph->c_sym. */
void d2o_cost_blocks(const d2o_phase *ph, const double *c_supp, double *C);

/*
 * d2 input files (the reference's d2_read, src/d2/clustering_io.c:14-201,
 * into the mph of its d2_allocate, src/d2/clustering_util.c:93-130).  The
 * mph is returned as an opaque pointer with the reference's layout
 * (include/d2/clustering.h:14-51); free it with the matching *_mph_free.
 *   d2o_read - d2_oracle.c, a restatement (token by token with fscanf).
 *   d2r_read - ref_harness.c, the reference's own d2_allocate + d2_read.
 */
int d2o_read(const char *filename, const char *meta_filename, int s_ph, size_t size,
             const int *avg_strides, const int *dims, const int *types, void **out_mph);
int d2o_mph_free(void *p_mph);

/* Exact transport cost between a row distribution wX[n] and a column
 * distribution wY[m] under C (column-major, C[i + j*n]), the linear program
 * of d2_match_by_distmat (src/d2/solver_mosek.cc:61-226) with the last column
 * constraint left free.  Successive shortest paths in FP64 (emd_oracle.c).
 * x_out (optional): the n*m plan, column-major. */
double d2o_emd(int n, int m, const double *C, const double *wX, const double *wY, double *x_out);

/* The assignment step restated (labeling_oracle.c, src/d2/clustering.c:33-376)
 * on the reference's structures (include/d2g.h); the mph / var_mph pointers
 * are passed as void * here so this header stays free of those types. */
double d2o_compute_distance(const void *a, size_t i, const void *b, size_t j, int selected_phase);
size_t d2o_labeling_prep(void *p_data, const void *centroids, void *var_work, int selected_phase,
                         size_t *dist_count);
void d2o_labeling_post(void *p_data, const void *c_old, const void *c_new, void *var_work,
                       int selected_phase);
size_t d2o_labeling(void *p_data, const void *centroids, void *var_work, int selected_phase,
                    double *cost);
int d2r_read(const char *filename, const char *meta_filename, int s_ph, size_t size,
             const int *avg_strides, const int *dims, const int *types, void **out_mph);
int d2r_mph_free(void *p_mph);

#ifdef __cplusplus
}
#endif
#endif
