/*
 * d2g - GB300-native B-ADMM Wasserstein-barycenter centroid update for
 * discrete-distribution (D2) clustering.  C ABI of libd2g.so.
 *
 * Two layers:
 *
 * 1. Drop-in entry points with the reference's own names, signatures and
 *    data layout (bobye/d2_kmeans, include/d2/clustering.h).  A program built
 *    against the reference links libd2g.so in place of
 *    src/d2/centroid_Bregman.o (and src/d2/centroid_util.o) and its
 *    d2_clustering() loop runs the centroid update on the GPU.
 *
 * 2. A resident API (d2g_phase_*, d2g_badmm_run) that keeps one phase's
 *    supports, weights and transport plans in HBM across calls, and a
 *    serving API (d2g_server_*) for fixed-centroid transport solves of
 *    arriving query distributions.
 *
 * All entry points return 0 on success and a negative D2G_E* code on failure;
 * none aborts the process (the reference assert()s instead).
 */
#ifndef D2G_H_
#define D2G_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ errors */
#define D2G_OK 0
#define D2G_E_INVAL (-1)         /* invalid argument or shape */
#define D2G_E_CUDA (-2)          /* CUDA runtime / launch failure */
#define D2G_E_NOMEM (-3)         /* device or pinned host allocation failed */
#define D2G_E_UNSUPPORTED (-4)   /* metric type or shape this build does not run */
#define D2G_E_EMPTY_CLUSTER (-5) /* a cluster has no instance (reference: assert, centroid_Bregman.c:144) */
#define D2G_E_NUMERIC (-6)       /* non-positive or non-finite normaliser (reference: assert, blas_like64.c:131,148) */
#define D2G_E_ADMISSION (-7)     /* serving: request refused by the HBM budget or queue bound */
#define D2G_E_NOTFOUND (-8)      /* serving: unknown ticket */

/* -------------------------------------------- reference data model (ABI) */
/* Layout-identical to include/d2/clustering.h:14-200 and include/d2/param.h:4-8
 * of the reference built with _D2_DOUBLE (SCALAR = double, the default of
 * make.inc.Linux64:14).  Skipped when the reference header is already
 * included, so reference code can include both. */
#ifndef _D2_CLUSTERING_H_
typedef struct {
  int dim, str, max_str;
  size_t col, max_col;
  int *p_str;
  size_t *p_str_cum;
  double *p_w;
  int metric_type;
  double *p_supp;
  int *p_supp_sym;
  double *dist_mat;
  int vocab_size;
  double *vocab_vec;
  char is_meta_allocated;
} sph;

typedef struct {
  double *l, *u, *s, *c;
  char *r;
} trieq;

typedef struct {
  int s_ph;
  size_t size;
  size_t global_size;
  int *label;
  int num_of_labels;
  sph *ph;
} mph;

typedef struct {
  double *C;
  double *X;
  double *L;
} var_sph;

typedef struct {
  double *X, *Z;
  double *Y;
  double *Xc, *Zr;
} var_sphBregman;

typedef struct {
  int s_ph;
  var_sph *g_var;
  var_sphBregman *l_var_sphBregman;
  char *label_switch;
  trieq tr;
} var_mph;
#endif /* _D2_CLUSTERING_H_ */

#ifndef _D2_PARAM_H_
typedef struct {
  int maxIters;
  double rhoCoeff;
  int updatePerLoops;
} BADMM_options;
#define D2_EUCLIDEAN_L2 (0)
#define D2_CITYBLOCK_L1 (1)
#define D2_HISTOGRAM (5)
#define D2_N_GRAM (6)
#define D2_WORD_EMBED (7)
#define D2_SPARSE_HISTOGRAM (12)
#endif /* _D2_PARAM_H_ */

/* ------------------------------------------------- drop-in entry points */

/* Replaces d2_allocate_work_sphBregman, src/d2/centroid_Bregman.c:26-35
 * (declared include/d2/clustering.h:223-224).  Allocates the same host work
 * buffers X, Z, Y (str*col), Xc (col) and Zr (str*size). */
int d2_allocate_work_sphBregman(sph *ph, size_t size, var_sphBregman *var_phwork);

/* Replaces d2_free_work_sphBregman, src/d2/centroid_Bregman.c:37-44
 * (clustering.h:225).  Also releases the device state kept for this work
 * object. */
int d2_free_work_sphBregman(var_sphBregman *var_phwork);

/* Replaces d2_centroid_sphBregman, src/d2/centroid_Bregman.c:51-325
 * (clustering.h:226-230).  Same inputs (phase idx_ph of p_data, labels,
 * label_switch, c0 as the warm start), same outputs: c->p_w and c->p_supp
 * updated in place (c->p_supp_sym for n-gram phases), the plans Z left in
 * var_work->l_var_sphBregman[idx_ph].Z for the next call's warm start.
 * Honours p_badmm_options (maxIters+1 iterations, rhoCoeff, updatePerLoops)
 * and the global time_budget.  Metric types: D2_EUCLIDEAN_L2, D2_WORD_EMBED,
 * D2_HISTOGRAM, D2_SPARSE_HISTOGRAM, D2_N_GRAM.  c0 == NULL
 * (:95-98) initialises c with d2_centroid_rands when the program links it
 * (src/d2/centroid_rand.c:161-295, found by dlsym), else with
 * d2g_centroid_rands.  The host X, Y
 * and C buffers are scratch for the reference's callers and are only written
 * back when d2g_config.sync_scratch is set. */
int d2_centroid_sphBregman(mph *p_data, var_mph *var_work, int idx_ph, sph *c0, sph *c);

/* Replaces calculate_distmat, src/d2/centroid_util.c:8-36 (declared
 * include/d2/centroid_util.h:40): the per-instance str x p_str[i] ground-cost
 * blocks between each instance and its labelled centroid, written into the
 * host array C at offset str*p_str_cum[i].  Computed on the GPU in FP64
 * (Euclidean, word-embedding and n-gram phases; histogram costs are fixed). */
void calculate_distmat(sph *data_ph, int *label, size_t size, sph *c, double *C);

/* No counterpart in the reference.  The ground costs of calculate_distmat for
 * callers that cannot allocate GPU memory (code that runs inside another
 * runtime's allocator or is handed only pre-allocated device buffers): every
 * pointer is a device pointer the caller owns - p_str [size], p_supp
 * [col*dim] or p_supp_sym [col] + vocab_vec [vocab_size*dim], label [size],
 * c_supp [num_of_labels*str*dim] in, C [str*col] out - and the working data
 * (prefix sums, column map) lives in an 8 MiB array fixed inside libd2g.so
 * on each GPU, so the call allocates no device memory.  Needs 8*size +
 * 4*col + 256 bytes of that array and returns D2G_E_INVAL beyond it.  Calls
 * share the array: calls whose GPU work overlaps race, so serialise them.
 * The first call on a device looks up the array's address; make it before
 * any stream capture.  Under CUDA's lazy module loading (the default unless
 * CUDA_MODULE_LOADING=EAGER) the array is created when the library's device
 * code first loads on a device, which may be that first call: make it at
 * set-up time.  Runs on `stream` (a cudaStream_t, NULL for the default stream)
 * and returns after the inputs are validated, with the cost kernel queued.
 * Euclidean and word-embedding phases only. */
int d2g_distmat_noalloc(int metric_type, int dim, int str, size_t size, size_t col,
                        const int *p_str, const double *p_supp, const int *p_supp_sym,
                        const double *vocab_vec, int vocab_size, const int *label,
                        int num_of_labels, const double *c_supp, double *C, void *stream);

/* The result of d2_centroid_rands, src/d2/centroid_rand.c:161-295 (declared
 * include/d2/clustering.h:216-218), for a program that does not link the
 * reference's own: random instances (glibc rand() order after srand(0), as
 * the reference's shuffle in a single process, src/d2/math.c:40-58) with at
 * least str supports become the centroids of phase idx_ph, larger ones
 * merged down to str (merge / merge_symbolic, centroid_rand.c:53-159).  c's
 * arrays are the caller's (d2_allocate_sph's layout); the process-wide rand()
 * state is not touched.  D2G_E_INVAL where the reference exit(1)s for too few
 * instances.  d2_centroid_sphBregman with c0 == NULL and d2g_clustering with
 * no centroids use the program's d2_centroid_rands when it links one, else
 * this. */
int d2g_centroid_rands(mph *p_data, int idx_ph, sph *c);

/* The result of d2_write_split, src/d2/clustering_io.c:329-480 (declared
 * include/d2/clustering.h:149), with the same signature: the shard files of
 * a sharded run.  The instances in the reference's shuffled order (its
 * shuffle after srand(0), one writing process) go to <filename>.ind and, in
 * contiguous batches of 1 + (size-1)/splits, to <filename>.0 ..
 * <filename>.<splits-1> in the d2 text format, byte for byte the reference's
 * files; is_pre_processed != 0 applies the reference's pre-processing
 * (embedding supports as vectors, supports merged down to str, dense
 * histograms as their non-zero bins) to Euclidean, word-embedding and dense
 * histogram phases and returns D2G_E_UNSUPPORTED for the others (where the
 * reference reads through a null pointer). */
int d2g_write_split(const char *filename, mph *p_data, int splits, char is_pre_processed);

/* Option structs of src/d2/centroid_Bregman.c:17-22 (the caller swaps
 * p_badmm_options, e.g. src/app/main.cc:234-236). */
extern BADMM_options badmm_clu_options;
extern BADMM_options badmm_cen_options;
extern BADMM_options *p_badmm_options;

/* Seconds after which the B-ADMM loop stops (centroid_Bregman.c:24,318).
 * The reference's driver defines and sets it (src/d2/clustering.c:21,240,373);
 * libd2g.so carries a weak definition, initialised to 1e300, for programs
 * that link it without that driver. */
extern double time_budget;

/* ------------------------------------------------------- library control */
typedef struct {
  int precision;    /* 0: FP32 plans + FP64 reductions (default); 1: FP64 throughout */
  int verbose;      /* 1: print the reference's iter/obj/primres/dualres lines */
  int use_graph;    /* 1: replay the iteration loop as one CUDA graph (default) */
  int sync_scratch; /* 1: also write the host X, Y and C back after a drop-in call */
  int profile;      /* 1: time every plan-update launch with CUDA events (no graph) */
  int cost_gemm;    /* word-embedding cost table of phases created afterwards:
                       0 tensor cores, 3xTF32 (default); 1 FP32 CUDA cores */
  int keep_time_budget; /* 0: the labelings set time_budget from their wall time as
                           the reference's do (default); 1: they leave it as it is */
  int pair_iterations;  /* 1: the batched form runs two iterations per pass over the
                           plans where that is exact (default); 0: one per pass */
} d2g_config;

int d2g_get_config(d2g_config *cfg);
int d2g_set_config(const d2g_config *cfg);
const char *d2g_error_string(int code);
/* last error message of this thread, "" if none */
const char *d2g_last_error(void);

/* ------------------------------------------------------------ resident API */
typedef struct d2g_phase d2g_phase;

typedef struct {
  int metric_type;          /* D2_EUCLIDEAN_L2, D2_WORD_EMBED, D2_HISTOGRAM, D2_SPARSE_HISTOGRAM,
                               D2_N_GRAM */
  int dim;                  /* support dimension (0 for histograms; n-gram length) */
  int str;                  /* centroid support size m */
  size_t size;              /* instances n */
  const int *p_str;         /* [size] */
  const double *p_w;        /* [col] */
  const double *p_supp;     /* [col*dim] Euclidean supports */
  const int *p_supp_sym;    /* [col] 0-based ids (embedding, sparse histogram);
                               [col*dim] symbols, dim per support point (n-gram) */
  const double *vocab_vec;  /* [vocab_size*dim] embedding vectors */
  const double *dist_mat;   /* [vocab_size*vocab_size] histogram bin cost, or the
                               symbol cost of an n-gram phase (row: centroid symbol) */
  int vocab_size;           /* vocabulary size / number of bins / n-gram alphabet size */
  const int *label;         /* [size] */
  int num_of_labels;        /* k */
  size_t global_size;       /* N normalising obj/primres/dualres (0 = size) */
} d2g_phase_desc;

typedef struct {
  int maxIters;             /* maxIters+1 iterations, as the reference */
  double rhoCoeff;
  int updatePerLoops;
  double time_budget;       /* seconds; <= 0 means unlimited */
} d2g_badmm_opts;

typedef struct {
  int iterations;           /* iterations run by the last call */
  double rho;
  double total_ms;          /* device time of the last call's iteration loop */
  double plan_ms_avg;       /* mean plan-update launch time (profile mode) */
  int plan_launches;        /* plan-update launches timed (profile mode) */
  long long kernel_launches;/* kernels launched by the last call */
  double plan_bytes;        /* algorithmic HBM bytes of one plan-update pass */
  size_t plan_entries;      /* str * col */
  int path;                 /* 0 batched FP32, 1 plain FP64 */
  double table_ms_avg;      /* mean word-embedding cost-table launch time (profile mode) */
  int table_launches;       /* cost-table launches timed (profile mode) */
  double table_flops;       /* algorithmic flops of one cost table: 2 * (k*str) * V * dim */
} d2g_run_stats;

/* Upload a phase.  Host arrays are copied; labels can change later. */
int d2g_phase_create(const d2g_phase_desc *desc, int precision, d2g_phase **out);
int d2g_phase_destroy(d2g_phase *ph);
/* Re-send weights, supports / ids, cost data and labels of a phase whose
 * shape (metric, dim, str, size, p_str) is unchanged. */
int d2g_phase_refresh(d2g_phase *ph, const d2g_phase_desc *desc);
/* new labels (k-means reassignment) */
int d2g_phase_set_labels(d2g_phase *ph, const int *label);
/* warm-start plans in the reference layout (str*col, column-major per instance) */
int d2g_phase_set_plans(d2g_phase *ph, const double *Z);
int d2g_phase_get_plans(d2g_phase *ph, double *Z);
/* One centroid update.  c_w [k*str] and c_supp [k*str*dim] (NULL for
 * histograms) are host arrays, read as the start point and overwritten with
 * the result.  label_switch [size] (NULL = all 1) selects plans to re-initialise.
 * N-gram phases use d2g_badmm_run_sym. */
int d2g_badmm_run(d2g_phase *ph, const d2g_badmm_opts *opt, double *c_w, double *c_supp,
                  const char *label_switch);
/* One centroid update of an n-gram phase (src/d2/centroid_Bregman.c:269-294):
 * c_sym [k*str*dim] holds the centroids' symbols (the reference's
 * c->p_supp_sym), read as the start point and overwritten with the result;
 * every updatePerLoops iterations after the first, each centroid symbol
 * moves to the symbol of least expected cost under the plans. */
int d2g_badmm_run_sym(d2g_phase *ph, const d2g_badmm_opts *opt, double *c_w, int *c_sym,
                      const char *label_switch);
/* obj/primres/dualres of the last run: 4 doubles (iter+1, obj, primres, dualres) per check */
int d2g_phase_trace(d2g_phase *ph, double *trace, int cap, int *n);
int d2g_phase_stats(d2g_phase *ph, d2g_run_stats *st);
/* the CUDA stream (cudaStream_t) every kernel of this phase is launched on */
void *d2g_phase_stream(d2g_phase *ph);
/* the last run's X (after step 1, or X-Z after a check iteration as the
 * reference leaves it), Y and C (divided by rho), reference layout, FP64 */
int d2g_phase_get_scratch(d2g_phase *ph, double *X, double *Y, double *C);
/* ------------------------------------------------- sharded centroid update
 * The reference's MPI build (src/d2/centroid_Bregman.c with __USE_MPI__)
 * splits the instances of a phase over ranks and all-reduces, by SUM, the
 * label counts (:142), the cluster weights (:188), the support numerators and
 * X row sums (:215-217) and obj / primres / dualres (:308-310).  A phase
 * created on one shard of the instances, with d2g_phase_desc.global_size set
 * to the instance count of all shards, runs the same update here once it has
 * an all-reduce: fn(buf, count, stream, ctx) must enqueue on `stream` (a
 * cudaStream_t) an in-place SUM of the count FP64 values of the device buffer
 * buf over all shards - e.g. ncclAllReduce(buf, buf, count, ncclDouble,
 * ncclSum, comm, stream) - and return 0.  It is called on the host while the
 * update is enqueued, the same calls in the same order on every shard; the
 * loop then runs without a CUDA graph.  Each shard takes rho from its own
 * instances, as the reference does; D2G_SHARD_GLOBAL_RHO takes it over all
 * shards (two more values exchanged).  Covers the batched form of Euclidean
 * and histogram phases without a time budget; fn == NULL turns it off. */
typedef int (*d2g_allreduce_fn)(double *buf, size_t count, void *stream, void *ctx);
#define D2G_SHARD_GLOBAL_RHO 1
int d2g_phase_set_allreduce(d2g_phase *ph, d2g_allreduce_fn fn, void *ctx, int flags);
/* The sharded update of nshard (<= 8) phases on the current device, one host
 * thread per shard, the all-reduce done between the shards' streams (a sum
 * over the shards' buffers in shard order).  c_w[s] and c_supp[s] are each
 * shard's centroids in and out (c_supp may be NULL for histograms); every
 * shard ends with the same centroids. */
int d2g_badmm_run_shards(d2g_phase *const *ph, int nshard, const d2g_badmm_opts *opt, int flags,
                         double *const *c_w, double *const *c_supp);

/* Test hook of the bounded device waits (no counterpart in the reference).
 * Every wait of the batched plan kernels for their bulk copies gives up after
 * wait_s seconds (0: one second), reports through the phase's control block
 * and the run returns D2G_E_CUDA; the phase and the CUDA context stay usable.
 * With unit >= 0 the plan pass of iteration iter withholds the tile copy of
 * that unit (its CTA's wait then runs out); unit < 0 turns the hook off.
 * Cluster launches (plans wider than one CTA, exchanged synchronously) ignore
 * the hook. */
int d2g_phase_test_wait(d2g_phase *ph, int iter, int unit, double wait_s);

/* ------------------------------------------------------------ d2 input files
 * Replaces d2_read, src/d2/clustering_io.c:14-201 (declared
 * include/d2/clustering.h:144), with the same signature and result: reads the
 * reference's d2 text formats (.d2 multi-phase Euclidean; dense histograms
 * with a .histN cost file; .d2s symbolic supports with a .vocabN embedding
 * file; sparse histograms) into an mph allocated by the reference's
 * d2_allocate (or by d2g_mph_alloc), growing its arrays when needed.  The
 * file is parsed in parallel (D2G_IO_THREADS threads, default all cores).
 * Malformed input returns D2G_E_INVAL (the reference asserts). */
int d2g_read(const char *filename, const char *meta_filename, mph *p_data);
/* The data part of d2_allocate (src/d2/clustering_util.c:93-130): phases,
 * labels (-1), per-phase arrays for size objects of avg_strides[n] + 0.6
 * support points on average.  d2g_mph_free releases it (and the cost /
 * vocabulary arrays d2g_read attached). */
int d2g_mph_alloc(int s_ph, size_t size, const int *avg_strides, const int *dims,
                  const int *types, mph **out);
int d2g_mph_free(mph *p_data);

/* ------------------------------------------- exact transport (assignment)
 * The assignment step's distances: the exact optimal transport cost of
 * d2_match_by_distmat (src/d2/solver_mosek.cc:61-226, a MOSEK network
 * simplex in the reference), computed on the GPU by a transportation simplex
 * (one warp per pair, FP32 pricing, FP64 optimality check and cost). */
typedef struct {
  size_t size;           /* objects */
  int str;               /* support count of every object when p_str is NULL */
  const int *p_str;      /* [size] support counts, or NULL */
  const double *p_w;     /* weights, object after object (each sums to 1) */
  const double *p_supp;  /* [.. * dim] Euclidean supports (D2_EUCLIDEAN_L2) */
  const int *p_supp_sym; /* bin ids (D2_SPARSE_HISTOGRAM); NULL: bin = support index */
} d2g_dists;

/* Exact transport cost of each pair (rows object pair_row[p], cols object
 * pair_col[p]) for metric D2_EUCLIDEAN_L2 (dim 1..7, squared Euclidean
 * ground cost in the difference form of _dpdist2, blas_like64.c:199-208),
 * D2_HISTOGRAM or D2_SPARSE_HISTOGRAM (ground cost dist_mat, vocab_size^2,
 * row-major by row bin).  Row sums are fixed to the row weights, column sums
 * to the column weights except the last column's, as in the reference's
 * program (solver_mosek.cc:64, :134-140).  cost[npairs]; pivots[npairs]
 * (optional): simplex pivots per pair.  D2G_E_NUMERIC if a pair did not
 * reach an optimal basis within 64 * (n + m rounded to 32) + 1024 pivots. */
int d2g_emd_pairs(int metric_type, int dim, const d2g_dists *rows, const d2g_dists *cols,
                  const double *dist_mat, int vocab_size, size_t npairs, const int *pair_row,
                  const int *pair_col, double *cost, int *pivots);

/* The assignment step on the reference's structures (src/d2/clustering.c:
 * 33-376); every distance is the square root of the phases' summed exact
 * transport costs, as d2_compute_distance returns it (an n-gram phase adds
 * 2 * cost / dim, clustering.c:102-115).  Metric types: D2_EUCLIDEAN_L2,
 * D2_HISTOGRAM, D2_SPARSE_HISTOGRAM, D2_WORD_EMBED, D2_N_GRAM.  The instances'
 * device copy is kept across calls while their arrays stay the same. */

/* out[p] = d2_compute_distance(a, ia[p], b, jb[p], selected_phase, ...) */
int d2g_compute_distances(mph *a, mph *b, int selected_phase, size_t npairs, const int *ia,
                          const int *jb, double *out);
/* d2_labeling (clustering.c:327-376): every instance to its nearest
 * centroid (first of equals), label_switch as the reference sets it;
 * *count = labels changed, *cost = sum of squared nearest distances. */
int d2g_labeling(mph *p_data, mph *centroids, var_mph *var_work, int selected_phase,
                 size_t *count, double *cost);
/* d2_labeling_prep (clustering.c:134-248), Elkan's pruning with the bounds in
 * var_work->tr: the same distances computed, bounds written and labels as
 * the reference's loop; *dist_count = distances computed. */
int d2g_labeling_prep(mph *p_data, mph *centroids, var_mph *var_work, int selected_phase,
                      size_t *count, size_t *dist_count);
/* d2_labeling_post (clustering.c:287-318): bounds after a centroid update */
int d2g_labeling_post(mph *p_data, mph *c_old, mph *c_new, var_mph *var_work, int selected_phase);

/* The reference's own entry points with its signatures (clustering.h); a
 * failure returns NaN / (size_t)-1 with the message in d2g_last_error.  The
 * labelings set time_budget as the reference does (clustering.c:245, :372). */
double d2_compute_distance(mph *a, size_t i, mph *b, size_t j, int selected_phase,
                           var_mph *var_work, size_t index_task);
size_t d2_labeling(mph *p_data, mph *centroids, var_mph *var_work, int selected_phase);
size_t d2_labeling_prep(mph *p_data, mph *centroids, var_mph *var_work, int selected_phase);
size_t d2_labeling_post(mph *p_data, mph *c_old, mph *c_new, var_mph *var_work, int selected_phase);
extern int d2_alg_type; /* clustering.c:24; label_switch is written when 0 (B-ADMM) */

/* The outer loop, d2_clustering (src/d2/clustering.c:409-525): rounds of
 * labeling (Elkan's pruning when use_triangle) and B-ADMM centroid updates
 * (p_badmm_options) until fewer than 0.1 % of the instances change label or
 * max_iter rounds; centroids->ph == NULL initialises them with the program's
 * d2_centroid_rands, or d2g_centroid_rands where it links none.  Log files <log_file>_c.d2 / <log_file>.label every
 * tenth round when log_file is given.  *rounds (optional): rounds run. */
int d2g_clustering(int num_of_clusters, int max_iter, mph *p_data, mph *centroids,
                   int selected_phase, int use_triangle, const char *log_file, int *rounds);
/* One labeling against given centroids (the labeling of d2_assignment,
 * clustering.c:528-548); *count = labels changed. */
int d2g_assignment(int num_of_clusters, mph *p_data, mph *centroids, int selected_phase,
                   size_t *count);
/* The reference's signature; returns 0 or a negative D2G_E* code. */
int d2_clustering(int num_of_clusters, int max_iter, mph *p_data, mph *centroids,
                  int selected_phase, char use_triangle, const char *log_file);

/* ------------------------------------------------------------- autotuning
 * Launch-shape choices of the batched form.  All choices compute the same
 * B-ADMM iteration; they differ in speed (and, for exchange, in the rounding
 * of Y's update: two FP32 roundings instead of one). */
typedef struct {
  int exchange;     /* plans wider than one CTA: 0 deferred row normalisation (one plain
                       launch over packed units), 1 synchronous DSMEM exchange on a
                       thread-block cluster per plan */
  int stage_costs;  /* table costs (16 <= padded str <= 128): the next unit's cost-table rows
                       copied into shared memory with cp.async while a unit computes (1,
                       default) or read through the cache (0) */
  int ctas_per_sm;  /* persistent plan-update grid: CTAs per SM, 0 = occupancy limit */
  int cost_gemm;    /* word-embedding cost table: 0 tensor cores (3xTF32), 1 CUDA cores */
  int pairs;        /* plans that all fit one CTA: 1 two iterations per pass over the plans
                       where the reference's schedule allows it, 0 one iteration per pass */
  int unit_order;   /* order in which the persistent grid walks the units of plans that fit
                       one CTA: 0 packing order, 1 largest unit first */
  int stage_scales; /* pair passes: 1 each unit's deferred row scales arrive in shared memory
                       with its tiles (where that keeps the CTAs per SM), 0 read by each thread */
} d2g_tuning;

int d2g_phase_get_tuning(d2g_phase *ph, d2g_tuning *t);
int d2g_phase_set_tuning(d2g_phase *ph, const d2g_tuning *t);
/* Time every candidate tuning on this phase with short runs (opt->maxIters
 * iterations from c_w / c_supp, which are not modified; plans re-initialised
 * and restored afterwards), keep the fastest on the phase and record it under
 * the phase's shape key: in this process, and in the text file named by the
 * environment variable D2G_TUNE_CACHE when set.  Phases created later with
 * the same shape start from the recorded tuning.  An n-gram phase (c_supp
 * NULL) starts every trial from the centroid symbols of its last
 * d2g_badmm_run_sym call.  Up to max_out candidates
 * and their loop times (ms, best of two graph replays) are written to cands /
 * ms (either may be NULL); *n_out receives the number of candidates. */
int d2g_phase_autotune(d2g_phase *ph, const d2g_badmm_opts *opt, const double *c_w,
                       const double *c_supp, d2g_tuning *cands, double *ms, int max_out,
                       int *n_out);

/* ------------------------------------------------------------- serving API */
typedef struct d2g_server d2g_server;

typedef struct {
  int num_of_labels;        /* k resident centroids */
  int str;                  /* centroid support size m */
  int dim;                  /* support dimension */
  const double *c_w;        /* [k*str] */
  const double *c_supp;     /* [k*str*dim] */
  int iters;                /* B-ADMM iterations per solve */
  double rhoCoeff;
  size_t hbm_budget_bytes;  /* admission bound on in-flight request state */
  int max_queue;            /* admission bound on queued requests */
  int max_batch_entries;    /* plan entries per device batch (0 = default) */
} d2g_server_desc;

int d2g_server_create(const d2g_server_desc *desc, d2g_server **out);
int d2g_server_destroy(d2g_server *s);
/* Admit one query distribution (m_q supports in R^dim).  Copies the data.
 * Returns D2G_E_ADMISSION when the HBM budget or queue bound refuses it. */
int d2g_server_submit(d2g_server *s, int m_q, const double *w_q, const double *supp_q,
                      long long *ticket);
/* Advance the device loop: launch whatever is admitted and collect finished
 * batches.  Non-blocking unless wait != 0.  Returns the number of requests
 * completed by this call. */
int d2g_server_progress(d2g_server *s, int wait);
/* 1 and the result when done, 0 while pending; costs [k] may be NULL.
 * A finished ticket is released by the call that returns 1. */
int d2g_server_result(d2g_server *s, long long ticket, int *label, double *costs,
                      double *latency_ms);

#ifdef __cplusplus
}
#endif
#endif /* D2G_H_ */
