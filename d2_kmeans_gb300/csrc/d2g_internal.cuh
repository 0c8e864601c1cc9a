// Internal declarations shared by the d2g CUDA translation units.
//
// Device layout of one phase in the batched (FP32-plan) form
// --------------------------------------------------------------
// Plans are stored "packed": the centroid support axis is padded to MP, a
// power of two >= max(str, 4), and each plan (instance) is column-major
// MP x m_i with its columns rounded up to whole groups of S columns.  Plans
// are reordered so that the plans sharing one thread block ("item") are
// contiguous; item sizes come from a best-fit-decreasing packing over the
// per-instance column counts.  A plan larger than one block's columns spans a
// thread-block cluster of 2, 4 or 8 CTAs and is an item on its own.
//
//   Z, Y        float [MP * ncols_packed]   transport plan and scaled dual
//   col_w       float [ncols_packed]        instance weights (0 in pad columns)
//   col_supp    float [ncols_packed * DS]   Euclidean supports (DS = 4 or 8)
//   col_sym     int   [ncols_packed]        table row (bin / vocabulary id)
//   grp_meta    int   [ngroups]             plan << 4 | valid columns (1..S)
//   grp_rec     int4  [ngroups]             {plan's slot, plan's first group, label,
//                                            plan's groups << 12 | plan's index
//                                            among its item's plans << 4 | valid}
//   plan_*      int   [nplans]              first group, group count, label,
//                                           instance id, m_i
//   rowsum      float [nplans * MP]         per-plan row sums of step 2, normalised
//                                           to sum 1 (step 4's Zr), by cluster slot
//   xmom        float [nplans * (dim+1) * MP]  per-plan X moments (step 5), by slot
//
// A plan's slot is its position in the cluster-sorted plan order (clusters in
// label order, plans in instance order), so the cluster reductions read each
// cluster's per-plan outputs as one contiguous run.
//
// Cluster-level state is FP64 (cw64 [k*str], cs64 [k*str*dim]) with FP32
// copies padded to MP for the plan kernel (cw32 [k*MP], cs32 [k*MP*DS]).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/d2g.h"

namespace d2g {

// Plan-update CTA shape per padded support size MP: S columns per thread (one
// column group), NT threads.  (512 threads of 2 columns for MP = 256 -- the same
// 32 columns per CTA with twice the warps -- measured 15-20 % slower than 256
// threads of 4 columns: the column shuffles and row-partial sums double.)
__host__ __device__ constexpr int plan_cols_per_thread(int /*MP*/) { return 4; }
__host__ __device__ constexpr int plan_threads(int /*MP*/) { return 256; }
constexpr int kMaxCluster = 8;
constexpr float kRoundoff = 1e-9f;  // ROUNDOFF, src/d2/centroid_Bregman.c:20

// Euclidean costs from supports padded to 4 or 8 coordinates (EUCLID3: d = 3,
// stored padded to 4, summed over 3), or read from a cost table
enum CostMode { COST_EUCLID4 = 0, COST_EUCLID8 = 1, COST_TABLE = 2, COST_EUCLID3 = 3 };

enum PlanFlags {
  PF_UPDATE = 1,   // support-update iteration: emit X moments (Euclidean)
  PF_WRITE_X = 2,  // store X (packed) for a later pass
  PF_CHECK = 4,    // residual-check iteration
  PF_IN_DEF = 8,   // wide plans arrive deferred: Z' and U = Y + X, scaled by rowsc on load
  PF_OUT_DEF = 16, // wide plans leave deferred: Z', U and per-slice row partials
  PF_STAGE_SC = 32,// pair pass with deferred input: each unit's row scales come with its tiles
};

// Device control block, one per phase.  Everything an iteration reads that
// changes between calls lives here, so a captured graph stays valid.
struct Ctl {
  double rho;
  float inv_rho;
  float inv_rho_l2;          // log2(e)/rho (the batched form works in base 2)
  int stop_iter;             // first iteration that must not run
  unsigned long long t_start_ns;
  unsigned long long budget_ns;
  int iters_done;
  int err;                   // nonzero: numeric failure seen on device
  double rho_coeff;
  double global_size;
  // bounded waits of the plan kernels: limit in ns (0 = one second), and a
  // test hook that withholds the tile copy of unit fault_unit in the plan
  // pass of iteration fault_iter (-1 = none), so that one wait runs out
  unsigned long long wait_ns;
  int fault_iter, fault_unit;
};

// record a device failure in the control block; the first one wins (later
// kernels of the same run may fail as a consequence and must not hide it)
__device__ __forceinline__ void ctl_fail(Ctl *c, int code) { atomicCAS(&c->err, 0, code); }

struct PlanArgs {
  float *Z, *Y;
  const float *col_w, *col_supp;
  const int *col_sym;
  const int *grp_meta, *plan_g0, *plan_ng, *plan_label;
  const int *item_g0, *item_ng;
  const float *cw32, *cs32;
  const float *ctab;
  long long ctab_lstride;   // floats between labels' tables (0: one shared table)
  float *rowsum_out, *xmom_out, *X_out;
  double *resid_part;       // 4 doubles per CTA (obj, primres, dualres, -)
  Ctl *ctl;
  int m, dim, flags, cs, iter, resid_off;
  // per group {plan slot, plan first group, label, plan groups << 12 | plan within its item << 4 | valid}
  const int4 *grp_rec;
  const int *plan_slot;     // plan -> slot: position in cluster-sorted order (row-sum outputs)
  float *rowpart;           // [slot][8][MP] per-slice row sums of Z' (deferred wide plans)
  // row scale c_w / rowsum(Z') of the previous iteration: [slot][MP] for wide
  // plans, [plan][MP] in packed order for pair passes
  const float *rowsc;
  int ctas_per_sm;          // persistent grid of plain launches: CTAs per SM (0: occupancy limit)
  const int *col_crow;      // per packed column: cost-table row (label * V + token, or the bin)
  int stage_costs;          // table costs (16 <= MP <= 128): next unit's rows by cp.async into smem
  int wide;                 // the phase has plans wider than one CTA
  float *rowsum2_out;       // pair pass: step-4 row sums of the second iteration, by slot
  float *rawsum_out;        // pair pass: raw row sums of the second iteration's Z', by slot
  int nplans_chk, nlab_chk; // plans and clusters of the phase (self-check of staged records)
  const int2 *item_pp;      // per item {first plan in packed order, plans}
  int ctab_rows;            // rows of MP floats in ctab (bound of the staged row gather)
  int stage_scales;         // pair passes: deferred row scales staged with the tiles where possible
};

// per-MP launch geometry
struct Geo {
  int MP, RPT, TPC, G, JC, S, NT;
};
Geo geo_for(int MP);

// kernels_plan.cu
cudaError_t launch_plan(int MP, int mode, bool check, const PlanArgs &a, int nitems,
                        size_t smem, cudaStream_t st);
size_t plan_smem_bytes(int MP, int dim, int cs);
cudaError_t launch_rho_partial(int MP, int mode, const PlanArgs &a, int nitems, double *part,
                               cudaStream_t st);
cudaError_t launch_pack_convert(int MP, int dir, const PlanArgs &a, int nitems,
                                double *ref, const long long *plan_refcol,
                                const char *plan_reinit, const double *cw64, int str,
                                cudaStream_t st);
cudaError_t launch_pack_columns(int MP, const PlanArgs &a, int nitems, const long long *plan_refcol,
                                const double *w_ref, const double *supp_ref, const int *sym_ref,
                                float *col_w, float *col_supp, int *col_sym, int dim, int DS,
                                int dense_hist, cudaStream_t st);
cudaError_t launch_obj(int MP, int mode, const PlanArgs &a, int nitems, cudaStream_t st);
// plan_pair.cuh: two iterations per pass (phases without plans wider than a CTA, MP <= 128)
cudaError_t launch_plan_pair(int MP, int mode, bool check, const PlanArgs &a, int nitems, cudaStream_t st);

// defer_kernels.cu: deferred row normalisation of plans wider than one CTA
cudaError_t launch_rowsum_combine(const int4 *wide, int nwide, const float *rowpart,
                                  const float *cw32, int MP, int m, float *rowsum_out,
                                  float *rowsc, const Ctl *ctl, int iter, cudaStream_t st);
cudaError_t launch_plan_finalize(float *Z, float *Y, const int *item_g0, const int *item_ng,
                                 int nitems, int cs, int G, int S, int MP, const int4 *grp_rec,
                                 const float *rowsc, const unsigned char *def_iter, const Ctl *ctl,
                                 cudaStream_t st);
// pair passes: the row scale c_w / rowsum(Z') of every plan (packed order, from
// the raw sums by slot), after the cluster reduction of the pair's first
// iteration; and Z = Z' * scale, Y = U - Z over every packed column, where a
// single pass or the end follows
cudaError_t launch_pair_scale(const float *rawsum, const int *plan_slot, const int *plan_label,
                              const float *cw32, int nplans, int MP, int m, float *rowsc, const Ctl *ctl,
                              int iter, int nlab, cudaStream_t st);
cudaError_t launch_pair_finalize(float *Z, float *Y, const int *grp_meta, int ngroups, int S, int MP,
                                 const float *rowsc, int nplans, int *err, cudaStream_t st);

// kernels_reduce.cu
struct ClusterArgs {
  const float *rowsum32;     // batched: [nplans * MP]
  const double *rowsum64;    // plain:   [nplans * str]
  const float *xmom32;       // batched: [nplans * (dim+1) * MP]
  const double *xmom64;      // plain:   [nplans * (dim+1) * str]
  int rstride;               // row stride of rowsum / xmom planes (MP or str)
  const int *cl_ptr, *cl_plans;  // cl_plans == nullptr: outputs already in slot order
  int K, m, dim, chunk, nchunk;
  double *part;              // [K][nplane][nchunk][m]
  double *cw64, *cs64;
  float *cw32, *cs32;
  int MP, DS;
  Ctl *ctl;
  int iter;
  int do_weights, do_moments;
  const double *xsum;        // sharded update: the cluster sums over all shards (else null)
};
cudaError_t launch_cluster_reduce(const ClusterArgs &a, cudaStream_t st);
// the same in three steps for a sharded update: partials, this shard's sums
// (cluster_xsum_count doubles into xsum), then, after the exchange, the final
cudaError_t launch_cluster_partial(const ClusterArgs &a, cudaStream_t st);
cudaError_t launch_cluster_local(const ClusterArgs &a, double *xsum, cudaStream_t st);
cudaError_t launch_cluster_final(const ClusterArgs &a, cudaStream_t st);
size_t cluster_xsum_count(const ClusterArgs &a);
cudaError_t launch_rho_final(const double *part, int n, Ctl *ctl, double nent,
                             cudaStream_t st);
cudaError_t launch_rho_local(const double *part, int n, double nent, double *xbuf, cudaStream_t st);
cudaError_t launch_rho_set(const double *xbuf, Ctl *ctl, cudaStream_t st);
cudaError_t launch_resid_final(const double *part, int n, Ctl *ctl, double *trace_slot,
                               int iter, bool obj_from_slot3, cudaStream_t st, int xmode = 0,
                               double *xbuf = nullptr);
// sharded update on one device: the shards' exchange buffers summed in shard order
// Launchers cache each kernel's shared-memory attribute and resident grid per
// device (both apply to the current device); device ordinals below this bound.
constexpr int kMaxDevices = 64;
inline cudaError_t launch_device(int *dev) {
  cudaError_t e = cudaGetDevice(dev);
  if (e == cudaSuccess && (*dev < 0 || *dev >= kMaxDevices)) e = cudaErrorInvalidDevice;
  return e;
}

constexpr int kMaxShards = 8;
struct ShardBufs {
  const double *p[kMaxShards];
  int n;
};
cudaError_t launch_shard_sum(const ShardBufs &b, size_t n, double *out, cudaStream_t st);
cudaError_t launch_centroid_to_f32(const double *cw64, const double *cs64, float *cw32,
                                   float *cs32, int K, int m, int dim, int MP, int DS,
                                   cudaStream_t st);

// kernels_plain.cu (FP64, reference layout)
struct PlainArgs {
  double *C, *X, *Y, *Z, *Z0;
  const double *w, *supp, *vocab, *dist;
  const int *sym, *col_inst, *p_str, *label;
  const int *csym;          // n-gram centroid symbols [K*str*dim]
  const long long *cum;     // p_str_cum
  const char *reinit;
  double *zr;               // [size * str] row sums
  double *xmom;             // [size * (dim+1) * str]
  double *cw64, *cs64;
  double *part;
  Ctl *ctl;
  long long col, nent;
  int size, str, dim, metric, vocab_size, iter;
};
cudaError_t plain_cost(const PlainArgs &a, cudaStream_t st);
cudaError_t plain_rho(const PlainArgs &a, cudaStream_t st);
cudaError_t plain_init(const PlainArgs &a, cudaStream_t st);
cudaError_t plain_iter_steps(const PlainArgs &a, bool update, cudaStream_t st);
cudaError_t plain_check(const PlainArgs &a, cudaStream_t st);
unsigned plain_check_blocks(long long nent);
int plain_launches_per_iter(bool update, bool check);

// serve_kernel.cu
struct ServeArgs {
  const float *q_w;       // [cols] query weights of the batch
  const float *q_supp;    // [cols * dim] query supports
  const float *c_w32;     // [K * MP] centroid weights (0 in padded rows)
  const float *c_supp32;  // [K * MP * dim] centroid supports
  const int4 *items;      // {request, first centroid, plans in the item, groups per plan}
  const float4 *reqs;     // per request {column offset (int bits), m_q (int bits), log2(e)/rho, 0}
  float *cost_out;        // [requests * K]
  int *err;               // set when a cluster exchange wait ran out
  int K, m, dim, iters, cs;
};
cudaError_t launch_serve(int MP, const ServeArgs &a, int nitems, cudaStream_t st);
constexpr int serve_groups_per_cta(int MP) { return 1024 / MP; }  // 256 threads, 4 rows x 4 columns

// embed_kernels.cu (word-embedding phase, batched form)
struct EmbedArgs {
  const int *pair_key, *pair_ptr, *occ_col;  // occupied (cluster, token) pairs and their columns
  int npairs;
  const float *X;        // packed X of the update iteration
  float *W;              // [K][V][MP]
  const float *vocab;    // [V][d]
  const float *vnorm;    // [V]
  float *cnorm;          // [K*m]
  float *part;           // [nchunk][K][MP][d+1]
  int nchunk, chunk;
  double *cs64;          // [K*m*d]
  float *cs32f;          // [K*m*d] row-major copy for the cost table
  float *T;              // [K][V][MP] cost table
  Ctl *ctl;
  int iter, K, m, MP, V, d;
  int gemm;              // cost table: 0 tensor cores (3xTF32), 1 FP32 CUDA cores
  const float *vsplit;   // vocabulary split into TF32 hi / lo tiles (tensor-core table)
  float *csplit;         // centroids split likewise, rebuilt per table
};
// Ctl::err value of a tensor-core wait that ran out
constexpr int kErrTcTimeout = 3;
cudaError_t launch_cost_table(const float *cs, int K, int m, const float *vocab, int V, int d,
                              float *cnorm, const float *vnorm, int MP, float *T, int gemm,
                              const float *vsplit, float *csplit, int *err, cudaStream_t st);
// tc_cost_table.cu: blocked TF32 hi / lo operands (rows in tiles of BR) and the table
size_t tf32_split_floats(int R, int d, int BR);
cudaError_t launch_tf32_split(const float *src, int R, int d, int BR, float *dst, cudaStream_t st);
cudaError_t launch_cost_table_tc(const float *cs, int nrows, const float *vsplit, int V, int d,
                                 const float *cnorm, const float *vnorm, int m, int MP, float *T,
                                 float *csplit, int *err, cudaStream_t st);
cudaError_t launch_vocab_norms(const float *vocab, int V, int d, float *vnorm, cudaStream_t st);
cudaError_t launch_to_f32(const double *a, size_t n, float *b, cudaStream_t st);
// step 5 of a word-embedding phase, then the new cost table (separate, so it can be timed)
cudaError_t launch_embed_support(const EmbedArgs &e, cudaStream_t st);
cudaError_t launch_embed_table(const EmbedArgs &e, cudaStream_t st);

// ngram_kernels.cu (n-gram phases, both forms)
struct NgramArgs {
  const int *key, *ptr, *occ;  // occurrence lists: key (l*dim + t)*V + v, columns in order
  int nlists;
  const float *Z32;            // batched: packed plans (column stride MP), or
  const double *Z64;           // plain: reference-layout plans (column stride str)
  long long zstride;
  double *cnt;                 // [K][m][dim][V] weighted symbol counts
  const double *dist;          // [V*V] symbol cost
  int *csym;                   // [K*m*dim] centroid symbols
  const int *tup;              // [U*dim] distinct instance tuples (batched table)
  float *T;                    // [K][U][MP] cost table (batched)
  Ctl *ctl;
  int iter, K, m, dim, V, U, MP;
  // batched plans left deferred by a pair pass: Z = Z' * rowsc[plan][row], the
  // plan of packed column c being grp_meta[c / S] >> 4 (null: Z is final)
  const float *rowsc;
  const int *grp_meta;
  int S, nplans;
};
// step 5: counts, then the new centroid symbols (skipped past the time budget)
cudaError_t launch_ngram_support(const NgramArgs &g, cudaStream_t st);
// the batched form's cost table of the current centroid symbols
cudaError_t launch_ngram_table(const NgramArgs &g, cudaStream_t st);
// the distinct tuples of count supports of dim symbols each, numbered in order
// of first appearance: key[e] = tuple of support e, tup [ntuples * dim];
// returns the number of tuples, or -1 for a symbol outside [0, V)
int number_tuples(const int *sym, size_t count, int dim, int V, std::vector<int> &key,
                  std::vector<int> &tup);
// assignment step: T[r * Uc + c] for row tuples rt [Ur*dim], column tuples ct [Uc*dim]
cudaError_t launch_ngram_pair_table(const int *rt, int Ur, const int *ct, int Uc, int dim, int V,
                                    const double *dist, double *T64, float *T32, cudaStream_t st);

// d2g_host.cu
int distmat_fp64(int dim, int str, size_t size, const int *p_str, int metric, const double *supp,
                 const int *sym, const double *vocab, int V, const int *label, const double *c_supp,
                 size_t K, double *C_host, const double *dist = nullptr, const int *c_sym = nullptr);

// d2g_init.cu: random centroids, the program's d2_centroid_rands where it
// links one, else d2g_centroid_rands
int centroid_rands(mph *p_data, int idx_ph, sph *c);

// error helpers (d2g_host.cu)
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

// exact transport (emd_kernel.cu): one warp per (row object, column object) pair
enum EmdMode { EMD_EUCLID = 0, EMD_TABLE = 1, EMD_EMBED = 2 };
struct EmdArgs {
  int mode, dim;
  // rows: weights, first support and support count per object (cum/str may
  // be null: every object has rfix supports), FP64 supports or table keys
  const double *rw;
  const size_t *rcum;
  const int *rstr;
  int rfix;
  const double *rsupp;
  const int *rsym;
  // columns, the same
  const double *cw;
  const size_t *ccum;
  const int *cstr;
  int cfix;
  const double *csupp;
  const int *csym;
  // table costs T[key_row * V + key_col] (EMD_TABLE); tscale >= every |T|.
  // EMD_EMBED: row objects are Euclidean (rsupp), column objects word ids
  // (csym) into vocab [V * dim]; FP32 costs T32[row object][word][row support]
  // with row-support stride tm
  const float *T32;
  const double *T64;
  int V;
  float tscale;
  const double *vocab;
  int tm;
  size_t key_off;  // EMD_EMBED without csym: column key = global support index - key_off
  const int *prow, *pcol;  // the pairs
  long long npairs;
  double *out;             // exact cost per pair
  int *piv;                // pivots per pair; -1: no optimum within max_piv
  int nmax;                // >= n + m of every pair, multiple of 32
  int max_piv;
};
size_t emd_slice(int nmax, int mode, int dim);
cudaError_t launch_emd(const EmdArgs &a, cudaStream_t st);

}  // namespace d2g

#define D2G_CUDA(call)                                     \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return d2g::cuda_fail(e_, #call); \
  } while (0)
