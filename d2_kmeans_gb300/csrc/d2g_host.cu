// Host side of libd2g: device state of one phase, packing of plans into
// thread blocks, the B-ADMM iteration loop (captured as one CUDA graph), and
// the resident C API (d2g_phase_*, d2g_badmm_run).
//
// Iteration loop, per iteration `it` (src/d2/centroid_Bregman.c:150-319):
//   plan_kernel            steps 1-3, row sums, [moments], [residual partials]
//   cluster_partial/final  step 4 (+ step 5 supports on update iterations)
//   [obj_kernel]           obj after a support update on a check iteration
//   [resid_final]          step 6 on check iterations
// The plain FP64 form runs one kernel per reference step instead.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <condition_variable>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "d2g_internal.cuh"

namespace d2g {

static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }
int cuda_fail(cudaError_t e, const char *what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  cudaGetLastError();  // clear a sticky launch error so the context stays usable
  return e == cudaErrorMemoryAllocation ? D2G_E_NOMEM : D2G_E_CUDA;
}
static int fail(int code, const std::string &msg) {
  set_error(msg);
  return code;
}

std::mutex g_cfg_mu;
d2g_config g_cfg = {0, 1, 1, 0, 0, 0, 0, 1};
d2g_config cfg_snapshot() {
  std::lock_guard<std::mutex> lk(g_cfg_mu);
  return g_cfg;
}

template <typename T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t cnt) {
    if (cnt == 0) cnt = 1;
    if (p && cnt <= n) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p, cnt * sizeof(T));
    if (e == cudaSuccess)
      n = cnt;
    else
      p = nullptr;
    return e;
  }
};

static inline bool is_check_iter(int it) { return (it % 100 == 99) || (it < 100 && it % 20 == 19); }
static inline int next_pow2(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

}  // namespace d2g

using namespace d2g;

struct d2g_phase {
  // ---- description
  int metric = 0, dim = 0, str = 0, K = 0, vocab_size = 0;
  size_t size = 0, col = 0, global_size = 0;
  int path = 0;  // 0 batched FP32, 1 plain FP64
  int cost_gemm = 0;  // word-embedding cost table: 0 tensor cores, 1 CUDA cores
  std::vector<int> p_str, label;
  std::vector<long long> cum;
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  // ---- test hook of the bounded device waits (d2g_phase_test_wait)
  unsigned long long wait_ns = 0;
  int fault_iter = -1, fault_unit = -1;

  // ---- sharded update: the exchange of the cluster sums between shards
  // (d2g_phase_set_allreduce, d2g_badmm_run_shards)
  d2g_allreduce_fn xfn = nullptr;
  void *xctx = nullptr;
  int xflags = 0;
  bool shard_pairs = false;  // every shard of the run can take pair passes
  DBuf<double> xbuf;
  std::vector<int> local_count;  // this shard's instances per cluster

  // ---- common device state
  DBuf<Ctl> ctl;
  DBuf<double> trace;
  int max_checks = 0;
  DBuf<double> cw64, cs64;
  DBuf<double> stage;  // reference-layout FP64 staging
  DBuf<double> colstage;  // reference-layout weights and supports on their way to the packed layout
  DBuf<int> symstage;
  DBuf<double> part;   // cluster partials
  int chunk = 256, nchunk = 1;
  std::vector<int> h_item_g0, h_item_ng;  // item arrays as packed (before any reordering)
  std::vector<int2> h_item_pp;
  int cur_order = 0;                      // the unit order the device item arrays hold
  DBuf<int> cl_ptr, cl_plans;
  DBuf<char> reinit;

  // ---- batched form
  Geo geo{};
  int MP = 0, DS = 4, mode = COST_EUCLID4;
  long long ncols_packed = 0;
  int ngroups = 0, nplans = 0;
  struct Bucket {
    int cs, nitems, item_off, block_off;
  };
  std::vector<Bucket> buckets;
  int total_blocks = 0;
  std::vector<int> plan_inst, inst_plan;
  DBuf<float> Z, Y, Xp, col_w, col_supp, rowsum, xmom, cw32, cs32, ctab;
  DBuf<int> col_sym, grp_meta, plan_g0, plan_ng, plan_label, item_g0, item_ng;
  DBuf<int2> item_pp;  // per item {first plan, plans} (packed order)
  DBuf<int> col_crow;  // word embeddings: cost-table row of each packed column
  DBuf<long long> plan_cum;
  DBuf<int4> grp_rec;
  DBuf<int> plan_slot;
  std::vector<int4> h_grp_rec;  // slot and label fields rewritten when labels change
  std::vector<int> h_grp_plan;  // plan of each group
  DBuf<double> resid_part, rho_part;
  size_t smem_plan = 0, smem_plan_upd = 0;
  // plans wider than one CTA: deferred row normalisation
  std::vector<int> h_wide_plans;  // packed ids
  Bucket units{1, 0, 0, 0};       // units of the deferred iterations
  int stage_costs = 0;
  d2g_tuning tune{0, 0, 0, 0};    // launch-shape choices (autotuner)
  int nwide = 0;
  bool defer = false;
  DBuf<float> rowpart, rowsc;
  DBuf<int4> wide;                       // {slot, slices with columns, label, 0} per wide plan
  // two iterations per pass (phases without wide plans): second-iteration row
  // sums (normalised / raw, by slot)
  bool pairs = false;
  DBuf<float> rowsum2, rawsum;
  DBuf<unsigned char> def_iter;          // per iteration: 1 if it ran deferred
  std::vector<unsigned char> h_def_iter;

  // ---- word-embedding and n-gram phases (batched form): per-cluster cost tables
  int ntab = 0;            // table rows per cluster: vocabulary size, or distinct n-gram tuples
  std::vector<int> h_sym;  // table row (token id / tuple id) per reference column
  DBuf<float> vocab32, vnorm, cnorm, cs32f, W, epart;
  DBuf<float> vsplit, csplit;  // TF32 hi / lo tiles of the vocabulary and of the centroids
  DBuf<int> pair_key, pair_ptr, occ_col;
  int npairs = 0, echunk = 0, enchunk = 0;

  // ---- n-gram phase (both forms)
  std::vector<int> h_nsym;        // [col*dim] instance symbols (host copy)
  std::vector<int> h_tup;         // [U*dim] distinct instance tuples (batched)
  std::vector<int> h_csym;        // centroid symbols of the last run (autotuner start point)
  DBuf<int> ntup, csym, nkey, nptr, nocc;
  DBuf<double> ndist, ncnt;
  int nlists = 0;

  // ---- plain form
  DBuf<double> pC, pX, pY, pZ, pZ0, pw, psupp, pvocab, pdist, pzr, pxmom;
  DBuf<int> psym, pcol_inst, pp_str, plabel;
  DBuf<long long> pcum;

  // ---- graph cache (valid while every buffer and value it captured is unchanged)
  cudaGraphExec_t gexec = nullptr;
  int g_maxIters = -1, g_upl = -1;
  std::vector<unsigned long long> g_sig;
  long long g_launches = 0;  // kernels in the captured loop

  // ---- last run
  d2g_run_stats stats{};
  std::vector<double> h_trace;
  int ntrace = 0;
  bool plans_valid = false;  // device Z holds plans from an earlier call / set_plans

  ~d2g_phase() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (st) cudaStreamDestroy(st);
  }
};

namespace d2g {

// ------------------------------------------------------------ tuning cache
// Key: the phase's shape.  Records live in this process and, when the
// environment names a file in D2G_TUNE_CACHE, in that file (one line per
// record: key exchange stage_costs ctas_per_sm cost_gemm; later lines win).
static std::string tune_key(const d2g_phase *ph) {
  char b[256];
  snprintf(b, sizeof b, "m%d.s%d.d%d.n%zu.c%zu.k%d.v%d", ph->metric, ph->str, ph->dim, ph->size,
           ph->col, ph->K, ph->vocab_size);
  return b;
}
static std::mutex g_tune_mu;
static std::vector<std::pair<std::string, d2g_tuning>> g_tune_mem;

static bool tune_cache_get(const std::string &key, d2g_tuning *t) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (auto it = g_tune_mem.rbegin(); it != g_tune_mem.rend(); ++it)
    if (it->first == key) {
      *t = it->second;
      return true;
    }
  const char *path = getenv("D2G_TUNE_CACHE");
  if (!path || !*path) return false;
  FILE *f = fopen(path, "r");
  if (!f) return false;
  bool found = false;
  char k[256];
  d2g_tuning r;
  while (fscanf(f, "%255s %d %d %d %d %d %d %d", k, &r.exchange, &r.stage_costs, &r.ctas_per_sm,
                &r.cost_gemm, &r.pairs, &r.unit_order, &r.stage_scales) == 8)
    if (key == k) {
      *t = r;
      found = true;
    }
  fclose(f);
  return found;
}

static void tune_cache_put(const std::string &key, const d2g_tuning &t) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_mem.emplace_back(key, t);
  const char *path = getenv("D2G_TUNE_CACHE");
  if (!path || !*path) return;
  FILE *f = fopen(path, "a");
  if (!f) return;
  fprintf(f, "%s %d %d %d %d %d %d %d\n", key.c_str(), t.exchange, t.stage_costs, t.ctas_per_sm,
          t.cost_gemm, t.pairs, t.unit_order, t.stage_scales);
  fclose(f);
}

// the run-time switches that follow from the phase's tuning
static int apply_tuning(d2g_phase *ph) {
  ph->defer = ph->path == 0 && ph->nwide > 0 && ph->units.nitems > 0 &&
              ph->tune.exchange == 0;
  ph->stage_costs = ph->tune.stage_costs;
  ph->cost_gemm = ph->tune.cost_gemm;
  // the walk order of the items that each fit one CTA (bucket 0): the item
  // arrays are permuted in place, the plans stay where they are
  if (ph->path == 0 && ph->tune.unit_order != ph->cur_order && !ph->h_item_g0.empty() &&
      !ph->buckets.empty() && ph->buckets[0].cs == 1) {
    const int n1 = ph->buckets[0].nitems;
    std::vector<int> idx(n1);
    for (int i = 0; i < n1; ++i) idx[i] = i;
    if (ph->tune.unit_order == 1)
      std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return ph->h_item_ng[a] > ph->h_item_ng[b]; });
    std::vector<int> g0(n1), ng(n1);
    std::vector<int2> pp(n1);
    for (int i = 0; i < n1; ++i) {
      g0[i] = ph->h_item_g0[idx[i]];
      ng[i] = ph->h_item_ng[idx[i]];
      pp[i] = ph->h_item_pp[idx[i]];
    }
    D2G_CUDA(cudaMemcpyAsync(ph->item_g0.p, g0.data(), n1 * 4, cudaMemcpyHostToDevice, ph->st));
    D2G_CUDA(cudaMemcpyAsync(ph->item_ng.p, ng.data(), n1 * 4, cudaMemcpyHostToDevice, ph->st));
    D2G_CUDA(cudaMemcpyAsync(ph->item_pp.p, pp.data(), n1 * sizeof(int2), cudaMemcpyHostToDevice, ph->st));
    D2G_CUDA(cudaStreamSynchronize(ph->st));
    ph->cur_order = ph->tune.unit_order;
  }
  return D2G_OK;
}

static bool batched_supported(const d2g_phase_desc *d, std::string *why) {
  if (d->str > 256) {
    *why = "str > 256";
    return false;
  }
  if (d->metric_type == D2_EUCLIDEAN_L2) {
    if (d->dim < 1 || d->dim > 8) {
      *why = "Euclidean dim outside 1..8";
      return false;
    }
    return true;
  }
  if (d->metric_type == D2_HISTOGRAM || d->metric_type == D2_SPARSE_HISTOGRAM) return true;
  if (d->metric_type == D2_WORD_EMBED || d->metric_type == D2_N_GRAM) return d->dim >= 1;
  *why = "metric type";
  return false;
}

// ------------------------------------------------------------------ packing
// Best-fit-decreasing packing of plans (in S-column groups) into items of G
// groups; plans needing more than G groups get a cluster of 2/4/8 CTAs.
// Packing of the plans into CTA work.  Plans of at most G column groups
// ("small") are packed best-fit-decreasing into units of G groups.  A plan of
// more than G groups ("wide") is cut into floor(ng/G) full slices of G groups
// and a remainder of ng mod G groups; with the deferred exchange the remainder
// opens a unit that small plans fill.  Layout: the small-only units, then per
// wide plan its groups followed by the small plans of its remainder unit.
// Three partitions of that one layout are launched:
//   - cs = 1 bucket: runs of whole small plans (synchronous iterations);
//   - cs = 2, 4, 8 buckets: one wide plan per item on a thread-block cluster
//     of next_pow2(ceil(ng/G)) CTAs (synchronous iterations);
//   - units: every range above of at most G groups, at most one wide slice
//     per unit and at its start (deferred iterations, one plain launch).
static int build_packing(d2g_phase *ph, bool with_units) {
  const int G = ph->geo.G, S = ph->geo.S;
  const size_t n = ph->size;
  std::vector<int> ng(n), csz(n);
  for (size_t i = 0; i < n; ++i) {
    ng[i] = (ph->p_str[i] + S - 1) / S;
    int c = (ng[i] + G - 1) / G;
    c = next_pow2(c);
    if (c > kMaxCluster) return fail(D2G_E_UNSUPPORTED, "instance support size exceeds 8 CTAs");
    csz[i] = c;
  }
  // bins of G groups: {anchor wide plan or -1, small plans}
  std::vector<int> bin_anchor;
  std::vector<std::vector<int>> bin_plans;
  std::vector<std::vector<int>> open(G + 1);  // bins by remaining capacity
  std::vector<int> anchor_bin(n, -1);
  if (with_units)
    for (size_t i = 0; i < n; ++i)
      if (csz[i] > 1 && ng[i] % G) {
        anchor_bin[i] = (int)bin_anchor.size();
        open[G - ng[i] % G].push_back((int)bin_anchor.size());
        bin_anchor.push_back((int)i);
        bin_plans.emplace_back();
      }
  std::vector<int> order;
  order.reserve(n);
  for (size_t i = 0; i < n; ++i)
    if (csz[i] == 1) order.push_back((int)i);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ng[a] > ng[b]; });
  for (int i : order) {
    int bi = -1, rem = -1;
    for (int r = ng[i]; r <= G; ++r)
      if (!open[r].empty()) {
        bi = open[r].back();
        open[r].pop_back();
        rem = r;
        break;
      }
    if (bi < 0) {
      bi = (int)bin_anchor.size();
      bin_anchor.push_back(-1);
      bin_plans.emplace_back();
      rem = G;
    }
    bin_plans[bi].push_back(i);
    rem -= ng[i];
    if (rem > 0) open[rem].push_back(bi);
  }
  // assign packed plan ids / groups
  ph->plan_inst.clear();
  ph->inst_plan.assign(n, -1);
  ph->h_grp_rec.clear();
  ph->h_grp_plan.clear();
  ph->h_wide_plans.clear();
  std::vector<int> h_plan_g0, h_plan_ng, h_meta;
  std::vector<long long> h_plan_cum;
  std::vector<int> it1_g0, it1_ng, unit_g0, unit_ng;
  std::vector<int> itc_g0[kMaxCluster + 1], itc_ng[kMaxCluster + 1];
  ph->buckets.clear();
  int g = 0;
  auto add_plan = [&](int i) {
    const int p = (int)ph->plan_inst.size();
    ph->plan_inst.push_back(i);
    ph->inst_plan[i] = p;
    h_plan_g0.push_back(g);
    h_plan_ng.push_back(ng[i]);
    h_plan_cum.push_back(ph->cum[i]);
    for (int q = 0; q < ng[i]; ++q) {
      const int nv = std::min(S, ph->p_str[i] - q * S);
      h_meta.push_back((p << 4) | nv);
      ph->h_grp_rec.push_back(make_int4(p, g, 0, (ng[i] << 12) | nv));
      ph->h_grp_plan.push_back(p);
    }
    g += ng[i];
  };
  auto add_small_run = [&](const std::vector<int> &pl, int unit_from) {
    const int g0 = g;
    for (int i : pl) add_plan(i);
    if (g > g0) {
      it1_g0.push_back(g0);
      it1_ng.push_back(g - g0);
    }
    if (g > unit_from) {
      unit_g0.push_back(unit_from);
      unit_ng.push_back(g - unit_from);
    }
  };
  for (size_t bi = 0; bi < bin_anchor.size(); ++bi)
    if (bin_anchor[bi] < 0) add_small_run(bin_plans[bi], g);
  for (size_t i = 0; i < n; ++i) {
    if (csz[i] == 1) continue;
    const int g0 = g;
    ph->h_wide_plans.push_back((int)ph->plan_inst.size());
    add_plan((int)i);
    itc_g0[csz[i]].push_back(g0);
    itc_ng[csz[i]].push_back(ng[i]);
    const int nfull = ng[i] / G;
    for (int k = 0; k < nfull; ++k) {
      unit_g0.push_back(g0 + k * G);
      unit_ng.push_back(G);
    }
    if (ng[i] % G) {
      static const std::vector<int> none;
      add_small_run(anchor_bin[i] >= 0 ? bin_plans[anchor_bin[i]] : none, g0 + nfull * G);
    }
  }
  // item arrays: cs = 1 items, cluster items by size, then the units
  std::vector<int> h_item_g0(it1_g0), h_item_ng(it1_ng);
  int blocks = 0;
  ph->buckets.push_back(d2g_phase::Bucket{1, (int)it1_g0.size(), 0, 0});
  blocks += (int)it1_g0.size();
  for (int c = 2; c <= kMaxCluster; c <<= 1) {
    if (itc_g0[c].empty()) continue;
    ph->buckets.push_back(d2g_phase::Bucket{c, (int)itc_g0[c].size(), (int)h_item_g0.size(), blocks});
    h_item_g0.insert(h_item_g0.end(), itc_g0[c].begin(), itc_g0[c].end());
    h_item_ng.insert(h_item_ng.end(), itc_ng[c].begin(), itc_ng[c].end());
    blocks += (int)itc_g0[c].size() * c;
  }
  ph->units = d2g_phase::Bucket{1, with_units ? (int)unit_g0.size() : 0, (int)h_item_g0.size(), 0};
  if (with_units) {
    h_item_g0.insert(h_item_g0.end(), unit_g0.begin(), unit_g0.end());
    h_item_ng.insert(h_item_ng.end(), unit_ng.begin(), unit_ng.end());
  }
  ph->nwide = (int)ph->h_wide_plans.size();
  if (ph->buckets[0].nitems == 0) ph->buckets.erase(ph->buckets.begin());
  ph->total_blocks = blocks;
  ph->ngroups = g;
  ph->nplans = (int)n;
  ph->ncols_packed = (long long)g * S;
  if (ph->ncols_packed * ph->MP > (1LL << 40)) return fail(D2G_E_UNSUPPORTED, "phase too large");
  // the plans of every item (contiguous in packed order); in the items of one
  // CTA, each group record carries its plan's index among the item's plans
  // (bits 4-11), which places the plan's row scale in the staged copy
  std::vector<int2> h_item_pp(h_item_g0.size());
  for (size_t it = 0; it < h_item_g0.size(); ++it) {
    const int g0 = h_item_g0[it], gl = g0 + h_item_ng[it] - 1;
    const int p0 = ph->h_grp_plan[g0];
    h_item_pp[it] = make_int2(p0, ph->h_grp_plan[gl] - p0 + 1);
    if (it >= it1_g0.size()) continue;
    for (int gi = g0; gi <= gl; ++gi) {
      const int lp = ph->h_grp_plan[gi] - p0;
      if (lp > 255) return fail(D2G_E_UNSUPPORTED, "more than 256 plans in one item");
      ph->h_grp_rec[gi].w |= lp << 4;
    }
  }

  D2G_CUDA(ph->grp_meta.alloc(h_meta.size()));
  D2G_CUDA(ph->plan_g0.alloc(n));
  D2G_CUDA(ph->plan_ng.alloc(n));
  D2G_CUDA(ph->plan_label.alloc(n));
  D2G_CUDA(ph->plan_cum.alloc(n));
  D2G_CUDA(ph->item_g0.alloc(h_item_g0.size()));
  D2G_CUDA(ph->item_ng.alloc(h_item_ng.size()));
  D2G_CUDA(ph->item_pp.alloc(h_item_pp.size()));
  D2G_CUDA(cudaMemcpyAsync(ph->grp_meta.p, h_meta.data(), h_meta.size() * 4, cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(cudaMemcpyAsync(ph->plan_g0.p, h_plan_g0.data(), n * 4, cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(cudaMemcpyAsync(ph->plan_ng.p, h_plan_ng.data(), n * 4, cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(cudaMemcpyAsync(ph->plan_cum.p, h_plan_cum.data(), n * 8, cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(cudaMemcpyAsync(ph->item_g0.p, h_item_g0.data(), h_item_g0.size() * 4, cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(cudaMemcpyAsync(ph->item_ng.p, h_item_ng.data(), h_item_ng.size() * 4, cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(cudaMemcpyAsync(ph->item_pp.p, h_item_pp.data(), h_item_pp.size() * sizeof(int2),
                           cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(cudaStreamSynchronize(ph->st));
  ph->h_item_g0 = h_item_g0;  // (the autotuner's unit order permutes copies of these)
  ph->h_item_ng = h_item_ng;
  ph->h_item_pp = h_item_pp;
  ph->cur_order = 0;
  return D2G_OK;
}

static PlanArgs base_args(d2g_phase *ph) {
  PlanArgs a{};
  a.Z = ph->Z.p;
  a.Y = ph->Y.p;
  a.col_w = ph->col_w.p;
  a.col_supp = ph->col_supp.p;
  a.col_sym = ph->col_sym.p;
  a.grp_meta = ph->grp_meta.p;
  a.plan_g0 = ph->plan_g0.p;
  a.plan_ng = ph->plan_ng.p;
  a.plan_label = ph->plan_label.p;
  a.cw32 = ph->cw32.p;
  a.cs32 = ph->cs32.p;
  a.ctab = ph->ctab.p;
  const bool tables = ph->metric == D2_WORD_EMBED || ph->metric == D2_N_GRAM;
  a.ctab_lstride = tables ? (long long)ph->ntab * ph->MP : 0;
  a.rowsum_out = ph->rowsum.p;
  a.xmom_out = ph->xmom.p;
  a.X_out = ph->Xp.p;
  a.resid_part = ph->resid_part.p;
  a.ctl = ph->ctl.p;
  a.ctas_per_sm = ph->tune.ctas_per_sm;
  a.stage_scales = ph->tune.stage_scales;
  a.m = ph->str;
  a.dim = ph->metric == D2_EUCLIDEAN_L2 ? ph->dim : 0;
  a.grp_rec = ph->grp_rec.p;
  a.plan_slot = ph->plan_slot.p;
  a.rowpart = ph->rowpart.p;
  a.rowsc = ph->rowsc.p;
  a.col_crow = tables ? ph->col_crow.p : ph->col_sym.p;
  a.stage_costs = ph->stage_costs;
  a.wide = ph->nwide > 0;
  a.rowsum2_out = ph->rowsum2.p;
  a.rawsum_out = ph->rawsum.p;
  a.nplans_chk = ph->nplans;
  a.nlab_chk = ph->K;
  a.ctab_rows = tables ? ph->K * ph->ntab
                       : ((ph->metric == D2_HISTOGRAM || ph->metric == D2_SPARSE_HISTOGRAM) ? ph->vocab_size : 0);
  return a;
}

static PlanArgs bucket_args(d2g_phase *ph, const PlanArgs &base, const d2g_phase::Bucket &b) {
  PlanArgs a = base;
  a.item_g0 = ph->item_g0.p + b.item_off;
  a.item_ng = ph->item_ng.p + b.item_off;
  a.item_pp = ph->item_pp.p + b.item_off;
  a.cs = b.cs;
  a.resid_off = b.block_off;
  return a;
}

// ---------------------------------------------------------- labels / lists
// Occurrence lists of an n-gram phase's support update: for every key
// (label * dim + t) * V + v, the columns whose symbol at position t is v, in
// increasing column order (packed columns in the batched form, reference
// columns in the plain form, so that the plain form adds in the reference's
// order).  col_label[c] < 0 marks a padding column; col_ref[c] is the column's
// reference column (its symbols).
static int build_ngram_lists(d2g_phase *ph, const std::vector<int> &col_label,
                             const std::vector<long long> &col_ref) {
  const int V = ph->vocab_size, dim = ph->dim;
  const size_t nkeys = (size_t)ph->K * dim * V, nc = col_label.size();
  if (nkeys >= (size_t)INT_MAX || nc * (size_t)dim >= (size_t)INT_MAX || nc >= (size_t)INT_MAX)
    return fail(D2G_E_UNSUPPORTED, "n-gram phase too large for 32-bit occurrence lists");
  std::vector<int> cnt(nkeys + 1, 0);
  for (size_t c = 0; c < nc; ++c) {
    if (col_label[c] < 0) continue;
    const int *x = ph->h_nsym.data() + (size_t)col_ref[c] * dim;
    for (int t = 0; t < dim; ++t) ++cnt[((size_t)col_label[c] * dim + t) * V + x[t] + 1];
  }
  std::vector<int> keys, ptr(1, 0);
  for (size_t k = 0; k < nkeys; ++k)
    if (cnt[k + 1]) {
      keys.push_back((int)k);
      ptr.push_back(ptr.back() + cnt[k + 1]);
    }
  for (size_t k = 1; k <= nkeys; ++k) cnt[k] += cnt[k - 1];
  std::vector<int> occ(ptr.back());
  for (size_t c = 0; c < nc; ++c) {
    if (col_label[c] < 0) continue;
    const int *x = ph->h_nsym.data() + (size_t)col_ref[c] * dim;
    for (int t = 0; t < dim; ++t) occ[cnt[((size_t)col_label[c] * dim + t) * V + x[t]]++] = (int)c;
  }
  ph->nlists = (int)keys.size();
  D2G_CUDA(ph->nkey.alloc(keys.size()));
  D2G_CUDA(ph->nptr.alloc(ptr.size()));
  D2G_CUDA(ph->nocc.alloc(occ.size()));
  D2G_CUDA(cudaMemcpyAsync(ph->nkey.p, keys.data(), keys.size() * 4, cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(cudaMemcpyAsync(ph->nptr.p, ptr.data(), ptr.size() * 4, cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(cudaMemcpyAsync(ph->nocc.p, occ.data(), occ.size() * 4, cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(cudaStreamSynchronize(ph->st));
  return D2G_OK;
}

static int set_labels_impl(d2g_phase *ph, const int *label) {
  const size_t n = ph->size;
  for (size_t i = 0; i < n; ++i)
    if (label[i] < 0 || label[i] >= ph->K) return fail(D2G_E_INVAL, "label out of range");
  ph->label.assign(label, label + n);
  std::vector<int> cnt(ph->K + 1, 0);
  for (size_t i = 0; i < n; ++i) ++cnt[label[i] + 1];
  int maxc = 0;
  ph->local_count.assign(cnt.begin() + 1, cnt.end());
  // a shard of a larger set (global_size > size) may hold no instance of a
  // cluster: the check then runs over all shards when the update starts
  const bool shard = ph->global_size > ph->size;
  for (int l = 0; l < ph->K; ++l) {
    if (cnt[l + 1] == 0 && !shard)
      return fail(D2G_E_EMPTY_CLUSTER, "cluster " + std::to_string(l) + " has no instance");
    maxc = std::max(maxc, cnt[l + 1]);
  }
  maxc = std::max(maxc, 1);
  for (int l = 0; l < ph->K; ++l) cnt[l + 1] += cnt[l];
  std::vector<int> pos(cnt.begin(), cnt.end() - 1), lists(n);
  const bool batched = ph->path == 0;
  for (size_t i = 0; i < n; ++i) lists[pos[label[i]]++] = batched ? ph->inst_plan[i] : (int)i;
  D2G_CUDA(ph->cl_ptr.alloc(ph->K + 1));
  D2G_CUDA(ph->cl_plans.alloc(n));
  D2G_CUDA(cudaMemcpyAsync(ph->cl_ptr.p, cnt.data(), (ph->K + 1) * 4, cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(cudaMemcpyAsync(ph->cl_plans.p, lists.data(), n * 4, cudaMemcpyHostToDevice, ph->st));
  ph->nchunk = (maxc + ph->chunk - 1) / ph->chunk;
  const int dimp = (ph->metric == D2_EUCLIDEAN_L2 || ph->metric == D2_WORD_EMBED) ? ph->dim : 0;
  D2G_CUDA(ph->part.alloc((size_t)ph->K * (dimp + 2) * ph->nchunk * ph->str));
  if (batched) {
    std::vector<int> pl(n);
    for (size_t p = 0; p < n; ++p) pl[p] = label[ph->plan_inst[p]];
    D2G_CUDA(cudaMemcpyAsync(ph->plan_label.p, pl.data(), n * 4, cudaMemcpyHostToDevice, ph->st));
    // slot of each plan: its position in the cluster-sorted order
    std::vector<int> slot(n);
    for (size_t q = 0; q < n; ++q) slot[lists[q]] = (int)q;
    D2G_CUDA(ph->plan_slot.alloc(n));
    D2G_CUDA(cudaMemcpyAsync(ph->plan_slot.p, slot.data(), n * 4, cudaMemcpyHostToDevice, ph->st));
    // group records: {slot, plan's first group, label, groups << 12 | plan in item << 4 | valid}
    const std::vector<int> &gplan = ph->h_grp_plan;
    for (size_t gi = 0; gi < ph->h_grp_rec.size(); ++gi) {
      const int p = gplan[gi];
      ph->h_grp_rec[gi].x = slot[p];
      ph->h_grp_rec[gi].z = pl[p];
    }
    if (ph->nwide > 0 && ph->path == 0) {  // wide plans: {slot, slices with columns, label}
      std::vector<int4> wl(ph->nwide);
      for (int q = 0; q < ph->nwide; ++q) {
        const int p = ph->h_wide_plans[q];
        const int ngp = (ph->p_str[ph->plan_inst[p]] + ph->geo.S - 1) / ph->geo.S;
        wl[q] = make_int4(slot[p], (ngp + ph->geo.G - 1) / ph->geo.G, pl[p], 0);
      }
      D2G_CUDA(ph->wide.alloc(ph->nwide));
      D2G_CUDA(cudaMemcpyAsync(ph->wide.p, wl.data(), wl.size() * sizeof(int4), cudaMemcpyHostToDevice,
                               ph->st));
      D2G_CUDA(cudaStreamSynchronize(ph->st));
    }
    if (ph->metric == D2_WORD_EMBED) {
      // occurrence lists: for each (cluster, token) the packed columns carrying it,
      // ordered by packed column (counting sort on the key label*V + token)
      const int V = ph->vocab_size;
      std::vector<int> key_of(ph->ncols_packed, -1);
      for (size_t gi = 0; gi < ph->h_grp_rec.size(); ++gi) {
        const int p = gplan[gi];
        const int nv = ph->h_grp_rec[gi].w & 15;
        const int jj0 = (int)(gi - ph->h_grp_rec[gi].y) * ph->geo.S;
        const long long c0 = ph->cum[ph->plan_inst[p]];
        for (int s2 = 0; s2 < nv; ++s2)
          key_of[gi * ph->geo.S + s2] = pl[p] * V + ph->h_sym[c0 + jj0 + s2];
      }
      std::vector<int> cnt((size_t)ph->K * V + 1, 0);
      for (int k2 : key_of)
        if (k2 >= 0) ++cnt[k2 + 1];
      std::vector<int> keys, ptr(1, 0);
      for (size_t k2 = 0; k2 < (size_t)ph->K * V; ++k2)
        if (cnt[k2 + 1]) {
          keys.push_back((int)k2);
          ptr.push_back(ptr.back() + cnt[k2 + 1]);
        }
      for (size_t k2 = 1; k2 < cnt.size(); ++k2) cnt[k2] += cnt[k2 - 1];
      std::vector<int> occ(ptr.back());
      for (long long pc = 0; pc < ph->ncols_packed; ++pc)
        if (key_of[pc] >= 0) occ[cnt[key_of[pc]]++] = (int)pc;
      // per packed column: its cost-table row label * V + token (0 in pad columns)
      for (auto &k2 : key_of) k2 = std::max(k2, 0);
      D2G_CUDA(ph->col_crow.alloc(key_of.size()));
      D2G_CUDA(cudaMemcpyAsync(ph->col_crow.p, key_of.data(), key_of.size() * 4, cudaMemcpyHostToDevice,
                               ph->st));
      ph->npairs = (int)keys.size();
      D2G_CUDA(ph->pair_key.alloc(keys.size()));
      D2G_CUDA(ph->pair_ptr.alloc(ptr.size()));
      D2G_CUDA(ph->occ_col.alloc(occ.size()));
      D2G_CUDA(cudaMemcpyAsync(ph->pair_key.p, keys.data(), keys.size() * 4, cudaMemcpyHostToDevice, ph->st));
      D2G_CUDA(cudaMemcpyAsync(ph->pair_ptr.p, ptr.data(), ptr.size() * 4, cudaMemcpyHostToDevice, ph->st));
      D2G_CUDA(cudaMemcpyAsync(ph->occ_col.p, occ.data(), occ.size() * 4, cudaMemcpyHostToDevice, ph->st));
      D2G_CUDA(cudaStreamSynchronize(ph->st));
    }
    if (ph->metric == D2_N_GRAM) {
      // per packed column: its cost-table row label * U + tuple (0 in pad
      // columns), its label and reference column for the occurrence lists
      const int U = ph->ntab;
      std::vector<int> crow(ph->ncols_packed, 0), clab(ph->ncols_packed, -1);
      std::vector<long long> cref(ph->ncols_packed, 0);
      for (size_t gi = 0; gi < ph->h_grp_rec.size(); ++gi) {
        const int p = gplan[gi];
        const int nv = ph->h_grp_rec[gi].w & 15;
        const int jj0 = (int)(gi - ph->h_grp_rec[gi].y) * ph->geo.S;
        const long long c0 = ph->cum[ph->plan_inst[p]];
        for (int s2 = 0; s2 < nv; ++s2) {
          const size_t pc = gi * ph->geo.S + s2;
          crow[pc] = pl[p] * U + ph->h_sym[c0 + jj0 + s2];
          clab[pc] = pl[p];
          cref[pc] = c0 + jj0 + s2;
        }
      }
      if ((size_t)ph->K * U >= (size_t)INT_MAX) return fail(D2G_E_UNSUPPORTED, "n-gram table too large");
      D2G_CUDA(ph->col_crow.alloc(crow.size()));
      D2G_CUDA(cudaMemcpyAsync(ph->col_crow.p, crow.data(), crow.size() * 4, cudaMemcpyHostToDevice, ph->st));
      int rc = build_ngram_lists(ph, clab, cref);
      if (rc) return rc;
    }
    D2G_CUDA(ph->grp_rec.alloc(ph->h_grp_rec.size()));
    D2G_CUDA(cudaMemcpyAsync(ph->grp_rec.p, ph->h_grp_rec.data(), ph->h_grp_rec.size() * sizeof(int4),
                             cudaMemcpyHostToDevice, ph->st));
  } else {
    D2G_CUDA(cudaMemcpyAsync(ph->plabel.p, label, n * 4, cudaMemcpyHostToDevice, ph->st));
    if (ph->metric == D2_N_GRAM) {  // lists over the reference columns, in order
      std::vector<int> clab(ph->col);
      std::vector<long long> cref(ph->col);
      for (size_t i = 0; i < n; ++i)
        for (int j = 0; j < ph->p_str[i]; ++j) {
          clab[ph->cum[i] + j] = label[i];
          cref[ph->cum[i] + j] = ph->cum[i] + j;
        }
      int rc = build_ngram_lists(ph, clab, cref);
      if (rc) return rc;
    }
  }
  D2G_CUDA(cudaStreamSynchronize(ph->st));
  return D2G_OK;
}

// ------------------------------------------------------------------ create
// per-column data: reference layout -> staging -> packed FP32 (+ histogram cost table)
static int upload_columns_batched(d2g_phase *ph, const d2g_phase_desc *d) {
  const bool euc = ph->metric == D2_EUCLIDEAN_L2;
  const size_t ns = ph->col * (size_t)(1 + (euc ? ph->dim : 0));
  // reference-layout staging, kept on the phase: a drop-in call re-sends the
  // columns every time, and a fresh allocation per call would cost more than
  // the copy
  DBuf<double> &tmp = ph->colstage;
  DBuf<int> &tsym = ph->symstage;
  D2G_CUDA(tmp.alloc(ns));
  D2G_CUDA(cudaMemcpyAsync(tmp.p, d->p_w, ph->col * 8, cudaMemcpyHostToDevice, ph->st));
  if (euc)
    D2G_CUDA(cudaMemcpyAsync(tmp.p + ph->col, d->p_supp, ph->col * ph->dim * 8, cudaMemcpyHostToDevice, ph->st));
  if (ph->metric == D2_SPARSE_HISTOGRAM || ph->metric == D2_WORD_EMBED) {
    D2G_CUDA(tsym.alloc(ph->col));
    D2G_CUDA(cudaMemcpyAsync(tsym.p, d->p_supp_sym, ph->col * 4, cudaMemcpyHostToDevice, ph->st));
  }
  if (ph->metric == D2_N_GRAM) {  // packed columns carry their tuple's table row
    ph->h_nsym.assign(d->p_supp_sym, d->p_supp_sym + ph->col * ph->dim);
    ph->ntab = number_tuples(ph->h_nsym.data(), ph->col, ph->dim, ph->vocab_size, ph->h_sym, ph->h_tup);
    if (ph->ntab < 0) return fail(D2G_E_INVAL, "n-gram symbol out of range");
    D2G_CUDA(tsym.alloc(ph->col));
    D2G_CUDA(cudaMemcpyAsync(tsym.p, ph->h_sym.data(), ph->col * 4, cudaMemcpyHostToDevice, ph->st));
    D2G_CUDA(ph->ntup.alloc(ph->h_tup.size()));
    D2G_CUDA(cudaMemcpyAsync(ph->ntup.p, ph->h_tup.data(), ph->h_tup.size() * 4, cudaMemcpyHostToDevice,
                             ph->st));
    const size_t VV = (size_t)ph->vocab_size * ph->vocab_size;
    D2G_CUDA(ph->ndist.alloc(VV));
    D2G_CUDA(cudaMemcpyAsync(ph->ndist.p, d->dist_mat, VV * 8, cudaMemcpyHostToDevice, ph->st));
    D2G_CUDA(ph->ctab.alloc((size_t)ph->K * ph->ntab * ph->MP));
    D2G_CUDA(cudaStreamSynchronize(ph->st));
  }
  PlanArgs base = base_args(ph);
  for (auto &b : ph->buckets) {
    PlanArgs a = bucket_args(ph, base, b);
    D2G_CUDA(launch_pack_columns(ph->MP, a, b.nitems, ph->plan_cum.p, tmp.p,
                                 euc ? tmp.p + ph->col : nullptr, tsym.p, ph->col_w.p,
                                 euc ? ph->col_supp.p : nullptr, euc ? nullptr : ph->col_sym.p,
                                 ph->dim, ph->DS, ph->metric == D2_HISTOGRAM ? 1 : 0, ph->st));
  }
  if (ph->metric == D2_WORD_EMBED) {  // vocabulary (FP32) and its norms; the cost table is per run
    const size_t vd = (size_t)ph->vocab_size * ph->dim;
    std::vector<float> v32(vd);
    for (size_t i = 0; i < vd; ++i) v32[i] = (float)d->vocab_vec[i];
    D2G_CUDA(ph->vocab32.alloc(vd));
    D2G_CUDA(cudaMemcpyAsync(ph->vocab32.p, v32.data(), vd * 4, cudaMemcpyHostToDevice, ph->st));
    D2G_CUDA(ph->vnorm.alloc(ph->vocab_size));
    D2G_CUDA(launch_vocab_norms(ph->vocab32.p, ph->vocab_size, ph->dim, ph->vnorm.p, ph->st));
    // tensor-core cost table operands: the vocabulary split once, centroid space per table
    D2G_CUDA(ph->vsplit.alloc(tf32_split_floats(ph->vocab_size, ph->dim, 256)));
    D2G_CUDA(launch_tf32_split(ph->vocab32.p, ph->vocab_size, ph->dim, 256, ph->vsplit.p, ph->st));
    D2G_CUDA(ph->csplit.alloc(tf32_split_floats(ph->K * ph->str, ph->dim, 128)));
    ph->h_sym.assign(d->p_supp_sym, d->p_supp_sym + ph->col);
    D2G_CUDA(cudaStreamSynchronize(ph->st));
  } else if (ph->metric == D2_HISTOGRAM || ph->metric == D2_SPARSE_HISTOGRAM) {
    // histogram cost table: row v = cost from bin v to every centroid bin
    const int V = ph->vocab_size;
    std::vector<float> t((size_t)V * ph->MP, 0.f);
    for (int v = 0; v < V; ++v)
      for (int k = 0; k < ph->str; ++k) t[(size_t)v * ph->MP + k] = (float)d->dist_mat[(size_t)v * V + k];
    D2G_CUDA(ph->ctab.alloc(t.size()));
    D2G_CUDA(cudaMemcpyAsync(ph->ctab.p, t.data(), t.size() * 4, cudaMemcpyHostToDevice, ph->st));
    D2G_CUDA(cudaStreamSynchronize(ph->st));
  }
  D2G_CUDA(cudaStreamSynchronize(ph->st));
  return D2G_OK;
}

static int create_batched(d2g_phase *ph, const d2g_phase_desc *d) {
  ph->MP = std::max(4, next_pow2(ph->str));
  ph->geo = geo_for(ph->MP);
  if (ph->metric == D2_EUCLIDEAN_L2) {
    ph->mode = ph->dim == 3 ? COST_EUCLID3 : (ph->dim <= 4 ? COST_EUCLID4 : COST_EUCLID8);
    ph->DS = ph->dim <= 4 ? 4 : 8;
  } else {
    ph->mode = COST_TABLE;
    ph->DS = 4;
  }
  int rc = build_packing(ph, true);
  if (rc) return rc;
  const size_t nz = (size_t)ph->ncols_packed * ph->MP;
  D2G_CUDA(ph->Z.alloc(nz));
  D2G_CUDA(ph->Y.alloc(nz));
  D2G_CUDA(cudaMemsetAsync(ph->Z.p, 0, nz * 4, ph->st));
  D2G_CUDA(cudaMemsetAsync(ph->Y.p, 0, nz * 4, ph->st));
  D2G_CUDA(ph->col_w.alloc(ph->ncols_packed));
  const bool euc = ph->metric == D2_EUCLIDEAN_L2;
  if (euc) D2G_CUDA(ph->col_supp.alloc((size_t)ph->ncols_packed * ph->DS));
  else D2G_CUDA(ph->col_sym.alloc(ph->ncols_packed));
  D2G_CUDA(ph->rowsum.alloc((size_t)ph->nplans * ph->MP));
  if (euc) D2G_CUDA(ph->xmom.alloc((size_t)ph->nplans * (ph->dim + 1) * ph->MP));
  D2G_CUDA(ph->cw32.alloc((size_t)ph->K * ph->MP));
  if (euc) D2G_CUDA(ph->cs32.alloc((size_t)ph->K * ph->MP * ph->DS));
  D2G_CUDA(ph->resid_part.alloc((size_t)ph->total_blocks * 4));
  D2G_CUDA(ph->rho_part.alloc(ph->total_blocks));
  D2G_CUDA(ph->reinit.alloc(ph->size));
  if (ph->metric == D2_WORD_EMBED) {
    ph->ntab = d->vocab_size;
    const size_t KV = (size_t)ph->K * d->vocab_size;
    D2G_CUDA(ph->ctab.alloc(KV * ph->MP));
    D2G_CUDA(cudaMemsetAsync(ph->ctab.p, 0, KV * ph->MP * 4, ph->st));  // padded rows stay 0
    D2G_CUDA(ph->W.alloc(KV * ph->MP));
    D2G_CUDA(ph->Xp.alloc(nz));
    D2G_CUDA(ph->cnorm.alloc((size_t)ph->K * ph->str));
    D2G_CUDA(ph->cs32f.alloc((size_t)ph->K * ph->str * d->dim));
    ph->enchunk = std::max(1, std::min(64, (d->vocab_size + 511) / 512));
    ph->echunk = (d->vocab_size + ph->enchunk - 1) / ph->enchunk;
    D2G_CUDA(ph->epart.alloc((size_t)ph->enchunk * ph->K * ph->MP * (d->dim + 1)));
  }
  if (ph->metric == D2_N_GRAM) {
    D2G_CUDA(ph->ncnt.alloc((size_t)ph->K * ph->str * ph->dim * ph->vocab_size));
    D2G_CUDA(ph->csym.alloc((size_t)ph->K * ph->str * ph->dim));
  }

  int rc2 = upload_columns_batched(ph, d);
  if (rc2) return rc2;
  // launch-shape defaults: the environment, the global configuration, then
  // whatever the autotuner recorded for this shape
  {
    const char *dx = getenv("D2G_WIDE_EXCHANGE");  // "cluster": synchronous DSMEM exchange
    const char *sc = getenv("D2G_STAGE_COSTS");    // "0": table costs through the cache
    ph->tune.exchange = (dx && std::string(dx) == "cluster") ? 1 : 0;
    ph->tune.stage_costs = (sc && std::string(sc) == "0") ? 0 : 1;
    ph->tune.ctas_per_sm = 0;
    ph->tune.cost_gemm = cfg_snapshot().cost_gemm;
    ph->tune.pairs = 1;
    ph->tune.unit_order = 0;
    ph->tune.stage_scales = 1;
    d2g_tuning rec;
    if (tune_cache_get(tune_key(ph), &rec)) ph->tune = rec;
  }
  if (ph->nwide > 0) {
    D2G_CUDA(ph->rowpart.alloc((size_t)ph->nplans * kMaxCluster * ph->MP));
    D2G_CUDA(ph->rowsc.alloc((size_t)ph->nplans * ph->MP));
  } else if (ph->MP <= 128) {  // pair passes possible
    D2G_CUDA(ph->rowsc.alloc((size_t)ph->nplans * ph->MP));
    D2G_CUDA(ph->rowsum2.alloc((size_t)ph->nplans * ph->MP));
    D2G_CUDA(ph->rawsum.alloc((size_t)ph->nplans * ph->MP));
  }
  PlanArgs base = base_args(ph);
  ph->smem_plan = plan_smem_bytes(ph->MP, 0, 1);
  ph->smem_plan_upd = plan_smem_bytes(ph->MP, euc ? ph->dim : 0, 1);
  // raise the shared-memory limits and size the persistent grids of the plan
  // kernels for every cluster size in use, before any stream capture
  std::vector<int> sizes = {1};
  for (auto &b : ph->buckets) sizes.push_back(b.cs);
  for (int cs : sizes) {
    PlanArgs a = base;
    a.cs = cs;
    for (int chk = 0; chk < 2; ++chk)
      D2G_CUDA(launch_plan(ph->MP, ph->mode, chk, a, 0, ph->smem_plan_upd, ph->st));
  }
  if (ph->rowsum2.n > 0) {  // the pair kernel too (its smem limit and grid), MP <= 128
    PlanArgs a = base;
    a.cs = 1;
    for (int chk = 0; chk < 2; ++chk) D2G_CUDA(launch_plan_pair(ph->MP, ph->mode, chk, a, 0, ph->st));
  }
  return D2G_OK;
}

static int upload_columns_plain(d2g_phase *ph, const d2g_phase_desc *d) {
  const size_t col = ph->col;
  D2G_CUDA(ph->pw.alloc(col));
  D2G_CUDA(cudaMemcpyAsync(ph->pw.p, d->p_w, col * 8, cudaMemcpyHostToDevice, ph->st));
  const bool euc = ph->metric == D2_EUCLIDEAN_L2, emb = ph->metric == D2_WORD_EMBED;
  if (euc) {
    D2G_CUDA(ph->psupp.alloc(col * ph->dim));
    D2G_CUDA(cudaMemcpyAsync(ph->psupp.p, d->p_supp, col * ph->dim * 8, cudaMemcpyHostToDevice, ph->st));
  }
  if (emb || ph->metric == D2_SPARSE_HISTOGRAM) {
    D2G_CUDA(ph->psym.alloc(col));
    D2G_CUDA(cudaMemcpyAsync(ph->psym.p, d->p_supp_sym, col * 4, cudaMemcpyHostToDevice, ph->st));
  }
  if (ph->metric == D2_N_GRAM) {  // dim symbols per column, the symbol cost, counts, centroids
    const size_t ns = col * (size_t)ph->dim, VV = (size_t)ph->vocab_size * ph->vocab_size;
    ph->h_nsym.assign(d->p_supp_sym, d->p_supp_sym + ns);
    D2G_CUDA(ph->psym.alloc(ns));
    D2G_CUDA(cudaMemcpyAsync(ph->psym.p, d->p_supp_sym, ns * 4, cudaMemcpyHostToDevice, ph->st));
    D2G_CUDA(ph->pdist.alloc(VV));
    D2G_CUDA(cudaMemcpyAsync(ph->pdist.p, d->dist_mat, VV * 8, cudaMemcpyHostToDevice, ph->st));
    D2G_CUDA(ph->ncnt.alloc((size_t)ph->K * ph->str * ph->dim * ph->vocab_size));
    D2G_CUDA(ph->csym.alloc((size_t)ph->K * ph->str * ph->dim));
  }
  if (emb) {
    D2G_CUDA(ph->pvocab.alloc((size_t)ph->vocab_size * ph->dim));
    D2G_CUDA(cudaMemcpyAsync(ph->pvocab.p, d->vocab_vec, (size_t)ph->vocab_size * ph->dim * 8,
                             cudaMemcpyHostToDevice, ph->st));
  }
  if (ph->metric == D2_HISTOGRAM || ph->metric == D2_SPARSE_HISTOGRAM) {
    D2G_CUDA(ph->pdist.alloc((size_t)ph->vocab_size * ph->vocab_size));
    D2G_CUDA(cudaMemcpyAsync(ph->pdist.p, d->dist_mat, (size_t)ph->vocab_size * ph->vocab_size * 8,
                             cudaMemcpyHostToDevice, ph->st));
  }
  D2G_CUDA(cudaStreamSynchronize(ph->st));
  return D2G_OK;
}

static int create_plain(d2g_phase *ph, const d2g_phase_desc *d) {
  const size_t n = ph->size, col = ph->col, nent = (size_t)ph->str * col;
  D2G_CUDA(ph->pC.alloc(nent));
  D2G_CUDA(ph->pX.alloc(nent));
  D2G_CUDA(ph->pY.alloc(nent));
  D2G_CUDA(ph->pZ.alloc(nent));
  D2G_CUDA(ph->pZ0.alloc(nent));
  D2G_CUDA(cudaMemsetAsync(ph->pZ.p, 0, nent * 8, ph->st));
  const bool euc = ph->metric == D2_EUCLIDEAN_L2, emb = ph->metric == D2_WORD_EMBED;
  int rc = upload_columns_plain(ph, d);
  if (rc) return rc;
  std::vector<int> ci(col);
  for (size_t i = 0; i < n; ++i)
    for (int j = 0; j < ph->p_str[i]; ++j) ci[ph->cum[i] + j] = (int)i;
  D2G_CUDA(ph->pcol_inst.alloc(col));
  D2G_CUDA(cudaMemcpyAsync(ph->pcol_inst.p, ci.data(), col * 4, cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(ph->pp_str.alloc(n));
  D2G_CUDA(cudaMemcpyAsync(ph->pp_str.p, ph->p_str.data(), n * 4, cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(ph->pcum.alloc(n));
  D2G_CUDA(cudaMemcpyAsync(ph->pcum.p, ph->cum.data(), n * 8, cudaMemcpyHostToDevice, ph->st));
  D2G_CUDA(ph->plabel.alloc(n));
  D2G_CUDA(ph->pzr.alloc(n * ph->str));
  if (euc || emb) D2G_CUDA(ph->pxmom.alloc(n * (ph->dim + 1) * ph->str));
  D2G_CUDA(ph->reinit.alloc(n));
  D2G_CUDA(ph->resid_part.alloc((size_t)plain_check_blocks((long long)nent) * 4));
  D2G_CUDA(ph->rho_part.alloc(plain_check_blocks((long long)nent)));
  D2G_CUDA(cudaStreamSynchronize(ph->st));
  return D2G_OK;
}

static PlainArgs plain_args(d2g_phase *ph, int iter) {
  PlainArgs a{};
  a.C = ph->pC.p;
  a.X = ph->pX.p;
  a.Y = ph->pY.p;
  a.Z = ph->pZ.p;
  a.Z0 = ph->pZ0.p;
  a.w = ph->pw.p;
  a.supp = ph->psupp.p;
  a.vocab = ph->pvocab.p;
  a.dist = ph->pdist.p;
  a.sym = ph->psym.p;
  a.csym = ph->csym.p;
  a.col_inst = ph->pcol_inst.p;
  a.p_str = ph->pp_str.p;
  a.label = ph->plabel.p;
  a.cum = ph->pcum.p;
  a.reinit = ph->reinit.p;
  a.zr = ph->pzr.p;
  a.xmom = ph->pxmom.p;
  a.cw64 = ph->cw64.p;
  a.cs64 = ph->cs64.p;
  a.part = ph->resid_part.p;
  a.ctl = ph->ctl.p;
  a.col = (long long)ph->col;
  a.nent = (long long)ph->col * ph->str;
  a.size = (int)ph->size;
  a.str = ph->str;
  a.dim = ph->dim;
  a.metric = ph->metric;
  a.vocab_size = ph->vocab_size;
  a.iter = iter;
  return a;
}

static ClusterArgs cluster_args(d2g_phase *ph, int iter, bool moments) {
  ClusterArgs c{};
  const bool batched = ph->path == 0;
  c.rowsum32 = batched ? ph->rowsum.p : nullptr;
  c.rowsum64 = batched ? nullptr : ph->pzr.p;
  c.xmom32 = batched ? ph->xmom.p : nullptr;
  c.xmom64 = batched ? nullptr : ph->pxmom.p;
  c.rstride = batched ? ph->MP : ph->str;
  c.cl_ptr = ph->cl_ptr.p;
  c.cl_plans = batched ? nullptr : ph->cl_plans.p;  // batched outputs are in slot order
  c.K = ph->K;
  c.m = ph->str;
  c.dim = (ph->metric == D2_EUCLIDEAN_L2 || ph->metric == D2_WORD_EMBED) ? ph->dim : 0;
  c.chunk = ph->chunk;
  c.nchunk = ph->nchunk;
  c.part = ph->part.p;
  c.cw64 = ph->cw64.p;
  c.cs64 = ph->cs64.p;
  c.cw32 = batched ? ph->cw32.p : nullptr;
  c.cs32 = batched ? ph->cs32.p : nullptr;
  c.MP = batched ? ph->MP : ph->str;
  c.DS = ph->DS;
  c.ctl = ph->ctl.p;
  c.iter = iter;
  c.do_weights = 1;
  c.do_moments = moments ? 1 : 0;
  return c;
}

// Everything the captured loop bakes into kernel arguments.
static std::vector<unsigned long long> loop_signature(d2g_phase *ph) {
  auto u = [](const void *p) { return (unsigned long long)(uintptr_t)p; };
  return {u(ph->part.p), u(ph->trace.p), u(ph->Xp.p), u(ph->cl_ptr.p), u(ph->cl_plans.p),
          u(ph->cw64.p), u(ph->cs64.p), u(ph->ctl.p), u(ph->resid_part.p), u(ph->ctab.p),
          u(ph->grp_rec.p), u(ph->plan_slot.p), u(ph->pair_key.p), u(ph->pair_ptr.p),
          u(ph->occ_col.p), (unsigned long long)ph->npairs, u(ph->vsplit.p), u(ph->csplit.p),
          (unsigned long long)ph->nchunk, (unsigned long long)ph->chunk,
          (unsigned long long)ph->global_size, (unsigned long long)ph->cost_gemm,
          u(ph->wide.p), u(ph->def_iter.p), u(ph->rowpart.p), u(ph->rowsc.p), u(ph->col_crow.p),
          (unsigned long long)ph->stage_costs, (unsigned long long)ph->tune.ctas_per_sm,
          (unsigned long long)ph->tune.stage_scales,
          (unsigned long long)ph->defer, u(ph->ncnt.p), u(ph->csym.p), u(ph->nkey.p), u(ph->nptr.p),
          u(ph->nocc.p), (unsigned long long)ph->nlists, u(ph->ntup.p), u(ph->ndist.p),
          (unsigned long long)ph->ntab, (unsigned long long)ph->pairs, u(ph->rowsum2.p), u(ph->rawsum.p),
          u(ph->plan_label.p), u(ph->item_pp.p)};
}

static bool has_collision(int maxIters, int upl) {
  for (int it = 0; it <= maxIters; ++it)
    if (it % upl == 0 && is_check_iter(it)) return true;
  return false;
}

static EmbedArgs embed_args(d2g_phase *ph, int iter) {
  EmbedArgs e{};
  e.pair_key = ph->pair_key.p;
  e.pair_ptr = ph->pair_ptr.p;
  e.occ_col = ph->occ_col.p;
  e.npairs = ph->npairs;
  e.X = ph->Xp.p;
  e.W = ph->W.p;
  e.vocab = ph->vocab32.p;
  e.vnorm = ph->vnorm.p;
  e.vsplit = ph->vsplit.p;
  e.csplit = ph->csplit.p;
  e.cnorm = ph->cnorm.p;
  e.part = ph->epart.p;
  e.nchunk = ph->enchunk;
  e.chunk = ph->echunk;
  e.cs64 = ph->cs64.p;
  e.cs32f = ph->cs32f.p;
  e.T = ph->ctab.p;
  e.ctl = ph->ctl.p;
  e.iter = iter;
  e.K = ph->K;
  e.m = ph->str;
  e.MP = ph->MP;
  e.V = ph->vocab_size;
  e.d = ph->dim;
  e.gemm = ph->cost_gemm;
  return e;
}

static NgramArgs ngram_args(d2g_phase *ph, int iter) {
  NgramArgs g{};
  const bool b = ph->path == 0;
  g.key = ph->nkey.p;
  g.ptr = ph->nptr.p;
  g.occ = ph->nocc.p;
  g.nlists = ph->nlists;
  g.Z32 = b ? ph->Z.p : nullptr;
  g.Z64 = b ? nullptr : ph->pZ.p;
  g.zstride = b ? ph->MP : ph->str;
  g.cnt = ph->ncnt.p;
  g.dist = b ? ph->ndist.p : ph->pdist.p;
  g.csym = ph->csym.p;
  g.tup = ph->ntup.p;
  g.T = ph->ctab.p;
  g.ctl = ph->ctl.p;
  g.iter = iter;
  g.K = ph->K;
  g.m = ph->str;
  g.dim = ph->dim;
  g.V = ph->vocab_size;
  g.U = ph->ntab;
  g.MP = ph->MP;
  return g;
}

// ------------------------------------------------------------- the loop
// Sharded update: SUM of n doubles of the phase's exchange buffer over all
// shards, in place, enqueued on the phase's stream by the exchange function.
static int xchg(d2g_phase *ph, double *buf, size_t n) {
  const int rc = ph->xfn(buf, n, (void *)ph->st, ph->xctx);
  if (rc) return fail(D2G_E_CUDA, "sharded update: the exchange between shards failed (" +
                                      std::to_string(rc) + ")");
  return D2G_OK;
}

// Step 4 (and 5) over the clusters; a shard adds its chunks first and the
// exchange sums those over all shards before the final.
static int cluster_reduce(d2g_phase *ph, ClusterArgs c) {
  if (!ph->xfn) {
    D2G_CUDA(launch_cluster_reduce(c, ph->st));
    return D2G_OK;
  }
  D2G_CUDA(launch_cluster_partial(c, ph->st));
  D2G_CUDA(launch_cluster_local(c, ph->xbuf.p, ph->st));
  int rc = xchg(ph, ph->xbuf.p, cluster_xsum_count(c));
  if (rc) return rc;
  c.xsum = ph->xbuf.p;
  D2G_CUDA(launch_cluster_final(c, ph->st));
  return D2G_OK;
}

// Step 6: obj, primres, dualres; a shard's three sums are exchanged first.
static int resid_final(d2g_phase *ph, const double *part, int n, double *slot, int iter, bool from3) {
  if (!ph->xfn) {
    D2G_CUDA(launch_resid_final(part, n, ph->ctl.p, slot, iter, from3, ph->st));
    return D2G_OK;
  }
  D2G_CUDA(launch_resid_final(part, n, ph->ctl.p, slot, iter, from3, ph->st, 1, ph->xbuf.p));
  int rc = xchg(ph, ph->xbuf.p, 3);
  if (rc) return rc;
  D2G_CUDA(launch_resid_final(part, n, ph->ctl.p, slot, iter, from3, ph->st, 2, ph->xbuf.p));
  return D2G_OK;
}

static int enqueue_loop(d2g_phase *ph, int maxIters, int upl, bool profile, long long *launches,
                        double *plan_ms, int *plan_timed) {
  const bool euc = ph->metric == D2_EUCLIDEAN_L2, emb = ph->metric == D2_WORD_EMBED;
  const bool ng = ph->metric == D2_N_GRAM;
  int chk_idx = 0;
  long long nl = 0;
  std::vector<cudaEvent_t> evs, tevs;  // plan launches, cost-table launches (profile mode)
  if (ph->path == 0) {
    PlanArgs base = base_args(ph);
    // Two iterations in one pass (plan_pair.cuh) where that is exact: `it` is
    // no support update and it + 1 no residual check.  Which pairs to take: the
    // fewest passes over the plans, counting the pass that applies a pair's
    // deferred scale before a single pass or at the end (a short dynamic
    // programme over the iterations).
    std::vector<char> pair_at((size_t)maxIters + 2, 0);
    if (ph->pairs) {
      const int N = maxIters + 1;
      auto upd_at = [&](int i) { return (i % upl == 0) && (euc || emb || (ng && i > 0)); };
      auto can_pair = [&](int i) { return i + 1 < N && !upd_at(i) && !is_check_iter(i + 1); };
      std::vector<int> f0((size_t)N + 2, 0), f1((size_t)N + 2, 1);  // passes left; f1: a pair is pending
      f0[N] = 0;
      f1[N] = 1;
      for (int i = N - 1; i >= 0; --i) {
        for (int pend = 0; pend < 2; ++pend) {
          int best = pend + 1 + f0[i + 1];                          // single pass (finalize first)
          if (can_pair(i)) best = std::min(best, 1 + f1[i + 2 <= N ? i + 2 : N]);
          (pend ? f1 : f0)[i] = best;
        }
      }
      int pend = 0;
      for (int i = 0; i < N;) {
        const int single = pend + 1 + f0[i + 1];
        if (can_pair(i) && 1 + f1[i + 2 <= N ? i + 2 : N] <= single) {
          pair_at[i] = 1;
          pend = 1;
          i += 2;
        } else {
          pend = 0;
          i += 1;
        }
      }
    }
    bool pend = false;  // Z / Y hold a pair pass's deferred output (its scale in rowsc)
    for (int it = 0; it <= maxIters; ++it) {
      // n-gram supports move from the second update iteration on (:270)
      const bool upd = (it % upl == 0) && (euc || emb || (ng && it > 0));
      if (pair_at[it]) {
        const int t1 = it + 1;
        const bool upd1 = (t1 % upl == 0) && (euc || emb || ng);  // t1 >= 1
        const bool chk0 = is_check_iter(it);
        if (profile) {
          cudaEvent_t a0, b0;
          cudaEventCreate(&a0);
          cudaEventCreate(&b0);
          evs.push_back(a0);
          evs.push_back(b0);
          cudaEventRecord(a0, ph->st);
        }
        const d2g_phase::Bucket &b = ph->buckets[0];
        PlanArgs a = bucket_args(ph, base, b);
        a.iter = it;
        a.flags = (pend ? PF_IN_DEF : 0) | (upd1 && euc ? PF_UPDATE : 0) | (upd1 && emb ? PF_WRITE_X : 0);
        D2G_CUDA(launch_plan_pair(ph->MP, ph->mode, chk0, a, b.nitems, ph->st));
        if (profile) cudaEventRecord(evs.back(), ph->st);
        // step 4 of `it` (c_w), the second iteration's row scale from that c_w,
        // then step 4 (and step 5) of it + 1
        {
          int rc = cluster_reduce(ph, cluster_args(ph, it, false));
          if (rc) return rc;
        }
        D2G_CUDA(launch_pair_scale(ph->rawsum.p, ph->plan_slot.p, ph->plan_label.p, ph->cw32.p, ph->nplans,
                                   ph->MP, ph->str, ph->rowsc.p, ph->ctl.p, t1, ph->K, ph->st));
        ClusterArgs c1 = cluster_args(ph, t1, upd1 && euc);
        c1.rowsum32 = ph->rowsum2.p;
        {
          int rc = cluster_reduce(ph, c1);
          if (rc) return rc;
        }
        nl += 6;
        if (upd1 && emb) {
          D2G_CUDA(launch_embed_support(embed_args(ph, t1), ph->st));
          D2G_CUDA(launch_embed_table(embed_args(ph, t1), ph->st));
          nl += 6;
        }
        if (upd1 && ng) {  // step 5 of it + 1 from its deferred Z (Z' * rowsc), then the new table
          NgramArgs g = ngram_args(ph, t1);
          g.rowsc = ph->rowsc.p;
          g.grp_meta = ph->grp_meta.p;
          g.S = ph->geo.S;
          g.nplans = ph->nplans;
          D2G_CUDA(launch_ngram_support(g, ph->st));
          D2G_CUDA(launch_ngram_table(g, ph->st));
          nl += 3;
        }
        if (chk0) {
          int rc = resid_final(ph, ph->resid_part.p, ph->total_blocks, ph->trace.p + 4 * chk_idx, it, false);
          if (rc) return rc;
          ++nl;
          ++chk_idx;
        }
        pend = true;
        ++it;  // the loop's increment moves past it + 1
        continue;
      }
      if (pend) {  // a single pass follows a pair: apply the pending scale first
        D2G_CUDA(launch_pair_finalize(ph->Z.p, ph->Y.p, ph->grp_meta.p, ph->ngroups, ph->geo.S, ph->MP,
                                      ph->rowsc.p, ph->nplans, &ph->ctl.p->err, ph->st));
        ++nl;
        pend = false;
      }
      const bool chk = is_check_iter(it);
      const bool collide = upd && chk;
      int flags = (upd && euc ? PF_UPDATE : 0) | (chk ? PF_CHECK : 0) |
                  ((collide || (upd && emb)) ? PF_WRITE_X : 0);
      // wide plans: deferred row normalisation except on check iterations and
      // Euclidean support updates (those exchange synchronously in a cluster)
      const bool def = ph->h_def_iter[it] != 0, prev_def = it > 0 && ph->h_def_iter[it - 1];
      if (profile) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        evs.push_back(a);
        evs.push_back(b);
        cudaEventRecord(a, ph->st);
      }
      if (def) {  // one plain launch over the units
        PlanArgs a = bucket_args(ph, base, ph->units);
        a.iter = it;
        a.flags = flags | PF_OUT_DEF | (prev_def ? PF_IN_DEF : 0);
        D2G_CUDA(launch_plan(ph->MP, ph->mode, chk, a, ph->units.nitems, ph->smem_plan, ph->st));
        ++nl;
      } else {
        for (auto &b : ph->buckets) {
          PlanArgs a = bucket_args(ph, base, b);
          a.iter = it;
          a.flags = flags | (prev_def ? PF_IN_DEF : 0);
          D2G_CUDA(launch_plan(ph->MP, ph->mode, chk, a, b.nitems,
                               (upd && euc) ? ph->smem_plan_upd : ph->smem_plan, ph->st));
          ++nl;
        }
      }
      if (def) {
        D2G_CUDA(launch_rowsum_combine(ph->wide.p, ph->nwide, ph->rowpart.p, ph->cw32.p, ph->MP,
                                       ph->str, ph->rowsum.p, ph->rowsc.p, ph->ctl.p, it, ph->st));
        ++nl;
      }
      if (profile) cudaEventRecord(evs.back(), ph->st);
      {
        int rc = cluster_reduce(ph, cluster_args(ph, it, upd && euc));
        if (rc) return rc;
      }
      nl += 2;
      if (upd && emb) {  // step 5 for word embeddings, then the new cost table
        D2G_CUDA(launch_embed_support(embed_args(ph, it), ph->st));
        cudaEvent_t t0 = nullptr, t1 = nullptr;
        if (profile) {
          cudaEventCreate(&t0);
          cudaEventCreate(&t1);
          cudaEventRecord(t0, ph->st);
        }
        D2G_CUDA(launch_embed_table(embed_args(ph, it), ph->st));
        if (profile) {
          cudaEventRecord(t1, ph->st);
          tevs.push_back(t0);
          tevs.push_back(t1);
        }
        nl += 6;
      }
      if (upd && ng) {  // step 5 of an n-gram phase from this iteration's Z, then the new table
        D2G_CUDA(launch_ngram_support(ngram_args(ph, it), ph->st));
        D2G_CUDA(launch_ngram_table(ngram_args(ph, it), ph->st));
        nl += 3;
      }
      if (collide) {
        for (auto &b : ph->buckets) {
          PlanArgs a = bucket_args(ph, base, b);
          a.iter = it;
          D2G_CUDA(launch_obj(ph->MP, ph->mode, a, b.nitems, ph->st));
          ++nl;
        }
      }
      if (chk) {
        int rc = resid_final(ph, ph->resid_part.p, ph->total_blocks, ph->trace.p + 4 * chk_idx, it, collide);
        if (rc) return rc;
        ++nl;
        ++chk_idx;
      }
    }
    if (pend) {  // the loop ended on a pair: its second iteration's scale
      D2G_CUDA(launch_pair_finalize(ph->Z.p, ph->Y.p, ph->grp_meta.p, ph->ngroups, ph->geo.S, ph->MP,
                                    ph->rowsc.p, ph->nplans, &ph->ctl.p->err, ph->st));
      ++nl;
    }
    if (ph->defer) {  // the scale of the last iteration that ran, if it ran deferred
      for (auto &b : ph->buckets)
        if (b.cs > 1) {
          D2G_CUDA(launch_plan_finalize(ph->Z.p, ph->Y.p, ph->item_g0.p + b.item_off,
                                        ph->item_ng.p + b.item_off, b.nitems, b.cs, ph->geo.G,
                                        ph->geo.S, ph->MP, ph->grp_rec.p, ph->rowsc.p, ph->def_iter.p,
                                        ph->ctl.p, ph->st));
          ++nl;
        }
    }
  } else {
    const unsigned nb = plain_check_blocks((long long)ph->col * ph->str);
    for (int it = 0; it <= maxIters; ++it) {
      const bool upd = (it % upl == 0) && (euc || emb || (ng && it > 0));
      const bool chk = is_check_iter(it);
      PlainArgs a = plain_args(ph, it);
      if (profile) {
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        evs.push_back(e0);
        evs.push_back(e1);
        cudaEventRecord(e0, ph->st);
      }
      D2G_CUDA(plain_iter_steps(a, upd && !ng, ph->st));
      D2G_CUDA(launch_cluster_reduce(cluster_args(ph, it, upd && !ng), ph->st));
      if (upd && ng) D2G_CUDA(launch_ngram_support(ngram_args(ph, it), ph->st));
      if (upd) D2G_CUDA(plain_cost(a, ph->st));
      if (chk) {
        D2G_CUDA(plain_check(a, ph->st));
        D2G_CUDA(launch_resid_final(ph->resid_part.p, (int)nb, ph->ctl.p, ph->trace.p + 4 * chk_idx,
                                    it, false, ph->st));
        ++chk_idx;
      }
      if (profile) cudaEventRecord(evs.back(), ph->st);
      nl += ng ? plain_launches_per_iter(false, chk) + (upd ? 3 : 0) : plain_launches_per_iter(upd, chk);
    }
  }
  if (profile) {
    D2G_CUDA(cudaStreamSynchronize(ph->st));
    double tot = 0;
    for (size_t i = 0; i + 1 < evs.size(); i += 2) {
      float ms = 0;
      cudaEventElapsedTime(&ms, evs[i], evs[i + 1]);
      tot += ms;
    }
    *plan_ms = evs.empty() ? 0 : tot / (evs.size() / 2);
    *plan_timed = (int)(evs.size() / 2);
    for (auto e : evs) cudaEventDestroy(e);
    double ttot = 0;
    for (size_t i = 0; i + 1 < tevs.size(); i += 2) {
      float ms = 0;
      cudaEventElapsedTime(&ms, tevs[i], tevs[i + 1]);
      ttot += ms;
    }
    ph->stats.table_ms_avg = tevs.empty() ? 0 : ttot / (tevs.size() / 2);
    ph->stats.table_launches = (int)(tevs.size() / 2);
    for (auto e : tevs) cudaEventDestroy(e);
  }
  *launches = nl;
  return D2G_OK;
}

// two iterations per pass are possible: plans that each fit one CTA
static bool pair_capable(const d2g_phase *ph, const d2g_config &cfg) {
  return cfg.pair_iterations && ph->path == 0 && ph->nwide == 0 && ph->buckets.size() == 1 &&
         ph->buckets[0].cs == 1 && ph->MP <= 128 && ph->rawsum.n > 0;
}

static int run_impl(d2g_phase *ph, const d2g_badmm_opts *opt, double *c_w, double *c_supp,
                    int *c_sym, const char *label_switch) {
  const d2g_config cfg = cfg_snapshot();
  {
    int rc = apply_tuning(ph);
    if (rc) return rc;
  }
  if (!opt || opt->maxIters < 0 || opt->updatePerLoops <= 0 || !(opt->rhoCoeff > 0) || !c_w)
    return fail(D2G_E_INVAL, "bad B-ADMM options");
  const bool euc = ph->metric == D2_EUCLIDEAN_L2, emb = ph->metric == D2_WORD_EMBED;
  const bool ng = ph->metric == D2_N_GRAM;
  if ((euc || emb) && !c_supp) return fail(D2G_E_INVAL, "c_supp required for this metric");
  const int K = ph->K, m = ph->str, dim = ph->dim;
  const size_t n = ph->size;
  if (ph->xfn) {  // sharded update: what it covers
    if (ph->path != 0) return fail(D2G_E_UNSUPPORTED, "sharded update: the batched form only");
    if (!euc && ph->metric != D2_HISTOGRAM && ph->metric != D2_SPARSE_HISTOGRAM)
      return fail(D2G_E_UNSUPPORTED, "sharded update: Euclidean and histogram phases only");
    if (opt->time_budget > 0 && opt->time_budget < 1.8e10)
      return fail(D2G_E_INVAL, "sharded update: no time budget (every shard must run every iteration)");
  } else {
    for (int l = 0; l < K; ++l)  // a shard run alone must hold every cluster
      if (l < (int)ph->local_count.size() && ph->local_count[l] == 0)
        return fail(D2G_E_EMPTY_CLUSTER, "cluster " + std::to_string(l) + " has no instance");
  }
  if (ng) {
    if (!c_sym) return fail(D2G_E_INVAL, "centroid symbols required for an n-gram phase");
    for (size_t q = 0; q < (size_t)K * m * dim; ++q)
      if (c_sym[q] < 0 || c_sym[q] >= ph->vocab_size) return fail(D2G_E_INVAL, "centroid symbol out of range");
  }

  // re-initialisation flags (per plan)
  std::vector<char> re(n, 1);
  bool any_warm = false;
  if (label_switch)
    for (size_t i = 0; i < n; ++i) {
      const size_t p = ph->path == 0 ? (size_t)ph->inst_plan[i] : i;
      re[p] = label_switch[i] == 1;
      any_warm |= !re[p];
    }
  if (any_warm && !ph->plans_valid)
    return fail(D2G_E_INVAL, "warm start requested but no plans were set");
  D2G_CUDA(cudaMemcpyAsync(ph->reinit.p, re.data(), n, cudaMemcpyHostToDevice, ph->st));

  // centroids and control block
  D2G_CUDA(ph->cw64.alloc((size_t)K * m));
  D2G_CUDA(cudaMemcpyAsync(ph->cw64.p, c_w, (size_t)K * m * 8, cudaMemcpyHostToDevice, ph->st));
  if (euc || emb) {
    D2G_CUDA(ph->cs64.alloc((size_t)K * m * dim));
    D2G_CUDA(cudaMemcpyAsync(ph->cs64.p, c_supp, (size_t)K * m * dim * 8, cudaMemcpyHostToDevice, ph->st));
  }
  if (ng)
    D2G_CUDA(cudaMemcpyAsync(ph->csym.p, c_sym, (size_t)K * m * dim * 4, cudaMemcpyHostToDevice, ph->st));
  ph->max_checks = opt->maxIters / 20 + 8;
  D2G_CUDA(ph->trace.alloc((size_t)4 * ph->max_checks));
  D2G_CUDA(ph->ctl.alloc(1));
  Ctl h{};
  h.stop_iter = INT_MAX;
  const double tb = opt->time_budget;
  h.budget_ns = (tb > 0 && tb < 1.8e10) ? (unsigned long long)(tb * 1e9) : ~0ULL;
  h.rho_coeff = opt->rhoCoeff;
  h.global_size = (double)ph->global_size;
  h.wait_ns = ph->wait_ns;
  h.fault_iter = ph->fault_iter;
  h.fault_unit = ph->fault_unit;
  D2G_CUDA(cudaMemcpyAsync(ph->ctl.p, &h, sizeof h, cudaMemcpyHostToDevice, ph->st));

  if (ph->xfn) {
    // exchange buffer: the largest exchange is the cluster sums with moments
    D2G_CUDA(ph->xbuf.alloc(std::max<size_t>((size_t)K * (dim + 2) * m, (size_t)K) + 8));
    // every cluster must hold an instance on some shard (:142-144)
    std::vector<double> cnt(K);
    for (int l = 0; l < K; ++l) cnt[l] = (double)ph->local_count[l];
    D2G_CUDA(cudaMemcpyAsync(ph->xbuf.p, cnt.data(), K * 8, cudaMemcpyHostToDevice, ph->st));
    int rc = xchg(ph, ph->xbuf.p, (size_t)K);
    if (rc) return rc;
    D2G_CUDA(cudaMemcpyAsync(cnt.data(), ph->xbuf.p, K * 8, cudaMemcpyDeviceToHost, ph->st));
    D2G_CUDA(cudaStreamSynchronize(ph->st));
    for (int l = 0; l < K; ++l)
      if (!(cnt[l] > 0)) return fail(D2G_E_EMPTY_CLUSTER, "cluster " + std::to_string(l) + " has no instance on any shard");
  }

  long long launches = 0;
  if (ph->path == 0 && (euc || emb || ng) && has_collision(opt->maxIters, opt->updatePerLoops))
    D2G_CUDA(ph->Xp.alloc((size_t)ph->ncols_packed * ph->MP));  // X kept for obj after step 5
  if (ph->path == 0) {
    D2G_CUDA(launch_centroid_to_f32(ph->cw64.p, euc ? ph->cs64.p : nullptr, ph->cw32.p,
                                    euc ? ph->cs32.p : nullptr, K, m, dim, ph->MP, ph->DS, ph->st));
    if (emb) {  // the cost table of the initial centroids
      D2G_CUDA(launch_to_f32(ph->cs64.p, (size_t)K * m * dim, ph->cs32f.p, ph->st));
      D2G_CUDA(launch_cost_table(ph->cs32f.p, K, m, ph->vocab32.p, ph->vocab_size, dim, ph->cnorm.p,
                                 ph->vnorm.p, ph->MP, ph->ctab.p, ph->cost_gemm, ph->vsplit.p,
                                 ph->csplit.p, &ph->ctl.p->err, ph->st));
      launches += 3;
    }
    if (ng) {  // the cost table of the initial centroid symbols
      D2G_CUDA(launch_ngram_table(ngram_args(ph, -1), ph->st));
      launches += 1;
    }
    PlanArgs base = base_args(ph);
    for (auto &b : ph->buckets) {
      PlanArgs a = bucket_args(ph, base, b);
      D2G_CUDA(launch_rho_partial(ph->MP, ph->mode, a, b.nitems, ph->rho_part.p + b.block_off, ph->st));
    }
    if (ph->xfn && (ph->xflags & D2G_SHARD_GLOBAL_RHO)) {  // rho over all shards' costs
      D2G_CUDA(launch_rho_local(ph->rho_part.p, ph->total_blocks, (double)ph->col * m, ph->xbuf.p, ph->st));
      int rc = xchg(ph, ph->xbuf.p, 2);
      if (rc) return rc;
      D2G_CUDA(launch_rho_set(ph->xbuf.p, ph->ctl.p, ph->st));
    } else {  // this shard's own, as the reference's MPI build does (:109)
      D2G_CUDA(launch_rho_final(ph->rho_part.p, ph->total_blocks, ph->ctl.p, (double)ph->col * m, ph->st));
    }
    D2G_CUDA(cudaMemsetAsync(ph->Y.p, 0, (size_t)ph->ncols_packed * ph->MP * 4, ph->st));
    for (auto &b : ph->buckets) {
      PlanArgs a = bucket_args(ph, base, b);
      D2G_CUDA(launch_pack_convert(ph->MP, 2, a, b.nitems, nullptr, ph->plan_cum.p, ph->reinit.p,
                                   ph->cw64.p, m, ph->st));
    }
    launches += 2 + 2 * (long long)ph->buckets.size() + 1;
  } else {
    PlainArgs a = plain_args(ph, -1);
    a.part = ph->rho_part.p;
    D2G_CUDA(plain_cost(a, ph->st));
    D2G_CUDA(plain_rho(a, ph->st));
    D2G_CUDA(plain_init(a, ph->st));
    launches += 5;
  }

  // two iterations per pass: phases whose plans fit in one CTA, no time budget
  // (the reference may stop after any iteration)
  ph->pairs = pair_capable(ph, cfg) && ph->tune.pairs && h.budget_ns == ~0ULL && (!ph->xfn || ph->shard_pairs);
  // deferred-exchange schedule of the wide plans
  ph->h_def_iter.assign((size_t)opt->maxIters + 1, 0);
  if (ph->path == 0 && ph->defer) {
    for (int it = 0; it <= opt->maxIters; ++it) {
      // Euclidean support updates need the moments of the same iteration, n-gram
      // updates its final Z: those iterations exchange synchronously
      const bool upd = (it % opt->updatePerLoops == 0) && (euc || (ng && it > 0));
      ph->h_def_iter[it] = !is_check_iter(it) && !upd;
    }
    if (ph->def_iter.n < ph->h_def_iter.size()) D2G_CUDA(ph->def_iter.alloc(ph->h_def_iter.size()));
    D2G_CUDA(cudaMemcpyAsync(ph->def_iter.p, ph->h_def_iter.data(), ph->h_def_iter.size(),
                             cudaMemcpyHostToDevice, ph->st));
    D2G_CUDA(cudaStreamSynchronize(ph->st));  // the host vector may change before the next call
  }
  const bool profile = cfg.profile != 0;
  double plan_ms = 0;
  int plan_timed = 0;
  long long nl = 0;
  D2G_CUDA(cudaEventRecord(ph->ev0, ph->st));
  if (profile || !cfg.use_graph || ph->xfn) {  // (a sharded update enqueues directly)
    int rc = enqueue_loop(ph, opt->maxIters, opt->updatePerLoops, profile, &nl, &plan_ms, &plan_timed);
    if (rc) return rc;
  } else {
    const std::vector<unsigned long long> sig = loop_signature(ph);
    if (!ph->gexec || ph->g_maxIters != opt->maxIters || ph->g_upl != opt->updatePerLoops ||
        ph->g_sig != sig) {
      if (ph->gexec) cudaGraphExecDestroy(ph->gexec);
      ph->gexec = nullptr;
      cudaGraph_t g;
      D2G_CUDA(cudaStreamBeginCapture(ph->st, cudaStreamCaptureModeThreadLocal));
      int rc = enqueue_loop(ph, opt->maxIters, opt->updatePerLoops, false, &nl, &plan_ms, &plan_timed);
      cudaError_t ce = cudaStreamEndCapture(ph->st, &g);
      if (rc) return rc;
      D2G_CUDA(ce);
      D2G_CUDA(cudaGraphInstantiate(&ph->gexec, g, 0));
      cudaGraphDestroy(g);
      ph->g_maxIters = opt->maxIters;
      ph->g_upl = opt->updatePerLoops;
      ph->g_sig = sig;
      ph->g_launches = nl;
    }
    nl = ph->g_launches;
    D2G_CUDA(cudaGraphLaunch(ph->gexec, ph->st));
  }
  D2G_CUDA(cudaEventRecord(ph->ev1, ph->st));

  // results
  D2G_CUDA(cudaMemcpyAsync(c_w, ph->cw64.p, (size_t)K * m * 8, cudaMemcpyDeviceToHost, ph->st));
  if (euc || emb)
    D2G_CUDA(cudaMemcpyAsync(c_supp, ph->cs64.p, (size_t)K * m * dim * 8, cudaMemcpyDeviceToHost, ph->st));
  if (ng)
    D2G_CUDA(cudaMemcpyAsync(c_sym, ph->csym.p, (size_t)K * m * dim * 4, cudaMemcpyDeviceToHost, ph->st));
  ph->h_trace.assign((size_t)4 * ph->max_checks, 0.0);
  D2G_CUDA(cudaMemcpyAsync(ph->h_trace.data(), ph->trace.p, ph->h_trace.size() * 8, cudaMemcpyDeviceToHost, ph->st));
  D2G_CUDA(cudaMemcpyAsync(&h, ph->ctl.p, sizeof h, cudaMemcpyDeviceToHost, ph->st));
  D2G_CUDA(cudaStreamSynchronize(ph->st));
  float ms = 0;
  cudaEventElapsedTime(&ms, ph->ev0, ph->ev1);
  int nchk = 0;
  for (int it = 0; it < h.iters_done; ++it) nchk += is_check_iter(it);
  ph->ntrace = nchk;
  ph->plans_valid = true;
  if (ng) ph->h_csym.assign(c_sym, c_sym + (size_t)K * m * dim);
  ph->stats.iterations = h.iters_done;
  ph->stats.rho = h.rho;
  ph->stats.total_ms = ms;
  ph->stats.plan_ms_avg = plan_ms;
  ph->stats.plan_launches = plan_timed;
  ph->stats.kernel_launches = launches + nl;
  ph->stats.plan_entries = ph->col * m;
  ph->stats.path = ph->path;
  if (!profile) {
    ph->stats.table_ms_avg = 0;
    ph->stats.table_launches = 0;
  }
  ph->stats.table_flops = (ph->path == 0 && emb) ? 2.0 * K * m * (double)ph->vocab_size * dim : 0.0;
  {
    const double ent = (double)ph->col * m;
    const double colb = ph->path == 0 ? (double)ph->col * (euc ? 4.0 * (1 + dim) : 8.0) : 0.0;
    // word-embedding and n-gram costs stream from the per-cluster table (4 B per
    // entry); histogram costs come from one str x str table that stays in L2
    ph->stats.plan_bytes = ph->path == 0 ? ((emb || ng) ? 20.0 : 16.0) * ent + colb + 4.0 * m * (double)n
                                         : 136.0 * ent;
  }
  if (h.err == 9)  // a plan-pass self-check: a staged plan record, slot or table row out of range
    return fail(D2G_E_CUDA, "device self-check failed: a plan record or table row out of range in a plan pass");
  if (h.err == 7)
    return fail(D2G_E_CUDA, "a plan pass gave up waiting for a bulk copy of its tiles (bounded wait ran out)");
  if (h.err == kErrTcTimeout)
    return fail(D2G_E_CUDA, "tensor-core cost table: wait for the MMA completion timed out");
  if (h.err) return fail(D2G_E_NUMERIC, "non-positive or non-finite normaliser (device code " +
                                            std::to_string(h.err) + ")");
  return D2G_OK;
}


// FP64 ground costs of every instance against its labelled centroid, the
// reference layout; backs the calculate_distmat drop-in.
int distmat_fp64(int dim, int str, size_t size, const int *p_str, int metric, const double *supp,
                 const int *sym, const double *vocab, int V, const int *label, const double *c_supp,
                 size_t K, double *C_host, const double *dist, const int *c_sym) {
  const bool ng = metric == D2_N_GRAM;
  if (dim < 1 || str < 1 || !p_str || !label || !C_host || (ng ? (!c_sym || !dist || !sym) : !c_supp))
    return fail(D2G_E_INVAL, "distmat args");
  std::vector<long long> cum(size);
  long long col = 0;
  for (size_t i = 0; i < size; ++i) {
    if (label[i] < 0 || (size_t)label[i] >= K) return fail(D2G_E_INVAL, "label out of range");
    if (p_str[i] < 0) return fail(D2G_E_INVAL, "negative support size");
    cum[i] = col;
    col += p_str[i];
  }
  // every id the cost kernel indexes with must lie inside its table (a
  // negative word-embedding id is the reference's ||centroid||^2 case)
  if (metric == D2_WORD_EMBED || ng) {
    if (!sym || V < 1 || (!ng && !vocab)) return fail(D2G_E_INVAL, "distmat: ids or vocabulary missing");
    const size_t nsym = ng ? (size_t)col * dim : (size_t)col;
    for (size_t j = 0; j < nsym; ++j)
      if (sym[j] >= V || (ng && sym[j] < 0)) return fail(D2G_E_INVAL, "distmat: id out of range");
    if (ng)
      for (size_t j = 0; j < K * str * (size_t)dim; ++j)
        if (c_sym[j] < 0 || c_sym[j] >= V) return fail(D2G_E_INVAL, "distmat: centroid symbol out of range");
  } else if (metric == D2_EUCLIDEAN_L2 && !supp && col > 0) {
    return fail(D2G_E_INVAL, "distmat: supports missing");
  }
  std::vector<int> ci(col);
  for (size_t i = 0; i < size; ++i)
    for (int j = 0; j < p_str[i]; ++j) ci[cum[i] + j] = (int)i;
  cudaStream_t st;
  D2G_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct Guard {
    cudaStream_t s;
    ~Guard() { cudaStreamDestroy(s); }
  } guard{st};
  DBuf<double> dC, dS, dV, dCS;
  DBuf<int> dSym, dCI, dL, dCsym;
  DBuf<long long> dCum;
  const size_t nent = (size_t)col * str;
  D2G_CUDA(dC.alloc(nent));
  if (ng) {  // symbols per column, centroid symbols, the symbol cost
    D2G_CUDA(dSym.alloc((size_t)col * dim));
    D2G_CUDA(cudaMemcpyAsync(dSym.p, sym, (size_t)col * dim * 4, cudaMemcpyHostToDevice, st));
    D2G_CUDA(dCsym.alloc(K * str * dim));
    D2G_CUDA(cudaMemcpyAsync(dCsym.p, c_sym, K * str * dim * 4, cudaMemcpyHostToDevice, st));
    D2G_CUDA(dV.alloc((size_t)V * V));
    D2G_CUDA(cudaMemcpyAsync(dV.p, dist, (size_t)V * V * 8, cudaMemcpyHostToDevice, st));
  } else {
    D2G_CUDA(dCS.alloc(K * str * dim));
    D2G_CUDA(cudaMemcpyAsync(dCS.p, c_supp, K * str * dim * 8, cudaMemcpyHostToDevice, st));
    if (metric == D2_EUCLIDEAN_L2) {
      D2G_CUDA(dS.alloc((size_t)col * dim));
      D2G_CUDA(cudaMemcpyAsync(dS.p, supp, (size_t)col * dim * 8, cudaMemcpyHostToDevice, st));
    } else {
      D2G_CUDA(dSym.alloc(col));
      D2G_CUDA(dV.alloc((size_t)V * dim));
      D2G_CUDA(cudaMemcpyAsync(dSym.p, sym, col * 4, cudaMemcpyHostToDevice, st));
      D2G_CUDA(cudaMemcpyAsync(dV.p, vocab, (size_t)V * dim * 8, cudaMemcpyHostToDevice, st));
    }
  }
  D2G_CUDA(dCI.alloc(col));
  D2G_CUDA(dL.alloc(size));
  D2G_CUDA(dCum.alloc(size));
  D2G_CUDA(cudaMemcpyAsync(dCI.p, ci.data(), col * 4, cudaMemcpyHostToDevice, st));
  D2G_CUDA(cudaMemcpyAsync(dL.p, label, size * 4, cudaMemcpyHostToDevice, st));
  D2G_CUDA(cudaMemcpyAsync(dCum.p, cum.data(), size * 8, cudaMemcpyHostToDevice, st));
  PlainArgs a{};
  a.C = dC.p;
  a.supp = dS.p;
  a.vocab = ng ? nullptr : dV.p;
  a.dist = ng ? dV.p : nullptr;
  a.csym = dCsym.p;
  a.sym = dSym.p;
  a.col_inst = dCI.p;
  a.label = dL.p;
  a.cum = dCum.p;
  a.cs64 = dCS.p;
  a.col = col;
  a.nent = (long long)nent;
  a.size = (int)size;
  a.str = str;
  a.dim = dim;
  a.metric = metric;
  a.vocab_size = V;
  a.iter = -1;
  D2G_CUDA(plain_cost(a, st));
  D2G_CUDA(cudaMemcpyAsync(C_host, dC.p, nent * 8, cudaMemcpyDeviceToHost, st));
  D2G_CUDA(cudaStreamSynchronize(st));
  return D2G_OK;
}

}  // namespace d2g

// =================================================================== C API
extern "C" {

int d2g_get_config(d2g_config *cfg) {
  if (!cfg) return D2G_E_INVAL;
  *cfg = cfg_snapshot();
  return D2G_OK;
}

int d2g_set_config(const d2g_config *cfg) {
  if (!cfg || cfg->precision < 0 || cfg->precision > 1 || cfg->cost_gemm < 0 || cfg->cost_gemm > 1 ||
      cfg->keep_time_budget < 0 || cfg->keep_time_budget > 1 || cfg->pair_iterations < 0 ||
      cfg->pair_iterations > 1)
    return D2G_E_INVAL;
  std::lock_guard<std::mutex> lk(g_cfg_mu);
  g_cfg = *cfg;
  return D2G_OK;
}

const char *d2g_error_string(int code) {
  switch (code) {
    case D2G_OK: return "ok";
    case D2G_E_INVAL: return "invalid argument";
    case D2G_E_CUDA: return "CUDA error";
    case D2G_E_NOMEM: return "out of memory";
    case D2G_E_UNSUPPORTED: return "unsupported metric type or shape";
    case D2G_E_EMPTY_CLUSTER: return "empty cluster";
    case D2G_E_NUMERIC: return "non-positive or non-finite normaliser";
    case D2G_E_ADMISSION: return "request refused by admission control";
    case D2G_E_NOTFOUND: return "unknown ticket";
    default: return "unknown error";
  }
}

const char *d2g_last_error(void) { return d2g::g_last_error.c_str(); }

int d2g_phase_create(const d2g_phase_desc *d, int precision, d2g_phase **out) {
  if (!d || !out || d->size == 0 || d->str <= 0 || d->num_of_labels <= 0 || !d->p_str || !d->p_w ||
      !d->label)
    return fail(D2G_E_INVAL, "incomplete phase description");
  const int mt = d->metric_type;
  if (mt == D2_CITYBLOCK_L1)
    return fail(D2G_E_UNSUPPORTED, "metric type " + std::to_string(mt) + " is not supported");
  if (mt != D2_EUCLIDEAN_L2 && mt != D2_WORD_EMBED && mt != D2_HISTOGRAM && mt != D2_SPARSE_HISTOGRAM &&
      mt != D2_N_GRAM)
    return fail(D2G_E_INVAL, "unknown metric type");
  if (mt == D2_N_GRAM && (d->dim < 1 || !d->p_supp_sym || !d->dist_mat || d->vocab_size < 1))
    return fail(D2G_E_INVAL, "n-gram phase needs symbols and a symbol cost matrix");
  if (mt == D2_EUCLIDEAN_L2 && (d->dim < 1 || !d->p_supp)) return fail(D2G_E_INVAL, "supports missing");
  if (mt == D2_WORD_EMBED && (d->dim < 1 || !d->p_supp_sym || !d->vocab_vec || d->vocab_size < 1))
    return fail(D2G_E_INVAL, "embedding phase needs ids and vocabulary");
  if ((mt == D2_HISTOGRAM || mt == D2_SPARSE_HISTOGRAM) && (!d->dist_mat || d->vocab_size != d->str))
    return fail(D2G_E_INVAL, "histogram phase needs a str x str cost matrix");
  if (mt == D2_SPARSE_HISTOGRAM && !d->p_supp_sym) return fail(D2G_E_INVAL, "sparse histogram ids missing");
  if (mt == D2_HISTOGRAM)  // the plan of a dense histogram indexes the cost by bin: m_i <= bins
    for (size_t i = 0; i < d->size; ++i)
      if (d->p_str[i] > d->vocab_size) return fail(D2G_E_INVAL, "histogram with more bins than the cost matrix");
  if (d->str > 256) return fail(D2G_E_UNSUPPORTED, "str > 256");

  d2g_phase *ph = new d2g_phase();
  ph->metric = mt;
  ph->dim = (mt == D2_EUCLIDEAN_L2 || mt == D2_WORD_EMBED || mt == D2_N_GRAM) ? d->dim : 0;
  ph->str = d->str;
  ph->K = d->num_of_labels;
  ph->vocab_size = d->vocab_size;
  ph->size = d->size;
  ph->global_size = d->global_size ? d->global_size : d->size;
  ph->p_str.assign(d->p_str, d->p_str + d->size);
  ph->cum.resize(d->size);
  long long c = 0;
  for (size_t i = 0; i < d->size; ++i) {
    if (d->p_str[i] < 1) {
      delete ph;
      return fail(D2G_E_INVAL, "instance with no support point");
    }
    ph->cum[i] = c;
    c += d->p_str[i];
  }
  ph->col = (size_t)c;
  if (mt == D2_SPARSE_HISTOGRAM || mt == D2_WORD_EMBED || mt == D2_N_GRAM) {
    const size_t nsym = mt == D2_N_GRAM ? ph->col * (size_t)d->dim : ph->col;
    for (size_t j = 0; j < nsym; ++j)
      if (d->p_supp_sym[j] < 0 || d->p_supp_sym[j] >= d->vocab_size) {
        delete ph;
        return fail(D2G_E_INVAL, "vocabulary id out of range");
      }
  }
  std::string why;
  ph->path = (precision == 1 || !batched_supported(d, &why)) ? 1 : 0;
  int rc = D2G_OK;
  if (cudaStreamCreateWithFlags(&ph->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&ph->ev0) != cudaSuccess || cudaEventCreate(&ph->ev1) != cudaSuccess) {
    delete ph;
    return fail(D2G_E_CUDA, "stream/event creation failed (no usable GPU?)");
  }
  rc = ph->path == 0 ? create_batched(ph, d) : D2G_E_UNSUPPORTED;
  if (rc == D2G_E_UNSUPPORTED) {  // shapes the batched form does not pack: FP64 form
    ph->path = 1;
    rc = create_plain(ph, d);
  }
  if (!rc) rc = set_labels_impl(ph, d->label);
  if (rc) {
    delete ph;
    return rc;
  }
  *out = ph;
  return D2G_OK;
}

int d2g_phase_refresh(d2g_phase *ph, const d2g_phase_desc *d) {
  if (!ph || !d || d->size != ph->size || d->str != ph->str || d->metric_type != ph->metric ||
      d->num_of_labels != ph->K || !d->p_w || !d->label)
    return fail(D2G_E_INVAL, "refresh needs the phase's own shape");
  for (size_t i = 0; i < ph->size; ++i)
    if (d->p_str[i] != ph->p_str[i]) return fail(D2G_E_INVAL, "support sizes changed");
  int rc = ph->path == 0 ? upload_columns_batched(ph, d) : upload_columns_plain(ph, d);
  if (rc) return rc;
  ph->global_size = d->global_size ? d->global_size : d->size;
  // what set_labels_impl derives (cluster lists, plan slots, group records)
  // depends on the labels alone for Euclidean and histogram phases: kept while
  // they are unchanged (word-embedding and n-gram lists also follow the ids)
  const bool label_only = ph->metric == D2_EUCLIDEAN_L2 || ph->metric == D2_HISTOGRAM ||
                          ph->metric == D2_SPARSE_HISTOGRAM;
  if (label_only && ph->label.size() == ph->size &&
      memcmp(ph->label.data(), d->label, ph->size * sizeof(int)) == 0)
    return D2G_OK;
  return set_labels_impl(ph, d->label);
}

int d2g_phase_destroy(d2g_phase *ph) {
  if (!ph) return D2G_E_INVAL;
  cudaStreamSynchronize(ph->st);
  delete ph;
  return D2G_OK;
}

int d2g_phase_set_labels(d2g_phase *ph, const int *label) {
  if (!ph || !label) return D2G_E_INVAL;
  return set_labels_impl(ph, label);
}

int d2g_phase_set_plans(d2g_phase *ph, const double *Z) {
  if (!ph || !Z) return D2G_E_INVAL;
  const size_t nent = ph->col * (size_t)ph->str;
  if (ph->path == 1) {
    D2G_CUDA(cudaMemcpyAsync(ph->pZ.p, Z, nent * 8, cudaMemcpyHostToDevice, ph->st));
  } else {
    D2G_CUDA(ph->stage.alloc(nent));
    D2G_CUDA(cudaMemcpyAsync(ph->stage.p, Z, nent * 8, cudaMemcpyHostToDevice, ph->st));
    PlanArgs base = base_args(ph);
    for (auto &b : ph->buckets) {
      PlanArgs a = bucket_args(ph, base, b);
      D2G_CUDA(launch_pack_convert(ph->MP, 0, a, b.nitems, ph->stage.p, ph->plan_cum.p, nullptr,
                                   nullptr, ph->str, ph->st));
    }
  }
  D2G_CUDA(cudaStreamSynchronize(ph->st));
  ph->plans_valid = true;
  return D2G_OK;
}

static int unpack_to_host(d2g_phase *ph, float *packed, double *out, int dir = 1) {
  const size_t nent = ph->col * (size_t)ph->str;
  D2G_CUDA(ph->stage.alloc(nent));
  PlanArgs base = base_args(ph);
  base.Z = packed;
  for (auto &b : ph->buckets) {
    PlanArgs a = bucket_args(ph, base, b);
    D2G_CUDA(launch_pack_convert(ph->MP, dir, a, b.nitems, ph->stage.p, ph->plan_cum.p, nullptr,
                                 nullptr, ph->str, ph->st));
  }
  D2G_CUDA(cudaMemcpyAsync(out, ph->stage.p, nent * 8, cudaMemcpyDeviceToHost, ph->st));
  D2G_CUDA(cudaStreamSynchronize(ph->st));
  return D2G_OK;
}

int d2g_phase_get_plans(d2g_phase *ph, double *Z) {
  if (!ph || !Z) return D2G_E_INVAL;
  if (ph->path == 1) {
    D2G_CUDA(cudaMemcpyAsync(Z, ph->pZ.p, ph->col * (size_t)ph->str * 8, cudaMemcpyDeviceToHost, ph->st));
    D2G_CUDA(cudaStreamSynchronize(ph->st));
    return D2G_OK;
  }
  return unpack_to_host(ph, ph->Z.p, Z);
}

int d2g_phase_get_scratch(d2g_phase *ph, double *X, double *Y, double *C) {
  if (!ph) return D2G_E_INVAL;
  const size_t nb = ph->col * (size_t)ph->str * 8;
  if (ph->path == 1) {
    if (X) D2G_CUDA(cudaMemcpyAsync(X, ph->pX.p, nb, cudaMemcpyDeviceToHost, ph->st));
    if (Y) D2G_CUDA(cudaMemcpyAsync(Y, ph->pY.p, nb, cudaMemcpyDeviceToHost, ph->st));
    if (C) D2G_CUDA(cudaMemcpyAsync(C, ph->pC.p, nb, cudaMemcpyDeviceToHost, ph->st));
    D2G_CUDA(cudaStreamSynchronize(ph->st));
    return D2G_OK;
  }
  if (X || C) return fail(D2G_E_UNSUPPORTED, "the batched form keeps neither X nor C");
  if (Y) return unpack_to_host(ph, ph->Y.p, Y, 3);  // stored times log2(e)
  return D2G_OK;
}

int d2g_badmm_run(d2g_phase *ph, const d2g_badmm_opts *opt, double *c_w, double *c_supp,
                  const char *label_switch) {
  if (!ph) return D2G_E_INVAL;
  if (ph->metric == D2_N_GRAM) return fail(D2G_E_INVAL, "n-gram phases run through d2g_badmm_run_sym");
  return run_impl(ph, opt, c_w, c_supp, nullptr, label_switch);
}

int d2g_badmm_run_sym(d2g_phase *ph, const d2g_badmm_opts *opt, double *c_w, int *c_sym,
                      const char *label_switch) {
  if (!ph) return D2G_E_INVAL;
  if (ph->metric != D2_N_GRAM) return fail(D2G_E_INVAL, "d2g_badmm_run_sym is for n-gram phases");
  return run_impl(ph, opt, c_w, nullptr, c_sym, label_switch);
}

int d2g_phase_set_allreduce(d2g_phase *ph, d2g_allreduce_fn fn, void *ctx, int flags) {
  if (!ph) return fail(D2G_E_INVAL, "null phase");
  if (flags & ~D2G_SHARD_GLOBAL_RHO) return fail(D2G_E_INVAL, "unknown sharding flags");
  ph->xfn = fn;
  ph->xctx = ctx;
  ph->xflags = fn ? flags : 0;
  ph->shard_pairs = false;  // shards in other processes may differ in shape
  return D2G_OK;
}

namespace {
// The exchange between the shards of d2g_badmm_run_shards, all on one device.
// Every shard's host thread reaches the same exchanges in the same order; at
// each, the shards' buffers are summed in shard order on every shard's stream
// (stream-ordered through events, no kernel waits on another).
struct ShardGroup {
  int n = 0;
  std::mutex mu;
  std::condition_variable cv;
  int arrived = 0;
  long long gen = 0;
  bool abort = false;
  std::vector<double *> buf, tmp;
  std::vector<size_t> cnt;
  std::vector<cudaEvent_t> ready, done;
  size_t tmp_cap = 0;
  bool meet() {  // host barrier of all shards; false once a shard has failed
    std::unique_lock<std::mutex> lk(mu);
    const long long g = gen;
    if (++arrived == n) {
      arrived = 0;
      ++gen;
      cv.notify_all();
    } else {
      cv.wait(lk, [&] { return gen != g || abort; });
    }
    return !abort;
  }
  void fail_all() {
    std::lock_guard<std::mutex> lk(mu);
    abort = true;
    cv.notify_all();
  }
};
struct ShardCtx {
  ShardGroup *g;
  int s;
};

int group_allreduce(double *buf, size_t count, void *stream, void *ctx) {
  ShardCtx *c = (ShardCtx *)ctx;
  ShardGroup *g = c->g;
  const int s = c->s;
  cudaStream_t st = (cudaStream_t)stream;
  if (count > g->tmp_cap) {
    g->fail_all();
    return 1;
  }
  g->buf[s] = buf;
  g->cnt[s] = count;
  if (cudaEventRecord(g->ready[s], st) != cudaSuccess) {
    g->fail_all();
    return 2;
  }
  if (!g->meet()) return 3;  // every shard's buffer is ready (in stream order)
  ShardBufs b{};
  b.n = g->n;
  for (int r = 0; r < g->n; ++r) {
    if (g->cnt[r] != count) {
      g->fail_all();
      return 4;
    }
    b.p[r] = g->buf[r];
    if (r != s && cudaStreamWaitEvent(st, g->ready[r], 0) != cudaSuccess) {
      g->fail_all();
      return 2;
    }
  }
  if (launch_shard_sum(b, count, g->tmp[s], st) != cudaSuccess ||
      cudaEventRecord(g->done[s], st) != cudaSuccess) {
    g->fail_all();
    return 2;
  }
  if (!g->meet()) return 3;  // every shard has read every buffer before any is overwritten
  for (int r = 0; r < g->n; ++r)
    if (r != s && cudaStreamWaitEvent(st, g->done[r], 0) != cudaSuccess) {
      g->fail_all();
      return 2;
    }
  if (cudaMemcpyAsync(buf, g->tmp[s], count * 8, cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
    g->fail_all();
    return 2;
  }
  return 0;
}
}  // namespace

int d2g_badmm_run_shards(d2g_phase *const *ph, int nshard, const d2g_badmm_opts *opt, int flags,
                         double *const *c_w, double *const *c_supp) {
  if (!ph || !opt || !c_w || nshard < 1 || nshard > kMaxShards)
    return fail(D2G_E_INVAL, "d2g_badmm_run_shards: 1 to 8 shards, options and outputs required");
  if (flags & ~D2G_SHARD_GLOBAL_RHO) return fail(D2G_E_INVAL, "unknown sharding flags");
  const d2g_config cfg = cfg_snapshot();
  size_t need = 8;
  bool pairs = true;
  for (int s = 0; s < nshard; ++s) {
    if (!ph[s] || !c_w[s]) return fail(D2G_E_INVAL, "d2g_badmm_run_shards: null shard");
    for (int r = 0; r < s; ++r)
      if (ph[r] == ph[s]) return fail(D2G_E_INVAL, "d2g_badmm_run_shards: a phase given twice");
    if (ph[s]->K != ph[0]->K || ph[s]->str != ph[0]->str || ph[s]->dim != ph[0]->dim ||
        ph[s]->metric != ph[0]->metric || ph[s]->path != ph[0]->path)
      return fail(D2G_E_INVAL, "d2g_badmm_run_shards: the shards differ in metric, k, str or dim");
    need = std::max(need, (size_t)ph[s]->K * (ph[s]->dim + 2) * ph[s]->str + 8);
    pairs = pairs && pair_capable(ph[s], cfg);
  }
  int dev = 0;
  D2G_CUDA(cudaGetDevice(&dev));
  ShardGroup g;
  g.n = nshard;
  g.buf.assign(nshard, nullptr);
  g.tmp.assign(nshard, nullptr);
  g.cnt.assign(nshard, 0);
  g.ready.assign(nshard, nullptr);
  g.done.assign(nshard, nullptr);
  g.tmp_cap = need;
  std::vector<ShardCtx> ctx(nshard);
  int rc = D2G_OK;
  for (int s = 0; s < nshard && !rc; ++s) {
    ctx[s] = {&g, s};
    if (cudaMalloc(&g.tmp[s], need * 8) != cudaSuccess ||
        cudaEventCreateWithFlags(&g.ready[s], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&g.done[s], cudaEventDisableTiming) != cudaSuccess)
      rc = fail(D2G_E_NOMEM, "d2g_badmm_run_shards: exchange buffers");
  }
  std::vector<int> rcs(nshard, D2G_OK);
  std::vector<std::string> msgs(nshard);
  if (!rc) {
    for (int s = 0; s < nshard; ++s) {
      ph[s]->xfn = group_allreduce;
      ph[s]->xctx = &ctx[s];
      ph[s]->xflags = flags;
      ph[s]->shard_pairs = pairs;
    }
    std::vector<std::thread> th;
    for (int s = 0; s < nshard; ++s)
      th.emplace_back([&, s] {
        cudaSetDevice(dev);
        rcs[s] = run_impl(ph[s], opt, c_w[s], c_supp ? c_supp[s] : nullptr, nullptr, nullptr);
        if (rcs[s]) {
          msgs[s] = g_last_error;
          g.fail_all();
        }
      });
    for (auto &t : th) t.join();
    for (int s = 0; s < nshard; ++s) {
      ph[s]->xfn = nullptr;
      ph[s]->xctx = nullptr;
      ph[s]->xflags = 0;
      ph[s]->shard_pairs = false;
    }
    // report the shard that failed first, not the ones stopped by it
    int first = -1;
    for (int s = 0; s < nshard; ++s)
      if (rcs[s] && (first < 0 || (msgs[first].find("failed (3)") != std::string::npos &&
                                   msgs[s].find("failed (3)") == std::string::npos)))
        first = s;
    if (first >= 0) {
      rc = rcs[first];
      set_error("shard " + std::to_string(first) + ": " + msgs[first]);
    }
  }
  for (int s = 0; s < nshard; ++s) {
    if (g.ready[s]) cudaStreamSynchronize(ph[s]->st);
    if (g.tmp[s]) cudaFree(g.tmp[s]);
    if (g.ready[s]) cudaEventDestroy(g.ready[s]);
    if (g.done[s]) cudaEventDestroy(g.done[s]);
  }
  return rc;
}

int d2g_phase_get_tuning(d2g_phase *ph, d2g_tuning *t) {
  if (!ph || !t) return D2G_E_INVAL;
  *t = ph->tune;
  return D2G_OK;
}

int d2g_phase_set_tuning(d2g_phase *ph, const d2g_tuning *t) {
  if (!ph || !t || t->exchange < 0 || t->exchange > 1 || t->stage_costs < 0 || t->stage_costs > 1 ||
      t->ctas_per_sm < 0 || t->ctas_per_sm > 32 || t->cost_gemm < 0 || t->cost_gemm > 1 ||
      t->pairs < 0 || t->pairs > 1 || t->unit_order < 0 || t->unit_order > 1 || t->stage_scales < 0 ||
      t->stage_scales > 1)
    return fail(D2G_E_INVAL, "bad tuning");
  ph->tune = *t;
  return D2G_OK;
}

int d2g_phase_autotune(d2g_phase *ph, const d2g_badmm_opts *opt, const double *c_w,
                       const double *c_supp, d2g_tuning *cands, double *ms, int max_out,
                       int *n_out) {
  if (!ph || !opt || !c_w || max_out < 0) return fail(D2G_E_INVAL, "bad autotune arguments");
  const bool euc = ph->metric == D2_EUCLIDEAN_L2, emb = ph->metric == D2_WORD_EMBED;
  const bool ng = ph->metric == D2_N_GRAM;
  if ((euc || emb) && !c_supp) return fail(D2G_E_INVAL, "c_supp required for this metric");
  if (ng && ph->h_csym.empty())
    return fail(D2G_E_INVAL, "an n-gram phase is tuned from the centroid symbols of its last run");
  if (n_out) *n_out = 0;
  if (ph->path != 0) return D2G_OK;  // the FP64 form has no launch-shape choices
  // candidates: every combination of the choices that apply to this phase
  const d2g_tuning base = ph->tune;
  std::vector<int> ex = {base.exchange}, sc = {0}, cp = {0}, cg = {base.cost_gemm}, pr = {0}, uo = {0};
  if (ph->nwide > 0 && ph->units.nitems > 0) ex = {0, 1};
  if (ph->mode == COST_TABLE && ph->MP >= 16 && ph->MP <= 128) sc = {0, 1};
  if (ph->MP < 256) cp = {0, 1};
  if (emb) cg = {0, 1};
  if (pair_capable(ph, cfg_snapshot())) pr = {1, 0};
  if (!ph->buckets.empty() && ph->buckets[0].cs == 1 && ph->buckets[0].nitems > 1) uo = {0, 1};
  std::vector<d2g_tuning> cand;
  for (int e : ex)
    for (int s2 : sc)
      for (int c : cp)
        for (int g : cg)
          for (int p2 : pr)
            for (int o2 : uo)
              for (int ss : (p2 ? std::vector<int>{1, 0} : std::vector<int>{1}))
                cand.push_back(d2g_tuning{e, s2, c, g, p2, o2, ss});
  // the phase's plans are re-initialised by the trial runs: keep them
  const size_t nz = (size_t)ph->ncols_packed * ph->MP;
  const bool had_plans = ph->plans_valid;
  DBuf<float> zsave;
  if (had_plans) {
    D2G_CUDA(zsave.alloc(nz));
    D2G_CUDA(cudaMemcpyAsync(zsave.p, ph->Z.p, nz * 4, cudaMemcpyDeviceToDevice, ph->st));
  }
  const size_t ncw = (size_t)ph->K * ph->str, ncs = (euc || emb) ? ncw * ph->dim : 0;
  std::vector<double> cw(ncw), cs(ncs);
  const std::vector<int> sym0 = ph->h_csym;
  std::vector<int> sym;
  d2g_badmm_opts o = *opt;
  o.time_budget = 0;
  std::vector<double> t(cand.size(), 1e300);
  int rc = D2G_OK;
  for (size_t i = 0; i < cand.size() && !rc; ++i) {
    ph->tune = cand[i];
    for (int rep = 0; rep < 3 && !rc; ++rep) {  // the first run captures the graph
      std::copy(c_w, c_w + ncw, cw.begin());
      if (ncs) std::copy(c_supp, c_supp + ncs, cs.begin());
      sym = sym0;
      rc = run_impl(ph, &o, cw.data(), ncs ? cs.data() : nullptr, ng ? sym.data() : nullptr, nullptr);
      if (!rc && rep > 0) t[i] = std::min(t[i], ph->stats.total_ms);
    }
  }
  size_t best = 0;
  for (size_t i = 1; i < cand.size(); ++i)
    if (t[i] < t[best]) best = i;
  ph->tune = rc ? base : cand[best];
  if (had_plans) {
    cudaMemcpyAsync(ph->Z.p, zsave.p, nz * 4, cudaMemcpyDeviceToDevice, ph->st);
    cudaStreamSynchronize(ph->st);
  }
  ph->plans_valid = had_plans;
  ph->h_csym = sym0;
  if (rc) return rc;
  tune_cache_put(tune_key(ph), ph->tune);
  for (int i = 0; i < (int)cand.size() && i < max_out; ++i) {
    if (cands) cands[i] = cand[i];
    if (ms) ms[i] = t[i];
  }
  if (n_out) *n_out = (int)cand.size();
  return D2G_OK;
}

int d2g_phase_trace(d2g_phase *ph, double *trace, int cap, int *n) {
  if (!ph || (!trace && cap > 0)) return D2G_E_INVAL;
  const int k = std::min(cap, ph->ntrace);
  for (int i = 0; i < 4 * k; ++i) trace[i] = ph->h_trace[i];
  if (n) *n = ph->ntrace;
  return D2G_OK;
}

void *d2g_phase_stream(d2g_phase *ph) { return ph ? (void *)ph->st : nullptr; }

int d2g_phase_test_wait(d2g_phase *ph, int iter, int unit, double wait_s) {
  if (!ph) return fail(D2G_E_INVAL, "null phase");
  if (!(wait_s >= 0 && wait_s <= 10)) return fail(D2G_E_INVAL, "wait limit outside 0..10 s");
  ph->fault_iter = unit >= 0 ? iter : -1;
  ph->fault_unit = unit >= 0 ? unit : -1;
  ph->wait_ns = (unsigned long long)(wait_s * 1e9);
  return D2G_OK;
}

int d2g_phase_stats(d2g_phase *ph, d2g_run_stats *st) {
  if (!ph || !st) return D2G_E_INVAL;
  *st = ph->stats;
  return D2G_OK;
}

}  // extern "C"
