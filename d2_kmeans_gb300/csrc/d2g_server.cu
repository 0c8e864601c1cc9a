// Serving loop: continuous batching of fixed-centroid transport solves.
//
// Centroids (weights and supports) stay resident in HBM.  d2g_server_submit
// admits a query distribution if the HBM budget and the queue bound allow it
// (its device footprint counts against the budget from admission until its
// result is collected), copies it into a pinned staging area and returns a
// ticket.  A worker thread keeps up to kSlots batches in flight, each on its
// own stream: whenever a slot is free it takes every queued request that fits
// (plan-entry bound per batch), uploads them, launches the solve kernels and
// moves on; when a batch's event completes it reads the costs back, takes the
// argmin per request and stamps the latency.  Requests that arrive while
// batches are on the GPU go into the next free slot, so work from successive
// batches overlaps on the device.  A request's result does not depend on the
// batch it ran in: its plans, its rho and its reductions are its own.
#include <chrono>
#include <condition_variable>
#include <cmath>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "d2g_internal.cuh"

namespace d2g {



namespace {

constexpr int kSlots = 2;
constexpr int kMaxQuerySupport = 512;

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  long long ticket = 0;
  int mq = 0;
  std::vector<float> w, supp;
  double rho = 0;
  double t_submit = 0, t_done = 0;
  size_t bytes = 0;
  int state = 0;  // 0 queued, 1 in flight, 2 done
  int label = -1;
  std::vector<double> costs;
};

struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  bool busy = false;
  std::vector<Request *> reqs;
  // device
  float *q_w = nullptr, *q_supp = nullptr, *cost = nullptr;
  int *err = nullptr, *h_err = nullptr;  // cluster exchange wait ran out (device, pinned copy)
  int4 *items = nullptr;
  float4 *rq = nullptr;
  size_t cap_cols = 0, cap_items = 0, cap_reqs = 0;
  // pinned host
  float *h_w = nullptr, *h_supp = nullptr, *h_cost = nullptr;
  int4 *h_items = nullptr;
  float4 *h_rq = nullptr;
};

}  // namespace
}  // namespace d2g

using namespace d2g;

struct d2g_server {
  int K = 0, m = 0, MP = 0, dim = 0, iters = 0, device = 0;
  double rho_coeff = 2.0;
  size_t budget = 0, inflight_bytes = 0;
  int max_queue = 0;
  long long max_batch_entries = 0;
  float *c_w32 = nullptr, *c_supp32 = nullptr;
  double c_sumsq = 0;            // sum over all centroid supports of |c|^2
  std::vector<double> c_sum;     // sum over all centroid supports of c
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Request *> queue;
  std::unordered_map<long long, Request *> table;
  long long next_ticket = 1;
  bool stop = false;
  int error = 0;
  std::string error_msg;
  Slot slots[kSlots];
  std::thread worker;
  long long completed = 0;
  std::condition_variable done_cv;
};

namespace d2g {
namespace {

int slot_reserve(d2g_server *s, Slot &sl, size_t cols, size_t nitems, size_t nreq) {
  if (!sl.err) {
    D2G_CUDA(cudaMalloc(&sl.err, sizeof(int)));
    D2G_CUDA(cudaMallocHost(&sl.h_err, sizeof(int)));
    D2G_CUDA(cudaMemset(sl.err, 0, sizeof(int)));
    *sl.h_err = 0;
  }
  auto grow = [](size_t want, size_t have) { return want <= have ? have : std::max(want, have * 2); };
  if (cols > sl.cap_cols) {
    const size_t c = grow(cols, sl.cap_cols);
    cudaFree(sl.q_w);
    cudaFree(sl.q_supp);
    cudaFreeHost(sl.h_w);
    cudaFreeHost(sl.h_supp);
    D2G_CUDA(cudaMalloc(&sl.q_w, c * 4));
    D2G_CUDA(cudaMalloc(&sl.q_supp, c * s->dim * 4));
    D2G_CUDA(cudaMallocHost(&sl.h_w, c * 4));
    D2G_CUDA(cudaMallocHost(&sl.h_supp, c * s->dim * 4));
    sl.cap_cols = c;
  }
  if (nitems > sl.cap_items) {
    const size_t c = grow(nitems, sl.cap_items);
    cudaFree(sl.items);
    cudaFreeHost(sl.h_items);
    D2G_CUDA(cudaMalloc(&sl.items, c * sizeof(int4)));
    D2G_CUDA(cudaMallocHost(&sl.h_items, c * sizeof(int4)));
    sl.cap_items = c;
  }
  if (nreq > sl.cap_reqs) {
    const size_t c = grow(nreq, sl.cap_reqs);
    cudaFree(sl.rq);
    cudaFree(sl.cost);
    cudaFreeHost(sl.h_rq);
    cudaFreeHost(sl.h_cost);
    D2G_CUDA(cudaMalloc(&sl.rq, c * sizeof(float4)));
    D2G_CUDA(cudaMalloc(&sl.cost, c * s->K * 4));
    D2G_CUDA(cudaMallocHost(&sl.h_rq, c * sizeof(float4)));
    D2G_CUDA(cudaMallocHost(&sl.h_cost, c * s->K * 4));
    sl.cap_reqs = c;
  }
  return D2G_OK;
}

// items of one request: several plans per CTA when they fit, else one plan
// per cluster of exactly ceil(ng / G) CTAs (2..8; any cluster size up to 8
// is a valid launch shape, so no slice of a wide plan is empty)
void request_items(int K, int G, int mq, int req, std::vector<int4> *by_cs) {
  const int ng = (mq + 3) / 4;
  if (ng <= G) {
    const int ppc = G / ng;
    for (int l = 0; l < K; l += ppc) by_cs[1].push_back(make_int4(req, l, std::min(ppc, K - l), ng));
  } else {
    const int cs = (ng + G - 1) / G;
    for (int l = 0; l < K; ++l) by_cs[cs].push_back(make_int4(req, l, 1, ng));
  }
}

int launch_batch(d2g_server *s, Slot &sl) {
  size_t cols = 0;
  for (Request *r : sl.reqs) cols += r->mq;
  std::vector<int4> by_cs[9];  // by cluster size 1..8
  const int G = serve_groups_per_cta(s->MP);
  for (size_t i = 0; i < sl.reqs.size(); ++i) request_items(s->K, G, sl.reqs[i]->mq, (int)i, by_cs);
  size_t nitems = 0;
  for (auto &v : by_cs) nitems += v.size();
  int rc = slot_reserve(s, sl, cols, nitems, sl.reqs.size());
  if (rc) return rc;
  size_t off = 0;
  for (size_t i = 0; i < sl.reqs.size(); ++i) {
    Request *r = sl.reqs[i];
    memcpy(sl.h_w + off, r->w.data(), r->mq * 4);
    memcpy(sl.h_supp + off * s->dim, r->supp.data(), (size_t)r->mq * s->dim * 4);
    float4 q;
    const int o = (int)off, mq = r->mq;
    memcpy(&q.x, &o, 4);
    memcpy(&q.y, &mq, 4);
    q.z = (float)(1.4426950408889634 / r->rho);  // log2(e)/rho
    q.w = 0.f;
    sl.h_rq[i] = q;
    off += r->mq;
  }
  size_t io = 0;
  for (auto &v : by_cs) {
    memcpy(sl.h_items + io, v.data(), v.size() * sizeof(int4));
    io += v.size();
  }
  D2G_CUDA(cudaMemcpyAsync(sl.q_w, sl.h_w, cols * 4, cudaMemcpyHostToDevice, sl.st));
  D2G_CUDA(cudaMemcpyAsync(sl.q_supp, sl.h_supp, cols * s->dim * 4, cudaMemcpyHostToDevice, sl.st));
  D2G_CUDA(cudaMemcpyAsync(sl.rq, sl.h_rq, sl.reqs.size() * sizeof(float4), cudaMemcpyHostToDevice, sl.st));
  D2G_CUDA(cudaMemcpyAsync(sl.items, sl.h_items, nitems * sizeof(int4), cudaMemcpyHostToDevice, sl.st));
  ServeArgs a{};
  a.q_w = sl.q_w;
  a.q_supp = sl.q_supp;
  a.c_w32 = s->c_w32;
  a.c_supp32 = s->c_supp32;
  a.reqs = sl.rq;
  a.cost_out = sl.cost;
  a.err = sl.err;
  a.K = s->K;
  a.m = s->m;
  a.dim = s->dim;
  a.iters = s->iters;
  io = 0;
  for (int cs = 1; cs <= 8; ++cs) {
    a.items = sl.items + io;
    a.cs = cs;
    D2G_CUDA(launch_serve(s->MP, a, (int)by_cs[cs].size(), sl.st));
    io += by_cs[cs].size();
  }
  D2G_CUDA(cudaMemcpyAsync(sl.h_cost, sl.cost, sl.reqs.size() * s->K * 4, cudaMemcpyDeviceToHost, sl.st));
  D2G_CUDA(cudaMemcpyAsync(sl.h_err, sl.err, sizeof(int), cudaMemcpyDeviceToHost, sl.st));
  D2G_CUDA(cudaEventRecord(sl.ev, sl.st));
  sl.busy = true;
  return D2G_OK;
}

void finish_batch(d2g_server *s, Slot &sl) {
  const double t = now_ms();
  std::lock_guard<std::mutex> lk(s->mu);
  if (*sl.h_err && !s->error) {
    s->error = D2G_E_CUDA;
    s->error_msg = "serving: a cluster exchange wait ran out";
  }
  for (size_t i = 0; i < sl.reqs.size(); ++i) {
    Request *r = sl.reqs[i];
    r->costs.resize(s->K);
    int best = 0;
    for (int l = 0; l < s->K; ++l) {
      r->costs[l] = sl.h_cost[i * s->K + l];
      if (r->costs[l] < r->costs[best]) best = l;
    }
    r->label = best;
    r->t_done = t;
    r->state = 2;
    ++s->completed;
  }
  sl.reqs.clear();
  sl.busy = false;
  s->done_cv.notify_all();
}

void worker_loop(d2g_server *s) {
  cudaSetDevice(s->device);
  for (;;) {
    bool idle = true;
    for (Slot &sl : s->slots) {
      if (sl.busy && cudaEventQuery(sl.ev) == cudaSuccess) {
        finish_batch(s, sl);
        idle = false;
      }
    }
    for (Slot &sl : s->slots) {
      if (sl.busy) continue;
      {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return;
        long long ent = 0;
        while (!s->queue.empty()) {
          Request *r = s->queue.front();
          const long long e = (long long)s->K * s->m * r->mq;
          if (!sl.reqs.empty() && ent + e > s->max_batch_entries) break;
          s->queue.pop_front();
          r->state = 1;
          sl.reqs.push_back(r);
          ent += e;
        }
      }
      if (sl.reqs.empty()) continue;
      int rc = launch_batch(s, sl);
      if (rc) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->error = rc;
        s->error_msg = d2g_last_error();
        s->stop = true;
        s->done_cv.notify_all();
        return;
      }
      idle = false;
    }
    if (idle) {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->stop) return;
      bool any_busy = false;
      for (Slot &sl : s->slots) any_busy |= sl.busy;
      if (any_busy)
        s->cv.wait_for(lk, std::chrono::microseconds(20));
      else
        s->cv.wait_for(lk, std::chrono::milliseconds(5), [s] { return s->stop || !s->queue.empty(); });
    }
  }
}

}  // namespace
}  // namespace d2g

extern "C" {

int d2g_server_create(const d2g_server_desc *d, d2g_server **out) {
  if (!d || !out || d->num_of_labels < 1 || d->str < 1 || d->str > 128 || d->dim < 1 ||
      !d->c_w || !d->c_supp || d->iters < 1 || !(d->rhoCoeff > 0)) {
    d2g::set_error("d2g_server_create: invalid description (str must be 1..128)");
    return D2G_E_INVAL;
  }
  d2g_server *s = new d2g_server();
  s->K = d->num_of_labels;
  s->m = d->str;
  s->MP = d->str <= 16 ? 16 : d->str <= 32 ? 32 : d->str <= 64 ? 64 : 128;
  // the widest query must fit an 8-CTA cluster
  if ((kMaxQuerySupport + 3) / 4 > 8 * serve_groups_per_cta(s->MP)) {
    delete s;
    d2g::set_error("d2g_server_create: str too large for 512-support queries");
    return D2G_E_UNSUPPORTED;
  }
  cudaGetDevice(&s->device);
  s->dim = d->dim;
  s->iters = d->iters;
  s->rho_coeff = d->rhoCoeff;
  s->budget = d->hbm_budget_bytes ? d->hbm_budget_bytes : ((size_t)1 << 30);
  s->max_queue = d->max_queue > 0 ? d->max_queue : 4096;
  s->max_batch_entries = d->max_batch_entries > 0 ? d->max_batch_entries : (64LL << 20);
  const size_t K = s->K, MP = s->MP, dim = s->dim;
  std::vector<float> cw(K * MP, 0.f), cs(K * MP * dim, 0.f);
  s->c_sum.assign(dim, 0.0);
  for (size_t l = 0; l < K; ++l)
    for (int k = 0; k < s->m; ++k) {
      cw[l * MP + k] = (float)d->c_w[l * s->m + k];
      for (size_t t = 0; t < dim; ++t) {
        const double v = d->c_supp[(l * s->m + k) * dim + t];
        cs[(l * MP + k) * dim + t] = (float)v;
        s->c_sum[t] += v;
        s->c_sumsq += v * v;
      }
    }
  if (cudaMalloc(&s->c_w32, cw.size() * 4) != cudaSuccess ||
      cudaMalloc(&s->c_supp32, cs.size() * 4) != cudaSuccess ||
      cudaMemcpy(s->c_w32, cw.data(), cw.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(s->c_supp32, cs.data(), cs.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
    d2g::set_error("d2g_server_create: centroid upload failed");
    cudaFree(s->c_w32);
    cudaFree(s->c_supp32);
    delete s;
    return D2G_E_CUDA;
  }
  for (Slot &sl : s->slots) {
    cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming);
  }
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return D2G_OK;
}

int d2g_server_destroy(d2g_server *s) {
  if (!s) return D2G_E_INVAL;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (Slot &sl : s->slots) {
    if (sl.st) cudaStreamSynchronize(sl.st);
    cudaFree(sl.q_w);
    cudaFree(sl.q_supp);
    cudaFree(sl.cost);
    cudaFree(sl.items);
    cudaFree(sl.rq);
    cudaFreeHost(sl.h_w);
    cudaFreeHost(sl.h_supp);
    cudaFreeHost(sl.h_cost);
    cudaFreeHost(sl.h_items);
    cudaFreeHost(sl.h_rq);
    cudaFree(sl.err);
    cudaFreeHost(sl.h_err);
    if (sl.ev) cudaEventDestroy(sl.ev);
    if (sl.st) cudaStreamDestroy(sl.st);
  }
  // every request not yet collected (queued, in flight or done) is in the
  // table exactly once; the queue and the slots only borrow those pointers
  for (auto &kv : s->table) delete kv.second;
  s->table.clear();
  s->queue.clear();
  cudaFree(s->c_w32);
  cudaFree(s->c_supp32);
  delete s;
  return D2G_OK;
}

int d2g_server_submit(d2g_server *s, int m_q, const double *w_q, const double *supp_q,
                      long long *ticket) {
  if (!s || m_q < 1 || m_q > kMaxQuerySupport || !w_q || !supp_q || !ticket) {
    d2g::set_error("d2g_server_submit: invalid request (m_q must be 1..512)");
    return D2G_E_INVAL;
  }
  const double t0 = now_ms();
  const size_t bytes = (size_t)m_q * (s->dim + 1) * 4 + (size_t)s->K * 4 + 64;
  // rho = rhoCoeff * mean over the request's K*m*m_q costs, from
  // sum |c - q|^2 = m_q*sum|c|^2 + K*m*sum|q|^2 - 2 (sum c).(sum q), in FP64
  double qsq = 0;
  std::vector<double> qsum(s->dim, 0.0);
  for (int j = 0; j < m_q; ++j)
    for (int t = 0; t < s->dim; ++t) {
      const double v = supp_q[(size_t)j * s->dim + t];
      qsq += v * v;
      qsum[t] += v;
    }
  double cross = 0;
  for (int t = 0; t < s->dim; ++t) cross += s->c_sum[t] * qsum[t];
  const double nent = (double)s->K * s->m * m_q;
  const double total = m_q * s->c_sumsq + (double)s->K * s->m * qsq - 2.0 * cross;
  Request *r = new Request();
  r->mq = m_q;
  r->w.assign(w_q, w_q + m_q);
  r->supp.resize((size_t)m_q * s->dim);
  for (size_t i = 0; i < r->supp.size(); ++i) r->supp[i] = (float)supp_q[i];
  r->rho = s->rho_coeff * total / nent;
  r->bytes = bytes;
  r->t_submit = t0;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->error) {
      delete r;
      d2g::set_error("d2g_server_submit: server stopped after an error: " + s->error_msg);
      return s->error;
    }
    if ((int)s->queue.size() >= s->max_queue || s->inflight_bytes + bytes > s->budget) {
      delete r;
      d2g::set_error("d2g_server_submit: refused by admission control (queue or HBM budget)");
      return D2G_E_ADMISSION;
    }
    if (!(r->rho > 0) || !std::isfinite(r->rho)) {
      delete r;
      d2g::set_error("d2g_server_submit: degenerate request (zero ground cost)");
      return D2G_E_INVAL;
    }
    r->ticket = s->next_ticket++;
    s->inflight_bytes += bytes;
    s->table[r->ticket] = r;
    s->queue.push_back(r);
  }
  s->cv.notify_one();
  *ticket = r->ticket;
  return D2G_OK;
}

int d2g_server_progress(d2g_server *s, int wait) {
  if (!s) return D2G_E_INVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  const long long before = s->completed;
  if (wait) {
    s->done_cv.wait_for(lk, std::chrono::seconds(30),
                        [&] { return s->completed > before || s->error || s->table.empty(); });
  }
  if (s->error) {
    d2g::set_error(s->error_msg);
    return s->error;
  }
  return (int)(s->completed - before);
}

int d2g_server_result(d2g_server *s, long long ticket, int *label, double *costs, double *latency_ms) {
  if (!s) return D2G_E_INVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->table.find(ticket);
  if (it == s->table.end()) {
    d2g::set_error("d2g_server_result: unknown ticket");
    return D2G_E_NOTFOUND;
  }
  Request *r = it->second;
  if (r->state != 2) return 0;
  if (label) *label = r->label;
  if (costs) memcpy(costs, r->costs.data(), s->K * sizeof(double));
  if (latency_ms) *latency_ms = r->t_done - r->t_submit;
  s->inflight_bytes -= r->bytes;
  s->table.erase(it);
  delete r;
  return 1;
}

}  // extern "C"
