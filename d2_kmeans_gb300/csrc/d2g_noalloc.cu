// d2g_distmat_noalloc: the ground-cost computation of calculate_distmat for
// callers that cannot allocate GPU memory.
//
// Some callers can't call cudaMalloc: code running inside another runtime's
// memory pool or under its allocator (a framework custom op, a plugin handed
// only pre-allocated device buffers), or code that must not grow the
// process's device footprint while a job is running.  They own their inputs
// and outputs in device memory but have nowhere to put the kernel's working
// data.  This entry point keeps that working data - the p_str prefix sums and
// the column-to-instance map that calculate_distmat builds in freshly
// allocated buffers - in one fixed, file-scope device array instead, so the
// call itself allocates no device memory: no cudaMalloc, no cudaFree, no
// allocating library routine.  (Its error paths do format their message on
// the host heap.)
//
// Limits and sharing rules:
//   * the scratch array is kNoallocScratchBytes (8 MiB) on every GPU that
//     loads libd2g.so, held until the process exits; a call needs
//     8*size + 4*col bytes of it plus 256 and is refused (D2G_E_INVAL) beyond;
//   * every call on a device shares the one array and it keeps the previous
//     call's contents; everything a call reads from it is rewritten by that
//     call first (the status word is cleared at the start), so results never
//     depend on an earlier call;
//   * calls whose GPU work overlaps (different streams or threads, no
//     ordering between them) race on the array: serialise them;
//   * the first call on each device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current); make that first call
//     before any stream capture on the device;
//   * with CUDA's lazy module loading (the default unless
//     CUDA_MODULE_LOADING=EAGER), the array itself comes into existence when
//     this library's device code is first loaded on a device, which can be
//     that same first call: it may then grow the device footprint by 8 MiB or
//     fail for lack of memory.  Callers that must not allocate during a job
//     make the first call at set-up time.
#include <climits>
#include <mutex>

#include "d2g_internal.cuh"

namespace d2g {

constexpr size_t kNoallocScratchBytes = 8u << 20;
constexpr int kNoallocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// status word layout (ints at the start of the scratch array)
enum { NA_BAD_SIZE = 1, NA_BAD_LABEL = 2, NA_BAD_SYM = 4, NA_BAD_COL = 8 };

// Exclusive prefix sum of p_str into cum and validation of the inputs, in
// one block (the sizes this entry point accepts fit one block's sweep).
__global__ void noalloc_prepare(const int *p_str, long long size, long long col, const int *label,
                                int K, const int *sym, int V, int *status, long long *cum) {
  __shared__ long long part[1024];
  __shared__ int flags;
  const int t = threadIdx.x;
  if (t == 0) flags = 0;
  __syncthreads();
  const long long chunk = (size + blockDim.x - 1) / blockDim.x;
  const long long b = (long long)t * chunk, e = min(size, b + chunk);
  long long s = 0;
  int f = 0;
  for (long long i = b; i < e; ++i) {
    const int v = p_str[i];
    if (v < 1) f |= NA_BAD_SIZE;
    s += v > 0 ? v : 0;
    const int l = label[i];
    if (l < 0 || l >= K) f |= NA_BAD_LABEL;
  }
  part[t] = s;
  if (f) atomicOr(&flags, f);
  __syncthreads();
  if (t == 0) {
    long long acc = 0;
    for (int k = 0; k < (int)blockDim.x; ++k) {
      const long long v = part[k];
      part[k] = acc;
      acc += v;
    }
    if (acc != col) flags |= NA_BAD_COL;
  }
  __syncthreads();
  long long acc = part[t];
  for (long long i = b; i < e; ++i) {
    cum[i] = acc;
    acc += p_str[i] > 0 ? p_str[i] : 0;
  }
  if (sym) {
    int g = 0;
    for (long long j = t; j < col; j += blockDim.x)
      if (sym[j] >= V) g = NA_BAD_SYM;
    if (g) atomicOr(&flags, g);
  }
  __syncthreads();
  if (t == 0) status[0] = flags;
}

__global__ void noalloc_fill(const int *p_str, const long long *cum, long long size, long long col,
                             int *col_inst) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < size;
       i += (long long)gridDim.x * blockDim.x)
    for (int j = 0; j < p_str[i]; ++j) {
      const long long c = cum[i] + j;
      if (c < col) col_inst[c] = (int)i;
    }
}

static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[kNoallocMaxDevices];

// Once per device, with that device current: the array's device address.
static int noalloc_scratch(void **out) {
  int dev = 0;
  D2G_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoallocMaxDevices) {
    set_error("d2g_distmat_noalloc: device index beyond the per-device table");
    return D2G_E_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    D2G_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return D2G_OK;
}

}  // namespace d2g

using namespace d2g;

extern "C" int d2g_distmat_noalloc(int metric_type, int dim, int str, size_t size, size_t col,
                                   const int *p_str, const double *p_supp, const int *p_supp_sym,
                                   const double *vocab_vec, int vocab_size, const int *label,
                                   int num_of_labels, const double *c_supp, double *C,
                                   void *stream) {
  if (metric_type != D2_EUCLIDEAN_L2 && metric_type != D2_WORD_EMBED) {
    set_error("d2g_distmat_noalloc: Euclidean and word-embedding phases only");
    return D2G_E_UNSUPPORTED;
  }
  if (dim < 1 || str < 1 || size == 0 || col == 0 || num_of_labels < 1 || !p_str || !label ||
      !c_supp || !C || (metric_type == D2_EUCLIDEAN_L2 && !p_supp) ||
      (metric_type == D2_WORD_EMBED && (!p_supp_sym || !vocab_vec || vocab_size < 1))) {
    set_error("d2g_distmat_noalloc: missing or invalid argument");
    return D2G_E_INVAL;
  }
  // refuse sizes whose scratch need would not even fit a size_t before
  // computing it (8 * size or 4 * col could wrap around)
  if (size > kNoallocScratchBytes / 8 || col > kNoallocScratchBytes / 4 || size > (size_t)INT_MAX) {
    set_error("d2g_distmat_noalloc: size or col beyond the 8 MiB fixed array");
    return D2G_E_INVAL;
  }
  const size_t need = 256 + 8 * size + 4 * col;
  if (need > kNoallocScratchBytes) {
    set_error("d2g_distmat_noalloc: needs 8*size + 4*col + 256 = " + std::to_string(need) +
              " bytes of scratch, more than the 8 MiB fixed array");
    return D2G_E_INVAL;
  }
  void *base = nullptr;
  int rc = noalloc_scratch(&base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char *sc = (unsigned char *)base;
  int *status = (int *)sc;
  long long *cum = (long long *)(sc + 256);
  int *col_inst = (int *)(sc + 256 + 8 * size);

  D2G_CUDA(cudaMemsetAsync(status, 0, sizeof(int), st));
  noalloc_prepare<<<1, 1024, 0, st>>>(p_str, (long long)size, (long long)col, label, num_of_labels,
                                      metric_type == D2_WORD_EMBED ? p_supp_sym : nullptr,
                                      vocab_size, status, cum);
  D2G_CUDA(cudaGetLastError());
  int h_status = 0;
  D2G_CUDA(cudaMemcpyAsync(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost, st));
  D2G_CUDA(cudaStreamSynchronize(st));
  if (h_status) {
    set_error("d2g_distmat_noalloc: invalid input (status " + std::to_string(h_status) +
              ": 1 support size < 1, 2 label out of range, 4 id >= vocab_size, 8 col != sum p_str)");
    return D2G_E_INVAL;
  }
  const int nb = (int)std::min<size_t>((size + 255) / 256, 152 * 8);
  noalloc_fill<<<nb, 256, 0, st>>>(p_str, cum, (long long)size, (long long)col, col_inst);
  D2G_CUDA(cudaGetLastError());

  PlainArgs a{};
  a.C = C;
  a.supp = p_supp;
  a.vocab = vocab_vec;
  a.sym = p_supp_sym;
  a.col_inst = col_inst;
  a.label = label;
  a.cum = cum;
  a.cs64 = const_cast<double *>(c_supp);
  a.col = (long long)col;
  a.nent = (long long)col * str;
  a.size = (int)size;
  a.str = str;
  a.dim = dim;
  a.metric = metric_type;
  a.vocab_size = vocab_size;
  a.iter = -1;  // unscaled costs, as calculate_distmat returns them
  D2G_CUDA(plain_cost(a, st));
  return D2G_OK;
}
