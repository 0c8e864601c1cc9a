// Reading the reference's d2 text formats into its `mph` structure.
//
// d2g_read has the signature and the result of d2_read
// (src/d2/clustering_io.c:14-201, declared include/d2/clustering.h:144):
// the same files (.d2 multi-phase Euclidean, dense histograms with a .histN
// cost file, .d2s symbolic supports with a .vocabN embedding file, sparse
// histograms), the same per-object checks and weight renormalisation
// (w / sum(w), summed in file order), the same id shift (ids start at one;
// id 0 becomes the vocabulary's last row), the same growth of the caller's
// arrays when the preallocated capacity is exceeded, and the same
// end-of-file rule (size drops to the objects read).  Differences: malformed
// or out-of-range input (including a file that ends inside an object) returns
// D2G_E_INVAL instead of asserting or reading on, and the per-rank file names
// of the MPI build are not used.
//
// The reference reads token by token with fscanf.  Here the file is read in
// one piece and parsed in three passes: token starts are found in parallel
// (one chunk of bytes per thread; a token belongs to the chunk holding its
// first byte), one sequential pass over the small integers (dimension,
// support size) lays out every object, and the numbers are converted in
// parallel with std::from_chars (correctly rounded like strtod; strtod itself
// is used where from_chars reports a value out of range, e.g. subnormals)
// straight into the caller's arrays.
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "d2g_internal.cuh"

namespace d2g {
namespace {

struct Text {
  std::vector<char> buf;     // file bytes + a terminating 0
  size_t len = 0;
  std::vector<size_t> tok;   // start offset of every token
};

inline bool is_ws(char c) {
  return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\f' || c == '\v';
}

int io_threads(size_t bytes) {
  int t = (int)std::thread::hardware_concurrency();
  if (const char *e = getenv("D2G_IO_THREADS")) t = atoi(e);
  t = std::max(1, std::min(t, 64));
  const size_t per = (size_t)1 << 20;  // at least 1 MB per thread
  return (int)std::max<size_t>(1, std::min<size_t>((size_t)t, (bytes + per - 1) / per));
}

template <typename F>
void parallel_for(int nt, F f) {
  if (nt <= 1) {
    f(0);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) th.emplace_back(f, t);
  f(0);
  for (auto &x : th) x.join();
}

bool load_text(const char *path, Text &tx) {
  FILE *f = fopen(path, "rb");
  if (!f) return false;
  // one read of the whole file (its size from the end offset; a stream that
  // cannot seek is read in pieces)
  std::vector<char> buf;
  long sz = -1;
  if (fseek(f, 0, SEEK_END) == 0) sz = ftell(f);
  if (sz >= 0 && fseek(f, 0, SEEK_SET) == 0) {
    buf.resize((size_t)sz + 1);
    const size_t r = fread(buf.data(), 1, (size_t)sz, f);
    buf.resize(r);
  } else {
    char tmp[1 << 16];
    size_t r;
    while ((r = fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + r);
  }
  fclose(f);
  tx.len = buf.size();
  buf.push_back(0);
  tx.buf.swap(buf);
  // token starts, in parallel over byte chunks
  const size_t n = tx.len;
  const int nt = io_threads(n);
  std::vector<std::vector<size_t>> part(nt);
  parallel_for(nt, [&](int t) {
    const size_t b = n * t / nt, e = n * (t + 1) / nt;
    const char *p = tx.buf.data();
    auto &v = part[t];
    for (size_t i = b; i < e; ++i)
      if (!is_ws(p[i]) && (i == 0 || is_ws(p[i - 1]))) v.push_back(i);
  });
  size_t tot = 0;
  for (auto &v : part) tot += v.size();
  tx.tok.clear();
  tx.tok.reserve(tot);
  for (auto &v : part) tx.tok.insert(tx.tok.end(), v.begin(), v.end());
  return true;
}

inline const char *tok_end(const Text &tx, size_t k) {
  const char *p = tx.buf.data() + tx.tok[k];
  while (*p && !is_ws(*p)) ++p;
  return p;
}

inline bool parse_int(const Text &tx, size_t k, int &v) {
  const char *p = tx.buf.data() + tx.tok[k], *e = tok_end(tx, k);
  if (p < e && *p == '+') ++p;
  auto r = std::from_chars(p, e, v);
  return r.ec == std::errc() && r.ptr == e;
}

inline bool parse_dbl(const Text &tx, size_t k, double &v) {
  const char *p = tx.buf.data() + tx.tok[k], *e = tok_end(tx, k);
  const char *q = (p < e && *p == '+') ? p + 1 : p;
  auto r = std::from_chars(q, e, v);
  if (r.ec == std::errc() && r.ptr == e) return true;
  if (r.ec == std::errc::result_out_of_range) {  // overflow / subnormal: strtod's value
    char *end = nullptr;
    v = strtod(p, &end);
    return end == e;
  }
  return false;
}

// numbers [k0, k0 + cnt) of a text into out[], in parallel
bool parse_dbl_range(const Text &tx, size_t k0, size_t cnt, double *out) {
  const int nt = io_threads(cnt * 8);
  std::vector<char> ok(nt, 1);
  parallel_for(nt, [&](int t) {
    const size_t b = cnt * t / nt, e = cnt * (t + 1) / nt;
    for (size_t i = b; i < e; ++i)
      if (!parse_dbl(tx, k0 + i, out[i])) {
        ok[t] = 0;
        return;
      }
  });
  for (char c : ok)
    if (!c) return false;
  return true;
}

int bad(const std::string &m) {
  set_error("d2g_read: " + m);
  return D2G_E_INVAL;
}

template <typename T>
bool grow(T *&p, size_t want) {
  T *q = (T *)realloc(p, want * sizeof(T));
  if (!q) return false;
  p = q;
  return true;
}

// the .histN / .vocabN file of a phase (src/d2/clustering_io.c:55-89)
int read_meta(const char *filename, const char *meta_filename, int s_ph, int n, sph *ph) {
  const bool hist = ph->metric_type == D2_HISTOGRAM || ph->metric_type == D2_SPARSE_HISTOGRAM;
  std::string path;
  if (meta_filename && s_ph == 1)
    path = meta_filename;
  else
    path = std::string(filename) + (hist ? ".hist" : ".vocab") + std::to_string(n);
  Text tx;
  if (!load_text(path.c_str(), tx)) return bad("cannot open " + path);
  if (hist) {
    int str = 0;
    if (tx.tok.empty() || !parse_int(tx, 0, str) || str <= 0) return bad(path + ": bad size");
    if (tx.tok.size() < 1 + (size_t)str * str) return bad(path + ": too few costs");
    double *dm = (double *)malloc((size_t)str * str * sizeof(double));
    if (!dm) return D2G_E_NOMEM;
    if (!parse_dbl_range(tx, 1, (size_t)str * str, dm)) {
      free(dm);
      return bad(path + ": bad number");
    }
    ph->dist_mat = dm;
    ph->vocab_size = str;
  } else {
    int dim = 0, V = 0;
    if (tx.tok.size() < 2 || !parse_int(tx, 0, dim) || !parse_int(tx, 1, V) || V <= 0)
      return bad(path + ": bad header");
    if (dim != ph->dim) return bad(path + ": dimension differs from the phase's");
    if (tx.tok.size() < 2 + (size_t)V * dim) return bad(path + ": too few vocabulary values");
    double *vv = (double *)malloc((size_t)V * dim * sizeof(double));
    if (!vv) return D2G_E_NOMEM;
    if (!parse_dbl_range(tx, 2, (size_t)V * dim, vv)) {
      free(vv);
      return bad(path + ": bad number");
    }
    ph->vocab_vec = vv;
    ph->vocab_size = V;
  }
  ph->is_meta_allocated = 1;
  return D2G_OK;
}

}  // namespace
}  // namespace d2g

using namespace d2g;

extern "C" {

int d2g_read(const char *filename, const char *meta_filename, mph *p_data) {
  if (!filename || !p_data || !p_data->ph || p_data->s_ph < 1) return bad("invalid arguments");
  const int s_ph = p_data->s_ph;
  size_t size = p_data->size;
  for (int n = 0; n < s_ph; ++n) {
    sph *ph = p_data->ph + n;
    ph->col = 0;
    const int mt = ph->metric_type;
    if (mt == D2_HISTOGRAM || mt == D2_SPARSE_HISTOGRAM || mt == D2_WORD_EMBED) {
      int rc = read_meta(filename, meta_filename, s_ph, n, ph);
      if (rc) return rc;
    } else if (mt != D2_EUCLIDEAN_L2) {
      return bad("metric type " + std::to_string(mt) + " has no d2 text format");
    }
  }
  Text tx;
  if (!load_text(filename, tx)) return bad(std::string("cannot open ") + filename);

  // layout pass: per phase, the token of each recorded object's first weight
  // and its first column (objects whose support size is 0 are skipped, as in
  // the reference, and leave their slot for the next object)
  std::vector<std::vector<size_t>> otok(s_ph), ocol(s_ph);
  std::vector<std::vector<int>> ostr(s_ph);
  std::vector<size_t> col(s_ph, 0);
  size_t k = 0, i = 0;
  const size_t ntok = tx.tok.size();
  for (i = 0; i < size; ++i) {
    bool eof = false;
    for (int n = 0; n < s_ph; ++n) {
      sph *ph = p_data->ph + n;
      int dim = 0, str = 0;
      if (k >= ntok) {  // the reference stops with a warning (size = objects read)
        if (n > 0) return bad("object " + std::to_string(i) + " is cut off after phase " +
                              std::to_string(n - 1));
        eof = true;
        break;
      }
      if (!parse_int(tx, k, dim)) return bad("object " + std::to_string(i) + ": bad dimension");
      if (dim != ph->dim)
        return bad("object " + std::to_string(i) + " phase " + std::to_string(n) + ": dimension " +
                   std::to_string(dim) + ", expected " + std::to_string(ph->dim));
      if (k + 1 >= ntok || !parse_int(tx, k + 1, str) || str < 0)
        return bad("object " + std::to_string(i) + ": bad support size");
      k += 2;
      if (str == 0) continue;
      const int mt = ph->metric_type;
      const size_t nsup = mt == D2_EUCLIDEAN_L2 ? (size_t)str * dim
                                                : (mt == D2_HISTOGRAM ? 0 : (size_t)str);
      if (k + str + nsup > ntok) return bad("object " + std::to_string(i) + ": truncated");
      otok[n].push_back(k);
      ocol[n].push_back(col[n]);
      ostr[n].push_back(str);
      col[n] += str;
      k += str + nsup;
    }
    if (eof) break;
  }
  if (i < size) {
    fprintf(stderr, "d2g_read warning: only read %zu d2!\n", i);
    p_data->size = size = i;
  }
  // capacity of the caller's arrays (allocated by d2_allocate)
  for (int n = 0; n < s_ph; ++n) {
    sph *ph = p_data->ph + n;
    if (ostr[n].size() > size) return bad("more objects than the preallocated size");
    if (col[n] > ph->max_col) {
      const size_t cap = std::max(col[n], 2 * ph->max_col);
      const int mt = ph->metric_type;
      if (!grow(ph->p_w, cap)) return D2G_E_NOMEM;
      if (mt == D2_EUCLIDEAN_L2 && !grow(ph->p_supp, cap * ph->dim)) return D2G_E_NOMEM;
      if ((mt == D2_WORD_EMBED || mt == D2_SPARSE_HISTOGRAM) && !grow(ph->p_supp_sym, cap))
        return D2G_E_NOMEM;
      ph->max_col = cap;
    }
  }
  // conversion pass, objects split over threads
  for (int n = 0; n < s_ph; ++n) {
    sph *ph = p_data->ph + n;
    const int mt = ph->metric_type, dim = ph->dim;
    const size_t nobj = ostr[n].size();
    const int nt = io_threads(col[n] * (mt == D2_EUCLIDEAN_L2 ? dim + 1 : 2) * 8);
    std::vector<std::string> err(nt);
    parallel_for(nt, [&](int t) {
      const size_t b = nobj * t / nt, e = nobj * (t + 1) / nt;
      for (size_t o = b; o < e; ++o) {
        const int str = ostr[n][o];
        const size_t kw = otok[n][o], c0 = ocol[n][o];
        double *w = ph->p_w + c0, wsum = 0.0;
        for (int j = 0; j < str; ++j) {
          if (!parse_dbl(tx, kw + j, w[j])) {
            err[t] = "bad weight";
            return;
          }
          // unless dense histograms, every support point needs a positive weight
          if (mt != D2_HISTOGRAM && !(w[j] > 1e-9)) {
            err[t] = "weight not above 1e-9";
            return;
          }
          wsum += w[j];
        }
        for (int j = 0; j < str; ++j) w[j] /= wsum;
        const size_t ks = kw + str;
        if (mt == D2_EUCLIDEAN_L2) {
          double *s = ph->p_supp + c0 * dim;
          for (size_t j = 0; j < (size_t)str * dim; ++j)
            if (!parse_dbl(tx, ks + j, s[j])) {
              err[t] = "bad support value";
              return;
            }
        } else if (mt == D2_WORD_EMBED || mt == D2_SPARSE_HISTOGRAM) {
          int *s = ph->p_supp_sym + c0;
          for (int j = 0; j < str; ++j) {
            int id = 0;
            if (!parse_int(tx, ks + j, id)) {
              err[t] = "bad support id";
              return;
            }
            id -= 1;  // ids start at one; id 0 is the vocabulary's last (zero) row
            s[j] = id < 0 ? ph->vocab_size - 1 : id;
          }
        }
      }
    });
    for (auto &m : err)
      if (!m.empty()) return bad("phase " + std::to_string(n) + ": " + m);
    for (size_t o = 0; o < nobj; ++o) {
      ph->p_str[o] = ostr[n][o];
      if (ostr[n][o] > ph->max_str) ph->max_str = ostr[n][o];
    }
    ph->col = col[n];
  }
  for (int n = 0; n < s_ph; ++n) {
    sph *ph = p_data->ph + n;
    if (ph->col > 0) {
      ph->p_str_cum[0] = 0;
      for (size_t o = 1; o < size; ++o) ph->p_str_cum[o] = ph->p_str_cum[o - 1] + ph->p_str[o - 1];
      if (ph->metric_type == D2_SPARSE_HISTOGRAM) ph->str = ph->vocab_size;  // centroid size
    }
  }
  p_data->global_size = p_data->size;
  return D2G_OK;
}

int d2g_mph_alloc(int s_ph, size_t size, const int *avg_strides, const int *dims, const int *types,
                  mph **out) {
  if (s_ph < 1 || size == 0 || !avg_strides || !dims || !types || !out) return bad("invalid arguments");
  mph *p = (mph *)calloc(1, sizeof(mph));
  if (!p) return D2G_E_NOMEM;
  p->s_ph = s_ph;
  p->size = size;
  p->ph = (sph *)calloc((size_t)s_ph, sizeof(sph));
  p->label = (int *)malloc(size * sizeof(int));
  bool ok = p->ph && p->label;
  if (ok)
    for (size_t i = 0; i < size; ++i) p->label[i] = -1;
  for (int n = 0; ok && n < s_ph; ++n) {
    // the data part of d2_allocate_sph (src/d2/clustering_util.c:18-59)
    sph *ph = p->ph + n;
    const size_t m = (size_t)(size * (avg_strides[n] + 0.6));
    ph->dim = dims[n];
    ph->str = ph->max_str = avg_strides[n];
    ph->max_col = m;
    ph->metric_type = types[n];
    ph->p_str = (int *)calloc(size, sizeof(int));
    ph->p_str_cum = (size_t *)calloc(size, sizeof(size_t));
    ph->p_w = (double *)malloc(std::max<size_t>(m, 1) * sizeof(double));
    ok = ph->p_str && ph->p_str_cum && ph->p_w;
    if (types[n] == D2_EUCLIDEAN_L2) {
      ph->p_supp = (double *)malloc(std::max<size_t>(m * dims[n], 1) * sizeof(double));
      ok = ok && ph->p_supp;
    } else if (types[n] == D2_WORD_EMBED || types[n] == D2_SPARSE_HISTOGRAM) {
      ph->p_supp_sym = (int *)malloc(std::max<size_t>(m, 1) * sizeof(int));
      ok = ok && ph->p_supp_sym;
    }
  }
  if (!ok) {
    d2g_mph_free(p);
    return D2G_E_NOMEM;
  }
  *out = p;
  return D2G_OK;
}

int d2g_mph_free(mph *p) {
  if (!p) return D2G_E_INVAL;
  for (int n = 0; p->ph && n < p->s_ph; ++n) {
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
  return D2G_OK;
}

}  // extern "C"
