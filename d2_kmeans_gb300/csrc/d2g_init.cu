// Random centroid initialisation for programs that do not link the
// reference's own: d2g_centroid_rands, the result of d2_centroid_rands
// (src/d2/centroid_rand.c:161-295) on the same input, with its helpers merge
// and merge_symbolic (:53-159) and shuffle (src/d2/math.c:40-58).  Host code:
// it runs once per clustering, before any device work.
//
// The reference draws its instance order from glibc's rand() after
// srand(time(NULL) * world_rank), i.e. srand(0) in a single-process run.  The
// same sequence comes from a private copy of that generator (below), so the
// process-wide rand() state is left alone.
#include <dlfcn.h>

#include <cfloat>
#include <cstdint>
#include <string>
#include <vector>

#include "d2g_internal.cuh"

namespace {

// glibc's rand() with its default state (random_r, TYPE_3): an additive
// lagged-Fibonacci generator over 31 words, r[i] = r[i-31] + r[i-3] (mod 2^32),
// each output the sum shifted right by one; the 31 seed words are successive
// 16807 * x mod (2^31 - 1) (computed without overflow by Schrage's method),
// and the first 310 sums are discarded.  Seed 0 is taken as 1.
class SeededRand {
 public:
  explicit SeededRand(unsigned seed) {
    int32_t word = seed == 0 ? 1 : (int32_t)seed;
    s_[0] = word;
    for (int i = 1; i < kDeg; ++i) {
      const int32_t hi = word / 127773, lo = word % 127773;
      word = 16807 * lo - 2836 * hi;
      if (word < 0) word += 2147483647;
      s_[i] = word;
    }
    f_ = kSep;
    r_ = 0;
    for (int k = 0; k < 10 * kDeg; ++k) next();
  }
  int next() {  // in [0, 2^31 - 1], as rand()
    const uint32_t v = (uint32_t)s_[f_] + (uint32_t)s_[r_];
    s_[f_] = (int32_t)v;
    f_ = f_ + 1 == kDeg ? 0 : f_ + 1;
    r_ = r_ + 1 == kDeg ? 0 : r_ + 1;
    return (int)(v >> 1);
  }
  static constexpr int kMax = 2147483647;  // RAND_MAX

 private:
  static constexpr int kDeg = 31, kSep = 3;
  int32_t s_[kDeg];
  int f_, r_;
};

// shuffle (src/d2/math.c:40-58): ten passes of swaps with j drawn in [i, n)
void shuffle(std::vector<size_t> &a, SeededRand &g) {
  const size_t n = a.size();
  if (n <= 1) return;
  for (int k = 0; k < 10; ++k)
    for (size_t i = 0; i < n - 1; ++i) {
      const size_t j = i + (size_t)g.next() / ((size_t)SeededRand::kMax / (n - i) + 1);
      const size_t t = a[j];
      a[j] = a[i];
      a[i] = t;
    }
}

// squared Euclidean distance as _dpdist2 sums it (src/utils/blas_like64.c:199-208)
double sqdist(const double *x, const double *y, int dim) {
  double s = 0;
  for (int t = 0; t < dim; ++t) s += (x[t] - y[t]) * (x[t] - y[t]);
  return s;
}

// merge (centroid_rand.c:108-159): m weighted supports in R^dim reduced to n
// by repeatedly joining the pair of least w_i w_j |x_i - x_j|^2 / (w_i + w_j)
// into their weighted mean (Ward's criterion); the survivors in index order
bool merge(int dim, const double *m_supp, const double *m_w, int m, double *c_supp, double *c_w, int n) {
  if (m <= n) return false;
  std::vector<double> D((size_t)m * m), supp(m_supp, m_supp + (size_t)m * dim), w(m_w, m_w + m);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) D[(size_t)i * m + j] = sqdist(&supp[(size_t)j * dim], &supp[(size_t)i * dim], dim);
  for (int mm = m; mm > n; --mm) {
    double mn = DBL_MAX;
    long long best = -1;
    for (int i = 0; i < m; ++i)
      for (int j = i + 1; j < m; ++j) {
        const double cost = w[i] * w[j] * D[(size_t)i * m + j] / (w[i] + w[j]);
        if (w[i] > 0 && w[j] > 0 && mn > cost) {
          mn = cost;
          best = (long long)i * m + j;
        }
      }
    if (best < 0) return false;  // fewer than two supports of positive weight left
    const int i = (int)(best / m), j = (int)(best % m);
    for (int k = 0; k < dim; ++k)
      supp[(size_t)i * dim + k] =
          (supp[(size_t)i * dim + k] * w[i] + supp[(size_t)j * dim + k] * w[j]) / (w[i] + w[j]);
    for (int k = 0; k < m; ++k) D[(size_t)i * m + k] = sqdist(&supp[(size_t)i * dim], &supp[(size_t)k * dim], dim);
    for (int k = 0; k < m; ++k) D[(size_t)k * m + i] = D[(size_t)i * m + k];
    w[i] = w[i] + w[j];
    w[j] = 0;
  }
  int j = 0;
  for (int i = 0; i < m; ++i)
    if (w[i] > 0) {
      if (j == n) return false;
      for (int k = 0; k < dim; ++k) c_supp[(size_t)j * dim + k] = supp[(size_t)i * dim + k];
      c_w[j] = w[i];
      ++j;
    }
  return j == n;
}

// merge_symbolic (centroid_rand.c:53-106): n-gram supports joined by least
// symbol cost; the joined support keeps the symbols of the heavier one; the
// costs are those of the original supports throughout (the reference does not
// recompute them after a join)
bool merge_symbolic(int dim, const int *m_supp, const double *m_w, int m, int *c_supp, double *c_w, int n,
                    int V, const double *dist) {
  if (m <= n) return false;
  std::vector<double> D((size_t)m * m), w(m_w, m_w + m);
  std::vector<int> supp(m_supp, m_supp + (size_t)m * dim);
  for (int i = 0; i < m; ++i)  // _dpdist_symbolic (blas_like64.c:232-242) of the supports with themselves
    for (int j = 0; j < m; ++j) {
      double s = 0;
      for (int k = 0; k < dim; ++k) s += dist[(size_t)supp[(size_t)j * dim + k] * V + supp[(size_t)i * dim + k]];
      D[(size_t)i * m + j] = s;
    }
  for (int mm = m; mm > n; --mm) {
    double mn = DBL_MAX;
    long long best = -1;
    for (int i = 0; i < m; ++i)
      for (int j = i + 1; j < m; ++j)
        if (w[i] > 0 && w[j] > 0 && mn > D[(size_t)i * m + j]) {
          mn = D[(size_t)i * m + j];
          best = (long long)i * m + j;
        }
    if (best < 0) return false;
    const int i = (int)(best / m), j = (int)(best % m);
    for (int k = 0; k < dim; ++k)
      supp[(size_t)i * dim + k] = w[i] > w[j] ? supp[(size_t)i * dim + k] : supp[(size_t)j * dim + k];
    w[i] = w[i] + w[j];
    w[j] = 0;
  }
  int j = 0;
  for (int i = 0; i < m; ++i)
    if (w[i] > 0) {
      if (j == n) return false;
      for (int k = 0; k < dim; ++k) c_supp[(size_t)j * dim + k] = supp[(size_t)i * dim + k];
      c_w[j] = w[i];
      ++j;
    }
  return j == n;
}

int fail(int code, const std::string &msg) {
  d2g::set_error(msg);
  return code;
}

}  // namespace

// d2_centroid_rands (centroid_rand.c:161-295) for one process (world_rank 0,
// nprocs 1): centroid j is the j-th instance, in shuffled order, with at
// least str supports (any size for sparse histograms); instances with more
// supports are merged down to str.  Where the reference exit(1)s for too few
// such instances this returns D2G_E_INVAL.  Reference behaviours kept as they
// are: a sparse-histogram instance is written into the first centroid's
// weights whatever j is (:262-264), and the first centroid then holds the
// last one taken.
extern "C" int d2g_centroid_rands(mph *p_data, int idx_ph, sph *c) {
  if (!p_data || !c || idx_ph < 0 || idx_ph >= p_data->s_ph || !c->p_str || !c->p_str_cum || !c->p_w)
    return fail(D2G_E_INVAL, "d2g_centroid_rands: bad arguments");
  const sph *data = p_data->ph + idx_ph;
  const size_t K = (size_t)p_data->num_of_labels, size = p_data->size;
  const int dim = data->dim, str = data->str;
  const int strxdim = str * dim;
  const int mt = data->metric_type;
  if (c->str != str) return fail(D2G_E_INVAL, "d2g_centroid_rands: c->str differs from the phase's str");
  if (c->metric_type == D2_EUCLIDEAN_L2 && !c->p_supp) return fail(D2G_E_INVAL, "d2g_centroid_rands: c->p_supp");
  if (c->metric_type == D2_N_GRAM && !c->p_supp_sym) return fail(D2G_E_INVAL, "d2g_centroid_rands: c->p_supp_sym");
  for (size_t i = 0; i < K; ++i) {  // :176-180
    c->p_str[i] = str;
    c->p_str_cum[i] = i * str;
  }
  c->col = (size_t)str * K;
  if (mt == D2_HISTOGRAM || mt == D2_SPARSE_HISTOGRAM || mt == D2_N_GRAM) {  // :186-191
    c->dist_mat = data->dist_mat;
    c->vocab_size = data->vocab_size;
  }
  std::vector<size_t> order(size);
  for (size_t i = 0; i < size; ++i) order[i] = i;
  SeededRand g(0);
  shuffle(order, g);
  for (size_t i = 0; i < c->col; ++i) c->p_w[i] = 0;
  if (c->metric_type == D2_EUCLIDEAN_L2)
    for (size_t i = 0; i < c->col * (size_t)c->dim; ++i) c->p_supp[i] = 0;
  else if (c->metric_type == D2_N_GRAM)
    for (size_t i = 0; i < c->col * (size_t)c->dim; ++i) c->p_supp_sym[i] = 0;

  size_t i = 0, j = 0;
  while (i < size && j < K) {
    while (i < size && data->p_str[order[i]] < str && mt != D2_SPARSE_HISTOGRAM) ++i;
    if (i == size) break;
    const int the_str = data->p_str[order[i]];
    const size_t cum = data->p_str_cum[order[i]];
    const double *m_w = data->p_w + cum;
    switch (mt) {
      case D2_HISTOGRAM:
        for (int k = 0; k < str; ++k) c->p_w[j * str + k] = m_w[k];
        break;
      case D2_EUCLIDEAN_L2: {
        const double *m_supp = data->p_supp + cum * dim;
        if (the_str == str) {
          for (int k = 0; k < strxdim; ++k) c->p_supp[j * strxdim + k] = m_supp[k];
          for (int k = 0; k < str; ++k) c->p_w[j * str + k] = m_w[k];
        } else if (!merge(dim, m_supp, m_w, the_str, c->p_supp + j * strxdim, c->p_w + j * str, str)) {
          return fail(D2G_E_NUMERIC, "d2g_centroid_rands: merge found no pair of positive weights");
        }
        break;
      }
      case D2_WORD_EMBED: {  // Euclidean centroids from the words' vectors
        const int *sym = data->p_supp_sym + cum;
        std::vector<double> supp((size_t)the_str * dim);
        for (int k = 0; k < the_str; ++k)
          for (int d = 0; d < dim; ++d) supp[(size_t)k * dim + d] = data->vocab_vec[(size_t)sym[k] * dim + d];
        if (the_str == str) {
          for (int k = 0; k < strxdim; ++k) c->p_supp[j * strxdim + k] = supp[k];
          for (int k = 0; k < str; ++k) c->p_w[j * str + k] = m_w[k];
        } else if (!merge(dim, supp.data(), m_w, the_str, c->p_supp + j * strxdim, c->p_w + j * str, str)) {
          return fail(D2G_E_NUMERIC, "d2g_centroid_rands: merge found no pair of positive weights");
        }
        break;
      }
      case D2_SPARSE_HISTOGRAM: {
        const int *sym = data->p_supp_sym + cum;
        for (int k = 0; k < str; ++k) c->p_w[k] = 0;
        for (int k = 0; k < the_str; ++k) c->p_w[sym[k]] = m_w[k];
        break;
      }
      case D2_N_GRAM: {
        const int *sym = data->p_supp_sym + cum * dim;
        if (the_str == str) {
          for (int k = 0; k < strxdim; ++k) c->p_supp_sym[j * strxdim + k] = sym[k];
          for (int k = 0; k < str; ++k) c->p_w[j * str + k] = m_w[k];
        } else if (!merge_symbolic(dim, sym, m_w, the_str, c->p_supp_sym + j * strxdim, c->p_w + j * str, str,
                                   c->vocab_size, c->dist_mat)) {
          return fail(D2G_E_NUMERIC, "d2g_centroid_rands: merge found no pair of positive weights");
        }
        break;
      }
      default:
        return fail(D2G_E_UNSUPPORTED, "d2g_centroid_rands: unknown metric type");
    }
    ++i;
    ++j;
  }
  if (j < K)
    return fail(D2G_E_INVAL, "d2g_centroid_rands: fewer instances with at least str supports than centroids");
  return D2G_OK;
}

// d2_write_split (src/d2/clustering_io.c:329-480): the instances in shuffled
// order (math.c's shuffle after srand(0), the writing process being rank 0),
// that order in <filename>.ind, and `splits` files <filename>.0 ... each with
// a contiguous batch of 1 + (n-1)/splits instances in the d2 text format the
// reader takes, one file per rank of a sharded run.  pre_processed != 0 writes
// them as the reference's pre-processing does: word-embedding supports as
// their vectors, Euclidean and embedding instances with more supports than
// the phase's str merged down to str (Ward), dense histograms as their
// non-zero bins.  The number formats are the reference's ("%lf", ids + 1), so
// the files are the reference's byte for byte.  Where the reference would
// read through a null pointer (pre-processed sparse histograms and n-grams)
// this returns D2G_E_UNSUPPORTED; where its merge finds too few positive
// weights (and writes uninitialised values), D2G_E_NUMERIC.
extern "C" int d2g_write_split(const char *filename, mph *p_data, int splits, char is_pre_processed) {
  if (!filename || !p_data || splits < 1 || (p_data->size > 0 && !p_data->ph))
    return fail(D2G_E_INVAL, "d2g_write_split: bad arguments");
  const int s_ph = p_data->s_ph;
  const size_t size = p_data->size;
  for (int j = 0; j < s_ph; ++j) {
    const sph &ph = p_data->ph[j];
    if (ph.col == 0) continue;
    const int mt = ph.metric_type;
    if (is_pre_processed && mt != D2_EUCLIDEAN_L2 && mt != D2_WORD_EMBED && mt != D2_HISTOGRAM)
      return fail(D2G_E_UNSUPPORTED, "d2g_write_split: pre-processing covers Euclidean, word-embedding "
                                     "and dense histogram phases");
  }
  std::vector<size_t> order(size);
  for (size_t i = 0; i < size; ++i) order[i] = i;
  SeededRand g(0);
  shuffle(order, g);
  const std::string base(filename);
  {
    FILE *f = fopen((base + ".ind").c_str(), "w+");
    if (!f) return fail(D2G_E_INVAL, "d2g_write_split: cannot write " + base + ".ind");
    for (size_t n = 0; n < size; ++n) fprintf(f, "%zd\n", order[n]);
    fclose(f);
  }
  const size_t batch = size ? 1 + (size - 1) / (size_t)splits : 1;
  std::vector<double> msupp, mw, csupp, cw;
  std::vector<int> ssym;
  for (int k = 0; k < splits; ++k) {
    const std::string name = base + "." + std::to_string(k);
    FILE *f = fopen(name.c_str(), "w+");
    if (!f) return fail(D2G_E_INVAL, "d2g_write_split: cannot write " + name);
    int rc = D2G_OK;
    for (size_t idx = batch * (size_t)k; idx < size && idx < batch * (size_t)(k + 1) && !rc; ++idx) {
      const size_t i = order[idx];
      for (int j = 0; j < s_ph && !rc; ++j) {
        const sph &ph = p_data->ph[j];
        if (ph.col == 0) continue;
        const int dim = ph.dim, mt = ph.metric_type;
        int str = ph.p_str[i];
        const size_t pos = ph.p_str_cum[i];
        if (!is_pre_processed) {
          if (mt == D2_HISTOGRAM)
            fprintf(f, "%d %d ", dim, str);
          else
            fprintf(f, "%d\n%d\n", dim, str);
          for (int q = 0; q < str; ++q) fprintf(f, "%lf ", ph.p_w[pos + q]);
          fprintf(f, "\n");
          if (mt == D2_EUCLIDEAN_L2) {
            for (int q = 0; q < str; ++q) {
              for (int d = 0; d < dim; ++d) fprintf(f, "%lf ", ph.p_supp[(pos + q) * dim + d]);
              fprintf(f, "\n");
            }
          } else if (mt == D2_WORD_EMBED || mt == D2_SPARSE_HISTOGRAM) {
            for (int q = 0; q < str; ++q) fprintf(f, "%d ", ph.p_supp_sym[pos + q] + 1);
            fprintf(f, "\n");
          }
          continue;
        }
        // pre-processed (:396-466)
        const double *w = ph.p_w + pos, *supp = nullptr, *pw = nullptr;
        const int *psym = nullptr;
        if (mt == D2_EUCLIDEAN_L2) {
          supp = ph.p_supp + pos * dim;
          pw = w;
        } else if (mt == D2_WORD_EMBED) {
          const int *sym = ph.p_supp_sym + pos;
          msupp.resize((size_t)str * dim);
          for (int q = 0; q < str; ++q)
            for (int d = 0; d < dim; ++d) msupp[(size_t)q * dim + d] = ph.vocab_vec[(size_t)sym[q] * dim + d];
          mw.assign(w, w + str);
          supp = msupp.data();
          pw = mw.data();
        }
        if ((mt == D2_EUCLIDEAN_L2 || mt == D2_WORD_EMBED) && str > ph.str) {
          csupp.resize((size_t)ph.str * dim);
          cw.resize(ph.str);
          if (!merge(dim, supp, pw, str, csupp.data(), cw.data(), ph.str)) {
            rc = fail(D2G_E_NUMERIC, "d2g_write_split: merge found no pair of positive weights");
            break;
          }
          str = ph.str;
          supp = csupp.data();
          pw = cw.data();
        }
        if (mt == D2_HISTOGRAM) {  // the non-zero bins
          ssym.clear();
          mw.clear();
          for (int q = 0; q < str; ++q)
            if (w[q] > 0) {
              ssym.push_back(q);
              mw.push_back(w[q]);
            }
          str = (int)ssym.size();
          psym = ssym.data();
          pw = mw.data();
        }
        fprintf(f, "%d\n", dim);
        fprintf(f, "%d\n", str);
        for (int q = 0; q < str; ++q) fprintf(f, "%lf ", pw[q]);
        fprintf(f, "\n");
        if (mt == D2_EUCLIDEAN_L2 || mt == D2_WORD_EMBED) {
          for (int q = 0; q < str; ++q) {
            for (int d = 0; d < dim; ++d) fprintf(f, "%lf ", supp[(size_t)q * dim + d]);
            fprintf(f, "\n");
          }
        } else if (mt == D2_HISTOGRAM) {
          for (int q = 0; q < str; ++q) fprintf(f, "%d ", psym[q] + 1);
          fprintf(f, "\n");
        }
      }
    }
    fclose(f);
    if (rc) return rc;
  }
  return D2G_OK;
}

namespace d2g {

// the program's d2_centroid_rands where it links one, else d2g_centroid_rands
int centroid_rands(mph *p_data, int idx_ph, sph *c) {
  typedef int (*rands_fn)(mph *, int, sph *);
  const rands_fn own = (rands_fn)dlsym(RTLD_DEFAULT, "d2_centroid_rands");
  return own ? own(p_data, idx_ph, c) : d2g_centroid_rands(p_data, idx_ph, c);
}

}  // namespace d2g
