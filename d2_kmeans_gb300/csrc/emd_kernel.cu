// Exact discrete transport for the assignment step: one warp per
// (row distribution, column distribution) pair, a transportation (network)
// primal simplex.
//
// The reference computes each instance-to-centroid distance with
// d2_match_by_distmat (src/d2/solver_mosek.cc:61-226): the linear program
//   min sum_ij C_ij x_ij  s.t.  sum_j x_ij = wR_i (rows),
//                               sum_i x_ij = wC_j (columns but the last),
//                               x >= 0,
// given to MOSEK's network primal simplex.  This kernel runs the same
// method on the GPU (Dantzig, "Linear Programming and Extensions", 1963,
// ch. 17; Ahuja, Magnanti and Orlin, "Network Flows", 1993, ch. 11):
//
//  * basis = spanning tree over the n + m row and column nodes, stored as a
//    parent array rooted at row 0 with the flow and FP32 cost of each node's
//    arc to its parent; initial tree from the row-minimum rule (the last
//    column's demand is what the rows supply beyond the other columns: its
//    constraint is the dropped one);
//  * node potentials (u_i + v_j = C_ij on tree arcs) by pointer jumping over
//    the parent array: log2(depth) rounds over all lanes, no traversal order
//    to maintain; depths come out of the same rounds;
//  * pricing: every cell's reduced cost, the lanes spread over rows, columns
//    or cells (whichever keeps more lanes busy), warp argmin (ties to the
//    lowest cell index).  Euclidean costs in the norm form
//    |x|^2 + |y|^2 - 2 x.y with the potentials folded into the norms, so a
//    cell is one dot product; supports are centred on the rows' mean (FP64)
//    before they are rounded to FP32 to keep the norms small;
//  * pivot: lane 0 walks both ends of the entering cell up to their common
//    ancestor and records the path; the ratio test (ties: the last blocking
//    arc met going round the cycle from the apex, the strongly-feasible-tree
//    choice that avoids cycling), the flow update and the re-hanging of the
//    cut-off subtree (parent pointers reversed from the entering node to the
//    leaving arc) run over the recorded path on all lanes;
//  * exactness: FP32 pricing enters only cells below -1e-5 of the cost
//    scale; when none is left the potentials are recomputed in FP64 from
//    FP64 costs (the reference's difference form) and every cell whose FP32
//    reduced cost is within a safe margin of zero is priced again in FP64;
//    pivots continue in FP64 until no reduced cost is below -1e-12 of the
//    scale.  The cost is then sum x_ij C_ij over the tree arcs in FP64, in a
//    fixed order.
//
// A pair that has not reached optimality after max_piv pivots reports -1
// pivots and a NaN cost (-3: a tree walk ran past the node count, which a
// correct tree cannot do); the host turns either into an error.
#include <math.h>

#include <mutex>

#include "d2g_internal.cuh"

namespace d2g {

namespace {

constexpr int kEmdWarps = 8;               // warps per block at most (fewer when the slices are large)
constexpr int kEmdSmemLimit = 220 * 1024;  // dynamic shared memory per block
constexpr int kSideJ = 1 << 20;            // ratio-test keys of the j side sort after the i side's

// per-node bytes of one warp's shared-memory slice: node data (DP floats:
// centred support + folded potential, or key + potential for tables), flow
// and FP64 potential (doubles), two FP32 jump accumulators (one FP64 buffer
// in the FP64 phase), two packed jump states, arc cost, parent, depth, path
__host__ __device__ constexpr int emd_node_bytes(int DP) {
  return (DP > 0 ? DP * 4 : 8) + 8 + 8 + 8 + 8 + 4 + 2 + 2 + 4;
}

__host__ __device__ inline size_t emd_slice_bytes(int nmax, int DP) {
  return ((size_t)nmax * emd_node_bytes(DP) + 15) & ~(size_t)15;
}

struct EmdWarp {
  float *dat;
  double *flow, *p64;
  float *jacc;   // [2][NM] FP32 accumulators; as double[NM]: the FP64 second buffer
  int *jad;      // [2][NM] packed (anc + 1) | dep << 16
  float *acost;
  short *parent, *depth, *path;
  int *stage;    // [NM] re-hang staging (aliases jad[0..NM))
};

__device__ inline EmdWarp carve(unsigned char *p, int NM, int DP) {
  EmdWarp w;
  w.dat = (float *)p;
  p += (size_t)NM * (DP > 0 ? DP * 4 : 8);
  w.flow = (double *)p;
  p += (size_t)NM * 8;
  w.p64 = (double *)p;
  p += (size_t)NM * 8;
  w.jacc = (float *)p;
  p += (size_t)NM * 8;
  w.jad = (int *)p;
  w.stage = (int *)p;
  p += (size_t)NM * 8;
  w.acost = (float *)p;
  p += (size_t)NM * 4;
  w.parent = (short *)p;
  p += (size_t)NM * 2;
  w.depth = (short *)p;
  p += (size_t)NM * 2;
  w.path = (short *)p;
  return w;
}

// one problem: sizes, where its supports live, and the staged node data
template <int MODE, int DP>
struct Prob {
  const EmdArgs *a;
  EmdWarp w;
  int n, m, N, NM;
  size_t r0, c0;  // first support of the row / column object
  // FP32 table view (tables, embeddings): cost(key_i, key_j) = tb[key_i * sR + key_j * sC]
  const float *tb;
  int sR, sC;

  // FP32 cost in the difference form, from the staged (centred) supports
  __device__ inline float c32(int i, int j) const {
    if constexpr (MODE == EMD_EUCLID) {
      const float *x = w.dat + (size_t)i * DP, *y = w.dat + (size_t)(n + j) * DP;
      float s = 0.f;
#pragma unroll
      for (int t = 0; t < DP - 1; ++t) {
        const float d = x[t] - y[t];
        s = fmaf(d, d, s);
      }
      return s;
    } else {
      const int ki = __float_as_int(w.dat[2 * i]), kj = __float_as_int(w.dat[2 * (n + j)]);
      return __ldg(tb + (size_t)ki * sR + (size_t)kj * sC);
    }
  }
  // FP64 cost, the reference's difference form (_dpdist2 / _dpdist2_sym,
  // blas_like64.c:199-220)
  __device__ inline double c64(int i, int j) const {
    if constexpr (MODE == EMD_EUCLID || MODE == EMD_EMBED) {
      const int d = a->dim;
      const double *x = a->rsupp + (r0 + i) * d;
      const double *y = MODE == EMD_EUCLID
                            ? a->csupp + (c0 + j) * d
                            : a->vocab + (size_t)__float_as_int(w.dat[2 * (n + j)]) * d;
      double s = 0.0;
      for (int t = 0; t < d; ++t) {
        const double v = __ldg(x + t) - __ldg(y + t);
        s += v * v;
      }
      return s;
    } else {
      const int ki = __float_as_int(w.dat[2 * i]), kj = __float_as_int(w.dat[2 * (n + j)]);
      return __ldg(a->T64 + (size_t)ki * a->V + kj);
    }
  }
  __device__ inline double arc_c64(int x, int px) const {
    return x < n ? c64(x, px - n) : c64(px, x - n);
  }
  // store node x's FP32 potential: folded into the norm (Euclidean) or kept
  __device__ inline void set_pot(int x, float p) const {
    if constexpr (MODE == EMD_EUCLID) {
      const float *v = w.dat + (size_t)x * DP;
      float nrm = 0.f;
#pragma unroll
      for (int t = 0; t < DP - 1; ++t) nrm = fmaf(v[t], v[t], nrm);
      w.dat[(size_t)x * DP + DP - 1] = nrm - p;
    } else {
      w.dat[2 * x + 1] = p;
    }
  }
};

// Potentials by pointer jumping: pot[x] = acc + (-1)^dep * pot[anc] until
// every anc is past the root.  FP32: the state of a node is one 8-byte word
// {acc, (anc + 1) | dep << 16} (two buffers: the jacc and jad regions), arc
// costs from acost.  FP64: acc in p64 and the jacc region as double, the
// packed anc/dep in the jad region, arc costs recomputed.  Leaves the depths
// in w.depth and the potentials in the node data (FP32) or p64.
template <int MODE, int DP, bool F64>
__device__ void potentials(const Prob<MODE, DP> &P, int lane) {
  const EmdWarp &w = P.w;
  const int N = P.N, NM = P.NM;
  if constexpr (!F64) {
    int2 *const b0 = (int2 *)w.jacc, *const b1 = (int2 *)w.jad;
    for (int x = lane; x < N; x += 32) {
      const int px = w.parent[x];
      b0[x] = make_int2(__float_as_int(px < 0 ? 0.f : w.acost[x]), (px + 1) | ((px < 0 ? 0 : 1) << 16));
    }
    __syncwarp();
    int cur = 0;
    for (int round = 0; round < 16; ++round) {
      const int2 *s = cur ? b1 : b0;
      int2 *d = cur ? b0 : b1;
      bool more = false;
      for (int x = lane; x < N; x += 32) {
        const int2 v = s[x];
        const int A = v.y & 0xffff;
        if (A == 0) {
          d[x] = v;
          continue;
        }
        const int2 u = s[A - 1];
        const float acc = (v.y >> 16) & 1 ? __int_as_float(v.x) - __int_as_float(u.x)
                                           : __int_as_float(v.x) + __int_as_float(u.x);
        const int A2 = u.y & 0xffff;
        d[x] = make_int2(__float_as_int(acc), A2 | (((v.y >> 16) + (u.y >> 16)) << 16));
        more |= A2 != 0;
      }
      __syncwarp();
      cur ^= 1;
      if (!__any_sync(0xffffffffu, more)) break;
    }
    const int2 *fin = cur ? b1 : b0;
    for (int x = lane; x < N; x += 32) {
      const int2 v = fin[x];
      w.depth[x] = (short)(v.y >> 16);
      P.set_pot(x, __int_as_float(v.x));
    }
    __syncwarp();
  } else {
    double *const a0 = w.p64, *const a1 = (double *)w.jacc;
    int *const j0 = w.jad, *const j1 = w.jad + NM;
    for (int x = lane; x < N; x += 32) {
      const int px = w.parent[x];
      j0[x] = (px + 1) | ((px < 0 ? 0 : 1) << 16);
      a0[x] = px < 0 ? 0.0 : P.arc_c64(x, px);
    }
    __syncwarp();
    int cur = 0;
    for (int round = 0; round < 16; ++round) {
      const int *s = cur ? j1 : j0;
      int *d = cur ? j0 : j1;
      const double *sa = cur ? a1 : a0;
      double *da = cur ? a0 : a1;
      bool more = false;
      for (int x = lane; x < N; x += 32) {
        const int v = s[x];
        const int A = v & 0xffff;
        if (A == 0) {
          d[x] = v;
          da[x] = sa[x];
          continue;
        }
        const int u = s[A - 1];
        const double q = sa[A - 1];
        da[x] = (v >> 16) & 1 ? sa[x] - q : sa[x] + q;
        const int A2 = u & 0xffff;
        d[x] = A2 | (((v >> 16) + (u >> 16)) << 16);
        more |= A2 != 0;
      }
      __syncwarp();
      cur ^= 1;
      if (!__any_sync(0xffffffffu, more)) break;
    }
    const int *fin = cur ? j1 : j0;
    for (int x = lane; x < N; x += 32) {
      w.depth[x] = (short)(fin[x] >> 16);
      if (cur) w.p64[x] = a1[x];
    }
    __syncwarp();
  }
}

struct Best {
  float v;
  int idx;
};

__device__ inline void better(Best &b, float v, int idx) {
  if (v < b.v || (v == b.v && idx < b.idx)) {
    b.v = v;
    b.idx = idx;
  }
}

__device__ inline Best warp_best(Best b) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const float v = __shfl_xor_sync(0xffffffffu, b.v, o);
    const int i = __shfl_xor_sync(0xffffffffu, b.idx, o);
    better(b, v, i);
  }
  return b;
}

// node data as registers: Euclidean (DP = 4: x, y, z, folded potential;
// DP = 8: two float4) or table (key, potential)
struct NodeV {
  float4 a, b;
};

template <int MODE, int DP>
__device__ inline NodeV load_node(const float *dat, int x) {
  NodeV v;
  if constexpr (MODE == EMD_EUCLID) {
    v.a = *(const float4 *)(dat + (size_t)x * DP);
    if constexpr (DP == 8) v.b = *(const float4 *)(dat + (size_t)x * DP + 4);
  } else {
    const float2 t = *(const float2 *)(dat + 2 * (size_t)x);
    v.a = make_float4(t.x, t.y, 0.f, 0.f);
  }
  return v;
}

// reduced cost of the cell (row node data r, column node data c)
template <int MODE, int DP>
__device__ inline float rcost(const NodeV &r, const NodeV &c, const Prob<MODE, DP> &P) {
  if constexpr (MODE == EMD_EUCLID) {
    if constexpr (DP == 4) {
      const float dot = fmaf(r.a.x, c.a.x, fmaf(r.a.y, c.a.y, r.a.z * c.a.z));
      return fmaf(-2.f, dot, r.a.w + c.a.w);
    } else {
      float dot = r.a.x * c.a.x;
      dot = fmaf(r.a.y, c.a.y, dot);
      dot = fmaf(r.a.z, c.a.z, dot);
      dot = fmaf(r.a.w, c.a.w, dot);
      dot = fmaf(r.b.x, c.b.x, dot);
      dot = fmaf(r.b.y, c.b.y, dot);
      dot = fmaf(r.b.z, c.b.z, dot);
      return fmaf(-2.f, dot, r.b.w + c.b.w);
    }
  } else {
    const float t = __ldg(P.tb + (size_t)__float_as_int(r.a.x) * P.sR + (size_t)__float_as_int(c.a.x) * P.sC);
    return t - r.a.y - c.a.y;
  }
}

// FP32 pricing: the cell with the most negative reduced cost.  map 0:
// lanes over rows, 1: over columns, 2: over cells.
template <int MODE, int DP>
__device__ Best price32(const Prob<MODE, DP> &P, int lane, int map) {
  const int n = P.n, m = P.m;
  const float *dat = P.w.dat;
  Best b{INFINITY, 0x7fffffff};
  if (map == 0) {
    for (int i = lane; i - lane < n; i += 32) {
      const bool ok = i < n;
      const NodeV r = load_node<MODE, DP>(dat, ok ? i : 0);
      for (int j = 0; j < m; ++j) {
        const float v = rcost<MODE, DP>(r, load_node<MODE, DP>(dat, n + j), P);
        if (ok && v < b.v) {
          b.v = v;
          b.idx = i * m + j;
        }
      }
    }
  } else if (map == 1) {
    for (int j = lane; j - lane < m; j += 32) {
      const bool ok = j < m;
      const NodeV c = load_node<MODE, DP>(dat, n + (ok ? j : 0));
      for (int i = 0; i < n; ++i) {
        const float v = rcost<MODE, DP>(load_node<MODE, DP>(dat, i), c, P);
        if (ok) better(b, v, i * m + j);
      }
    }
  } else {
    int i = lane / m, j = lane - (lane / m) * m;
    const int di = 32 / m, dj = 32 - di * m;
    while (i < n) {
      const float v = rcost<MODE, DP>(load_node<MODE, DP>(dat, i), load_node<MODE, DP>(dat, n + j), P);
      if (v < b.v) {
        b.v = v;
        b.idx = i * m + j;
      }
      i += di;
      j += dj;
      if (j >= m) {
        j -= m;
        ++i;
      }
    }
  }
  return warp_best(b);
}

// FP64 pricing, potentials in p64: the most negative reduced cost below
// -tol.  The potentials are folded into the FP32 node data too; a cell whose
// FP32 reduced cost is above thr (far above the FP32 rounding error of the
// norms, dot products and potentials) is nonnegative in exact arithmetic and
// is not evaluated in FP64.
template <int MODE, int DP>
__device__ Best price64(const Prob<MODE, DP> &P, int lane, double tol, float scale) {
  const int n = P.n, m = P.m, N = P.N;
  float pmax = 0.f;
  for (int x = lane; x < N; x += 32) {
    const float pv = (float)P.w.p64[x];
    P.set_pot(x, pv);
    pmax = fmaxf(pmax, fabsf(pv));
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) pmax = fmaxf(pmax, __shfl_xor_sync(0xffffffffu, pmax, o));
  __syncwarp();
  const float thr = 1e-3f * scale + 1e-5f * pmax;
  const float *dat = P.w.dat;
  double bv = INFINITY;
  int bi = 0x7fffffff;
  int i = lane / m, j = lane - (lane / m) * m;
  const int di = 32 / m, dj = 32 - di * m;
  while (i < n) {
    const float r32 = rcost<MODE, DP>(load_node<MODE, DP>(dat, i), load_node<MODE, DP>(dat, n + j), P);
    if (r32 < thr) {
      const double r = P.c64(i, j) - P.w.p64[i] - P.w.p64[n + j];
      const int c = i * m + j;
      if (r < bv || (r == bv && c < bi)) {
        bv = r;
        bi = c;
      }
    }
    i += di;
    j += dj;
    if (j >= m) {
      j -= m;
      ++i;
    }
  }
  // rank by the value in units of tol (ties to the lowest index)
  Best b{bv < -tol ? (float)(bv / tol) : INFINITY, bv < -tol ? bi : 0x7fffffff};
  return warp_best(b);
}

// Starting basis by the row-minimum rule (Dantzig 1963, ch. 18): rows in
// order, each ships to its cheapest open column until the row or the column
// is used up, crossing out exactly one line per cell (never the last open
// row or column), which gives n + m - 1 cells forming a spanning tree.  It
// needs about half the pivots of the north-west corner on Euclidean costs.
// The last column's demand is what the rows supply beyond the other columns
// (its constraint is the dropped one).  Weights staged in p64; the cells go
// to scratch (rows, columns in jad, flows in jacc), then lane 0 roots the
// tree at row 0 by a breadth-first walk over an adjacency list.  False if
// the cells do not span every node (not for a correct allocation).
template <int MODE, int DP>
__device__ bool row_min_start(const Prob<MODE, DP> &P, int lane) {
  const EmdWarp &w = P.w;
  const int n = P.n, m = P.m, N = P.N, NM = P.NM;
  int *const crow = w.jad, *const ccol = w.jad + NM;
  double *const cflow = (double *)w.jacc;
  short *const coldone = w.parent + n;
  // last column's demand: total supply minus the other columns' demands
  double tot = 0.0;
  for (int x = lane; x < N - 1; x += 32) tot += x < n ? w.p64[x] : -w.p64[x];
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  for (int j = lane; j < m; j += 32) coldone[j] = 0;
  __syncwarp();
  if (lane == 0) w.p64[N - 1] = fmax(tot, 0.0);
  __syncwarp();
  int count = 0, nr = n, nc = m;
  for (int i = 0; i < n && count < N - 1; ++i) {
    double si = w.p64[i];
    for (;;) {
      float bv = INFINITY;
      int bj = 0x7fffffff;
      for (int j = lane; j < m; j += 32)
        if (!coldone[j]) {
          const float c = P.c32(i, j);
          if (c < bv) {
            bv = c;
            bj = j;
          }
        }
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        const float v = __shfl_xor_sync(0xffffffffu, bv, o);
        const int jj = __shfl_xor_sync(0xffffffffu, bj, o);
        if (v < bv || (v == bv && jj < bj)) {
          bv = v;
          bj = jj;
        }
      }
      if (bj >= m) return false;  // no open column: not for a correct allocation
      const int j = bj;
      double dj = w.p64[n + j];
      const double f = fmin(si, dj);
      si -= f;
      dj -= f;
      __syncwarp();
      if (lane == 0) {
        crow[count] = i;
        ccol[count] = j;
        cflow[count] = f;
        w.p64[n + j] = dj;
      }
      ++count;
      bool row_done = false;
      if (count == N - 1) {
        row_done = true;
      } else if (si <= dj && nr > 1) {
        --nr;
        row_done = true;
      } else if (nc > 1) {
        if (lane == 0) coldone[j] = 1;
        --nc;
      } else {
        --nr;
        row_done = true;
      }
      __syncwarp();
      if (row_done) break;
    }
  }
  // root the tree at row 0: adjacency list (degrees in acost as ints,
  // offsets in depth, entries in p64 as ints), then a breadth-first walk
  int spanned = 0;
  if (lane == 0 && count == N - 1) {
    int *const deg = (int *)w.acost;
    short *const off = w.depth;
    int *const adj = (int *)w.p64;
    for (int x = 0; x < N; ++x) deg[x] = 0;
    for (int k = 0; k < N - 1; ++k) {
      ++deg[crow[k]];
      ++deg[n + ccol[k]];
    }
    int acc = 0;
    for (int x = 0; x < N; ++x) {
      off[x] = (short)acc;
      acc += deg[x];
      deg[x] = off[x];  // fill cursor
    }
    for (int k = 0; k < N - 1; ++k) {
      const int r = crow[k], c = n + ccol[k];
      adj[deg[r]++] = c | (k << 16);
      adj[deg[c]++] = r | (k << 16);
    }
    for (int x = 0; x < N; ++x) w.parent[x] = -2;
    w.parent[0] = -1;
    w.flow[0] = 0.0;
    w.acost[0] = 0.f;
    int head = 0, tail = 0;
    w.path[tail++] = 0;
    while (head < tail) {
      const int u = w.path[head++];
      const int end = u + 1 < N ? off[u + 1] : 2 * (N - 1);
      for (int e = off[u]; e < end; ++e) {
        const int v = adj[e] & 0xffff, k = adj[e] >> 16;
        if (w.parent[v] != -2) continue;
        w.parent[v] = (short)u;
        w.flow[v] = cflow[k];
        w.acost[v] = P.c32(crow[k], ccol[k]);
        if (tail < N) w.path[tail++] = (short)v;
      }
    }
    spanned = tail == N;
  }
  __syncwarp();
  return __shfl_sync(0xffffffffu, spanned, 0) != 0;
}

// One pivot on cell (ei, ej).  Lane 0 records the cycle's tree path (i side
// at path[0..ta), j side at path[N-1], path[N-2], ...); the ratio test, flow
// update and re-hang run on all lanes.  Returns false if a walk outgrows the
// tree (every walk is bounded by the node count).
template <int MODE, int DP>
__device__ bool pivot(const Prob<MODE, DP> &P, int lane, int ei, int ej) {
  const EmdWarp &w = P.w;
  const int n = P.n, N = P.N;
  const int ni = ei, nj = n + ej;
  int packed = 0;
  if (lane == 0) {
    int a = ni, b = nj, ta = 0, tb = 0;
    int da = w.depth[a], db = w.depth[b];
    bool ok = da < N && db < N;
    while (ok && da > db) {
      w.path[ta++] = (short)a;
      a = w.parent[a];
      --da;
    }
    while (ok && db > da) {
      w.path[N - 1 - tb++] = (short)b;
      b = w.parent[b];
      --db;
    }
    while (ok && a != b) {
      if (a < 0 || b < 0 || ta + tb + 2 > N) {
        ok = false;
        break;
      }
      w.path[ta++] = (short)a;
      a = w.parent[a];
      w.path[N - 1 - tb++] = (short)b;
      b = w.parent[b];
    }
    packed = ok ? (ta | (tb << 16)) : -1;
  }
  __syncwarp();
  packed = __shfl_sync(0xffffffffu, packed, 0);
  if (packed < 0) return false;
  const int ta = packed & 0xffff, tb = packed >> 16;
  // ratio test over the arcs at even positions (they lose flow).  Flows are
  // nonnegative, so they order like their bit patterns (sign bit cleared for
  // -0): integer compares, off the narrow FP64 pipe.
  unsigned long long tbits = 0x7ff0000000000000ull;  // +inf
  int qkey = -0x7fffffff;
  for (int t = lane; t < ta + tb; t += 32) {
    const bool iside = t < ta;
    const int pos = iside ? t : t - ta;
    if (pos & 1) continue;
    const int x = iside ? w.path[t] : w.path[N - 1 - pos];
    const unsigned long long f = (unsigned long long)__double_as_longlong(w.flow[x]) & 0x7fffffffffffffffull;
    const int key = iside ? -pos : kSideJ + pos;
    if (f < tbits || (f == tbits && key > qkey)) {
      tbits = f;
      qkey = key;
    }
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const unsigned long long f = __shfl_xor_sync(0xffffffffu, tbits, o);
    const int k = __shfl_xor_sync(0xffffffffu, qkey, o);
    if (f < tbits || (f == tbits && k > qkey)) {
      tbits = f;
      qkey = k;
    }
  }
  if (qkey == -0x7fffffff) return false;
  const double theta = __longlong_as_double((long long)tbits);
  // flows along the cycle
  for (int t = lane; t < ta + tb; t += 32) {
    const bool iside = t < ta;
    const int pos = iside ? t : t - ta;
    const int x = iside ? w.path[t] : w.path[N - 1 - pos];
    w.flow[x] += (pos & 1) ? theta : -theta;
  }
  __syncwarp();
  // the leaving arc's lower node q is at position tq on its side; the
  // endpoint e on that side is re-hung from the other endpoint o and the
  // parent pointers from e to q reversed (arc data move one node down)
  const bool jside = qkey >= kSideJ;
  const int tq = jside ? qkey - kSideJ : -qkey;
  const int e = jside ? nj : ni, o = jside ? ni : nj;
  auto node_at = [&](int t) -> int { return jside ? w.path[N - 1 - t] : w.path[t]; };
  // stage the new (parent, flow, cost) of every reversed node
  double *sflow = (double *)w.jacc;
  float *scost = (float *)(w.stage + P.NM);
  for (int t = lane; t <= tq; t += 32) {
    if (t == 0) {
      w.stage[0] = o;
      sflow[0] = theta;
      scost[0] = P.c32(ei, ej);
    } else {
      const int prev = node_at(t - 1);
      w.stage[t] = prev;
      sflow[t] = w.flow[prev];
      scost[t] = w.acost[prev];
    }
  }
  __syncwarp();
  for (int t = lane; t <= tq; t += 32) {
    const int x = t == 0 ? e : node_at(t);
    w.parent[x] = (short)w.stage[t];
    w.flow[x] = sflow[t];
    w.acost[x] = scost[t];
  }
  __syncwarp();
  return true;
}

template <int MODE, int DP>
__global__ void __launch_bounds__(kEmdWarps * 32, 3) emd_kernel(const __grid_constant__ EmdArgs a) {
  extern __shared__ __align__(16) unsigned char emd_smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const int NM = a.nmax;
  Prob<MODE, DP> P;
  P.a = &a;
  P.w = carve(emd_smem + (size_t)wib * emd_slice_bytes(NM, DP), NM, DP);
  P.NM = NM;
  const EmdWarp &w = P.w;
  for (long long p = (long long)blockIdx.x * wpb + wib; p < a.npairs; p += (long long)gridDim.x * wpb) {
    const int ro = __ldg(a.prow + p), co = __ldg(a.pcol + p);
    const int n = a.rstr ? __ldg(a.rstr + ro) : a.rfix;
    const int m = a.cstr ? __ldg(a.cstr + co) : a.cfix;
    const size_t r0 = a.rcum ? __ldg(a.rcum + ro) : (size_t)ro * a.rfix;
    const size_t c0 = a.ccum ? __ldg(a.ccum + co) : (size_t)co * a.cfix;
    const int N = n + m;
    if (n <= 0 || m <= 0 || N > NM) {
      if (lane == 0) {
        a.out[p] = n <= 0 || m <= 0 ? 0.0 : NAN;
        a.piv[p] = n <= 0 || m <= 0 ? 0 : -2;
      }
      continue;
    }
    P.n = n;
    P.m = m;
    P.N = N;
    P.r0 = r0;
    P.c0 = c0;
    if constexpr (MODE == EMD_TABLE) {
      P.tb = a.T32;
      P.sR = a.V;
      P.sC = 1;
    } else if constexpr (MODE == EMD_EMBED) {  // T[row object][word][row support]
      P.tb = a.T32 + (size_t)ro * a.V * a.tm;
      P.sR = 1;
      P.sC = a.tm;
    }
    // stage weights (p64) and supports (centred on the rows' mean, FP32) or
    // table keys; the cost scale bounds every cell's cost
    float scale;
    if constexpr (MODE == EMD_EUCLID) {
      const int d = a.dim;
      double ctr[DP - 1];
#pragma unroll
      for (int t = 0; t < DP - 1; ++t) ctr[t] = 0.0;
      for (int x = lane; x < n; x += 32)
#pragma unroll
        for (int t = 0; t < DP - 1; ++t)
          if (t < d) ctr[t] += __ldg(a.rsupp + (r0 + x) * d + t);
#pragma unroll
      for (int t = 0; t < DP - 1; ++t) {
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) ctr[t] += __shfl_xor_sync(0xffffffffu, ctr[t], o);
        ctr[t] /= n;
      }
      float nr = 0.f, nc = 0.f;
      for (int x = lane; x < N; x += 32) {
        const bool row = x < n;
        const size_t g = row ? r0 + x : c0 + (x - n);
        w.p64[x] = __ldg((row ? a.rw : a.cw) + g);
        const double *s = (row ? a.rsupp : a.csupp) + g * d;
        float *dst = w.dat + (size_t)x * DP;
        float nrm = 0.f;
#pragma unroll
        for (int t = 0; t < DP - 1; ++t) {
          const float v = t < d ? (float)(__ldg(s + t) - ctr[t]) : 0.f;
          dst[t] = v;
          nrm = fmaf(v, v, nrm);
        }
        dst[DP - 1] = 0.f;
        if (row)
          nr = fmaxf(nr, nrm);
        else
          nc = fmaxf(nc, nrm);
      }
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        nr = fmaxf(nr, __shfl_xor_sync(0xffffffffu, nr, o));
        nc = fmaxf(nc, __shfl_xor_sync(0xffffffffu, nc, o));
      }
      const float rad = sqrtf(nr) + sqrtf(nc);
      scale = rad * rad;
    } else {
      for (int x = lane; x < N; x += 32) {
        const bool row = x < n;
        const size_t g = row ? r0 + x : c0 + (x - n);
        w.p64[x] = __ldg((row ? a.rw : a.cw) + g);
        const int *sym = row ? a.rsym : a.csym;
        // keys: bin / word ids, else the support's index in its object (rows,
        // tables) or its global index less key_off (embedding-mode columns)
        const int key = sym ? __ldg(sym + g)
                            : (row ? x : (MODE == EMD_EMBED ? (int)(g - a.key_off) : x - n));
        w.dat[2 * x] = __int_as_float(key);
        w.dat[2 * x + 1] = 0.f;
      }
      scale = a.tscale;
    }
    __syncwarp();
    int piv = 0, status = row_min_start(P, lane) ? 0 : -3;
    scale = fmaxf(scale, 1e-30f);
    const float tol32 = 1e-5f * scale;
    const double tol64 = 1e-12 * (double)scale;
    // lanes over rows, columns or cells: whichever keeps more lanes busy
    const float ur = (float)n / (32 * ((n + 31) / 32)), uc = (float)m / (32 * ((m + 31) / 32));
    const int map = fmaxf(ur, uc) < 0.7f ? 2 : (ur >= uc ? 0 : 1);
    bool f64 = false;
    while (status == 0) {
      Best b;
      if (!f64) {
        potentials<MODE, DP, false>(P, lane);
        b = price32(P, lane, map);
        if (!(b.v < -tol32)) {
          f64 = true;
          continue;
        }
      } else {
        potentials<MODE, DP, true>(P, lane);
        b = price64(P, lane, tol64, scale);
        if (b.idx == 0x7fffffff) break;
      }
      if (++piv > a.max_piv) {
        status = -1;
        break;
      }
      if (!pivot(P, lane, b.idx / m, b.idx % m)) {
        status = -3;
        break;
      }
    }
    // cost over the tree arcs, FP64, fixed order
    double obj = 0.0;
    if (status == 0) {
      for (int x = lane; x < N; x += 32) {
        const int px = w.parent[x];
        if (px >= 0) obj += w.flow[x] * P.arc_c64(x, px);
      }
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) obj += __shfl_xor_sync(0xffffffffu, obj, o);
    }
    if (lane == 0) {
      a.out[p] = status == 0 ? obj : NAN;
      a.piv[p] = status == 0 ? piv : status;
    }
    __syncwarp();
  }
}

template <int MODE, int DP>
cudaError_t launch_emd_t(const EmdArgs &a, cudaStream_t st) {
  const size_t slice = emd_slice_bytes(a.nmax, DP);
  auto kern = emd_kernel<MODE, DP>;
  int dev = 0, sms = 0, smem_sm = 0;
  if (cudaError_t e = launch_device(&dev); e != cudaSuccess) return e;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  // warps per block: the most warps per SM that the shared memory holds
  int best_w = 0, wpb = 0;
  for (int cand = kEmdWarps; cand >= 1; --cand) {
    const size_t smem = (size_t)cand * slice;
    if (smem > (size_t)kEmdSmemLimit) continue;
    const int blocks = (int)((size_t)smem_sm / (smem + 1024));
    const int warps = blocks * cand > 64 ? 64 : blocks * cand;
    if (warps > best_w) {
      best_w = warps;
      wpb = cand;
    }
  }
  if (wpb < 1) return cudaErrorInvalidValue;
  const size_t smem = (size_t)wpb * slice;
  static size_t configured[kMaxDevices] = {};
  {  // the attribute only grows; calls from other host threads see it set first
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (smem > configured[dev]) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      configured[dev] = smem;
    }
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, wpb * 32, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const long long need = (a.npairs + wpb - 1) / wpb;
  const long long grid = need < (long long)per_sm * sms ? need : (long long)per_sm * sms;
  if (grid <= 0) return cudaSuccess;
  kern<<<(unsigned)grid, wpb * 32, smem, st>>>(a);
  return cudaGetLastError();
}

}  // namespace

size_t emd_slice(int nmax, int mode, int dim) {
  const int DP = mode == EMD_EUCLID ? (dim <= 3 ? 4 : 8) : 0;
  return emd_slice_bytes(nmax, DP);
}

cudaError_t launch_emd(const EmdArgs &a, cudaStream_t st) {
  if (a.npairs <= 0) return cudaSuccess;
  if (a.mode == EMD_EUCLID) {
    if (a.dim <= 3) return launch_emd_t<EMD_EUCLID, 4>(a, st);
    if (a.dim <= 7) return launch_emd_t<EMD_EUCLID, 8>(a, st);
    return cudaErrorInvalidValue;
  }
  if (a.mode == EMD_EMBED) return launch_emd_t<EMD_EMBED, 0>(a, st);
  return launch_emd_t<EMD_TABLE, 0>(a, st);
}

}  // namespace d2g
