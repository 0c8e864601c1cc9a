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
//    arc to its parent; initial tree from the north-west corner rule (the
//    last column takes whatever the rows still hold: its constraint is the
//    dropped one);
//  * node potentials (u_i + v_j = C_ij on tree arcs) by pointer jumping over
//    the parent array: log2(depth) rounds, all lanes, no traversal order to
//    maintain; depths come out of the same rounds;
//  * pricing: every cell's reduced cost C_ij - u_i - v_j, spread over the
//    warp's lanes, warp argmin (ties to the lowest cell index); FP32 costs
//    from supports staged in shared memory;
//  * pivot (lane 0): walk both ends of the entering cell up to their common
//    ancestor, ratio test over the arcs that lose flow (ties: the last
//    blocking arc met going round the cycle from the apex, the
//    strongly-feasible-tree choice that avoids cycling), update the flows,
//    re-hang the cut-off subtree by reversing the parent pointers from the
//    entering node to the leaving arc;
//  * exactness: when FP32 pricing finds no cell below -1e-5 of the cost
//    scale, the potentials are recomputed in FP64 from FP64 costs and every
//    cell is priced again in FP64; pivots continue in FP64 until no reduced
//    cost is below -1e-12 of the scale.  The cost is then sum x_ij C_ij over
//    the tree arcs in FP64, in a fixed order.
//
// A pair that has not reached optimality after max_piv pivots reports -1
// pivots and a NaN cost (-3: a tree walk ran past the node count, which a
// correct tree cannot do); the host turns either into an error.
#include <math.h>

#include "d2g_internal.cuh"

namespace d2g {

namespace {

constexpr int kEmdWarps = 8;               // warps per block at most (fewer when the slices are large)
constexpr int kEmdSmemLimit = 220 * 1024;  // dynamic shared memory per block

// per-node bytes of the shared-memory slice of one warp
__host__ __device__ constexpr int emd_node_bytes(int DP) {
  // flow, pot64 (weights first), acc64 second buffer: 3 doubles
  // acost, jacc[2]: 3 floats; jan[2], jdep[2], parent, depth: 6 shorts
  // data: DP floats (supports + potential), or key + potential for tables
  return 3 * 8 + 3 * 4 + 6 * 2 + (DP > 0 ? DP * 4 : 8);
}

__host__ __device__ inline size_t emd_slice_bytes(int nmax, int DP) {
  return ((size_t)nmax * emd_node_bytes(DP) + 15) & ~(size_t)15;
}

struct EmdWarp {
  double *flow, *p64, *q64;
  float *acost, *jacc0, *jacc1;
  short *jan0, *jan1, *jdep0, *jdep1, *parent, *depth;
  float *dat;  // DP floats per node (EUCLID) or {key bits, pot} (TABLE)
};

__device__ inline EmdWarp carve(unsigned char *p, int NM, int DP) {
  EmdWarp w;
  w.dat = (float *)p;
  p += (size_t)NM * (DP > 0 ? DP * 4 : 8);
  w.flow = (double *)p;
  p += (size_t)NM * 8;
  w.p64 = (double *)p;
  p += (size_t)NM * 8;
  w.q64 = (double *)p;
  p += (size_t)NM * 8;
  w.acost = (float *)p;
  p += (size_t)NM * 4;
  w.jacc0 = (float *)p;
  p += (size_t)NM * 4;
  w.jacc1 = (float *)p;
  p += (size_t)NM * 4;
  w.jan0 = (short *)p;
  p += (size_t)NM * 2;
  w.jan1 = (short *)p;
  p += (size_t)NM * 2;
  w.jdep0 = (short *)p;
  p += (size_t)NM * 2;
  w.jdep1 = (short *)p;
  p += (size_t)NM * 2;
  w.parent = (short *)p;
  p += (size_t)NM * 2;
  w.depth = (short *)p;
  return w;
}

// cost access for one problem
template <int MODE, int DP>
struct Costs {
  const EmdArgs *a;
  EmdWarp w;
  int n;
  size_t r0, c0;  // first support of the row / column object
  const float *T32;
  const double *T64;

  // FP32 cost from the staged node data
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
      return __ldg(T32 + (size_t)ki * a->V + kj);
    }
  }
  // FP64 cost, the reference's difference form (_dpdist2, blas_like64.c:199-208)
  __device__ inline double c64(int i, int j) const {
    if constexpr (MODE == EMD_EUCLID) {
      const int d = a->dim;
      const double *x = a->rsupp + (r0 + i) * d, *y = a->csupp + (c0 + j) * d;
      double s = 0.0;
      for (int t = 0; t < d; ++t) {
        const double v = __ldg(x + t) - __ldg(y + t);
        s += v * v;
      }
      return s;
    } else {
      const int ki = __float_as_int(w.dat[2 * i]), kj = __float_as_int(w.dat[2 * (n + j)]);
      return __ldg(T64 + (size_t)ki * a->V + kj);
    }
  }
  __device__ inline void set_pot(int x, float p) const {
    if constexpr (MODE == EMD_EUCLID)
      w.dat[(size_t)x * DP + DP - 1] = p;
    else
      w.dat[2 * x + 1] = p;
  }
  __device__ inline float pot(int x) const {
    if constexpr (MODE == EMD_EUCLID)
      return w.dat[(size_t)x * DP + DP - 1];
    else
      return w.dat[2 * x + 1];
  }
};

// cost of node x's tree arc (x and its parent: one row, one column)
template <int MODE, int DP>
__device__ inline double arc_c64(const Costs<MODE, DP> &cs, int x, int px) {
  const int n = cs.n;
  return x < n ? cs.c64(x, px - n) : cs.c64(px, x - n);
}

// Potentials by pointer jumping: pot[x] = acc + (-1)^dep * pot[anc] until
// every anc is the root's -1.  FP32 (acc in jacc, costs from acost) or FP64
// (acc in p64 / q64, costs recomputed).  Leaves depths in w.depth.
template <int MODE, int DP, bool F64>
__device__ void potentials(const Costs<MODE, DP> &cs, int N, int lane) {
  const EmdWarp &w = cs.w;
  for (int x = lane; x < N; x += 32) {
    const int px = w.parent[x];
    w.jan0[x] = (short)px;
    w.jdep0[x] = px < 0 ? 0 : 1;
    if (F64)
      w.p64[x] = px < 0 ? 0.0 : arc_c64(cs, x, px);
    else
      w.jacc0[x] = px < 0 ? 0.f : w.acost[x];
  }
  __syncwarp();
  int cur = 0;
  for (int round = 0; round < 16; ++round) {
    const short *an = cur ? w.jan1 : w.jan0;
    const short *dp = cur ? w.jdep1 : w.jdep0;
    short *an2 = cur ? w.jan0 : w.jan1;
    short *dp2 = cur ? w.jdep0 : w.jdep1;
    bool more = false;
    for (int x = lane; x < N; x += 32) {
      const int a0 = an[x];
      const int d0 = dp[x];
      if (a0 < 0) {
        an2[x] = -1;
        dp2[x] = (short)d0;
        if (F64)
          (cur ? w.p64 : w.q64)[x] = (cur ? w.q64 : w.p64)[x];
        else
          (cur ? w.jacc0 : w.jacc1)[x] = (cur ? w.jacc1 : w.jacc0)[x];
        continue;
      }
      const int a1 = an[a0];
      if (F64) {
        const double *ac = cur ? w.q64 : w.p64;
        double *ac2 = cur ? w.p64 : w.q64;
        ac2[x] = (d0 & 1) ? ac[x] - ac[a0] : ac[x] + ac[a0];
      } else {
        const float *ac = cur ? w.jacc1 : w.jacc0;
        float *ac2 = cur ? w.jacc0 : w.jacc1;
        ac2[x] = (d0 & 1) ? ac[x] - ac[a0] : ac[x] + ac[a0];
      }
      an2[x] = (short)a1;
      dp2[x] = (short)(d0 + dp[a0]);
      more |= a1 >= 0;
    }
    __syncwarp();
    cur ^= 1;
    if (!__any_sync(0xffffffffu, more)) break;
  }
  // results in buffer `cur`
  const short *dp = cur ? w.jdep1 : w.jdep0;
  for (int x = lane; x < N; x += 32) {
    w.depth[x] = dp[x];
    if (F64) {
      if (cur) w.p64[x] = w.q64[x];
    } else {
      cs.set_pot(x, cur ? w.jacc1[x] : w.jacc0[x]);
    }
  }
  __syncwarp();
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

// FP32 pricing: the cell with the most negative reduced cost
template <int MODE, int DP>
__device__ Best price32(const Costs<MODE, DP> &cs, int n, int m, int lane) {
  Best b{INFINITY, 0x7fffffff};
  if (m <= 32) {
    const int mp = m <= 1 ? 1 : 1 << (32 - __clz(m - 1));
    const int R = 32 / mp;
    const int j = lane & (mp - 1);
    if (j < m) {
      const float vj = cs.pot(n + j);
      for (int i = lane / mp; i < n; i += R) {
        const float r = cs.c32(i, j) - cs.pot(i) - vj;
        better(b, r, i * m + j);
      }
    }
  } else {
    for (int j = lane; j < m; j += 32) {
      const float vj = cs.pot(n + j);
      for (int i = 0; i < n; ++i) {
        const float r = cs.c32(i, j) - cs.pot(i) - vj;
        better(b, r, i * m + j);
      }
    }
  }
  return warp_best(b);
}

// FP64 pricing, potentials in p64
template <int MODE, int DP>
__device__ Best price64(const Costs<MODE, DP> &cs, int n, int m, int lane, double tol) {
  double bv = INFINITY;
  int bi = 0x7fffffff;
  const int cells = n * m;
  for (int c = lane; c < cells; c += 32) {
    const int i = c / m, j = c - i * m;
    const double r = cs.c64(i, j) - cs.w.p64[i] - cs.w.p64[n + j];
    if (r < bv) {
      bv = r;
      bi = c;
    }
  }
  Best b{bv < -tol ? (float)(bv / tol) : INFINITY, bv < -tol ? bi : 0x7fffffff};
  // ties on the scaled value fall to the lowest index
  return warp_best(b);
}

// the maximum FP32 cost (tolerance scale)
template <int MODE, int DP>
__device__ float cost_scale(const Costs<MODE, DP> &cs, int n, int m, int lane) {
  float s = 0.f;
  for (int c = lane; c < n * m; c += 32) {
    const int i = c / m, j = c - i * m;
    s = fmaxf(s, fabsf(cs.c32(i, j)));
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) s = fmaxf(s, __shfl_xor_sync(0xffffffffu, s, o));
  return s;
}

// north-west corner start (lane 0); weights staged in p64
template <int MODE, int DP>
__device__ void nw_corner(const Costs<MODE, DP> &cs, int n, int m) {
  const EmdWarp &w = cs.w;
  w.parent[0] = -1;
  w.flow[0] = 0.0;
  w.acost[0] = 0.f;
  int r = 0, c = 0, cur = n;  // node holding the current cell's arc
  double s = w.p64[0], d = m == 1 ? INFINITY : w.p64[n];
  w.parent[n] = 0;
  w.acost[n] = cs.c32(0, 0);
  for (;;) {
    const double f = fmin(s, d);
    w.flow[cur] = f;
    s -= f;
    d -= f;
    if (r == n - 1 && c == m - 1) break;
    if (c == m - 1 || (r < n - 1 && s <= d)) {
      ++r;
      s = w.p64[r];
      w.parent[r] = (short)(n + c);
      w.acost[r] = cs.c32(r, c);
      cur = r;
    } else {
      ++c;
      d = c == m - 1 ? INFINITY : w.p64[n + c];
      w.parent[n + c] = (short)r;
      w.acost[n + c] = cs.c32(r, c);
      cur = n + c;
    }
  }
}

// one pivot on cell (ei, ej) (lane 0); false if a walk outgrows the tree
// (a broken tree: every walk is bounded by the node count)
template <int MODE, int DP>
__device__ bool pivot(const Costs<MODE, DP> &cs, int n, int N, int ei, int ej) {
  const EmdWarp &w = cs.w;
  const int ni = ei, nj = n + ej;
  // ratio test: arcs at even positions from either end lose flow
  double theta = INFINITY;
  int q = -1, qkey = -2147483647;
  {
    int a = ni, b = nj, ta = 0, tb = 0;
    int da = w.depth[a], db = w.depth[b];
    auto visit_i = [&](int x, int t) {  // i side, position t from ei
      if (t & 1) return;
      const double f = w.flow[x];
      const int key = -t;  // nearest ei is last on this side
      if (f < theta || (f == theta && key > qkey)) {
        theta = f;
        q = x;
        qkey = key;
      }
    };
    auto visit_j = [&](int x, int t) {  // j side, position t from ej
      if (t & 1) return;
      const double f = w.flow[x];
      const int key = 1000000 + t;  // j side after i side, nearest the apex last
      if (f < theta || (f == theta && key > qkey)) {
        theta = f;
        q = x;
        qkey = key;
      }
    };
    if (da >= N || db >= N) return false;
    while (da > db) {
      visit_i(a, ta++);
      a = w.parent[a];
      --da;
    }
    while (db > da) {
      visit_j(b, tb++);
      b = w.parent[b];
      --db;
    }
    while (a != b) {
      if (a < 0 || b < 0 || ta + tb > N) return false;
      visit_i(a, ta++);
      a = w.parent[a];
      visit_j(b, tb++);
      b = w.parent[b];
    }
    if (q < 0) return false;
  }
  // flows along the cycle
  {
    int a = ni, b = nj, ta = 0, tb = 0;
    int da = w.depth[a], db = w.depth[b];
    while (da > db) {
      w.flow[a] += (ta++ & 1) ? theta : -theta;
      a = w.parent[a];
      --da;
    }
    while (db > da) {
      w.flow[b] += (tb++ & 1) ? theta : -theta;
      b = w.parent[b];
      --db;
    }
    while (a != b) {
      w.flow[a] += (ta++ & 1) ? theta : -theta;
      a = w.parent[a];
      w.flow[b] += (tb++ & 1) ? theta : -theta;
      b = w.parent[b];
    }
  }
  // q's arc leaves; the endpoint below it is re-hung from the other endpoint
  const bool jside = qkey >= 1000000;
  const int e = jside ? nj : ni, o = jside ? ni : nj;
  double pf = theta;
  float pc = cs.c32(ei, ej);
  int px = o, x = e;
  for (int step = 0;; ++step) {
    if (x < 0 || step > N) return false;
    const int nx = w.parent[x];
    const double tf = w.flow[x];
    const float tc = w.acost[x];
    w.parent[x] = (short)px;
    w.flow[x] = pf;
    w.acost[x] = pc;
    if (x == q) break;
    px = x;
    pf = tf;
    pc = tc;
    x = nx;
  }
  return true;
}

template <int MODE, int DP>
__global__ void __launch_bounds__(kEmdWarps * 32) emd_kernel(const __grid_constant__ EmdArgs a) {
  extern __shared__ __align__(16) unsigned char emd_smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const int NM = a.nmax;
  Costs<MODE, DP> cs;
  cs.a = &a;
  cs.w = carve(emd_smem + (size_t)wib * emd_slice_bytes(NM, DP), NM, DP);
  cs.T32 = a.T32;
  cs.T64 = a.T64;
  const EmdWarp &w = cs.w;
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
    cs.n = n;
    cs.r0 = r0;
    cs.c0 = c0;
    // stage weights (p64) and FP32 supports / table keys
    for (int x = lane; x < N; x += 32) {
      const bool row = x < n;
      const size_t g = row ? r0 + x : c0 + (x - n);
      w.p64[x] = __ldg((row ? a.rw : a.cw) + g);
      if constexpr (MODE == EMD_EUCLID) {
        const double *s = (row ? a.rsupp : a.csupp) + g * a.dim;
        float *dst = w.dat + (size_t)x * DP;
#pragma unroll
        for (int t = 0; t < DP - 1; ++t) dst[t] = t < a.dim ? (float)__ldg(s + t) : 0.f;
        dst[DP - 1] = 0.f;
      } else {
        const int *sym = row ? a.rsym : a.csym;
        const int key = sym ? __ldg(sym + g) : (row ? x : x - n);
        w.dat[2 * x] = __int_as_float(key);
        w.dat[2 * x + 1] = 0.f;
      }
    }
    __syncwarp();
    if (lane == 0) nw_corner(cs, n, m);
    __syncwarp();
    const float scale = fmaxf(cost_scale(cs, n, m, lane), 1e-30f);
    const float tol32 = 1e-5f * scale;
    const double tol64 = 1e-12 * (double)scale;
    int piv = 0, status = 0;
    bool f64 = false;
    for (;;) {
      Best b;
      if (!f64) {
        potentials<MODE, DP, false>(cs, N, lane);
        b = price32(cs, n, m, lane);
        if (!(b.v < -tol32)) {
          f64 = true;
          continue;
        }
      } else {
        potentials<MODE, DP, true>(cs, N, lane);
        b = price64(cs, n, m, lane, tol64);
        if (b.idx == 0x7fffffff) break;
      }
      if (++piv > a.max_piv) {
        status = -1;
        break;
      }
      int ok = 1;
      if (lane == 0) ok = pivot(cs, n, N, b.idx / m, b.idx % m);
      __syncwarp();
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) {
        status = -3;
        break;
      }
    }
    // cost over the tree arcs, FP64, fixed order
    double obj = 0.0;
    if (status == 0) {
      for (int x = lane; x < N; x += 32) {
        const int px = w.parent[x];
        if (px >= 0) obj += w.flow[x] * arc_c64(cs, x, px);
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
  int wpb = (int)((size_t)kEmdSmemLimit / slice);
  if (wpb > kEmdWarps) wpb = kEmdWarps;
  if (wpb < 1) return cudaErrorInvalidValue;
  const size_t smem = (size_t)wpb * slice;
  auto kern = emd_kernel<MODE, DP>;
  static size_t configured = 0;
  if (smem > configured) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = smem;
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, wpb * 32, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
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
  return launch_emd_t<EMD_TABLE, 0>(a, st);
}

}  // namespace d2g
