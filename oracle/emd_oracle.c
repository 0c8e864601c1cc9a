/*
 * TEST INFRASTRUCTURE ONLY: exact discrete transport for the CPU oracle.
 *
 * The reference computes every instance-to-centroid distance of the
 * assignment step with d2_match_by_distmat (src/d2/solver_mosek.cc:61-226):
 * the linear program
 *     minimise  sum_ij C[i + j*n] x_ij
 *     s.t.      sum_j x_ij = wX[i]            (i < n, rows)
 *               sum_i x_ij = wY[j]            (j < m-1; the last column is
 *                                              left free, :64, :134-140)
 *               x >= 0
 * solved by MOSEK 7.1's network primal simplex (:115; MOSEK is a closed
 * third-party library, not part of the reference tree).  The optimum value
 * is unique, whatever the algorithm, so this oracle solves the same program
 * by successive shortest paths (Ahuja, Magnanti and Orlin, "Network Flows",
 * 1993, ch. 9.7): Dijkstra on reduced costs from a row with supply left,
 * augment to the nearest column with demand left, update the potentials;
 * each augmentation exhausts a row, a column or a reverse arc.  The last
 * column's demand is set to what the rows supply beyond the other columns,
 * which is the reference's dropped constraint.  All arithmetic is FP64.
 * Checked against scipy's HiGHS LP solver in tests/test_oracle_emd.py.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "d2_oracle.h"

double d2o_emd(int n, int m, const double *C, const double *wX, const double *wY, double *x_out) {
  if (n <= 0 || m <= 0) return 0.0;
  const int N = n + m;
  double *sup = (double *)malloc(sizeof(double) * n);
  double *dem = (double *)malloc(sizeof(double) * m);
  double *x = (double *)calloc((size_t)n * m, sizeof(double));
  double *pot = (double *)calloc(N, sizeof(double));
  double *dist = (double *)malloc(sizeof(double) * N);
  int *prev = (int *)malloc(sizeof(int) * N);
  char *done = (char *)malloc(N);
  double tot = 0.0;
  for (int i = 0; i < n; ++i) {
    sup[i] = wX[i];
    tot += wX[i];
  }
  double rest = tot;
  for (int j = 0; j < m - 1; ++j) {
    dem[j] = wY[j];
    rest -= wY[j];
  }
  dem[m - 1] = rest > 0.0 ? rest : 0.0;
  const double eps = 1e-14 * (tot > 0.0 ? tot : 1.0);
  /* nonnegative reduced costs for the empty flow: column potentials at their
     cheapest incoming arc */
  for (int j = 0; j < m; ++j) {
    double mn = DBL_MAX;
    for (int i = 0; i < n; ++i) mn = fmin(mn, C[i + (size_t)j * n]);
    pot[n + j] = mn;
  }
  for (int guard = 0; guard < 4 * N * N + 64; ++guard) {
    double left = 0.0;
    for (int i = 0; i < n; ++i) left += sup[i] > eps ? sup[i] : 0.0;
    if (left <= eps) break;
    /* Dijkstra over the residual graph; node ids: rows 0..n-1, columns n.. */
    for (int v = 0; v < N; ++v) {
      dist[v] = DBL_MAX;
      prev[v] = -1;
      done[v] = 0;
    }
    for (int i = 0; i < n; ++i)
      if (sup[i] > eps) { /* single source: the first row with supply left */
        dist[i] = 0.0;
        break;
      }
    int target = -1;
    for (;;) {
      int u = -1;
      double best = DBL_MAX;
      for (int v = 0; v < N; ++v)
        if (!done[v] && dist[v] < best) {
          best = dist[v];
          u = v;
        }
      if (u < 0) break;
      done[u] = 1;
      if (u >= n && dem[u - n] > eps) {
        target = u;
        break;
      }
      if (u < n) { /* forward arcs row u -> every column */
        for (int j = 0; j < m; ++j) {
          const int v = n + j;
          if (done[v]) continue;
          double rc = C[u + (size_t)j * n] + pot[u] - pot[v];
          if (rc < 0.0) rc = 0.0; /* rounding */
          if (dist[u] + rc < dist[v]) {
            dist[v] = dist[u] + rc;
            prev[v] = u;
          }
        }
      } else { /* reverse arcs column -> rows that ship to it */
        const int j = u - n;
        for (int i = 0; i < n; ++i) {
          if (done[i] || x[i + (size_t)j * n] <= 0.0) continue;
          double rc = -C[i + (size_t)j * n] - pot[i] + pot[u];
          if (rc < 0.0) rc = 0.0;
          if (dist[u] + rc < dist[i]) {
            dist[i] = dist[u] + rc;
            prev[i] = u;
          }
        }
      }
    }
    if (target < 0) break; /* nothing reachable: totals exhausted up to eps */
    const double dt = dist[target];
    for (int v = 0; v < N; ++v) pot[v] += (done[v] ? dist[v] : dt) - dt;
    /* bottleneck along the path */
    double delta = dem[target - n];
    int v = target;
    while (prev[v] >= 0) {
      const int u = prev[v];
      if (u >= n) { /* reverse arc column u -> row v */
        const double f = x[v + (size_t)(u - n) * n];
        if (f < delta) delta = f;
      }
      v = u;
    }
    if (sup[v] < delta) delta = sup[v];
    /* augment */
    v = target;
    while (prev[v] >= 0) {
      const int u = prev[v];
      if (u < n)
        x[u + (size_t)(v - n) * n] += delta;
      else
        x[v + (size_t)(u - n) * n] -= delta;
      v = u;
    }
    sup[v] -= delta;
    dem[target - n] -= delta;
  }
  double obj = 0.0;
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < n; ++i) obj += C[i + (size_t)j * n] * x[i + (size_t)j * n];
  if (x_out) memcpy(x_out, x, sizeof(double) * (size_t)n * m);
  free(sup);
  free(dem);
  free(x);
  free(pot);
  free(dist);
  free(prev);
  free(done);
  return obj;
}
