/*
 * TEST INFRASTRUCTURE ONLY: what src/d2/clustering.c needs from the MOSEK
 * solver module (src/d2/solver_mosek.cc, include/d2/solver.h) when the
 * reference is compiled here without MOSEK (a closed third-party library,
 * absent from the container).  d2_match_by_distmat solves the same linear
 * program (row sums wX, column sums wY but the last, x >= 0, cost C
 * column-major n x m) exactly with the oracle's successive-shortest-path
 * solver (emd_oracle.c); the optimum value is MOSEK's up to its tolerances.
 * The ADMM and gradient-descent centroid updates, deprecated in the
 * reference and not on the tested path, are stubs that refuse to run.
 */
#include <stdio.h>
#include <stdlib.h>

#include "d2/solver.h"
#include "d2_oracle.h"

void d2_solver_setup() {}
void d2_solver_release() {}

double d2_match_by_distmat(int n, int m, SCALAR *C, SCALAR *wX, SCALAR *wY, SCALAR *x,
                           SCALAR *lambda, size_t index) {
  (void)lambda;
  (void)index;
  return d2o_emd(n, m, C, wX, wY, x);
}

int d2_centroid_sphADMM() {
  fprintf(stderr, "ref_solver: the ADMM centroid update is not built\n");
  abort();
}
int d2_centroid_sphGradDecent() {
  fprintf(stderr, "ref_solver: the gradient-descent centroid update is not built\n");
  abort();
}
