"""The assignment step's exact transport costs (d2g_emd_pairs) from Python.

Mirrors the reference's d2_match_by_distmat (src/d2/solver_mosek.cc:61-226)
as d2_compute_distance calls it (src/d2/clustering.c:33-122): rows are the
first argument's supports (the centroid, or any object), columns the second
(the instance)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

EUCLIDEAN, HISTOGRAM, SPARSE_HISTOGRAM = 0, 5, 12


def _dists(keep, p_w, p_str=None, str_=0, p_supp=None, p_supp_sym=None):
    def arr(a, t):
        if a is None:
            return None
        a = np.ascontiguousarray(a, t)
        keep.append(a)
        return a.ctypes.data
    p_w = np.ascontiguousarray(p_w, np.float64)
    size = len(p_str) if p_str is not None else p_w.size // max(str_, 1)
    return L.d2g_dists(size, int(str_), arr(p_str, np.int32), arr(p_w, np.float64),
                       arr(p_supp, np.float64), arr(p_supp_sym, np.int32))


def emd_pairs(metric: int, rows: dict, cols: dict, pair_row, pair_col, dim: int = 0,
              dist_mat=None, with_pivots: bool = False):
    """Exact transport cost of each (rows object, cols object) pair.  ``rows``
    / ``cols``: dicts with ``p_w`` and either ``p_str`` or ``str`` (every
    object the same size), plus ``p_supp`` (Euclidean) or ``p_supp_sym``
    (sparse histogram bins)."""
    lib = L.load()
    keep = []
    R = _dists(keep, rows["p_w"], rows.get("p_str"), rows.get("str", 0), rows.get("p_supp"),
               rows.get("p_supp_sym"))
    Cc = _dists(keep, cols["p_w"], cols.get("p_str"), cols.get("str", 0), cols.get("p_supp"),
                cols.get("p_supp_sym"))
    pr = np.ascontiguousarray(pair_row, np.int32)
    pc = np.ascontiguousarray(pair_col, np.int32)
    npairs = pr.size
    cost = np.zeros(npairs)
    piv = np.zeros(npairs, np.int32)
    dm = None if dist_mat is None else np.ascontiguousarray(dist_mat, np.float64)
    V = 0 if dm is None else int(round(np.sqrt(dm.size)))
    L.check(lib.d2g_emd_pairs(int(metric), int(dim), C.byref(R), C.byref(Cc),
                              None if dm is None else dm.ctypes.data, V, npairs, pr.ctypes.data,
                              pc.ctypes.data, cost.ctypes.data, piv.ctypes.data), "d2g_emd_pairs")
    return (cost, piv) if with_pivots else cost
