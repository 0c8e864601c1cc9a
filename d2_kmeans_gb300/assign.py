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


# ---------------------------------------------------------------------------
# the reference's structures for the assignment step (include/d2g.h, the
# layout of include/d2/clustering.h)

class Mph:
    """An mph (instances or centroids) built from per-phase dicts: ``metric``,
    ``dim``, ``str``, ``p_w`` and ``p_str`` (or every object ``str``
    supports), plus ``p_supp`` / ``p_supp_sym`` / ``dist_mat`` +
    ``vocab_size`` as the metric needs."""

    def __init__(self, phases, size: int, label=None, num_of_labels: int = 0):
        self.keep = []
        self.size = int(size)
        self.arrays = []  # per phase: the numpy arrays the mph points into
        sphs = (L.sph * len(phases))()
        for n, ph in enumerate(phases):
            s = sphs[n]
            arrs = {}
            self.arrays.append(arrs)
            p_str = np.ascontiguousarray(ph["p_str"] if ph.get("p_str") is not None
                                         else np.full(self.size, ph["str"]), np.int32)
            cum = np.zeros(self.size, np.uint64)
            cum[1:] = np.cumsum(p_str[:-1])
            s.dim = int(ph.get("dim", 0))
            s.str = int(ph["str"])
            s.max_str = int(p_str.max()) if p_str.size else 0
            s.col = int(p_str.sum())
            s.max_col = s.col
            s.p_str = self._ptr(p_str, C.c_int)
            s.p_str_cum = self._ptr(cum, C.c_size_t)
            arrs["p_w"] = np.array(ph["p_w"], np.float64)
            s.p_w = self._ptr(arrs["p_w"], C.c_double)
            s.metric_type = int(ph["metric"])
            if ph.get("p_supp") is not None:
                arrs["p_supp"] = np.array(ph["p_supp"], np.float64)
                s.p_supp = self._ptr(arrs["p_supp"], C.c_double)
            if ph.get("p_supp_sym") is not None:
                arrs["p_supp_sym"] = np.array(ph["p_supp_sym"], np.int32)
                s.p_supp_sym = self._ptr(arrs["p_supp_sym"], C.c_int)
            if ph.get("dist_mat") is not None:
                s.dist_mat = self._ptr(np.ascontiguousarray(ph["dist_mat"], np.float64), C.c_double)
            if ph.get("vocab_vec") is not None:
                s.vocab_vec = self._ptr(np.ascontiguousarray(ph["vocab_vec"], np.float64), C.c_double)
            s.vocab_size = int(ph.get("vocab_size", 0))
        self.sphs = sphs
        self.label = np.ascontiguousarray(label if label is not None else np.full(self.size, -1),
                                          np.int32)
        m = L.mph()
        m.s_ph = len(phases)
        m.size = self.size
        m.global_size = self.size
        m.label = self.label.ctypes.data_as(C.POINTER(C.c_int))
        m.num_of_labels = int(num_of_labels)
        m.ph = C.cast(sphs, C.POINTER(L.sph))
        self.mph = m

    def _ptr(self, a, t):
        self.keep.append(a)
        return a.ctypes.data_as(C.POINTER(t))


class Work:
    """A var_mph holding what the assignment step reads and writes:
    label_switch and the triangle-inequality bounds (tr), initialised as
    d2_allocate_work does (clustering_util.c:218-228)."""

    def __init__(self, size: int, k: int, s_ph: int, cost_scratch=None):
        """``cost_scratch``: per phase, the g_var[n].C array the reference's
        own d2_compute_distance writes its cost blocks into (and reads the
        precomputed sparse-histogram costs from); this library needs none."""
        self.label_switch = np.zeros(size, np.int8)
        self.l = np.zeros(size * k)
        self.u = np.full(size, np.finfo(np.float64).max)
        self.s = np.zeros(k)
        self.c = np.zeros(k * k)
        self.r = np.ones(size, np.int8)
        w = L.var_mph()
        w.s_ph = s_ph
        w.label_switch = self.label_switch.ctypes.data_as(C.POINTER(C.c_char))
        w.tr.l = self.l.ctypes.data_as(C.POINTER(C.c_double))
        w.tr.u = self.u.ctypes.data_as(C.POINTER(C.c_double))
        w.tr.s = self.s.ctypes.data_as(C.POINTER(C.c_double))
        w.tr.c = self.c.ctypes.data_as(C.POINTER(C.c_double))
        w.tr.r = C.cast(self.r.ctypes.data, C.c_char_p)
        if cost_scratch is not None:
            self.scratch = [np.ascontiguousarray(a, np.float64) for a in cost_scratch]
            gv = (L.var_sph * s_ph)()
            for n, a in enumerate(self.scratch):
                gv[n].C = a.ctypes.data_as(C.POINTER(C.c_double))
            self.gv = gv
            w.g_var = C.cast(gv, C.POINTER(L.var_sph))
        self.var = w

    def state(self):
        return {k: getattr(self, k).copy() for k in ("label_switch", "l", "u", "s", "c", "r")}


def labeling(data: Mph, cents: Mph, work: Work, selected_phase: int = -1):
    """d2g_labeling: returns (labels changed, sum of squared nearest distances)."""
    lib = L.load()
    cnt, cost = C.c_size_t(), C.c_double()
    L.check(lib.d2g_labeling(C.byref(data.mph), C.byref(cents.mph), C.byref(work.var),
                             int(selected_phase), C.byref(cnt), C.byref(cost)), "d2g_labeling")
    return cnt.value, cost.value


def labeling_prep(data: Mph, cents: Mph, work: Work, selected_phase: int = -1):
    """d2g_labeling_prep: returns (labels changed, distances computed)."""
    lib = L.load()
    cnt, dc = C.c_size_t(), C.c_size_t()
    L.check(lib.d2g_labeling_prep(C.byref(data.mph), C.byref(cents.mph), C.byref(work.var),
                                  int(selected_phase), C.byref(cnt), C.byref(dc)),
            "d2g_labeling_prep")
    return cnt.value, dc.value


def labeling_post(data: Mph, c_old: Mph, c_new: Mph, work: Work, selected_phase: int = -1):
    lib = L.load()
    L.check(lib.d2g_labeling_post(C.byref(data.mph), C.byref(c_old.mph), C.byref(c_new.mph),
                                  C.byref(work.var), int(selected_phase)), "d2g_labeling_post")


def compute_distances(a: Mph, b: Mph, ia, jb, selected_phase: int = -1):
    lib = L.load()
    ia = np.ascontiguousarray(ia, np.int32)
    jb = np.ascontiguousarray(jb, np.int32)
    out = np.zeros(ia.size)
    L.check(lib.d2g_compute_distances(C.byref(a.mph), C.byref(b.mph), int(selected_phase), ia.size,
                                      ia.ctypes.data, jb.ctypes.data, out.ctypes.data),
            "d2g_compute_distances")
    return out


def clustering(data: Mph, cents: Mph, k: int, max_iter: int, use_triangle: bool = True,
               selected_phase: int = -1, log_file: str | None = None) -> int:
    """d2g_clustering (the reference's d2_clustering loop) on the GPU; the
    centroids' arrays and the instances' labels are updated in place.
    Returns the number of rounds run."""
    lib = L.load()
    rounds = C.c_int()
    L.check(lib.d2g_clustering(int(k), int(max_iter), C.byref(data.mph), C.byref(cents.mph),
                               int(selected_phase), int(bool(use_triangle)),
                               log_file.encode() if log_file else None, C.byref(rounds)),
            "d2g_clustering")
    return rounds.value
