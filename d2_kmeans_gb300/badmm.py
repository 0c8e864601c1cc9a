"""Python mirror of the reference's B-ADMM centroid-update interface.

Two ways in, both through libd2g.so's C ABI:

* :class:`DropIn` builds the reference's own structures (``mph``, ``sph``,
  ``var_mph``, ``var_sphBregman``) and calls the drop-in
  ``d2_centroid_sphBregman`` exactly as the reference's ``d2_clustering``
  does (src/d2/clustering.c:488-498), including the warm start through
  ``label_switch`` and the plans ``Z`` kept in the work object.
* :class:`Phase` is the resident API: supports, weights and plans stay in HBM
  across calls.

A phase is described by a dict with the reference's array names (``p_str``,
``p_w``, ``p_supp`` or ``p_supp_sym`` + ``vocab_vec``, ``dist_mat``,
``label``, ``num_of_labels``, ``metric``, ``dim``, ``str``); centroids by a
dict with ``c_w`` (k*str) and ``c_supp`` (k*str*dim), or for n-gram phases
the integer symbols ``c_sym`` (k*str*dim).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def _arr(a, dtype):
    return None if a is None else np.ascontiguousarray(a, dtype=dtype)


def set_config(**kw) -> dict:
    """Update the library configuration (precision, verbose, use_graph,
    sync_scratch, profile, cost_gemm, keep_time_budget); returns the previous
    values."""
    lib = L.load()
    cfg = L.d2g_config()
    L.check(lib.d2g_get_config(C.byref(cfg)), "d2g_get_config")
    old = {f: getattr(cfg, f) for f, _ in L.d2g_config._fields_}
    for k, v in kw.items():
        setattr(cfg, k, int(v))
    L.check(lib.d2g_set_config(C.byref(cfg)), "d2g_set_config")
    return old


def get_config() -> dict:
    lib = L.load()
    cfg = L.d2g_config()
    L.check(lib.d2g_get_config(C.byref(cfg)), "d2g_get_config")
    return {f: getattr(cfg, f) for f, _ in L.d2g_config._fields_}


def _metric(v):
    names = {"euclidean": 0, "histogram": 5, "ngram": 6, "embed": 7, "sparse_histogram": 12}
    return names[v] if isinstance(v, str) else int(v)


class Phase:
    """One phase resident on the GPU (d2g_phase_*)."""

    def __init__(self, phase: dict, precision: int = 0):
        self.lib = L.load()
        self._keep = []
        p_str = _arr(phase["p_str"], np.int32)
        self.size = p_str.size
        self.col = int(p_str.sum())
        self.str = int(phase["str"])
        self.dim = int(phase.get("dim", 0))
        self.k = int(phase["num_of_labels"])
        self.metric = _metric(phase["metric"])
        d = L.d2g_phase_desc()
        d.metric_type = self.metric
        d.dim = self.dim
        d.str = self.str
        d.size = self.size
        arrays = dict(p_str=p_str, p_w=_arr(phase["p_w"], np.float64),
                      p_supp=_arr(phase.get("p_supp"), np.float64),
                      p_supp_sym=_arr(phase.get("p_supp_sym"), np.int32),
                      vocab_vec=_arr(phase.get("vocab_vec"), np.float64),
                      dist_mat=_arr(phase.get("dist_mat"), np.float64),
                      label=_arr(phase["label"], np.int32))
        for name, a in arrays.items():
            setattr(d, name, None if a is None else a.ctypes.data)
        d.vocab_size = int(phase.get("vocab_size", 0))
        d.num_of_labels = self.k
        d.global_size = int(phase.get("global_size", 0))
        h = C.c_void_p()
        L.check(self.lib.d2g_phase_create(C.byref(d), int(precision), C.byref(h)), "d2g_phase_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.d2g_phase_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_labels(self, label):
        lab = _arr(label, np.int32)
        L.check(self.lib.d2g_phase_set_labels(self.h, lab.ctypes.data), "d2g_phase_set_labels")

    def set_plans(self, Z):
        Z = _arr(Z, np.float64)
        L.check(self.lib.d2g_phase_set_plans(self.h, Z.ctypes.data), "d2g_phase_set_plans")

    def get_plans(self) -> np.ndarray:
        Z = np.empty(self.str * self.col)
        L.check(self.lib.d2g_phase_get_plans(self.h, Z.ctypes.data), "d2g_phase_get_plans")
        return Z

    def get_scratch(self, X=True, Y=True, Cm=True):
        n = self.str * self.col
        out = {k: (np.empty(n) if want else None) for k, want in (("X", X), ("Y", Y), ("C", Cm))}
        L.check(self.lib.d2g_phase_get_scratch(
            self.h, *(None if out[k] is None else out[k].ctypes.data for k in ("X", "Y", "C"))),
            "d2g_phase_get_scratch")
        return out

    def stream(self) -> int:
        """cudaStream_t (as an integer) that this phase's kernels run on."""
        return self.lib.d2g_phase_stream(self.h) or 0

    def tuning(self) -> dict:
        """Launch-shape choices of this phase (d2g_tuning)."""
        t = L.d2g_tuning()
        L.check(self.lib.d2g_phase_get_tuning(self.h, C.byref(t)), "d2g_phase_get_tuning")
        return {f: getattr(t, f) for f, _ in L.d2g_tuning._fields_}

    def set_tuning(self, **kw) -> dict:
        old = self.tuning()
        t = L.d2g_tuning(**dict(old, **{k: int(v) for k, v in kw.items()}))
        L.check(self.lib.d2g_phase_set_tuning(self.h, C.byref(t)), "d2g_phase_set_tuning")
        return old

    def autotune(self, centroids: dict, opts: dict) -> dict:
        """Time every candidate tuning with short runs of ``opts`` (the plans
        are restored afterwards), keep the fastest; returns the chosen tuning
        and the candidates with their loop times in ms.  An n-gram phase
        starts every trial from the symbols of its last run."""
        o = L.d2g_badmm_opts()
        o.maxIters = int(opts.get("maxIters", 20))
        o.rhoCoeff = float(opts.get("rhoCoeff", 2.0))
        o.updatePerLoops = int(opts.get("updatePerLoops", 10))
        o.time_budget = 0.0
        c_w = np.ascontiguousarray(centroids["c_w"], dtype=np.float64).reshape(-1)
        cs = centroids.get("c_supp")
        c_supp = None if cs is None else np.ascontiguousarray(cs, dtype=np.float64).reshape(-1)
        cap = 64
        cands = (L.d2g_tuning * cap)()
        ms = np.zeros(cap)
        n = C.c_int(0)
        L.check(self.lib.d2g_phase_autotune(self.h, C.byref(o), c_w.ctypes.data,
                                            None if c_supp is None else c_supp.ctypes.data,
                                            cands, ms.ctypes.data, cap, C.byref(n)),
                "d2g_phase_autotune")
        rows = [({f: getattr(cands[i], f) for f, _ in L.d2g_tuning._fields_}, float(ms[i]))
                for i in range(min(n.value, cap))]
        return {"best": self.tuning(), "candidates": rows}

    def test_wait(self, iter: int = -1, unit: int = -1, wait_s: float = 0.0):
        """Test hook of the bounded device waits (d2g_phase_test_wait): the plan
        pass of iteration ``iter`` withholds the tile copy of ``unit`` and every
        wait gives up after ``wait_s`` seconds (0: one second)."""
        L.check(self.lib.d2g_phase_test_wait(self.h, int(iter), int(unit), float(wait_s)),
                "d2g_phase_test_wait")

    def stats(self) -> dict:
        st = L.d2g_run_stats()
        L.check(self.lib.d2g_phase_stats(self.h, C.byref(st)), "d2g_phase_stats")
        return {f: getattr(st, f) for f, _ in L.d2g_run_stats._fields_}

    def trace(self) -> np.ndarray:
        n = C.c_int(0)
        self.lib.d2g_phase_trace(self.h, None, 0, C.byref(n))
        t = np.zeros(4 * max(n.value, 1))
        L.check(self.lib.d2g_phase_trace(self.h, t.ctypes.data, n.value, C.byref(n)), "d2g_phase_trace")
        return t[: 4 * n.value].reshape(-1, 4)

    def run(self, centroids: dict, opts: dict, label_switch=None, c_w_out=None, c_supp_out=None):
        """One centroid update; returns the updated centroids and the trace."""
        o = L.d2g_badmm_opts()
        o.maxIters = int(opts.get("maxIters", 100))
        o.rhoCoeff = float(opts.get("rhoCoeff", 2.0))
        o.updatePerLoops = int(opts.get("updatePerLoops", 10))
        o.time_budget = float(opts.get("time_budget", 0.0))
        c_w = c_w_out if c_w_out is not None else np.array(centroids["c_w"], np.float64).reshape(-1)
        if c_w_out is not None:
            c_w[:] = np.asarray(centroids["c_w"]).reshape(-1)
        cs = centroids.get("c_supp")
        c_supp = None
        if cs is not None:
            c_supp = c_supp_out if c_supp_out is not None else np.array(cs, np.float64).reshape(-1)
            if c_supp_out is not None:
                c_supp[:] = np.asarray(cs).reshape(-1)
        ls = None if label_switch is None else _arr(label_switch, np.int8)
        if self.metric == 6:  # n-gram: integer centroid symbols
            c_sym = np.array(centroids["c_sym"], np.int32).reshape(-1)
            L.check(self.lib.d2g_badmm_run_sym(self.h, C.byref(o), c_w.ctypes.data, c_sym.ctypes.data,
                                               None if ls is None else ls.ctypes.data),
                    "d2g_badmm_run_sym")
            return {"c_w": c_w, "c_supp": None, "c_sym": c_sym, "trace": self.trace(),
                    "stats": self.stats()}
        L.check(self.lib.d2g_badmm_run(self.h, C.byref(o), c_w.ctypes.data,
                                       None if c_supp is None else c_supp.ctypes.data,
                                       None if ls is None else ls.ctypes.data), "d2g_badmm_run")
        return {"c_w": c_w, "c_supp": c_supp, "trace": self.trace(), "stats": self.stats()}


def run_shards(phases, centroids: dict, opts: dict, global_rho: bool = False):
    """The sharded centroid update of several phases on this device
    (d2g_badmm_run_shards): each phase holds one shard of the instances, with
    ``global_size`` the instance count of all shards.  Returns each shard's
    centroids, trace and statistics (the centroids are the same on every
    shard)."""
    lib = L.load()
    n = len(phases)
    o = L.d2g_badmm_opts()
    o.maxIters = int(opts.get("maxIters", 100))
    o.rhoCoeff = float(opts.get("rhoCoeff", 2.0))
    o.updatePerLoops = int(opts.get("updatePerLoops", 10))
    o.time_budget = float(opts.get("time_budget", 0.0))
    cws = [np.array(centroids["c_w"], np.float64).reshape(-1) for _ in range(n)]
    cs = centroids.get("c_supp")
    css = None if cs is None else [np.array(cs, np.float64).reshape(-1) for _ in range(n)]
    hs = (C.c_void_p * n)(*[p.h.value for p in phases])
    pw = (C.c_void_p * n)(*[a.ctypes.data for a in cws])
    ps = None if css is None else (C.c_void_p * n)(*[a.ctypes.data for a in css])
    L.check(lib.d2g_badmm_run_shards(hs, n, C.byref(o), L.D2G_SHARD_GLOBAL_RHO if global_rho else 0, pw, ps),
            "d2g_badmm_run_shards")
    return [{"c_w": cws[i], "c_supp": None if css is None else css[i], "trace": phases[i].trace(),
             "stats": phases[i].stats()} for i in range(n)]


class DropIn:
    """The reference's own calling convention for d2_centroid_sphBregman.

    Holds the mph / var_mph / work objects like d2_clustering does, so that
    successive calls warm-start from the plans left in the work object.
    """

    def __init__(self, phase: dict, centroids: dict):
        self.lib = L.load()
        self.keep = []
        p_str = _arr(phase["p_str"], np.int32)
        n = p_str.size
        col = int(p_str.sum())
        m = int(phase["str"])
        dim = int(phase.get("dim", 0))
        k = int(phase["num_of_labels"])
        cum = np.zeros(n, np.uint64)
        cum[1:] = np.cumsum(p_str[:-1])
        self.n, self.col, self.m, self.dim, self.k = n, col, m, dim, k

        def keep(a):
            self.keep.append(a)
            return a

        def ptr(a, t):
            return None if a is None else keep(a).ctypes.data_as(C.POINTER(t))

        ph = L.sph()
        ph.dim = dim
        ph.str = m
        ph.max_str = int(p_str.max())
        ph.col = col
        ph.max_col = col
        ph.p_str = ptr(p_str, C.c_int)
        ph.p_str_cum = ptr(cum, C.c_size_t)
        ph.p_w = ptr(_arr(phase["p_w"], np.float64), C.c_double)
        ph.metric_type = _metric(phase["metric"])
        ph.p_supp = ptr(_arr(phase.get("p_supp"), np.float64), C.c_double)
        ph.p_supp_sym = ptr(_arr(phase.get("p_supp_sym"), np.int32), C.c_int)
        ph.dist_mat = ptr(_arr(phase.get("dist_mat"), np.float64), C.c_double)
        ph.vocab_size = int(phase.get("vocab_size", 0))
        ph.vocab_vec = ptr(_arr(phase.get("vocab_vec"), np.float64), C.c_double)
        self.ph = ph
        self.label = keep(_arr(phase["label"], np.int32))
        md = L.mph()
        md.s_ph = 1
        md.size = n
        md.global_size = int(phase.get("global_size", n))
        md.label = self.label.ctypes.data_as(C.POINTER(C.c_int))
        md.num_of_labels = k
        md.ph = C.pointer(ph)
        self.mph = md
        # centroids (c0 and c are the same object, clustering.c:493)
        self.c_w = np.array(centroids["c_w"], np.float64).reshape(-1)
        cs = centroids.get("c_supp")
        self.c_supp = None if cs is None else np.array(cs, np.float64).reshape(-1)
        sy = centroids.get("c_sym")
        self.c_sym = None if sy is None else np.array(sy, np.int32).reshape(-1)
        c = L.sph()
        c.dim = dim
        c.str = m
        c.max_str = m
        c.col = k * m
        # strides as d2_allocate_sph + d2_centroid_rands leave them
        c.p_str = ptr(np.full(k, m, np.int32), C.c_int)
        c.p_str_cum = ptr(np.arange(k, dtype=np.uint64) * m, C.c_size_t)
        c.p_w = self.c_w.ctypes.data_as(C.POINTER(C.c_double))
        c.p_supp = (None if self.c_supp is None
                    else self.c_supp.ctypes.data_as(C.POINTER(C.c_double)))
        c.p_supp_sym = (None if self.c_sym is None
                        else self.c_sym.ctypes.data_as(C.POINTER(C.c_int)))
        c.vocab_size = ph.vocab_size
        c.dist_mat = ph.dist_mat
        c.metric_type = ph.metric_type % 7
        self.c = c
        # work: C sized as d2_allocate_work does (clustering_util.c:179)
        self.Cbuf = keep(np.zeros(m * (col + k * m)))
        gv = L.var_sph()
        gv.C = self.Cbuf.ctypes.data_as(C.POINTER(C.c_double))
        self.gv = gv
        bw = L.var_sphBregman()
        L.check(self.lib.d2_allocate_work_sphBregman(C.byref(ph), max(n, k), C.byref(bw)),
                "d2_allocate_work_sphBregman")
        self.bw = bw
        self.ls = keep(np.ones(n, np.int8))
        vw = L.var_mph()
        vw.s_ph = 1
        vw.g_var = C.pointer(gv)
        vw.l_var_sphBregman = C.pointer(bw)
        vw.label_switch = self.ls.ctypes.data_as(C.POINTER(C.c_char))
        self.vw = vw

    def Z(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.bw.Z, shape=(self.m * self.col,)).copy()

    def set_Z(self, Z):
        np.ctypeslib.as_array(self.bw.Z, shape=(self.m * self.col,))[:] = np.asarray(Z).reshape(-1)

    def X(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.bw.X, shape=(self.m * self.col,)).copy()

    def Y(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.bw.Y, shape=(self.m * self.col,)).copy()

    def call(self, opts: dict, label_switch=None, labels=None, random_init=False) -> int:
        """One d2_centroid_sphBregman call with the given BADMM options;
        ``random_init`` passes c0 = NULL (centroid_Bregman.c:95-98)."""
        if label_switch is not None:
            self.ls[:] = np.asarray(label_switch, np.int8)
        if labels is not None:
            self.label[:] = np.asarray(labels, np.int32)
        opt = L.BADMM_options.in_dll(self.lib, "badmm_clu_options")
        opt.maxIters = int(opts.get("maxIters", 100))
        opt.rhoCoeff = float(opts.get("rhoCoeff", 2.0))
        opt.updatePerLoops = int(opts.get("updatePerLoops", 10))
        C.c_double.in_dll(self.lib, "time_budget").value = float(opts.get("time_budget", 1e300))
        c = self.c
        return self.lib.d2_centroid_sphBregman(C.byref(self.mph), C.byref(self.vw), 0,
                                               None if random_init else C.byref(c), C.byref(c))

    def close(self):
        if getattr(self, "bw", None) is not None:
            self.lib.d2_free_work_sphBregman(C.byref(self.bw))
            self.bw = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def centroid_sphBregman(phase: dict, centroids: dict, opts: dict, Z=None, label_switch=None):
    """One drop-in call through the reference structures; returns c_w, c_supp, Z."""
    d = DropIn(phase, centroids)
    try:
        if Z is not None:
            d.set_Z(Z)
        rc = d.call(opts, label_switch)
        L.check(rc, "d2_centroid_sphBregman")
        return {"c_w": d.c_w.copy(), "c_supp": None if d.c_supp is None else d.c_supp.copy(),
                "c_sym": None if d.c_sym is None else d.c_sym.copy(), "Z": d.Z()}
    finally:
        d.close()
