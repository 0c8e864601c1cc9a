"""TEST INFRASTRUCTURE ONLY: ctypes front end of the CPU oracle.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
legs may import this module, and only as the checker or as the timed CPU
baseline.  The product path (``d2_kmeans_gb300``) never imports it.

Two back ends share one plain-array C interface (``d2_oracle.h``):

* ``port``      - ``liboracle.so``, the C restatement of the reference B-ADMM
                  update (src/d2/centroid_Bregman.c:95-318); builds anywhere.
* ``reference`` - ``_ref/libd2ref.so``, the reference's own sources compiled
                  unmodified by ``oracle/Makefile``; exists only where the
                  reference tree was present at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libd2ref.so")
# where the reference's source tree is read from (the build of oracle/_ref and
# the tests that read its data files); absent trees are skipped
REF_TREE = os.environ.get("D2_REFERENCE_TREE", "/root/reference")

METRIC = {"euclidean": 0, "histogram": 5, "ngram": 6, "embed": 7, "sparse_histogram": 12}


class _Phase(C.Structure):
    _fields_ = [
        ("metric", C.c_int), ("dim", C.c_int), ("str", C.c_int),
        ("size", C.c_size_t), ("col", C.c_size_t),
        ("p_str", C.c_void_p), ("p_w", C.c_void_p), ("p_supp", C.c_void_p),
        ("p_supp_sym", C.c_void_p), ("vocab_vec", C.c_void_p), ("vocab_size", C.c_int),
        ("dist_mat", C.c_void_p), ("label", C.c_void_p), ("num_of_labels", C.c_int),
        ("label_switch", C.c_void_p), ("global_size", C.c_size_t), ("c_sym", C.c_void_p),
    ]


class _Opts(C.Structure):
    _fields_ = [("maxIters", C.c_int), ("rhoCoeff", C.c_double),
                ("updatePerLoops", C.c_int), ("time_budget", C.c_double)]


def build(reference: bool | None = None) -> None:
    """Compile the restatement (always) and the reference (when its tree exists)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if reference is None:
        reference = os.path.isdir(os.path.join(REF_TREE, "src", "d2"))
    if reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_TREE}"], check=True)


_libs: dict[str, C.CDLL] = {}


def available(kind: str) -> bool:
    return os.path.exists(PORT_LIB if kind == "port" else REF_LIB)


def _lib(kind: str) -> C.CDLL:
    if kind not in _libs:
        path = PORT_LIB if kind == "port" else REF_LIB
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library {path} not built")
        lib = C.CDLL(path)
        fn = lib.d2o_badmm if kind == "port" else lib.d2r_badmm
        fn.restype = C.c_int
        fn.argtypes = [C.POINTER(_Phase), C.POINTER(_Opts)] + [C.c_void_p] * 10
        if kind == "port":
            lib.d2o_serve_query.restype = C.c_int
            lib.d2o_serve_query.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                            C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                            C.c_double, C.c_void_p]
        _libs[kind] = lib
    return _libs[kind]


def _ptr(a):
    return None if a is None else a.ctypes.data


def badmm(phase: dict, centroids: dict, opts: dict, kind: str = "port",
          want=("X", "Y", "C")) -> dict:
    """Run one B-ADMM centroid update on the CPU.

    ``phase`` holds the reference's d2 arrays (``p_str``, ``p_w``, ``p_supp`` or
    ``p_supp_sym`` + ``vocab_vec`` or ``dist_mat``, ``label``, ``num_of_labels``,
    ``label_switch``, ``metric``, ``dim``, ``str``); ``centroids`` holds ``c_w``
    (k*str) and ``c_supp`` (k*str*dim) - or, for n-gram phases, the integer
    symbols ``c_sym`` (k*str*dim) - plus optionally a warm-start ``Z``.
    Returns the updated centroids, Z, optional X/Y/C, the obj/primres/dualres
    trace and rho.
    """
    lib = _lib(kind)
    p_str = np.ascontiguousarray(phase["p_str"], dtype=np.int32)
    size = p_str.size
    col = int(p_str.sum())
    m = int(phase["str"])
    dim = int(phase.get("dim", 0))
    k = int(phase["num_of_labels"])
    keep = []

    def arr(name, dtype):
        a = phase.get(name)
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dtype)
        keep.append(a)
        return a

    ph = _Phase()
    ph.metric = METRIC[phase["metric"]] if isinstance(phase["metric"], str) else int(phase["metric"])
    ph.dim, ph.str, ph.size, ph.col = dim, m, size, col
    ph.p_str = p_str.ctypes.data
    ph.p_w = _ptr(arr("p_w", np.float64))
    ph.p_supp = _ptr(arr("p_supp", np.float64))
    ph.p_supp_sym = _ptr(arr("p_supp_sym", np.int32))
    ph.vocab_vec = _ptr(arr("vocab_vec", np.float64))
    ph.vocab_size = int(phase.get("vocab_size", 0))
    ph.dist_mat = _ptr(arr("dist_mat", np.float64))
    ph.label = _ptr(arr("label", np.int32))
    ph.num_of_labels = k
    ls = phase.get("label_switch")
    ls = np.ones(size, np.int8) if ls is None else np.ascontiguousarray(ls, dtype=np.int8)
    keep.append(ls)
    ph.label_switch = ls.ctypes.data
    ph.global_size = int(phase.get("global_size", size))

    op = _Opts()
    op.maxIters = int(opts.get("maxIters", 100))
    op.rhoCoeff = float(opts.get("rhoCoeff", 2.0))
    op.updatePerLoops = int(opts.get("updatePerLoops", 10))
    op.time_budget = float(opts.get("time_budget", 1e300))

    c_w = np.array(centroids["c_w"], dtype=np.float64, copy=True).reshape(-1)
    cs = centroids.get("c_supp")
    c_supp = (np.zeros(max(k * m * dim, 1)) if cs is None
              else np.array(cs, dtype=np.float64, copy=True).reshape(-1))
    c_sym = None
    if centroids.get("c_sym") is not None:
        c_sym = np.array(centroids["c_sym"], dtype=np.int32, copy=True).reshape(-1)
        ph.c_sym = c_sym.ctypes.data
    Z = centroids.get("Z")
    Z = np.zeros(m * col) if Z is None else np.array(Z, dtype=np.float64, copy=True).reshape(-1)
    outs = {n: (np.empty(m * col) if n in want else None) for n in ("X", "Y", "C")}
    nchk = op.maxIters // 20 + 8
    trace = np.zeros(4 * nchk)
    ntrace = C.c_int(0)
    rho = C.c_double(0)
    iters = C.c_int(0)
    fn = lib.d2o_badmm if kind == "port" else lib.d2r_badmm
    rc = fn(C.byref(ph), C.byref(op), c_w.ctypes.data, c_supp.ctypes.data, Z.ctypes.data,
            _ptr(outs["X"]), _ptr(outs["Y"]), _ptr(outs["C"]), trace.ctypes.data,
            C.addressof(ntrace), C.addressof(rho), C.addressof(iters))
    res = {"rc": rc, "c_w": c_w, "c_supp": c_supp, "c_sym": c_sym, "Z": Z,
           "trace": trace[: 4 * ntrace.value].reshape(-1, 4), "rho": rho.value,
           "iters": iters.value}
    res.update({n: v for n, v in outs.items() if v is not None})
    return res


ALLREDUCE_FN = C.CFUNCTYPE(C.c_int, C.POINTER(C.c_double), C.c_size_t, C.c_void_p)


def badmm_mpi(phase: dict, centroids: dict, opts: dict, allreduce, global_rho: bool = False) -> dict:
    """The reference's MPI build of the update on this process's shard
    (d2o_badmm_mpi): ``allreduce(buf)`` must sum the float64 numpy array
    ``buf`` in place over all ranks.  ``phase["global_size"]`` is the number
    of instances of all ranks together."""
    lib = _lib("port")
    fn = lib.d2o_badmm_mpi
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(_Phase), C.POINTER(_Opts)] + [C.c_void_p] * 7 + [ALLREDUCE_FN, C.c_void_p,
                                                                              C.c_int]
    keep = []

    def arr(a, dtype):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dtype)
        keep.append(a)
        return a
    p_str = arr(phase["p_str"], np.int32)
    m, k = int(phase["str"]), int(phase["num_of_labels"])
    dim = int(phase.get("dim", 0))
    col = int(p_str.sum())
    ph = _Phase()
    ph.metric = METRIC[phase["metric"]] if isinstance(phase["metric"], str) else int(phase["metric"])
    ph.dim, ph.str, ph.size, ph.col = dim, m, p_str.size, col
    ph.p_str = p_str.ctypes.data
    ph.p_w = _ptr(arr(phase["p_w"], np.float64))
    ph.p_supp = _ptr(arr(phase.get("p_supp"), np.float64))
    ph.p_supp_sym = _ptr(arr(phase.get("p_supp_sym"), np.int32))
    ph.vocab_vec = _ptr(arr(phase.get("vocab_vec"), np.float64))
    ph.vocab_size = int(phase.get("vocab_size", 0))
    ph.dist_mat = _ptr(arr(phase.get("dist_mat"), np.float64))
    ph.label = _ptr(arr(phase["label"], np.int32))
    ph.num_of_labels = k
    ls = arr(phase.get("label_switch", np.ones(p_str.size, np.int8)), np.int8)
    ph.label_switch = ls.ctypes.data
    ph.global_size = int(phase.get("global_size", p_str.size))
    c_sym = None
    if centroids.get("c_sym") is not None:
        c_sym = np.array(centroids["c_sym"], dtype=np.int32, copy=True).reshape(-1)
        ph.c_sym = c_sym.ctypes.data
    op = _Opts()
    op.maxIters = int(opts.get("maxIters", 100))
    op.rhoCoeff = float(opts.get("rhoCoeff", 2.0))
    op.updatePerLoops = int(opts.get("updatePerLoops", 10))
    op.time_budget = 1e300
    c_w = np.array(centroids["c_w"], dtype=np.float64, copy=True).reshape(-1)
    cs = centroids.get("c_supp")
    c_supp = np.zeros(max(k * m * dim, 1)) if cs is None else np.array(cs, np.float64, copy=True).reshape(-1)
    Z = np.zeros(m * col)
    trace = np.zeros(4 * (op.maxIters // 20 + 8))
    ntrace, rho, iters = C.c_int(0), C.c_double(0), C.c_int(0)
    errors = []

    def cb(buf, n, _ctx):
        try:
            allreduce(np.ctypeslib.as_array(buf, shape=(n,)))
            return 0
        except Exception as e:  # reported after the call
            errors.append(e)
            return 1
    cfn = ALLREDUCE_FN(cb)
    rc = fn(C.byref(ph), C.byref(op), c_w.ctypes.data, c_supp.ctypes.data, Z.ctypes.data,
            trace.ctypes.data, C.addressof(ntrace), C.addressof(rho), C.addressof(iters), cfn, None,
            1 if global_rho else 0)
    if errors:
        raise errors[0]
    return {"rc": rc, "c_w": c_w, "c_supp": c_supp, "c_sym": c_sym, "Z": Z,
            "trace": trace[: 4 * ntrace.value].reshape(-1, 4), "rho": rho.value, "iters": iters.value}


def shard_phase(phase: dict, lo: int, hi: int) -> dict:
    """Instances [lo, hi) of a phase as one rank's shard, global_size kept at
    the whole phase's instance count.  (The reference's d2_write_split writes
    contiguous batches of 1 + (n-1)/splits instances of a shuffled order,
    src/d2/clustering_io.c:329-362, and rank r reads file.r, :20-28.)"""
    p_str = np.asarray(phase["p_str"])
    cum = np.concatenate([[0], np.cumsum(p_str, dtype=np.int64)])
    a, b = int(cum[lo]), int(cum[hi])
    d = int(phase.get("dim", 0))
    out = dict(phase, p_str=p_str[lo:hi], p_w=np.asarray(phase["p_w"])[a:b],
               label=np.asarray(phase["label"])[lo:hi],
               label_switch=np.asarray(phase.get("label_switch", np.ones(p_str.size, np.int8)))[lo:hi],
               global_size=int(phase.get("global_size", p_str.size)))
    if phase.get("p_supp") is not None:
        out["p_supp"] = np.asarray(phase["p_supp"])[a * d:b * d]
    if phase.get("p_supp_sym") is not None:
        w = d if int(phase["metric"] if not isinstance(phase["metric"], str) else METRIC[phase["metric"]]) == 6 else 1
        out["p_supp_sym"] = np.asarray(phase["p_supp_sym"])[a * w:b * w]
    return out


def cost_blocks(phase: dict, centroids: dict) -> np.ndarray:
    """Every instance's ground-cost block against its cluster's centroid
    (d2o_cost_blocks): C [str*col], the blocks of calculate_distmat."""
    lib = _lib("port")
    lib.d2o_cost_blocks.restype = None
    lib.d2o_cost_blocks.argtypes = [C.POINTER(_Phase), C.c_void_p, C.c_void_p]
    keep = []

    def arr(a, dtype):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dtype)
        keep.append(a)
        return a
    p_str = arr(phase["p_str"], np.int32)
    m = int(phase["str"])
    col = int(p_str.sum())
    ph = _Phase()
    ph.metric = METRIC[phase["metric"]] if isinstance(phase["metric"], str) else int(phase["metric"])
    ph.dim, ph.str, ph.size, ph.col = int(phase.get("dim", 0)), m, p_str.size, col
    ph.p_str = p_str.ctypes.data
    ph.p_w = _ptr(arr(phase.get("p_w"), np.float64))
    ph.p_supp = _ptr(arr(phase.get("p_supp"), np.float64))
    ph.p_supp_sym = _ptr(arr(phase.get("p_supp_sym"), np.int32))
    ph.vocab_vec = _ptr(arr(phase.get("vocab_vec"), np.float64))
    ph.vocab_size = int(phase.get("vocab_size", 0))
    ph.dist_mat = _ptr(arr(phase.get("dist_mat"), np.float64))
    ph.label = _ptr(arr(phase["label"], np.int32))
    ph.num_of_labels = int(phase["num_of_labels"])
    ph.global_size = p_str.size
    ph.c_sym = _ptr(arr(centroids.get("c_sym"), np.int32))
    cs = arr(centroids.get("c_supp"), np.float64)
    out = np.zeros(m * col)
    lib.d2o_cost_blocks(C.byref(ph), _ptr(cs), out.ctypes.data)
    return out


def serve_query(c_w, c_supp, w_q, supp_q, iters=200, rho_coeff=2.0):
    """Fixed-centroid transport solve of one query against all k centroids."""
    lib = _lib("port")
    c_w = np.ascontiguousarray(c_w, dtype=np.float64)
    k, m = c_w.shape
    c_supp = np.ascontiguousarray(c_supp, dtype=np.float64)
    dim = c_supp.shape[-1]
    w_q = np.ascontiguousarray(w_q, dtype=np.float64)
    supp_q = np.ascontiguousarray(supp_q, dtype=np.float64)
    cost = np.zeros(k)
    best = lib.d2o_serve_query(dim, m, k, c_w.ctypes.data, c_supp.ctypes.data, w_q.size,
                               w_q.ctypes.data, supp_q.ctypes.data, int(iters),
                               float(rho_coeff), cost.ctypes.data)
    return best, cost


def read(kind: str, filename: str, size: int, dims, types, avg_strides=None, meta_filename=None):
    """d2 input file through the restatement (``port``: d2o_read) or the
    reference's own d2_allocate + d2_read (``ref``); returns the mph's arrays
    (d2_kmeans_gb300.d2io.mph_arrays layout) and the call's return code."""
    import numpy as np
    from d2_kmeans_gb300 import _lib as L
    from d2_kmeans_gb300.d2io import mph_arrays
    lib = _lib(kind)
    fn = lib.d2o_read if kind == "port" else lib.d2r_read
    free = lib.d2o_mph_free if kind == "port" else lib.d2r_mph_free
    fn.restype = C.c_int
    fn.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_size_t] + [C.c_void_p] * 3 + \
        [C.POINTER(C.c_void_p)]
    free.restype = C.c_int
    free.argtypes = [C.c_void_p]
    s_ph = len(dims)
    avg = np.ascontiguousarray(avg_strides if avg_strides is not None else [8] * s_ph, np.int32)
    dims = np.ascontiguousarray(dims, np.int32)
    types = np.ascontiguousarray(types, np.int32)
    out = C.c_void_p()
    rc = fn(filename.encode(), meta_filename.encode() if meta_filename else None, s_ph, int(size),
            avg.ctypes.data, dims.ctypes.data, types.ctypes.data, C.byref(out))
    try:
        arrays = mph_arrays(C.cast(out, C.POINTER(L.mph))) if out.value else None
    finally:
        if out.value:
            free(out)
    return rc, arrays


def emd(C_nm, wX, wY, want_plan=False):
    """Exact transport cost (d2o_emd) between wX (rows) and wY (columns) under
    the n x m cost matrix C_nm (row i, column j); the last column's constraint
    is left free, as in the reference's d2_match_by_distmat."""
    import numpy as np
    lib = _lib("port")
    lib.d2o_emd.restype = C.c_double
    lib.d2o_emd.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 4
    Cc = np.asfortranarray(C_nm, dtype=np.float64)  # column-major, C[i + j*n]
    n, m = Cc.shape
    wX = np.ascontiguousarray(wX, np.float64)
    wY = np.ascontiguousarray(wY, np.float64)
    x = np.zeros((n, m), order="F") if want_plan else None
    v = lib.d2o_emd(n, m, Cc.ctypes.data, wX.ctypes.data, wY.ctypes.data,
                    x.ctypes.data if want_plan else None)
    return (v, x) if want_plan else v


class Labeling:
    """The assignment step on the reference's structures (mph / var_mph built
    by d2_kmeans_gb300.assign.Mph / Work): ``port`` = the oracle's
    restatement (labeling_oracle.c), ``ref`` = the reference's own
    clustering.c functions compiled into oracle/_ref with the oracle's exact
    transport under d2_match_by_distmat (ref_solver.c)."""

    def __init__(self, kind: str):
        self.kind = kind
        lib = _lib(kind)
        vp, sz = C.c_void_p, C.c_size_t
        if kind == "port":
            self._lab = lib.d2o_labeling
            self._lab.restype, self._lab.argtypes = sz, [vp, vp, vp, C.c_int, C.POINTER(C.c_double)]
            self._prep = lib.d2o_labeling_prep
            self._prep.restype, self._prep.argtypes = sz, [vp, vp, vp, C.c_int, C.POINTER(sz)]
            self._post = lib.d2o_labeling_post
            self._post.restype, self._post.argtypes = None, [vp, vp, vp, vp, C.c_int]
            self._dist = lib.d2o_compute_distance
            self._dist.restype, self._dist.argtypes = C.c_double, [vp, sz, vp, sz, C.c_int]
        else:
            self._lab = lib.d2_labeling
            self._lab.restype, self._lab.argtypes = sz, [vp, vp, vp, C.c_int]
            self._prep = lib.d2_labeling_prep
            self._prep.restype, self._prep.argtypes = sz, [vp, vp, vp, C.c_int]
            self._post = lib.d2_labeling_post
            self._post.restype, self._post.argtypes = sz, [vp, vp, vp, vp, C.c_int]
            self._dist = lib.d2_compute_distance
            self._dist.restype, self._dist.argtypes = C.c_double, [vp, sz, vp, sz, C.c_int, vp, sz]

    @staticmethod
    def _p(x):
        return C.cast(C.pointer(x), C.c_void_p)

    def labeling(self, data, cents, work, selected_phase=-1):
        """(labels changed, sum of squared nearest distances or None)"""
        if self.kind == "port":
            cost = C.c_double()
            n = self._lab(self._p(data.mph), self._p(cents.mph), self._p(work.var), selected_phase,
                          C.byref(cost))
            return n, cost.value
        return self._lab(self._p(data.mph), self._p(cents.mph), self._p(work.var), selected_phase), None

    def labeling_prep(self, data, cents, work, selected_phase=-1):
        """(labels changed, distances computed or None)"""
        if self.kind == "port":
            dc = C.c_size_t()
            n = self._prep(self._p(data.mph), self._p(cents.mph), self._p(work.var), selected_phase,
                           C.byref(dc))
            return n, dc.value
        return self._prep(self._p(data.mph), self._p(cents.mph), self._p(work.var),
                          selected_phase), None

    def labeling_post(self, data, c_old, c_new, work, selected_phase=-1):
        self._post(self._p(data.mph), self._p(c_old.mph), self._p(c_new.mph), self._p(work.var),
                   selected_phase)

    def distance(self, a, i, b, j, selected_phase=-1):
        if self.kind == "port":
            return self._dist(self._p(a.mph), i, self._p(b.mph), j, selected_phase)
        return self._dist(self._p(a.mph), i, self._p(b.mph), j, selected_phase, None, 0)
