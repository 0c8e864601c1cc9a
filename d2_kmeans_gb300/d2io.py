"""The reference's d2 text formats: read with d2g_read, write for tests and
benchmarks.

Formats (data/README.md of bobye/d2_kmeans): per object and phase
``dim  n  w_1 .. w_n  [supports]`` with Euclidean supports as n rows of dim
values, symbolic supports (word embeddings, sparse histograms) as n ids
starting at one, dense histograms (dim 0) without supports.  A histogram
phase has a ``<file>.hist<phase>`` cost file (``str`` then str x str
costs); an embedding phase a ``<file>.vocab<phase>`` file (``dim V`` then
V x dim values).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

EUCLIDEAN, HISTOGRAM, WORD_EMBED, SPARSE_HISTOGRAM = 0, 5, 7, 12


def mph_arrays(p) -> dict:
    """Copy the data of an mph (ctypes pointer, the reference's layout) into numpy."""
    m = p.contents
    out = {"size": int(m.size), "global_size": int(m.global_size), "phases": []}
    for n in range(m.s_ph):
        ph = m.ph[n]
        size, col = int(m.size), int(ph.col)
        d = {"metric": int(ph.metric_type), "dim": int(ph.dim), "str": int(ph.str),
             "max_str": int(ph.max_str), "col": col, "vocab_size": int(ph.vocab_size),
             "p_str": np.ctypeslib.as_array(ph.p_str, (size,)).copy() if size else np.zeros(0, np.int32),
             "p_str_cum": np.ctypeslib.as_array(ph.p_str_cum, (size,)).copy() if size else np.zeros(0),
             "p_w": np.ctypeslib.as_array(ph.p_w, (col,)).copy() if col else np.zeros(0)}
        if ph.metric_type == EUCLIDEAN and col:
            d["p_supp"] = np.ctypeslib.as_array(ph.p_supp, (col * ph.dim,)).copy()
        if ph.metric_type in (WORD_EMBED, SPARSE_HISTOGRAM) and col:
            d["p_supp_sym"] = np.ctypeslib.as_array(ph.p_supp_sym, (col,)).copy()
        if ph.metric_type in (HISTOGRAM, SPARSE_HISTOGRAM) and ph.dist_mat:
            d["dist_mat"] = np.ctypeslib.as_array(ph.dist_mat, (ph.vocab_size ** 2,)).copy()
        if ph.metric_type == WORD_EMBED and ph.vocab_vec:
            d["vocab_vec"] = np.ctypeslib.as_array(ph.vocab_vec, (ph.vocab_size * ph.dim,)).copy()
        out["phases"].append(d)
    return out


def read(filename: str, size: int, dims, types, avg_strides=None, meta_filename=None) -> dict:
    """d2g_read into a fresh mph (d2g_mph_alloc); returns its arrays."""
    lib = L.load()
    s_ph = len(dims)
    avg = np.ascontiguousarray(avg_strides if avg_strides is not None else [8] * s_ph, np.int32)
    dims = np.ascontiguousarray(dims, np.int32)
    types = np.ascontiguousarray(types, np.int32)
    p = C.POINTER(L.mph)()
    L.check(lib.d2g_mph_alloc(s_ph, int(size), avg.ctypes.data_as(L.ip), dims.ctypes.data_as(L.ip),
                              types.ctypes.data_as(L.ip), C.byref(p)), "d2g_mph_alloc")
    try:
        L.check(lib.d2g_read(filename.encode(), meta_filename.encode() if meta_filename else None, p),
                "d2g_read")
        return mph_arrays(p)
    finally:
        lib.d2g_mph_free(p)


def phase_dict(data: dict, phase: int, str_: int, label, num_of_labels: int) -> dict:
    """A phase description (the form badmm.Phase / DropIn take) from read data."""
    ph = data["phases"][phase]
    n = data["size"]
    out = dict(metric=ph["metric"], dim=ph["dim"], str=str_, p_str=ph["p_str"][:n].astype(np.int32),
               p_w=ph["p_w"], label=np.ascontiguousarray(label, np.int32), num_of_labels=num_of_labels,
               label_switch=np.ones(n, np.int8), vocab_size=ph["vocab_size"])
    for k in ("p_supp", "p_supp_sym", "dist_mat", "vocab_vec"):
        if k in ph:
            out[k] = ph[k]
    return out


def _fmt(a) -> list:
    return [repr(float(v)) for v in np.asarray(a, np.float64).reshape(-1)]


def write(filename: str, phases, vocab=None, dist_mats=None) -> None:
    """Write objects in the d2 format.  ``phases``: one dict per phase with
    ``metric``, ``dim``, ``p_str`` and ``p_w`` plus ``p_supp`` (Euclidean) or
    ``p_supp_sym`` (0-based ids, written from one); ``vocab`` / ``dist_mats``:
    {phase: array} for the .vocabN / .histN files.  Floats are written with
    17 significant digits, so they read back exactly."""
    size = len(phases[0]["p_str"])
    cum = [np.concatenate([[0], np.cumsum(ph["p_str"])]) for ph in phases]
    lines = []
    for i in range(size):
        for n, ph in enumerate(phases):
            s = int(ph["p_str"][i])
            a, b = int(cum[n][i]), int(cum[n][i + 1])
            lines.append(f"{ph['dim']}")
            lines.append(f"{s}")
            lines.append(" ".join(_fmt(ph["p_w"][a:b])))
            if ph["metric"] == EUCLIDEAN:
                sup = np.asarray(ph["p_supp"]).reshape(-1, ph["dim"])[a:b]
                lines.extend(" ".join(_fmt(r)) for r in sup)
            elif ph["metric"] in (WORD_EMBED, SPARSE_HISTOGRAM):
                lines.append(" ".join(str(int(v) + 1) for v in ph["p_supp_sym"][a:b]))
    with open(filename, "w") as f:
        f.write("\n".join(lines) + "\n")
    for n, v in (vocab or {}).items():
        v = np.asarray(v, np.float64)
        with open(f"{filename}.vocab{n}", "w") as f:
            f.write(f"{v.shape[1]} {v.shape[0]}\n")
            f.write("\n".join(" ".join(_fmt(r)) for r in v) + "\n")
    for n, dm in (dist_mats or {}).items():
        dm = np.asarray(dm, np.float64)
        k = dm.shape[0]
        with open(f"{filename}.hist{n}", "w") as f:
            f.write(f"{k}\n")
            f.write("\n".join(" ".join(_fmt(r)) for r in dm) + "\n")
