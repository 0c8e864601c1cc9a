"""calculate_distmat (src/d2/centroid_util.c:8-36) through libd2g.so's C ABI
against the oracle's cost blocks (oracle/d2_oracle.c cost_block, which
restates _dpdist2 / _dpdist2_sym / _dpdist_symbolic of
src/utils/blas_like64.c:199-242): every instance's str x m_i block against
its labelled centroid, column-major at str*p_str_cum[i].

Both sides are FP64; the GPU may contract the squared differences into FMAs,
so the bound is 1e-12 relative per entry (n-gram costs, sums of table
entries in the same order, are held to equality).  Histogram phases have
fixed costs: like the reference, calculate_distmat leaves C as it was.
"""
import ctypes as C

import numpy as np
import pytest

from d2_kmeans_gb300 import _lib as L
from d2_kmeans_gb300 import synth

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def calculate_distmat(ph, c, C_in=None):
    """calculate_distmat on the reference's sph structures (host arrays)."""
    lib = L.load()
    p_str = np.ascontiguousarray(ph["p_str"], np.int32)
    col = int(p_str.sum())
    m, dim = int(ph["str"]), int(ph.get("dim", 0))
    keep = []

    def k(a, dt):
        a = None if a is None else np.ascontiguousarray(a, dt)
        keep.append(a)
        return a
    data = L.sph()
    data.dim, data.str, data.col = dim, m, col
    data.p_str = _ptr(p_str, C.c_int)
    data.p_w = _ptr(k(ph["p_w"], np.float64), C.c_double)
    data.metric_type = int(ph["metric"])
    data.p_supp = _ptr(k(ph.get("p_supp"), np.float64), C.c_double)
    data.p_supp_sym = _ptr(k(ph.get("p_supp_sym"), np.int32), C.c_int)
    data.vocab_size = int(ph.get("vocab_size", 0))
    data.vocab_vec = _ptr(k(ph.get("vocab_vec"), np.float64), C.c_double)
    data.dist_mat = _ptr(k(ph.get("dist_mat"), np.float64), C.c_double)
    cen = L.sph()
    cen.dim, cen.str, cen.col = dim, m, int(ph["num_of_labels"]) * m
    cen.p_supp = _ptr(k(c.get("c_supp"), np.float64), C.c_double)
    cen.p_supp_sym = _ptr(k(c.get("c_sym"), np.int32), C.c_int)
    label = k(ph["label"], np.int32)
    out = np.zeros(m * col) if C_in is None else np.array(C_in, np.float64)
    lib.calculate_distmat(C.byref(data), _ptr(label, C.c_int), p_str.size, C.byref(cen),
                          _ptr(out, C.c_double))
    return out


def _euclid(dim, seed):
    return synth.euclidean_phase(300, 6, 16, dim, (1, 40), False, 8, 1.0, seed=seed)


@pytest.mark.parametrize("dim", [1, 3, 5, 8, 64])
def test_euclidean_costs(oracle_mod, dim):
    ph, c = _euclid(dim, 60 + dim)
    got = calculate_distmat(ph, c)
    ref = oracle_mod.cost_blocks(ph, c)
    np.testing.assert_allclose(got, ref, rtol=RTOL, atol=0)


def test_config1_shape(oracle_mod):
    ph, c, _ = synth.workload("plain", seed=1)
    np.testing.assert_allclose(calculate_distmat(ph, c), oracle_mod.cost_blocks(ph, c), rtol=RTOL, atol=0)


def test_word_embedding_costs_with_negative_ids(oracle_mod):
    """d = 300 embeddings; ids < 0 take the reference's ||centroid||^2 branch
    (blas_like64.c:214-216)."""
    ph, c = synth.embed_phase(80, 4, 16, V=1500, dim=300, sizes=(5, 60), seed=61)
    sym = np.array(ph["p_supp_sym"], np.int32)
    rng = np.random.default_rng(62)
    sym[rng.choice(sym.size, size=sym.size // 10, replace=False)] = -1
    ph = dict(ph, p_supp_sym=sym)
    got = calculate_distmat(ph, c)
    ref = oracle_mod.cost_blocks(ph, c)
    np.testing.assert_allclose(got, ref, rtol=RTOL, atol=0)
    # the negative ids really took the norm branch
    p_str = np.asarray(ph["p_str"])
    cum = np.concatenate([[0], np.cumsum(p_str)])
    m = ph["str"]
    cs = np.asarray(c["c_supp"]).reshape(ph["num_of_labels"], m, -1)
    i = int(np.searchsorted(cum, int(np.nonzero(sym < 0)[0][0]), side="right") - 1)
    j = int(np.nonzero(sym < 0)[0][0]) - cum[i]
    blk = got[m * cum[i]: m * cum[i + 1]].reshape(p_str[i], m)
    np.testing.assert_allclose(blk[j], (cs[ph["label"][i]] ** 2).sum(1), rtol=RTOL)


def test_ngram_costs(oracle_mod):
    ph, c = synth.ngram_phase(120, 5, 16, dim=3, V=20, lengths=(20, 120), seed=63)
    got = calculate_distmat(ph, c)
    ref = oracle_mod.cost_blocks(ph, c)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("sparse", [False, True])
def test_histogram_costs_are_left_alone(sparse):
    """centroid_util.c:27-29: histogram costs were filled when the work was
    allocated; calculate_distmat does not touch them."""
    ph, c = synth.histogram_phase(20, 3, side=4, seed=64)
    if sparse:
        ph = dict(ph, metric=12, p_supp_sym=np.tile(np.arange(16, dtype=np.int32), 20))
    col = int(np.sum(ph["p_str"]))
    sentinel = np.random.default_rng(65).random(ph["str"] * col)
    got = calculate_distmat(ph, c, C_in=sentinel)
    np.testing.assert_array_equal(got, sentinel)


def test_out_of_range_ids_are_refused_before_the_gpu_reads_them():
    """The reference would read past its vocabulary; the drop-in refuses (the
    C array is left alone and the error is recorded)."""
    ph, c = synth.embed_phase(30, 2, 8, V=200, dim=16, sizes=(3, 20), seed=66)
    sym = np.array(ph["p_supp_sym"], np.int32)
    sym[5] = 200
    col = int(np.sum(ph["p_str"]))
    sentinel = np.full(ph["str"] * col, 7.0)
    got = calculate_distmat(dict(ph, p_supp_sym=sym), c, C_in=sentinel)
    np.testing.assert_array_equal(got, sentinel)
    assert b"out of range" in L.load().d2g_last_error()
