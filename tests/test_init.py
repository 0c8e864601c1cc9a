"""Random centroid initialisation (d2g_centroid_rands, host code in libd2g.so)
against the reference's own d2_centroid_rands (src/d2/centroid_rand.c:161-295,
compiled from the reference tree into oracle/_ref): weights and supports bit
for bit on every metric type, including instances merged down to the
centroid size.  Where the reference tree is absent, the instance order is
checked against glibc's rand() after srand(0), the reference's shuffle
(src/d2/math.c:40-58) restated here.  CPU only: no device work."""
import ctypes as C

import numpy as np
import pytest

import assign_data as AD
from d2_kmeans_gb300 import _lib as L
from d2_kmeans_gb300 import synth
from d2_kmeans_gb300.assign import Mph


@pytest.fixture(scope="module")
def lib():
    from d2_kmeans_gb300.build import build
    build()
    return L.load()


class Cent:
    """an sph laid out as d2_allocate_sph leaves it for k centroids of str supports"""

    def __init__(self, metric, dim, m, k):
        self.w = np.full(k * m, np.nan)
        self.supp = np.full(k * m * max(dim, 1), np.nan)
        self.sym = np.full(k * m * max(dim, 1), -7, np.int32)
        self.p_str = np.zeros(k, np.int32)
        self.cum = np.zeros(k, np.uint64)
        s = L.sph()
        s.dim, s.str, s.max_str, s.metric_type = dim, m, m, metric % 7
        s.p_str = self.p_str.ctypes.data_as(C.POINTER(C.c_int))
        s.p_str_cum = self.cum.ctypes.data_as(C.POINTER(C.c_size_t))
        s.p_w = self.w.ctypes.data_as(C.POINTER(C.c_double))
        if metric % 7 == 0:
            s.p_supp = self.supp.ctypes.data_as(C.POINTER(C.c_double))
        if metric == 6:
            s.p_supp_sym = self.sym.ctypes.data_as(C.POINTER(C.c_int))
        self.s = s


def data_case(metric, seed):
    rng = np.random.default_rng(seed)
    k = 4
    if metric == 0:   # sizes around str, so that some instances are merged down
        ph, _ = synth.euclidean_phase(60, k, 6, 3, (3, 12), False, 5, 1.0, seed=seed)
        return ph, k, 6
    if metric == 5:
        ph, _ = synth.histogram_phase(30, k, side=3, alpha=0.3, seed=seed)
        return ph, k, 9
    if metric == 7:
        ph, _ = synth.embed_phase(40, k, 5, V=60, dim=4, sizes=(3, 10), seed=seed)
        return ph, k, 5
    if metric == 12:
        d, _ = AD.hist_phase(rng, 30, k, 3, sparse=True)
        d = dict(d, str=9)
        return d, k, 9
    ph, _ = synth.ngram_phase(50, k, 6, 2, 9, (6, 30), 3, seed=seed)
    return ph, k, 6


def run(fn, ph, k, m):
    metric, dim = int(ph["metric"]), int(ph.get("dim", 0))
    data = Mph([dict(ph, str=m)], len(ph["p_str"]), label=np.zeros(len(ph["p_str"]), np.int32),
               num_of_labels=k)
    c = Cent(metric, dim, m, k)
    rc = fn(C.byref(data.mph), 0, C.byref(c.s))
    return rc, c


@pytest.mark.parametrize("metric", [0, 5, 6, 7, 12])
def test_matches_the_reference_build(lib, oracle_mod, metric):
    if not oracle_mod.available("ref"):
        pytest.skip("the reference tree is not present")
    ref = oracle_mod._lib("ref").d2_centroid_rands
    ref.restype = C.c_int
    ref.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    ph, k, m = data_case(metric, 3)
    rc, ours = run(lib.d2g_centroid_rands, ph, k, m)
    assert rc == 0, lib.d2g_last_error()
    rr, theirs = run(lambda a, i, c: ref(C.cast(a, C.c_void_p), i, C.cast(c, C.c_void_p)), ph, k, m)
    assert rr == 0
    np.testing.assert_array_equal(ours.w, theirs.w)
    np.testing.assert_array_equal(ours.supp, theirs.supp)
    np.testing.assert_array_equal(ours.sym, theirs.sym)
    np.testing.assert_array_equal(ours.p_str, theirs.p_str)
    np.testing.assert_array_equal(ours.cum, theirs.cum)
    assert ours.s.col == theirs.s.col == k * m
    if metric in (0, 6, 7):  # some centroids came from merges
        assert (np.asarray(ph["p_str"]) > m).any()


def glibc_order(n):
    """the instance order of the reference's shuffle with glibc's rand() after srand(0)"""
    libc = C.CDLL(None)
    libc.srand(0)
    a = list(range(n))
    rand_max = 2147483647
    for _ in range(10):
        for i in range(n - 1):
            j = i + libc.rand() // (rand_max // (n - i) + 1)
            a[i], a[j] = a[j], a[i]
    return a


def test_instance_order_is_glibc_rand_after_srand0(lib):
    """every instance has exactly str supports: centroid j is instance order[j]"""
    rng = np.random.default_rng(5)
    n, k, m, dim = 40, 7, 3, 2
    supp = rng.normal(size=n * m * dim)
    ph = dict(metric=0, dim=dim, str=m, p_str=np.full(n, m, np.int32),
              p_w=np.tile(np.full(m, 1.0 / m), n), p_supp=supp)
    rc, c = run(lib.d2g_centroid_rands, ph, k, m)
    assert rc == 0
    order = glibc_order(n)
    exp = np.concatenate([supp.reshape(n, m * dim)[order[j]] for j in range(k)])
    np.testing.assert_array_equal(c.supp, exp)


def test_too_few_instances_is_an_error(lib):
    ph, k, m = data_case(0, 4)
    ph = dict(ph, p_str=np.minimum(ph["p_str"], 4).astype(np.int32))
    col = int(ph["p_str"].sum())
    ph["p_w"] = np.full(col, 0.25)
    ph["p_supp"] = np.zeros(col * 3)
    rc, _ = run(lib.d2g_centroid_rands, ph, k, 6)  # no instance has 6 supports
    assert rc == L.D2G_E_INVAL
    assert b"fewer instances" in lib.d2g_last_error()
