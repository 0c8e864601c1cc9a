"""The outer loop on the GPU (d2g_clustering / d2_clustering in libd2g.so)
against the reference's loop composed from the oracle's restatements
(assign_data.oracle_clustering, itself bit-identical to the reference's
d2_clustering): same rounds, same labels, centroids within the B-ADMM
tolerances (c_w L1 <= 1e-4 per cluster, supports <= 1e-4 relative), plain
and pruned labeling; random initialisation through the program's
d2_centroid_rands."""
import ctypes as C

import numpy as np
import pytest

import assign_data as AD
from d2_kmeans_gb300 import _lib as L
from d2_kmeans_gb300 import assign
from d2_kmeans_gb300.assign import Mph

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(oracle_mod):
    from d2_kmeans_gb300 import badmm
    from d2_kmeans_gb300.build import build
    build()
    # the reference's rule ties the update's time budget to the labeling's
    # wall time; keep it fixed so that the runs repeat
    badmm.set_config(verbose=0, precision=0, use_graph=1, profile=0, sync_scratch=0, cost_gemm=0,
                     keep_time_budget=1)
    lib = L.load()
    C.c_double.in_dll(lib, "time_budget").value = 1e300
    # the update runs with p_badmm_options -> badmm_clu_options, the
    # reference's defaults {100, 2.0, 10} (centroid_Bregman.c:17), which other
    # tests may have changed
    opt = L.BADMM_options.in_dll(lib, "badmm_clu_options")
    opt.maxIters, opt.rhoCoeff, opt.updatePerLoops = 100, 2.0, 10
    C.c_void_p.in_dll(lib, "p_badmm_options").value = C.addressof(opt)
    yield lib
    badmm.set_config(keep_time_budget=0)


def case(seed, n, k, dims=(2,)):
    rng = np.random.default_rng(seed)
    dph, cph = [], []
    for d in dims:
        d0, c0 = AD.euclid_phase(rng, n, d, 2, 10, k, 5, spread=1.5)
        c0["p_supp"] = rng.normal(size=c0["p_supp"].size) * 1.5
        dph.append(d0)
        cph.append(c0)
    return dph, cph, np.full(n, -1)


def close_centroids(a, b, k, m):
    for pa, pb in zip(a.arrays, b.arrays):
        l1 = np.abs(pa["p_w"].reshape(k, m) - pb["p_w"].reshape(k, m)).sum(1)
        assert l1.max() <= 1e-4, l1.max()
        if "p_supp" in pa:
            sa, sb = pa["p_supp"], pb["p_supp"]
            scale = max(1e-3 * np.abs(sb).max(), 1e-12)
            assert np.max(np.abs(sa - sb) / np.maximum(np.abs(sb), scale)) <= 1e-4


@pytest.mark.parametrize("tri,dims", [(0, (2,)), (1, (2,)), (1, (3, 2))])
def test_clustering_matches_oracle_loop(lib, oracle_mod, tri, dims):
    n, k = 150, 4
    dph, cph, label = case(3 + tri, n, k, dims)
    lab_o, cents_o, rounds_o = AD.oracle_clustering(oracle_mod, dph, cph, n, k, label, 6, tri)
    data = Mph(dph, n, label=label.copy(), num_of_labels=k)
    cents = Mph(cph, k, num_of_labels=k)
    rounds = assign.clustering(data, cents, k, 6, use_triangle=bool(tri))
    assert rounds == rounds_o
    assert np.array_equal(data.label, lab_o)
    close_centroids(cents, cents_o, k, 5)


def test_reference_entry_point(lib, oracle_mod):
    n, k = 150, 4
    dph, cph, label = case(9, n, k)
    lab_o, cents_o, _ = AD.oracle_clustering(oracle_mod, dph, cph, n, k, label, 5, 1)
    data = Mph(dph, n, label=label.copy(), num_of_labels=k)
    cents = Mph(cph, k, num_of_labels=k)
    assert lib.d2_clustering(k, 5, C.byref(data.mph), C.byref(cents.mph), -1, b"\x01", None) == 0
    assert np.array_equal(data.label, lab_o)
    close_centroids(cents, cents_o, k, 5)


def test_random_initialisation(lib, rands_stub):
    """centroids->ph == NULL: the program's d2_centroid_rands fills them; the
    loop then runs as from those centroids given explicitly."""
    from conftest import rands_stub_init
    n, k, m = 150, 4, 5
    dph, _, label = case(11, n, k)
    data = Mph(dph, n, label=label.copy(), num_of_labels=k)
    empty = L.mph()
    rounds = C.c_int()
    L.check(lib.d2g_clustering(k, 4, C.byref(data.mph), C.byref(empty), -1, 1, None, C.byref(rounds)),
            "d2g_clustering")
    got_w = np.ctypeslib.as_array(empty.ph[0].p_w, (k * m,)).copy()
    got_s = np.ctypeslib.as_array(empty.ph[0].p_supp, (k * m * 2,)).copy()
    init = rands_stub_init(dict(dph[0]), k, m)
    data2 = Mph(dph, n, label=label.copy(), num_of_labels=k)
    cents2 = Mph([dict(metric=0, dim=2, str=m, p_w=init["c_w"], p_supp=init["c_supp"])], k,
                 num_of_labels=k)
    assert assign.clustering(data2, cents2, k, 4, use_triangle=True) == rounds.value
    assert np.array_equal(data.label, data2.label)
    assert np.array_equal(got_w, cents2.arrays[0]["p_w"])
    assert np.array_equal(got_s, cents2.arrays[0]["p_supp"])


@pytest.mark.parametrize("tri", [0, 1])
def test_ngram_clustering_matches_oracle_loop(lib, oracle_mod, tri):
    """n-gram phases through the whole loop: exact-transport labels (2 * cost /
    dim) and B-ADMM rounds with symbol updates; labels and symbols identical,
    weights within the B-ADMM tolerance"""
    rng = np.random.default_rng(40 + tri)
    n, k, m = 120, 3, 6
    dph, cph = AD.ngram_phase(rng, n, k, m, 2, 10, lo=10, hi=60)
    label = np.full(n, -1)
    lab_o, cents_o, rounds_o = AD.oracle_clustering(oracle_mod, [dph], [cph], n, k, label, 5, tri)
    data = Mph([dph], n, label=label.copy(), num_of_labels=k)
    cents = Mph([cph], k, num_of_labels=k)
    rounds = assign.clustering(data, cents, k, 5, use_triangle=bool(tri))
    assert rounds == rounds_o and rounds >= 2
    assert np.array_equal(data.label, lab_o)
    assert np.array_equal(cents.arrays[0]["p_supp_sym"], cents_o.arrays[0]["p_supp_sym"])
    close_centroids(cents, cents_o, k, m)
