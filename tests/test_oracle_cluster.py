"""The reference's outer loop composed from the oracle's restatements
(assign_data.oracle_clustering) against the reference's own d2_clustering
(src/d2/clustering.c:409-525, compiled from the reference tree into
oracle/_ref with the oracle's exact transport standing in for MOSEK): labels,
centroids and round count bit for bit, plain and pruned labeling.  CPU only."""
import ctypes as C

import numpy as np
import pytest

import assign_data as AD
from d2_kmeans_gb300.assign import Mph


@pytest.fixture(scope="module")
def ref(oracle_mod):
    if not oracle_mod.available("ref"):
        pytest.skip("the reference tree is not present")
    lib = oracle_mod._lib("ref")
    lib.d2_clustering.restype = C.c_int
    lib.d2_clustering.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_char,
                                  C.c_char_p]
    C.c_double.in_dll(lib, "time_budget").value = 1e300
    return lib


def case(seed, n, k):
    """overlapping clusters and centroids started away from them, so that the
    loop runs several rounds"""
    rng = np.random.default_rng(seed)
    d0, c0 = AD.euclid_phase(rng, n, 2, 2, 10, k, 5, spread=1.5)
    c0["p_supp"] = rng.normal(size=c0["p_supp"].size) * 1.5
    return [d0], [c0], np.full(n, -1)


@pytest.mark.parametrize("tri", [0, 1])
def test_clustering_loop_bit_identical(oracle_mod, ref, tri):
    n, k = 150, 4
    dph, cph, label = case(3 + tri, n, k)
    lab_o, cents_o, rounds = AD.oracle_clustering(oracle_mod, dph, cph, n, k, label, 6, tri)
    data = Mph(dph, n, label=label.copy(), num_of_labels=k)
    cents = Mph(cph, k, num_of_labels=k)
    rc = ref.d2_clustering(k, 6, C.cast(C.pointer(data.mph), C.c_void_p),
                           C.cast(C.pointer(cents.mph), C.c_void_p), -1, bytes([tri]), None)
    assert rc == 0
    assert np.array_equal(data.label, lab_o)
    assert np.array_equal(cents.arrays[0]["p_w"], cents_o.arrays[0]["p_w"])
    assert np.array_equal(cents.arrays[0]["p_supp"], cents_o.arrays[0]["p_supp"])
    assert rounds >= 2


def test_ngram_clustering_loop_bit_identical(oracle_mod, ref):
    """n-gram phases: labels from 2 * cost / dim, symbol updates in the B-ADMM
    rounds (the protein application's path, plain labeling as it runs it,
    data/protein_seq/d2_protein_ngram.cc:341).  The reference's pruned
    labeling cannot run on n-gram phases: its d2_copy (clustering_util.c:
    280-282) copies the centroid symbols into p_supp_sym, which d2_allocate_sph
    (:41-55) leaves unallocated for n-grams; the GPU tests cover that case
    against the composed oracle loop."""
    tri = 0
    rng = np.random.default_rng(30)
    n, k = 90, 3
    dph, cph = AD.ngram_phase(rng, n, k, 6, 2, 8, lo=10, hi=40)
    label = np.full(n, -1)
    opts = dict(maxIters=100, rhoCoeff=2.0, updatePerLoops=10)
    lab_o, cents_o, rounds = AD.oracle_clustering(oracle_mod, [dph], [cph], n, k, label, 5, tri, opts)
    data = Mph([dph], n, label=label.copy(), num_of_labels=k)
    cents = Mph([cph], k, num_of_labels=k)
    rc = ref.d2_clustering(k, 5, C.cast(C.pointer(data.mph), C.c_void_p),
                           C.cast(C.pointer(cents.mph), C.c_void_p), -1, bytes([tri]), None)
    assert rc == 0
    assert np.array_equal(data.label, lab_o)
    assert np.array_equal(cents.arrays[0]["p_w"], cents_o.arrays[0]["p_w"])
    assert np.array_equal(cents.arrays[0]["p_supp_sym"], cents_o.arrays[0]["p_supp_sym"])
    assert rounds >= 2
