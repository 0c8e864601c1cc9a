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
