"""The assignment step on the GPU (d2g_labeling / d2g_labeling_prep /
d2g_labeling_post / d2g_compute_distances and the reference-signature
d2_labeling family in libd2g.so) against the oracle's restatement
(oracle/labeling_oracle.c, itself bit-identical to the reference's
clustering.c): labels, label_switch, counts and distances computed exactly,
distances and bounds to 1e-9 relative, over several rounds of
labeling_prep -> centroid change -> labeling_post."""
import ctypes as C

import numpy as np
import pytest

import assign_data as AD
from d2_kmeans_gb300 import _lib as L
from d2_kmeans_gb300 import assign
from d2_kmeans_gb300.assign import Mph, Work

pytestmark = pytest.mark.gpu
RTOL = 1e-9


@pytest.fixture(scope="module")
def port(oracle_mod):
    from d2_kmeans_gb300.build import build
    build()
    return oracle_mod.Labeling("port")


def close_state(a, b):
    for key in ("label_switch", "r"):
        assert np.array_equal(a[key], b[key]), key
    for key in ("l", "u", "s", "c"):
        x, y = a[key], b[key]
        big = y > 1e300
        assert np.array_equal(x > 1e300, big), key
        np.testing.assert_allclose(x[~big], y[~big], rtol=RTOL, atol=1e-12, err_msg=key)


def rounds(port, data_ph, cent_ph, n, k, label, nround, rng, selected_phase=-1, prep=True):
    dg, cg = AD.build(data_ph, cent_ph, n, k, label.copy())
    dp, cp = AD.build(data_ph, cent_ph, n, k, label.copy())
    wg, wp = Work(n, k, len(data_ph)), Work(n, k, len(data_ph))
    for rnd in range(nround):
        if prep:
            a, da = assign.labeling_prep(dg, cg, wg, selected_phase)
            b, db = port.labeling_prep(dp, cp, wp, selected_phase)
            assert da == db
        else:
            a, ca = assign.labeling(dg, cg, wg, selected_phase)
            b, cb = port.labeling(dp, cp, wp, selected_phase)
            np.testing.assert_allclose(ca, cb, rtol=RTOL)
        assert a == b, rnd
        assert np.array_equal(dg.label, dp.label), rnd
        close_state(wg.state(), wp.state())
        new_ph = AD.perturb(cent_ph, rng, 0.05)
        cng, cnp = Mph(new_ph, k, num_of_labels=k), Mph(new_ph, k, num_of_labels=k)
        if prep:
            assign.labeling_post(dg, cg, cng, wg, selected_phase)
            port.labeling_post(dp, cp, cnp, wp, selected_phase)
            close_state(wg.state(), wp.state())
        cent_ph, cg, cp = new_ph, cng, cnp
    return dg.label


def euclid_case(seed, n, k):
    rng = np.random.default_rng(seed)
    d0, c0 = AD.euclid_phase(rng, n, 3, 2, 15, k, 6)
    d1, c1 = AD.euclid_phase(rng, n, 2, 1, 9, k, 4)
    return rng, [d0, d1], [c0, c1], rng.integers(-1, k, size=n)


def test_compute_distances(port):
    rng, dph, cph, label = euclid_case(1, 40, 4)
    d, c = AD.build(dph, cph, 40, 4, label)
    ia, jb = np.meshgrid(np.arange(40), np.arange(4), indexing="ij")
    got = assign.compute_distances(d, c, ia.reshape(-1), jb.reshape(-1))
    ref = np.array([port.distance(d, i, c, j) for i, j in zip(ia.reshape(-1), jb.reshape(-1))])
    np.testing.assert_allclose(got, ref, rtol=RTOL)
    got1 = assign.compute_distances(d, c, ia.reshape(-1), jb.reshape(-1), selected_phase=1)
    ref1 = np.array([port.distance(d, i, c, j, 1) for i, j in zip(ia.reshape(-1), jb.reshape(-1))])
    np.testing.assert_allclose(got1, ref1, rtol=RTOL)


def test_labeling(port):
    rng, dph, cph, label = euclid_case(2, 300, 6)
    rounds(port, dph, cph, 300, 6, label, 2, rng, prep=False)


def test_labeling_prep_post_rounds(port):
    rng, dph, cph, label = euclid_case(3, 300, 6)
    rounds(port, dph, cph, 300, 6, label, 4, rng, prep=True)


def test_selected_phase(port):
    rng, dph, cph, label = euclid_case(4, 200, 5)
    rounds(port, dph, cph, 200, 5, label, 2, rng, selected_phase=0, prep=True)


@pytest.mark.parametrize("sparse", [False, True])
def test_histograms(port, sparse):
    rng = np.random.default_rng(5)
    dph, cph = AD.hist_phase(rng, 80, 4, 5, sparse=sparse, asym=True)
    label = rng.integers(-1, 4, size=80)
    rounds(port, [dph], [cph], 80, 4, label, 2, rng, prep=True)


def test_word_embeddings(port):
    """word-embedding phases: FP32 costs from the (centroid, word) table, FP64
    check against the vocabulary"""
    rng = np.random.default_rng(12)
    dph, cph = AD.embed_phase(rng, 120, 5, 300, 24, 8, lo=3, hi=60)
    label = rng.integers(-1, 5, size=120)
    rounds(port, [dph], [cph], 120, 5, label, 3, rng, prep=True)
    rounds(port, [dph], [cph], 120, 5, label, 1, rng, prep=False)


def test_high_dimensional_euclidean(port):
    """Euclidean supports of d = 12 (beyond the direct-cost kernel's 7): costs
    through a (centroid support, instance support) table"""
    rng = np.random.default_rng(13)
    d0, c0 = AD.euclid_phase(rng, 100, 12, 2, 20, 4, 6)
    label = rng.integers(-1, 4, size=100)
    rounds(port, [d0], [c0], 100, 4, label, 3, rng, prep=True)


def test_plain_config_shape(port):
    """n = 2 000 instances, d = 3, m_i 4-16, k = 10, m = 16: every label and
    the cost against the oracle."""
    rng = np.random.default_rng(6)
    d0, c0 = AD.euclid_phase(rng, 2000, 3, 4, 16, 10, 16)
    label = rng.integers(0, 10, size=2000)
    rounds(port, [d0], [c0], 2000, 10, label, 1, rng, prep=False)


def test_reference_entry_points(port):
    """d2_labeling / d2_labeling_prep / d2_labeling_post / d2_compute_distance
    with the reference's signatures; the labelings set time_budget."""
    lib = L.load()
    rng, dph, cph, label = euclid_case(7, 150, 4)
    dg, cg = AD.build(dph, cph, 150, 4, label.copy())
    dp, cp = AD.build(dph, cph, 150, 4, label.copy())
    wg, wp = Work(150, 4, 2), Work(150, 4, 2)
    tb = C.c_double.in_dll(lib, "time_budget")
    tb.value = -1.0
    n = lib.d2_labeling_prep(C.byref(dg.mph), C.byref(cg.mph), C.byref(wg.var), -1)
    assert n == port.labeling_prep(dp, cp, wp)[0]
    assert tb.value >= 0.0
    assert np.array_equal(dg.label, dp.label)
    new_ph = AD.perturb(cph, rng, 0.1)
    cng, cnp = Mph(new_ph, 4, num_of_labels=4), Mph(new_ph, 4, num_of_labels=4)
    assert lib.d2_labeling_post(C.byref(dg.mph), C.byref(cg.mph), C.byref(cng.mph), C.byref(wg.var), -1) == 0
    port.labeling_post(dp, cp, cnp, wp)
    close_state(wg.state(), wp.state())
    n = lib.d2_labeling(C.byref(dg.mph), C.byref(cng.mph), C.byref(wg.var), -1)
    assert n == port.labeling(dp, cnp, wp)[0]
    assert np.array_equal(dg.label, dp.label)
    d = lib.d2_compute_distance(C.byref(dg.mph), 3, C.byref(cng.mph), 1, -1, None, 0)
    assert abs(d - port.distance(dp, 3, cnp, 1)) <= RTOL * d


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_ngrams(port, dim):
    """n-gram phases: exact transport between the distinct centroid and
    instance tuples, 2 * cost / dim per phase (clustering.c:102-115)"""
    rng = np.random.default_rng(20 + dim)
    dph, cph = AD.ngram_phase(rng, 150, 5, 8, dim, 20, lo=10, hi=120)
    label = rng.integers(-1, 5, size=150)
    rounds(port, [dph], [cph], 150, 5, label, 3, rng, prep=True)
    rounds(port, [dph], [cph], 150, 5, label, 1, rng, prep=False)


def test_unsupported_metric_is_refused(port):
    from d2_kmeans_gb300._lib import D2GError
    rng = np.random.default_rng(8)
    d0, c0 = AD.euclid_phase(rng, 10, 3, 2, 5, 2, 3)
    d0 = dict(d0, metric=1)  # D2_CITYBLOCK_L1: no exact-transport path
    dg, cg = AD.build([d0], [c0], 10, 2, np.zeros(10, int))
    with pytest.raises(D2GError):
        assign.labeling(dg, cg, Work(10, 2, 1))
