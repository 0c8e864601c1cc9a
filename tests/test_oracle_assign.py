"""The oracle's assignment step (oracle/labeling_oracle.c) against the
reference's own d2_compute_distance / d2_labeling / d2_labeling_prep /
d2_labeling_post (src/d2/clustering.c:33-376, compiled from the reference
tree into oracle/_ref with the oracle's exact transport standing in for
MOSEK): bit for bit on labels, label_switch, counts and every bound of the
triangle-inequality state, over several rounds.  CPU only."""
import copy

import numpy as np
import pytest

import assign_data as AD
from d2_kmeans_gb300.assign import Mph, Work


@pytest.fixture(scope="module")
def both(oracle_mod):
    if not oracle_mod.available("ref"):
        pytest.skip("the reference tree is not present")
    return oracle_mod.Labeling("port"), oracle_mod.Labeling("ref")


def euclid_case(seed, n=120, k=5):
    rng = np.random.default_rng(seed)
    d0, c0 = AD.euclid_phase(rng, n, 3, 2, 15, k, 6)
    d1, c1 = AD.euclid_phase(rng, n, 2, 1, 9, k, 4)
    label = rng.integers(-1, k, size=n)
    return rng, [d0, d1], [c0, c1], label


def run_both(both, data_ph, cent_ph, n, k, label, rounds, rng, selected_phase=-1, prep=True):
    port, ref = both
    labels = label.copy()
    dp, cp = AD.build(data_ph, cent_ph, n, k, labels.copy())
    dr, cr = AD.build(data_ph, cent_ph, n, k, labels.copy())
    wp = Work(n, k, len(data_ph))
    wr = Work(n, k, len(data_ph), cost_scratch=AD.ref_scratch(data_ph, n, k))
    for rnd in range(rounds):
        if prep:
            a = port.labeling_prep(dp, cp, wp, selected_phase)[0]
            b = ref.labeling_prep(dr, cr, wr, selected_phase)[0]
        else:
            a = port.labeling(dp, cp, wp, selected_phase)[0]
            b = ref.labeling(dr, cr, wr, selected_phase)[0]
        assert a == b
        assert np.array_equal(dp.label, dr.label)
        sp, sr = wp.state(), wr.state()
        for key in sp:
            assert np.array_equal(sp[key], sr[key]), (rnd, key)
        new_ph = AD.perturb(cent_ph, rng, 0.05)
        cnp = Mph(new_ph, k, num_of_labels=k)
        cnr = Mph(new_ph, k, num_of_labels=k)
        if prep:
            port.labeling_post(dp, cp, cnp, wp, selected_phase)
            ref.labeling_post(dr, cr, cnr, wr, selected_phase)
            sp, sr = wp.state(), wr.state()
            for key in sp:
                assert np.array_equal(sp[key], sr[key]), (rnd, "post", key)
        cent_ph, cp, cr = new_ph, cnp, cnr
    return dp.label


def test_compute_distance_bit_identical(both):
    port, ref = both
    rng, dph, cph, label = euclid_case(1, n=20, k=3)
    d, c = AD.build(dph, cph, 20, 3, label)
    wr = Work(20, 3, 2, cost_scratch=AD.ref_scratch(dph, 20, 3))
    for i in range(20):
        for j in range(3):
            a = port.distance(d, i, c, j)
            b = ref._dist(ref._p(d.mph), i, ref._p(c.mph), j, -1, ref._p(wr.var), i)
            assert a == b


def test_labeling_bit_identical(both):
    rng, dph, cph, label = euclid_case(2)
    run_both(both, dph, cph, 120, 5, label, rounds=2, rng=rng, prep=False)


def test_labeling_prep_post_rounds_bit_identical(both):
    rng, dph, cph, label = euclid_case(3)
    run_both(both, dph, cph, 120, 5, label, rounds=4, rng=rng, prep=True)


def test_selected_phase(both):
    rng, dph, cph, label = euclid_case(4)
    run_both(both, dph, cph, 120, 5, label, rounds=2, rng=rng, selected_phase=1)


def test_word_embeddings(both):
    rng = np.random.default_rng(6)
    dph, cph = AD.embed_phase(rng, 60, 4, 80, 6, 5)
    label = rng.integers(-1, 4, size=60)
    run_both(both, [dph], [cph], 60, 4, label, rounds=2, rng=rng, prep=True)


@pytest.mark.parametrize("sparse", [False, True])
def test_histograms(both, sparse):
    rng = np.random.default_rng(5)
    dph, cph = AD.hist_phase(rng, 60, 4, 4, sparse=sparse, asym=True)
    label = rng.integers(-1, 4, size=60)
    run_both(both, [dph], [cph], 60, 4, label, rounds=2, rng=rng, prep=True)


@pytest.mark.parametrize("dim", [1, 3])
def test_ngrams(both, dim):
    """n-gram phases: 2 * transport cost / dim per phase (clustering.c:102-115)"""
    rng = np.random.default_rng(9 + dim)
    dph, cph = AD.ngram_phase(rng, 60, 4, 6, dim, 12)
    label = rng.integers(-1, 4, size=60)
    run_both(both, [dph], [cph], 60, 4, label, rounds=2, rng=rng, prep=True)
