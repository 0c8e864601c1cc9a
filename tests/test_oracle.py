"""The CPU oracle, pinned: the C restatement against the reference compiled
from its own sources, and against the committed golden fixtures."""
import os
import sys

import numpy as np
import pytest

from conftest import golden_names, load_golden

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from golden.make_golden import digest  # noqa: E402

from d2_kmeans_gb300 import synth  # noqa: E402


def _port_warm(oracle, ph, c0, opts, exp):
    """The fixture's two-call warm-start sequence on the port."""
    first = dict(ph, label=exp["first_label"], label_switch=np.ones(len(ph["p_str"]), np.int8))
    r1 = oracle.badmm(first, {"c_w": exp["first_c_w"], "c_supp": exp["first_c_supp"]}, opts,
                      "port", want=())
    return oracle.badmm(ph, {"c_w": r1["c_w"], "c_supp": r1["c_supp"], "Z": r1["Z"]}, opts,
                        "port", want=())


@pytest.mark.parametrize("name", golden_names())
def test_port_matches_golden_bitwise(oracle_mod, name):
    ph, c0, opts, exp = load_golden(name)
    if "first_label" in exp:
        r = _port_warm(oracle_mod, ph, c0, opts, exp)
    else:
        r = oracle_mod.badmm(ph, c0, opts, "port", want=())
    assert r["rc"] == 0
    np.testing.assert_array_equal(r["c_w"], exp["out_c_w"])
    if "out_c_supp" in exp:
        np.testing.assert_array_equal(r["c_supp"], exp["out_c_supp"])
    if "out_c_sym" in exp:
        np.testing.assert_array_equal(r["c_sym"], exp["out_c_sym"])
    np.testing.assert_array_equal(digest(r["Z"]), exp["out_Z_digest"])
    # the reference prints the trace with %f: 6 decimals
    np.testing.assert_allclose(r["trace"][:, 1:], exp["out_trace"][:, 1:], atol=5.1e-7, rtol=0)
    np.testing.assert_array_equal(r["trace"][:, 0], exp["out_trace"][:, 0])


@pytest.mark.parametrize("metric", ["euclidean", "hist", "embed", "ngram"])
def test_port_matches_reference_build(oracle_mod, metric):
    """Bit-identical to the reference's own d2_centroid_sphBregman, all outputs."""
    if not oracle_mod.available("reference"):
        pytest.skip("reference tree not present on this host")
    if metric == "euclidean":
        ph, c = synth.euclidean_phase(150, 5, 16, 3, (8, 128), True, 12, 0.5, seed=3)
        opts = dict(maxIters=30, rhoCoeff=2.0, updatePerLoops=7)
    elif metric == "hist":
        ph, c = synth.histogram_phase(40, 3, side=6, alpha=0.1, seed=4)
        opts = dict(maxIters=25, rhoCoeff=2.0, updatePerLoops=10)
    elif metric == "embed":
        ph, c = synth.embed_phase(30, 3, 8, V=500, dim=12, sizes=(5, 40), seed=5)
        opts = dict(maxIters=25, rhoCoeff=2.0, updatePerLoops=10)
    else:
        ph, c = synth.ngram_phase(60, 3, 10, 3, 9, (8, 60), 4, seed=6)
        opts = dict(maxIters=45, rhoCoeff=2.0, updatePerLoops=4)
    a = oracle_mod.badmm(ph, c, opts, "port")
    b = oracle_mod.badmm(ph, c, opts, "reference")
    assert a["rc"] == 0 and b["rc"] == 0
    if metric == "ngram":  # the symbols moved, identically
        assert np.any(a["c_sym"] != c["c_sym"])
        np.testing.assert_array_equal(a["c_sym"], b["c_sym"])
    for k in ("c_w", "c_supp", "Z", "X", "Y", "C"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    np.testing.assert_allclose(a["trace"][:, 1:], b["trace"][:, 1:], atol=5.1e-7, rtol=0)


def test_port_time_budget_stops_after_one_iteration(oracle_mod):
    ph, c = synth.euclidean_phase(50, 3, 8, 3, (4, 10), seed=8)
    r = oracle_mod.badmm(ph, c, dict(maxIters=50, rhoCoeff=2.0, updatePerLoops=10,
                                      time_budget=-1.0), "port", want=())
    assert r["iters"] == 1
    r0 = oracle_mod.badmm(ph, c, dict(maxIters=0, rhoCoeff=2.0, updatePerLoops=10), "port",
                          want=())
    np.testing.assert_array_equal(r["c_w"], r0["c_w"])


def test_port_empty_cluster_is_an_error(oracle_mod):
    ph, c = synth.euclidean_phase(20, 4, 8, 3, (4, 10), seed=9)
    ph["label"][:] = 0
    ph["label"][1] = 1
    r = oracle_mod.badmm(ph, c, dict(maxIters=5), "port", want=())
    assert r["rc"] == -5


def test_serve_oracle_argmin_is_nearest(oracle_mod):
    c_w, c_supp, means = synth.serving_centroids(k=4, m=8, dim=6, n_comp=4, seed=0)
    q = synth.serving_queries(3, means, sizes=(4, 20), seed=2)
    for w, s in q:
        best, cost = oracle_mod.serve_query(c_w, c_supp, w, s, iters=50)
        assert best == int(np.argmin(cost)) and np.all(cost > 0)
