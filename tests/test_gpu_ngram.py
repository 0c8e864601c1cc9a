"""N-gram phases (D2_N_GRAM) on the GPU through the C ABI against the oracle
(the C restatement, bit-identical to the reference's src/d2/centroid_Bregman.c
:269-294 and blas_like64.c:232-242) on the same seeded inputs.

Tolerances: the batched FP32 form to the metric's bounds (objective 1e-5
relative, c_w L1 1e-4 per cluster), the FP64 form to 1e-9; the centroid
symbols must be identical in both forms.  The reference's own protein
1-gram fixtures run through test_gpu_badmm's golden tests."""
import ctypes as C

import numpy as np
import pytest

from test_gpu_badmm import _exchange, _plan_l1, _port, assert_close, EXCHANGES
from d2_kmeans_gb300 import _lib as L
from d2_kmeans_gb300 import synth
from d2_kmeans_gb300._lib import D2GError

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("exchange", EXCHANGES)
@pytest.mark.parametrize("n,k,m,dim,V,lengths,upl,seed", [
    (300, 6, 32, 3, 20, (30, 400), 10, 61),   # 3-grams, plans up to ~400 columns (wide)
    (200, 5, 20, 2, 20, (20, 200), 7, 62),    # 2-grams, m = 20 padded to 32
    (150, 4, 7, 1, 23, (10, 60), 5, 63),      # 1-grams over 23 symbols, m = 7 padded to 8
    (80, 3, 64, 3, 6, (40, 300), 10, 64),     # small alphabet, m = 64
])
def test_ngram_matches_oracle(d2g, oracle_mod, monkeypatch, exchange, n, k, m, dim, V, lengths,
                              upl, seed):
    _exchange(monkeypatch, exchange)
    ph, c = synth.ngram_phase(n, k, m, dim, V, lengths, 5, seed=seed)
    opts = dict(maxIters=60, rhoCoeff=2.0, updatePerLoops=upl)
    ref = _port(oracle_mod, ph, c, opts)
    assert np.any(ref["c_sym"] != c["c_sym"])  # the symbols moved
    for precision in (0, 1):
        P = d2g.Phase(ph, precision)
        r = P.run(c, opts)
        assert r["stats"]["path"] == precision
        assert_close(r, ref, k, m, fp64=precision == 1)
        if precision == 1:
            np.testing.assert_allclose(P.get_plans(), ref["Z"], rtol=1e-9, atol=1e-15)
        P.close()


def test_ngram_warm_start_and_time_budget(d2g, oracle_mod):
    ph, c = synth.ngram_phase(120, 4, 16, 2, 20, (20, 300), 4, seed=65)
    o1 = dict(maxIters=30, rhoCoeff=2.0, updatePerLoops=10)
    r1 = _port(oracle_mod, ph, c, o1)
    ph2 = dict(ph, label_switch=np.zeros(len(ph["p_str"]), np.int8))
    c2 = dict(c_w=r1["c_w"], c_sym=r1["c_sym"], c_supp=None, Z=r1["Z"])
    r2 = _port(oracle_mod, ph2, c2, o1)
    P = d2g.Phase(ph, 0)
    g1 = P.run(c, o1)
    assert_close(g1, r1, 4, 16)
    assert _plan_l1(P.get_plans(), r1["Z"]) <= 1e-4
    g2 = P.run(dict(c_w=g1["c_w"], c_sym=g1["c_sym"]), o1, label_switch=ph2["label_switch"])
    assert_close(g2, r2, 4, 16)
    # the time budget stops the loop after iteration 0: no support update ran
    r0 = _port(oracle_mod, ph, c, dict(maxIters=0, rhoCoeff=2.0, updatePerLoops=10))
    g0 = P.run(c, dict(maxIters=40, rhoCoeff=2.0, updatePerLoops=10, time_budget=1e-9))
    assert g0["stats"]["iterations"] == 1
    np.testing.assert_array_equal(g0["c_sym"], c["c_sym"])
    assert np.abs(g0["c_w"] - r0["c_w"]).reshape(4, 16).sum(1).max() < 1e-5
    P.close()


def test_ngram_graph_replay_is_bitwise_and_autotune_keeps_results(d2g):
    ph, c = synth.ngram_phase(200, 5, 32, 3, 20, (30, 300), 5, seed=66)
    opts = dict(maxIters=40, rhoCoeff=2.0, updatePerLoops=10)
    P = d2g.Phase(ph, 0)
    a = P.run(c, opts)
    b = P.run(c, opts)
    np.testing.assert_array_equal(a["c_w"], b["c_w"])
    np.testing.assert_array_equal(a["c_sym"], b["c_sym"])
    np.testing.assert_array_equal(a["trace"], b["trace"])
    t = P.autotune(c, dict(opts, maxIters=12))
    assert len(t["candidates"]) >= 2
    P.set_tuning(**t["best"])
    r = P.run(c, opts)
    assert np.abs(r["c_w"] - a["c_w"]).reshape(5, 32).sum(1).max() < 1e-5
    np.testing.assert_array_equal(r["c_sym"], a["c_sym"])
    P.close()


def test_ngram_entry_points_check_the_metric(d2g):
    ph, c = synth.ngram_phase(20, 2, 8, 2, 10, (5, 20), 2, seed=67)
    P = d2g.Phase(ph, 0)
    o = L.d2g_badmm_opts(10, 2.0, 10, 0.0)
    cw = np.array(c["c_w"])
    assert P.lib.d2g_badmm_run(P.h, C.byref(o), cw.ctypes.data, None, None) == L.D2G_E_INVAL
    P.close()
    bad = dict(c, c_sym=np.full_like(c["c_sym"], 10))  # symbol == V
    P = d2g.Phase(ph, 0)
    with pytest.raises(D2GError):
        P.run(bad, dict(maxIters=5))
    P.close()
    pe, ce = synth.euclidean_phase(20, 2, 8, 3, (4, 10), seed=68)
    P = d2g.Phase(pe, 0)
    sym = np.zeros(16, np.int32)
    assert P.lib.d2g_badmm_run_sym(P.h, C.byref(o), np.array(ce["c_w"]).ctypes.data,
                                   sym.ctypes.data, None) == L.D2G_E_INVAL
    P.close()


def test_ngram_calculate_distmat(d2g):
    """calculate_distmat (src/d2/centroid_util.c:31-33) on an n-gram phase,
    FP64 on the GPU, against the sum of symbol costs computed here."""
    lib = L.load()
    ph, c = synth.ngram_phase(50, 3, 12, 3, 20, (10, 80), 3, seed=69)
    p_str = np.ascontiguousarray(ph["p_str"], np.int32)
    col, m, dim, V = int(p_str.sum()), 12, 3, 20
    sym = np.ascontiguousarray(ph["p_supp_sym"], np.int32)
    dist = np.ascontiguousarray(ph["dist_mat"], np.float64)
    csym = np.ascontiguousarray(c["c_sym"], np.int32)
    label = np.ascontiguousarray(ph["label"], np.int32)
    data = L.sph()
    data.dim, data.str, data.col, data.metric_type, data.vocab_size = dim, m, col, L.D2_N_GRAM, V
    data.p_str = p_str.ctypes.data_as(C.POINTER(C.c_int))
    data.p_supp_sym = sym.ctypes.data_as(C.POINTER(C.c_int))
    data.dist_mat = dist.ctypes.data_as(C.POINTER(C.c_double))
    cen = L.sph()
    cen.dim, cen.str, cen.col = dim, m, 3 * m
    cen.p_supp_sym = csym.ctypes.data_as(C.POINTER(C.c_int))
    out = np.zeros(m * col)
    lib.calculate_distmat(C.byref(data), label.ctypes.data_as(C.POINTER(C.c_int)), p_str.size,
                          C.byref(cen), out.ctypes.data_as(C.POINTER(C.c_double)))
    inst = np.repeat(np.arange(p_str.size), p_str)
    A = csym.reshape(3, m, dim)[label[inst]]            # [col, m, dim] centroid symbols
    B = sym.reshape(col, 1, dim)                        # [col, 1, dim] instance symbols
    ref = dist.reshape(V, V)[A, B].sum(-1)              # [col, m]
    np.testing.assert_allclose(out, ref.reshape(-1), rtol=1e-15, atol=0)


@pytest.mark.parametrize("n,k,m,dim,V,lengths,upl,iters,seed", [
    (200, 5, 16, 1, 23, (10, 60), 10, 60, 67),   # 1-grams (the protein application's form)
    (150, 4, 8, 2, 8, (10, 80), 7, 45, 68),      # 2-grams over 8 symbols, odd updatePerLoops
])
def test_ngram_pair_passes_match_the_oracle_and_single_passes(d2g, oracle_mod, n, k, m, dim, V, lengths,
                                                               upl, iters, seed):
    """Plans that fit one CTA run two iterations per pass; a symbol update on
    a pair's second iteration counts its deferred Z (Z' times the plan's row
    scale).  Same symbols and bounds as the oracle, with about half the passes."""
    ph, c = synth.ngram_phase(n, k, m, dim, V, lengths, 4, seed=seed)
    opts = dict(maxIters=iters, rhoCoeff=2.0, updatePerLoops=upl)
    ref = _port(oracle_mod, ph, c, opts)
    assert np.any(ref["c_sym"] != c["c_sym"])  # the symbols moved
    passes = {}
    for pairs in (1, 0):
        d2g.set_config(pair_iterations=pairs)
        try:
            P = d2g.Phase(ph, 0)
            r = P.run(c, opts)
            r["Z"] = P.get_plans()
            d2g.set_config(profile=1)  # one timed launch per pass over the plans
            P.run(c, opts)
            passes[pairs] = P.stats()["plan_launches"]
            P.close()
        finally:
            d2g.set_config(pair_iterations=1, profile=0)
        assert r["stats"]["iterations"] == iters + 1
        assert_close(r, ref, k, m)
        assert _plan_l1(r["Z"], ref["Z"]) <= 1e-4
    assert passes[0] == iters + 1
    assert passes[1] <= 0.75 * passes[0], passes
