"""Parity of the CUDA B-ADMM centroid update (libd2g.so, through its C ABI)
against the reference's FP64 results: the committed golden fixtures (made by
the reference compiled from its own sources) and the C restatement of the
oracle on the same seeded inputs.

Tolerances (FP32 plans + FP64 cross-plan reductions against FP64):
  relative objective error            <= 1e-5   (every residual check)
  centroid weights, L1 per cluster    <= 1e-4
  support locations                   <= 1e-4 relative: |c_k - c_k,ref| / |c_k,ref| per
                                      support point (Euclidean norm over the d
                                      coordinates, floored at 1e-3 of the largest
                                      |c_k,ref| of the phase)
  n-gram centroid symbols             identical
The FP64 path (precision=1) is held to 1e-9.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from golden.make_golden import digest
from d2_kmeans_gb300 import synth
from d2_kmeans_gb300._lib import D2GError, D2G_E_EMPTY_CLUSTER

pytestmark = pytest.mark.gpu

OBJ_TOL, CW_TOL, SUPP_TOL = 1e-5, 1e-4, 1e-4


def assert_close(res, ref, k, m, fp64=False, trace_atol=0.0):
    """res / ref: dicts with c_w, c_supp, trace (iter, obj, primres, dualres)."""
    cw = np.asarray(res["c_w"]).reshape(k, m)
    cwr = np.asarray(ref["c_w"]).reshape(k, m)
    l1 = np.abs(cw - cwr).sum(axis=1).max()
    assert l1 <= (1e-10 if fp64 else CW_TOL), f"c_w L1 {l1}"
    if ref.get("c_supp") is not None and res.get("c_supp") is not None:
        s = np.asarray(res["c_supp"]).reshape(k * m, -1)
        sr = np.asarray(ref["c_supp"]).reshape(k * m, -1)
        nrm = np.linalg.norm(sr, axis=1)
        rel = (np.linalg.norm(s - sr, axis=1) / np.maximum(nrm, 1e-3 * nrm.max())).max()
        assert rel <= (1e-9 if fp64 else SUPP_TOL), f"support rel err {rel}"
    if ref.get("c_sym") is not None:
        np.testing.assert_array_equal(np.asarray(res["c_sym"]).reshape(-1),
                                      np.asarray(ref["c_sym"]).reshape(-1), err_msg="c_sym")
    tr, trr = np.asarray(res["trace"]), np.asarray(ref["trace"])
    assert tr.shape == trr.shape, (tr.shape, trr.shape)
    if trr.size == 0:
        return
    np.testing.assert_array_equal(tr[:, 0], trr[:, 0])
    obj_err = np.abs(tr[:, 1] - trr[:, 1]) / np.abs(trr[:, 1])
    assert obj_err.max() <= (1e-9 if fp64 else OBJ_TOL) + trace_atol / np.abs(trr[:, 1]).min(), \
        f"objective rel err {obj_err}"


def golden_ref(exp):
    return {"c_w": exp["out_c_w"], "c_supp": exp.get("out_c_supp"), "c_sym": exp.get("out_c_sym"),
            "trace": exp["out_trace"]}


def run_phase(d2g, ph, c0, opts, precision, exp=None):
    """One resident-API call; for the warm fixture, the two-call sequence."""
    if exp is not None and "first_label" in exp:
        first = dict(ph, label=exp["first_label"])
        P = d2g.Phase(first, precision)
        r1 = P.run({"c_w": exp["first_c_w"], "c_supp": exp["first_c_supp"]}, opts)
        P.set_labels(ph["label"])
        r = P.run({"c_w": r1["c_w"], "c_supp": r1["c_supp"]}, opts, label_switch=ph["label_switch"])
    else:
        P = d2g.Phase(ph, precision)
        r = P.run(c0, opts)
    r["Z"] = P.get_plans()
    P.close()
    return r


@pytest.mark.parametrize("name", golden_names())
def test_batched_fp32_matches_golden(d2g, name):
    ph, c0, opts, exp = load_golden(name)
    r = run_phase(d2g, ph, c0, opts, 0, exp)
    assert r["stats"]["path"] == 0
    assert_close(r, golden_ref(exp), ph["num_of_labels"], ph["str"], trace_atol=5.1e-7)


@pytest.mark.parametrize("name", golden_names())
def test_plain_fp64_matches_golden(d2g, name):
    ph, c0, opts, exp = load_golden(name)
    r = run_phase(d2g, ph, c0, opts, 1, exp)
    assert r["stats"]["path"] == 1
    assert_close(r, golden_ref(exp), ph["num_of_labels"], ph["str"], fp64=True, trace_atol=5.1e-7)
    np.testing.assert_allclose(digest(r["Z"]), exp["out_Z_digest"], rtol=1e-9, atol=1e-15)


@pytest.mark.parametrize("name", golden_names())
def test_dropin_matches_golden(d2g, name):
    """Through d2_centroid_sphBregman with the reference's own structures."""
    ph, c0, opts, exp = load_golden(name)
    if "first_label" in exp:
        first = dict(ph, label=exp["first_label"])
        d = d2g.DropIn(first, {"c_w": exp["first_c_w"], "c_supp": exp["first_c_supp"]})
        assert d.call(opts) == 0
        assert d.call(opts, label_switch=ph["label_switch"], labels=ph["label"]) == 0
    else:
        d = d2g.DropIn(ph, c0)
        assert d.call(opts) == 0
    res = {"c_w": d.c_w, "c_supp": d.c_supp, "c_sym": d.c_sym}
    Z = d.Z()
    d.close()
    ref = golden_ref(exp)
    ref["trace"] = np.zeros((0, 4))
    res["trace"] = np.zeros((0, 4))
    assert_close(res, ref, ph["num_of_labels"], ph["str"])
    dz = digest(Z)
    np.testing.assert_allclose(dz[:3], exp["out_Z_digest"][:3], rtol=1e-4)


def _port(oracle_mod, ph, c, opts):
    r = oracle_mod.badmm(ph, c, opts, "port", want=())
    assert r["rc"] == 0
    return r


def test_plain_config_full_size(d2g, oracle_mod):
    """The n=2000, d=3, m_i 4..16, k=10, m=16, 100-iteration workload, both forms."""
    ph, c, opts = synth.workload("plain", seed=0)
    ref = _port(oracle_mod, ph, c, opts)
    for precision in (0, 1):
        P = d2g.Phase(ph, precision)
        r = P.run(c, opts)
        assert_close(r, ref, 10, 16, fp64=precision == 1)
        assert r["stats"]["iterations"] == 101
        np.testing.assert_allclose(r["stats"]["rho"], ref["rho"], rtol=1e-6 if precision == 0 else 1e-13)
        P.close()


@pytest.mark.parametrize("m,dim,lo,hi,k,seed", [
    (5, 1, 1, 9, 3, 21), (12, 2, 3, 40, 4, 22), (40, 6, 10, 300, 3, 23),
    (100, 8, 2, 64, 3, 24), (64, 3, 200, 700, 2, 25), (3, 4, 1, 4, 2, 26),
])
def test_batched_odd_shapes(d2g, oracle_mod, m, dim, lo, hi, k, seed):
    ph, c = synth.euclidean_phase(40, k, m, dim, (lo, hi), False, 5, 1.0, seed=seed)
    opts = dict(maxIters=30, rhoCoeff=2.0, updatePerLoops=10)
    ref = _port(oracle_mod, ph, c, opts)
    P = d2g.Phase(ph, 0)
    r = P.run(c, opts)
    # plans wider than an 8-CTA cluster run on the FP64 form
    assert_close(r, ref, k, m, fp64=r["stats"]["path"] == 1)
    P.close()


EXCHANGES = ["deferred", "cluster"]


def _exchange(monkeypatch, exchange):
    """Plans wider than one CTA: deferred row normalisation (default) or the
    synchronous DSMEM exchange on a thread-block cluster."""
    if exchange == "cluster":
        monkeypatch.setenv("D2G_WIDE_EXCHANGE", "cluster")
    else:
        monkeypatch.delenv("D2G_WIDE_EXCHANGE", raising=False)


@pytest.mark.parametrize("exchange", EXCHANGES)
def test_histogram_256_bins_cluster_path(d2g, oracle_mod, monkeypatch, exchange):
    """256-bin plans span 8 CTA slices (row sums exchanged deferred or in a cluster)."""
    _exchange(monkeypatch, exchange)
    ph, c = synth.histogram_phase(10, 2, side=16, alpha=0.1, seed=31)
    opts = dict(maxIters=30, rhoCoeff=2.0, updatePerLoops=10)
    ref = _port(oracle_mod, ph, c, opts)
    P = d2g.Phase(ph, 0)
    assert_close(P.run(c, opts), ref, 2, 256)
    P.close()


def _plan_l1(Z, Zr):
    return np.abs(np.asarray(Z) - np.asarray(Zr)).sum() / np.abs(np.asarray(Zr)).sum()


@pytest.mark.parametrize("exchange", EXCHANGES)
def test_wide_plans_warm_start(d2g, oracle_mod, monkeypatch, exchange):
    """Two calls on wide plans, the second warm-started (label_switch = 0) from
    the Z the first left.  The first call ends on iteration 25, which runs
    deferred, so its Z must be the row-scaled plan; Z within 1e-4 relative L1."""
    _exchange(monkeypatch, exchange)
    ph, c = synth.histogram_phase(12, 3, side=16, alpha=0.1, seed=33)
    o1 = dict(maxIters=25, rhoCoeff=2.0, updatePerLoops=10)
    o2 = dict(maxIters=12, rhoCoeff=2.0, updatePerLoops=10)
    r1 = oracle_mod.badmm(ph, c, o1, "port", want=())
    ph2 = dict(ph, label_switch=np.zeros(len(ph["p_str"]), np.int8))
    r2 = oracle_mod.badmm(ph2, dict(c_w=r1["c_w"], c_supp=None, Z=r1["Z"]), o2, "port", want=())
    P = d2g.Phase(ph, 0)
    g1 = P.run(c, o1)
    assert_close(g1, r1, 3, 256)
    assert _plan_l1(P.get_plans(), r1["Z"]) <= 1e-4
    g2 = P.run(dict(c_w=g1["c_w"], c_supp=None), o2, label_switch=ph2["label_switch"])
    assert_close(g2, r2, 3, 256)
    assert _plan_l1(P.get_plans(), r2["Z"]) <= 1e-4
    P.close()


@pytest.mark.parametrize("exchange", EXCHANGES)
def test_wide_plans_time_budget(d2g, oracle_mod, monkeypatch, exchange):
    """The loop stops after iteration 0 (deferred for wide plans): c_w and the
    plans left behind equal one iteration of the reference."""
    _exchange(monkeypatch, exchange)
    ph, c = synth.histogram_phase(8, 2, side=16, alpha=0.1, seed=34)
    ref = oracle_mod.badmm(ph, c, dict(maxIters=0, rhoCoeff=2.0, updatePerLoops=10), "port", want=())
    P = d2g.Phase(ph, 0)
    r = P.run(c, dict(maxIters=50, rhoCoeff=2.0, updatePerLoops=10, time_budget=1e-9))
    assert r["stats"]["iterations"] == 1
    cw = np.asarray(r["c_w"]).reshape(2, 256)
    assert np.abs(cw - ref["c_w"].reshape(2, 256)).sum(1).max() < 1e-5
    assert _plan_l1(P.get_plans(), ref["Z"]) <= 1e-5
    P.close()


def test_sparse_histogram(d2g, oracle_mod):
    rng = np.random.default_rng(5)
    V, n, k = 24, 30, 3
    D = synth.grid_cost(int(np.sqrt(V))) if False else np.abs(
        np.subtract.outer(np.arange(V), np.arange(V))).astype(float) ** 1.5
    p_str = rng.integers(2, 10, size=n).astype(np.int32)
    syms = np.concatenate([np.sort(rng.choice(V, size=s, replace=False)) for s in p_str]).astype(np.int32)
    w = np.concatenate([rng.dirichlet(np.ones(s)) for s in p_str])
    lab = np.concatenate([np.arange(k), rng.integers(0, k, size=n - k)]).astype(np.int32)
    ph = dict(metric=12, dim=0, str=V, p_str=p_str, p_w=w, p_supp_sym=syms, dist_mat=D.reshape(-1),
              vocab_size=V, label=lab, num_of_labels=k, label_switch=np.ones(n, np.int8))
    c = dict(c_w=rng.dirichlet(np.ones(V), size=k).reshape(-1), c_supp=None)
    opts = dict(maxIters=40, rhoCoeff=2.0, updatePerLoops=10)
    ref = _port(oracle_mod, ph, c, opts)
    for precision in (0, 1):
        P = d2g.Phase(ph, precision)
        assert_close(P.run(c, opts), ref, k, V, fp64=precision == 1)
        P.close()


def test_time_budget_stops_after_first_iteration(d2g, oracle_mod):
    ph, c = synth.euclidean_phase(60, 3, 8, 3, (4, 12), seed=41)
    ref = _port(oracle_mod, ph, c, dict(maxIters=0, rhoCoeff=2.0, updatePerLoops=10))
    for precision in (0, 1):
        P = d2g.Phase(ph, precision)
        r = P.run(c, dict(maxIters=50, rhoCoeff=2.0, updatePerLoops=10, time_budget=1e-9))
        assert r["stats"]["iterations"] == 1
        cw = np.asarray(r["c_w"]).reshape(3, 8)
        assert np.abs(cw - ref["c_w"].reshape(3, 8)).sum(1).max() < 1e-5
        P.close()


def test_empty_cluster_is_an_error(d2g):
    ph, c = synth.euclidean_phase(30, 4, 8, 3, (4, 10), seed=42)
    ph["label"][:] = 0
    ph["label"][1] = 1
    with pytest.raises(D2GError) as e:
        d2g.Phase(ph, 0)
    assert e.value.code == D2G_E_EMPTY_CLUSTER


def test_bitwise_reproducible_and_graph_equals_direct(d2g):
    ph, c, opts = synth.workload("plain", seed=3, scale=0.5)
    outs = []
    for graph in (1, 1, 0):
        d2g.set_config(use_graph=graph)
        P = d2g.Phase(ph, 0)
        r = P.run(c, opts)
        outs.append((r["c_w"], r["c_supp"], P.get_plans(), r["trace"]))
        P.close()
    d2g.set_config(use_graph=1)
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            np.testing.assert_array_equal(a, b)


def test_repeated_runs_reuse_the_graph(d2g):
    ph, c, opts = synth.workload("plain", seed=4, scale=0.3)
    P = d2g.Phase(ph, 0)
    a = P.run(c, opts)
    b = P.run(c, opts)
    np.testing.assert_array_equal(a["c_w"], b["c_w"])
    P.close()


@pytest.mark.parametrize("gemm", [0, 1], ids=["tcgen05_3xtf32", "fp32_cuda_cores"])
@pytest.mark.parametrize("n,k,m,V,dim,sizes,seed", [
    (60, 3, 8, 300, 12, (3, 25), 61),       # small: several plans per CTA
    (120, 4, 64, 2000, 300, (20, 400), 62),  # the embedding workload's shape: d=300, m=64, plans up to 400 wide
    (80, 5, 24, 517, 13, (5, 60), 63),      # ragged: d % 4 != 0, k*m and V not multiples of the 128 x 256 tile
])
def test_word_embedding_batched(d2g, oracle_mod, gemm, n, k, m, V, dim, sizes, seed):
    """Cost table T[l][v][k] from a (k*m) x V x d contraction (tensor cores in
    3xTF32, or FP32 CUDA cores), support update from the stored X through
    per-(cluster, token) occurrence lists."""
    ph, c = synth.embed_phase(n, k, m, V=V, dim=dim, sizes=sizes, seed=seed)
    opts = dict(maxIters=30, rhoCoeff=2.0, updatePerLoops=10)
    ref = _port(oracle_mod, ph, c, opts)
    old = d2g.set_config(cost_gemm=gemm)
    try:
        P = d2g.Phase(ph, 0)
        r = P.run(c, opts)
    finally:
        d2g.set_config(**old)
    assert r["stats"]["path"] == 0
    assert_close(r, ref, k, m)
    P.close()


def test_word_embedding_cost_table_paths_agree(d2g):
    """The tensor-core (3xTF32) and CUDA-core (FP32) cost tables give the same
    B-ADMM run up to FP32 rounding: objectives within 2e-6 relative, centroid
    weights within 1e-5 in L1."""
    ph, c = synth.embed_phase(200, 6, 64, V=3000, dim=300, sizes=(20, 200), seed=64)
    opts = dict(maxIters=40, rhoCoeff=2.0, updatePerLoops=10)
    out = []
    for gemm in (0, 1):
        old = d2g.set_config(cost_gemm=gemm)
        try:
            P = d2g.Phase(ph, 0)
            out.append(P.run(c, opts))
            P.close()
        finally:
            d2g.set_config(**old)
    a, b = out
    np.testing.assert_allclose(a["trace"][:, 1], b["trace"][:, 1], rtol=2e-6)
    assert np.abs(a["c_w"] - b["c_w"]).sum() <= 1e-5 * 6


def test_autotune_times_every_candidate_and_keeps_results(d2g, oracle_mod, tmp_path, monkeypatch):
    """The autotuner times every candidate tuning (wide-plan exchange x table-cost
    staging x CTAs per SM x cost-table GEMM x unit order for an embedding phase
    with plans wider than one CTA), keeps the fastest, leaves the phase's plans as they
    were, records the choice in the D2G_TUNE_CACHE file, and a new phase of the
    same shape starts from it.  The tuned phase still matches the oracle."""
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("D2G_TUNE_CACHE", str(cache))
    ph, c = synth.embed_phase(100, 4, 64, V=1500, dim=300, sizes=(20, 400), seed=65)
    opts = dict(maxIters=30, rhoCoeff=2.0, updatePerLoops=10)
    ref = _port(oracle_mod, ph, c, opts)
    P = d2g.Phase(ph, 0)
    P.run(c, opts)
    z0 = P.get_plans()
    out = P.autotune(c, dict(maxIters=12, rhoCoeff=2.0, updatePerLoops=10))
    cands = out["candidates"]
    assert len(cands) == 32
    assert all(0 < ms < 1e9 for _, ms in cands)
    fastest = min(cands, key=lambda r: r[1])[0]
    assert out["best"] == fastest
    np.testing.assert_array_equal(P.get_plans(), z0)
    assert_close(P.run(c, opts), ref, 4, 64)
    P.close()
    rec = cache.read_text().split()
    keys = ("exchange", "stage_costs", "ctas_per_sm", "cost_gemm", "pairs", "unit_order", "stage_scales")
    assert len(rec) == 8 and [int(v) for v in rec[1:]] == [fastest[k] for k in keys]
    Q = d2g.Phase(ph, 0)
    assert Q.tuning() == fastest
    Q.close()


def test_autotune_tile_schedule_of_the_batched_phase(d2g, oracle_mod):
    """Plans that all fit one CTA: the autotuner also chooses two iterations per
    pass or one, the walk order of the units and whether a pair pass stages its
    row scales (12 candidates with the CTAs per SM); every choice matches the
    oracle."""
    ph, c, opts = synth.workload("batched", seed=41, scale=0.01)
    opts = dict(opts, maxIters=40)
    ref = _port(oracle_mod, ph, c, opts)
    P = d2g.Phase(ph, 0)
    out = P.autotune(c, dict(opts, maxIters=12))
    cands = [t for t, _ in out["candidates"]]
    assert len(cands) == 12
    assert {t["pairs"] for t in cands} == {0, 1} and {t["unit_order"] for t in cands} == {0, 1}
    for t in cands:
        P.set_tuning(**t)
        assert_close(P.run(c, opts), ref, 64, 32)
    P.close()


@pytest.mark.parametrize("exchange", EXCHANGES)
def test_widest_packable_plan_and_one_more(d2g, oracle_mod, monkeypatch, exchange):
    """m = 32 packs 128 columns per CTA and a plan over at most 8 CTAs: a
    1024-column plan runs batched (8 slices); a 1025-column plan runs on the
    FP64 form.  Both match the oracle."""
    _exchange(monkeypatch, exchange)
    for width, path in ((1024, 0), (1025, 1)):
        ph, c = synth.euclidean_phase(6, 2, 32, 3, (4, 40), False, 5, 1.0, seed=71)
        ph["p_str"][0] = width
        rng = np.random.default_rng(72)
        cum = np.concatenate([[0], np.cumsum(ph["p_str"])])
        ph["p_w"] = np.concatenate([rng.dirichlet(np.ones(s)) for s in ph["p_str"]])
        ph["p_supp"] = rng.normal(size=(int(cum[-1]), 3)).reshape(-1) * 3.0
        opts = dict(maxIters=20, rhoCoeff=2.0, updatePerLoops=10)
        ref = _port(oracle_mod, ph, c, opts)
        P = d2g.Phase(ph, 0)
        r = P.run(c, opts)
        assert r["stats"]["path"] == path
        assert_close(r, ref, 2, 32, fp64=path == 1)
        P.close()


def test_read_file_then_update(d2g, oracle_mod, tmp_path):
    """A d2 file read by d2g_read feeds the batched centroid update; the result
    matches the oracle on the same arrays."""
    from d2_kmeans_gb300 import d2io
    ph, c = synth.euclidean_phase(300, 5, 16, 3, (4, 30), False, 8, 1.0, seed=81)
    f = str(tmp_path / "p.d2")
    d2io.write(f, [dict(metric=d2io.EUCLIDEAN, dim=3, p_str=ph["p_str"], p_w=ph["p_w"], p_supp=ph["p_supp"])])
    data = d2io.read(f, 300, [3], [d2io.EUCLIDEAN], avg_strides=[17])
    rd = d2io.phase_dict(data, 0, 16, ph["label"], 5)
    np.testing.assert_array_equal(rd["p_str"], ph["p_str"])
    opts = dict(maxIters=30, rhoCoeff=2.0, updatePerLoops=10)
    ref = _port(oracle_mod, rd, c, opts)
    P = d2g.Phase(rd, 0)
    assert_close(P.run(c, opts), ref, 5, 16)
    P.close()


def test_dropin_random_init_uses_the_programs_rands(d2g, rands_stub):
    """c0 == NULL initialises c with the program's d2_centroid_rands, then runs
    the same update as a call whose c0 holds that initialisation."""
    from conftest import rands_stub_init
    ph, c = synth.euclidean_phase(400, 4, 8, 3, (4, 12), False, 6, 1.0, seed=91)
    opts = dict(maxIters=40, rhoCoeff=2.0, updatePerLoops=10)
    a = d2g.DropIn(ph, c)
    assert a.call(opts, random_init=True) == 0
    b = d2g.DropIn(ph, rands_stub_init(ph, 4, 8))
    assert b.call(opts) == 0
    assert np.array_equal(a.c_w, b.c_w) and np.array_equal(a.c_supp, b.c_supp)
    assert np.array_equal(a.Z(), b.Z())
    a.close()
    b.close()


@pytest.mark.parametrize("case", ["euclid_upl10", "euclid_upl7_odd", "euclid_d8", "hist16", "embed_small", "m6_d2"])
def test_pair_passes_match_the_oracle_and_single_passes(d2g, oracle_mod, case):
    """Two iterations per HBM pass (plan_pair.cuh) against the oracle and
    against one iteration per pass: the same bounds; odd updatePerLoops and
    odd iteration counts put single passes after pairs (their deferred scale
    applied first)."""
    if case == "euclid_upl10":
        ph, c = synth.euclidean_phase(300, 5, 32, 3, (8, 128), True, 12, 0.5, seed=71)
        opts = dict(maxIters=60, rhoCoeff=2.0, updatePerLoops=10)
    elif case == "euclid_upl7_odd":
        ph, c = synth.euclidean_phase(250, 4, 16, 3, (4, 60), False, 8, 1.0, seed=72)
        opts = dict(maxIters=45, rhoCoeff=2.0, updatePerLoops=7)
    elif case == "euclid_d8":
        ph, c = synth.euclidean_phase(200, 4, 12, 7, (3, 40), False, 6, 1.0, seed=73)
        opts = dict(maxIters=40, rhoCoeff=1.5, updatePerLoops=5)
    elif case == "hist16":
        ph, c = synth.histogram_phase(150, 4, side=4, alpha=0.2, seed=74)
        opts = dict(maxIters=50, rhoCoeff=2.0, updatePerLoops=10)
    elif case == "embed_small":
        ph, c = synth.embed_phase(120, 3, 8, V=400, dim=16, sizes=(3, 30), seed=75)
        opts = dict(maxIters=40, rhoCoeff=2.0, updatePerLoops=10)
    else:
        ph, c = synth.euclidean_phase(180, 3, 6, 2, (2, 20), False, 5, 1.0, seed=76)
        opts = dict(maxIters=33, rhoCoeff=2.0, updatePerLoops=4)
    k, m = ph["num_of_labels"], ph["str"]
    ref = _port(oracle_mod, ph, c, opts)
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
        assert r["stats"]["iterations"] == opts["maxIters"] + 1
        assert_close(r, ref, k, m)
        assert _plan_l1(r["Z"], ref["Z"]) <= 1e-4
    # about half the passes over the plans with pairs
    assert passes[0] == opts["maxIters"] + 1
    assert passes[1] <= 0.75 * passes[0], passes


def test_pair_passes_warm_start_and_budget(d2g, oracle_mod):
    """A warm-started second call on plans left by a pair pass; with a time
    budget the loop runs single passes and stops after iteration 0."""
    ph, c = synth.euclidean_phase(200, 4, 16, 3, (4, 40), False, 8, 1.0, seed=77)
    o1 = dict(maxIters=30, rhoCoeff=2.0, updatePerLoops=10)
    r1 = _port(oracle_mod, ph, c, o1)
    ph2 = dict(ph, label_switch=np.zeros(len(ph["p_str"]), np.int8))
    r2 = _port(oracle_mod, ph2, dict(c_w=r1["c_w"], c_supp=r1["c_supp"], Z=r1["Z"]), o1)
    P = d2g.Phase(ph, 0)
    g1 = P.run(c, o1)
    assert_close(g1, r1, 4, 16)
    assert _plan_l1(P.get_plans(), r1["Z"]) <= 1e-4
    g2 = P.run(dict(c_w=g1["c_w"], c_supp=g1["c_supp"]), o1, label_switch=ph2["label_switch"])
    assert_close(g2, r2, 4, 16)
    r0 = _port(oracle_mod, ph, c, dict(maxIters=0, rhoCoeff=2.0, updatePerLoops=10))
    g0 = P.run(c, dict(maxIters=30, rhoCoeff=2.0, updatePerLoops=10, time_budget=1e-9))
    assert g0["stats"]["iterations"] == 1
    assert np.abs(g0["c_w"] - r0["c_w"]).reshape(4, 16).sum(1).max() < 1e-5
    P.close()
