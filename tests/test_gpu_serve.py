"""Serving: fixed-centroid transport solves through d2g_server_* against the
oracle's restatement (d2o_serve_query: B-ADMM steps 1-3 of
src/d2/centroid_Bregman.c:155-175 with the centroid weights held fixed), the
same result alone and in a mix, and admission control.

Tolerance: transport costs within 1e-4 relative of the FP64 oracle after 200
iterations (FP32 plans); the argmin agrees wherever the oracle's best and
second-best costs differ by more than that.  Alone vs in a mix: the same
arithmetic runs for a request whatever batch it lands in, so the costs must
agree to 1e-6 relative (they are bitwise equal in practice)."""
import numpy as np
import pytest

from d2_kmeans_gb300 import synth
from d2_kmeans_gb300._lib import D2G_E_ADMISSION

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def serve_mod(d2g):
    from d2_kmeans_gb300 import serve
    return serve


def test_serve_matches_oracle(serve_mod, oracle_mod):
    c_w, c_supp, means = synth.serving_centroids(k=8, m=64, dim=16, n_comp=8, seed=3)
    S = serve_mod.Server(c_w, c_supp, iters=200)
    qs = synth.serving_queries(6, means, sizes=(4, 16), seed=4)
    rng = np.random.default_rng(7)
    # widths across the packing: several plans per CTA, 2-, 4- and 8-CTA clusters
    for mq in (70, 130, 300, 512):
        comp = rng.integers(0, means.shape[0], size=mq)
        w = rng.dirichlet(np.ones(mq))
        qs.append((w / w.sum(), means[comp] + rng.normal(size=(mq, means.shape[1]))))
    for w, s in qs:
        lab, cost, _ = S.solve(w, s)
        best, ref = oracle_mod.serve_query(c_w, c_supp, w, s, iters=200)
        np.testing.assert_allclose(cost, ref, rtol=1e-4)
        order = np.sort(ref)
        if (order[1] - order[0]) / order[0] > 1e-4:
            assert lab == best
    S.close()


@pytest.mark.parametrize("m", [12, 16, 32, 50])
def test_serve_support_sizes(serve_mod, oracle_mod, m):
    """Centroid supports of every padded size the server takes (16, 32, 64),
    full (m = 16, 32) and with padded rows (m = 12, 50), each with queries
    from one column group to 512 supports (several plans per CTA up to
    clusters of 8 CTAs); the same tolerances as above."""
    c_w, c_supp, means = synth.serving_centroids(k=8, m=m, dim=8, n_comp=6, seed=40 + m)
    S = serve_mod.Server(c_w, c_supp, iters=200)
    rng = np.random.default_rng(m)
    try:
        for mq in (3, 37, 130, 300, 512):
            comp = rng.integers(0, means.shape[0], size=mq)
            w = rng.dirichlet(np.ones(mq))
            s = means[comp] + rng.normal(size=(mq, means.shape[1]))
            lab, cost, _ = S.solve(w / w.sum(), s)
            best, ref = oracle_mod.serve_query(c_w, c_supp, w / w.sum(), s, iters=200)
            np.testing.assert_allclose(cost, ref, rtol=1e-4, err_msg=f"m={m} m_q={mq}")
            order = np.sort(ref)
            if (order[1] - order[0]) / order[0] > 1e-4:
                assert lab == best
    finally:
        S.close()


def test_same_result_alone_and_in_a_mix(serve_mod):
    c_w, c_supp, means = synth.serving_centroids(k=64, m=64, dim=32, n_comp=16, seed=5)
    S = serve_mod.Server(c_w, c_supp, iters=100)
    probe = synth.serving_queries(3, means, sizes=(4, 512), seed=6)
    alone = [S.solve(w, s)[:2] for w, s in probe]
    mix = synth.serving_queries(60, means, sizes=(4, 512), seed=8)
    tickets = []
    for i, (w, s) in enumerate(mix):
        tickets.append(("mix", S.submit(w, s)))
        if i % 20 == 10:
            j = i // 20
            tickets.append(("probe%d" % j, S.submit(*probe[j])))
    got = {}
    while tickets:
        rest = []
        for tag, t in tickets:
            r = S.result(t)
            if r is None:
                rest.append((tag, t))
            elif tag != "mix":
                got[tag] = r
        tickets = rest
        if tickets:
            S.wait()
    for j in range(3):
        lab, cost, _ = got["probe%d" % j]
        assert lab == alone[j][0]
        np.testing.assert_allclose(cost, alone[j][1], rtol=1e-6)
    S.close()


def test_admission_control_refuses_then_recovers(serve_mod):
    c_w, c_supp, means = synth.serving_centroids(k=16, m=64, dim=8, n_comp=4, seed=9)
    q = synth.serving_queries(3, means, sizes=(64, 64), seed=10)
    one = 64 * 9 * 4 + 16 * 4 + 64  # bytes one such request holds
    S = serve_mod.Server(c_w, c_supp, iters=50, hbm_budget_bytes=one + 10)
    t = S.submit(*q[0])
    assert S.try_submit(*q[1]) is None  # over the budget while the first is held
    while S.result(t) is None:
        S.wait()
    assert S.try_submit(*q[2]) is not None  # budget released with the result
    S.close()


def test_poisson_arrivals_all_complete(serve_mod):
    c_w, c_supp, means = synth.serving_centroids(k=256, m=64, dim=64, n_comp=32, seed=0)
    S = serve_mod.Server(c_w, c_supp, iters=200)
    qs = synth.serving_queries(200, means, sizes=(4, 512), seed=1)
    out = serve_mod.poisson_run(S, qs, rate=2000.0, seed=2)
    assert out["completed"] + out["refused"] == 200 and out["completed"] > 0
    assert out["p99_ms"] >= out["p50_ms"] > 0
    S.close()
