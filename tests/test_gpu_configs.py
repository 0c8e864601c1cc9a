"""Parity at the shapes of the five benchmark workloads, against the oracle
(the C restatement, bit-identical to the reference's own FP64 update), on the
same seeded inputs and iteration counts.  Each case keeps its workload's
support sizes, centroid size, dimension, cluster count, metric and iteration
schedule and cuts only the number of instances so that the FP64 oracle ends
in seconds:

  batched Euclidean   n = 5 000 (of 200 000), m_i log-uniform 8-128, d = 3,
                      k = 64, m = 32, 201 iterations, updates every 10
  word embeddings     100 documents (of 20 000) of 20-400 tokens over a
                      20 000 x 300 vocabulary, k = 20, m = 64, 101 iterations
  256-bin histograms  200 histograms (of 100 000), 16 x 16 grid cost, k = 32,
                      61 iterations (of 101)
  two-phase, phase 2  n = 10 000 (of 100 000), d = 3, m_i 4-32, k = 32,
                      m = 16, 101 iterations
  serving             k = 256 resident centroids, m = 64, d = 64; three
                      requests of 8, 120 and 512 supports; 60 B-ADMM
                      iterations per solve (of 200)
  mountaindat.d2      the reference's own data file, phase 0 (n = 2 000,
                      k = 10, m = 6, labels i % 10, centroids from the
                      reference's d2_centroid_rands), 101 iterations: the
                      reference's objective trace 949.944316 ... 731.139455

Tolerances (the parity bounds of every batched test): objective 1e-5
relative at every check, c_w L1 1e-4 per cluster, supports 1e-4 relative
per support point; serving costs 1e-4 relative, argmin identical wherever
the oracle's two best costs differ by more than that.  The oracle runs for all cases start together on host
threads when the module loads (the C oracle releases the GIL).
"""
import concurrent.futures as cf

import numpy as np
import pytest

from conftest import load_golden
from d2_kmeans_gb300 import synth
from test_gpu_badmm import assert_close

pytestmark = pytest.mark.gpu

REF_TRACE = [949.944316, 800.134253, 751.011049, 737.562036, 731.139455]


def _cases():
    out = {}
    ph, c, o = synth.workload("batched", seed=5, scale=0.025)
    out["batched"] = (ph, c, o)
    ph, c = synth.embed_phase(100, 20, 64, 20000, 300, (20, 400), 1.1, seed=6)
    out["embed"] = (ph, c, dict(maxIters=100, rhoCoeff=2.0, updatePerLoops=10))
    ph, c = synth.histogram_phase(200, 32, 16, 0.1, seed=7)
    out["hist"] = (ph, c, dict(maxIters=60, rhoCoeff=2.0, updatePerLoops=10))
    ph, c, o = synth.workload("twophase_euclid", seed=8, scale=0.1)
    out["twophase_euclid"] = (ph, c, o)
    return out


def _queries():
    c_w, c_supp, means = synth.serving_centroids(k=256, m=64, dim=64, n_comp=32, seed=0)
    rng = np.random.default_rng(3)
    qs = []
    for mq in (8, 120, 512):
        comp = rng.integers(0, means.shape[0], size=mq)
        w = rng.dirichlet(np.ones(mq))
        qs.append((w, means[comp] + rng.normal(size=(mq, means.shape[1]))))
    return c_w, c_supp, qs


SERVE_ITERS = 60


@pytest.fixture(scope="module")
def refs(oracle_mod):
    """Every oracle result of this module, computed on host threads at once."""
    cases = _cases()
    c_w, c_supp, qs = _queries()
    ex = cf.ThreadPoolExecutor(max_workers=8)
    fut = {name: ex.submit(oracle_mod.badmm, ph, c, o, "port", ()) for name, (ph, c, o) in cases.items()}
    for i, (w, s) in enumerate(qs):
        fut["serve%d" % i] = ex.submit(oracle_mod.serve_query, c_w, c_supp, w, s, SERVE_ITERS)
    yield cases, (c_w, c_supp, qs), fut
    ex.shutdown(wait=True)


@pytest.mark.parametrize("name", ["batched", "embed", "hist", "twophase_euclid"])
@pytest.mark.parametrize("pairs", [1, 0])
def test_workload_shape_matches_oracle(d2g, refs, name, pairs):
    cases, _, fut = refs
    ph, c, opts = cases[name]
    old = d2g.set_config(pair_iterations=pairs)
    try:
        P = d2g.Phase(ph, precision=0)
        r = P.run(c, opts)
        P.close()
    finally:
        d2g.set_config(pair_iterations=old["pair_iterations"])
    ref = fut[name].result()
    assert ref["rc"] == 0
    assert r["stats"]["path"] == 0 and r["stats"]["iterations"] == opts["maxIters"] + 1
    assert_close(r, ref, ph["num_of_labels"], ph["str"])


def test_serving_shape_matches_oracle(d2g, refs):
    from d2_kmeans_gb300 import serve
    _, (c_w, c_supp, qs), fut = refs
    S = serve.Server(c_w, c_supp, iters=SERVE_ITERS)
    try:
        for i, (w, s) in enumerate(qs):
            lab, cost, _ = S.solve(w, s)
            best, ref = fut["serve%d" % i].result()
            np.testing.assert_allclose(cost, ref, rtol=1e-4)
            order = np.sort(ref)
            if (order[1] - order[0]) / order[0] > 1e-4:
                assert lab == best
    finally:
        S.close()


@pytest.mark.parametrize("pairs", [1, 0])
def test_mountaindat_reference_trace(d2g, pairs):
    """The reference's data/mountaindat.d2 example: the objective trace of the
    reference's own run (stored in tests/golden/mountain_kat.npz by
    make_golden.py from the compiled reference)."""
    ph, c0, opts, exp = load_golden("mountain_kat")
    np.testing.assert_allclose(exp["out_trace"][:, 1], REF_TRACE, rtol=0, atol=5e-7)
    old = d2g.set_config(pair_iterations=pairs)
    try:
        P = d2g.Phase(ph, precision=0)
        r = P.run(c0, opts)
        P.close()
    finally:
        d2g.set_config(pair_iterations=old["pair_iterations"])
    obj = r["trace"][:, 1]
    np.testing.assert_allclose(obj, REF_TRACE, rtol=1e-5)
    assert_close(r, {"c_w": exp["out_c_w"], "c_supp": exp["out_c_supp"], "trace": exp["out_trace"]},
                 10, 6, trace_atol=5.1e-7)
