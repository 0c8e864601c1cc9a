"""Bounded device waits: a plan pass whose bulk copy never lands gives up,
reports, and leaves the phase and the CUDA context usable.

Every wait of the batched plan kernels on a bulk-copy mbarrier is bounded
(one second by default).  The test hook d2g_phase_test_wait withholds the
tile copy of one unit in the pass of one iteration and lowers the limit to a
few milliseconds, so the wait runs out without any fault: the run must return
D2G_E_CUDA with the wait's own message, and the next run on the same phase,
hook off, must match the oracle under the usual tolerances (objective 1e-5
relative, c_w L1 1e-4 per cluster, supports 1e-4 relative).
"""
import numpy as np
import pytest

from d2_kmeans_gb300 import synth
from d2_kmeans_gb300._lib import D2GError, D2G_E_CUDA
from test_gpu_badmm import assert_close

pytestmark = pytest.mark.gpu

WAIT_S = 0.003


def _case(name, scale, maxIters=None):
    ph, c, opts = synth.workload(name, seed=3, scale=scale)
    if maxIters is not None:
        opts = dict(opts, maxIters=maxIters)
    return ph, c, opts


# (workload, scale, iterations, faulted iteration, unit, pair passes)
CASES = [
    ("batched", 0.01, 30, 1, 0, 1),    # pair pass of iterations (1, 2), first unit of CTA 0
    ("batched", 0.01, 30, 1, 350, 1),  # a later unit of its CTA: the stage issued one unit ahead
    ("batched", 0.01, 30, 0, 0, 1),    # the single pass of iteration 0
    ("batched", 0.01, 30, 4, 3, 0),    # one iteration per pass
    ("embed", 0.005, 20, 1, 0, 1),     # pair pass with staged cost-table rows
    ("hist", 0.0005, 20, 1, 0, 1),     # 256-bin plans wider than a CTA, deferred exchange
]


@pytest.mark.parametrize("name,scale,iters,fit,unit,pairs", CASES)
def test_wait_runs_out_then_recovers(d2g, oracle_mod, name, scale, iters, fit, unit, pairs):
    ph, c, opts = _case(name, scale, iters)
    k, m = ph["num_of_labels"], ph["str"]
    old = d2g.set_config(pair_iterations=pairs)
    P = d2g.Phase(ph, precision=0)
    try:
        P.test_wait(iter=fit, unit=unit, wait_s=WAIT_S)
        with pytest.raises(D2GError) as e:
            P.run(c, opts)
        assert e.value.code == D2G_E_CUDA, str(e.value)
        assert "bounded wait ran out" in str(e.value), str(e.value)
        P.test_wait()  # hook off, default limit
        r = P.run(c, opts)
    finally:
        P.close()
        d2g.set_config(pair_iterations=old["pair_iterations"])
    ref = oracle_mod.badmm(ph, c, opts, "port", want=())
    assert_close(r, ref, k, m)


def test_hook_rejects_bad_limit(d2g):
    ph, c, opts = _case("batched", 0.002, 5)
    P = d2g.Phase(ph, precision=0)
    try:
        with pytest.raises(D2GError):
            P.test_wait(iter=0, unit=0, wait_s=-1.0)
        with pytest.raises(D2GError):
            P.test_wait(iter=0, unit=0, wait_s=100.0)
    finally:
        P.close()
