"""Phases updated at once from several host threads through the resident API
(each phase on its own stream, graphs captured thread-locally, the launchers'
cached launch shapes shared under a lock): every result equals the result of
the same update run alone, bit for bit."""
import threading

import numpy as np
import pytest

from d2_kmeans_gb300 import synth

pytestmark = pytest.mark.gpu


def _cases():
    e_ph, e_c = synth.euclidean_phase(3000, 6, 32, 3, (8, 128), True, 12, 0.5, seed=201)
    n_ph, n_c = synth.ngram_phase(400, 5, 16, 1, 23, (10, 60), 4, seed=202)
    h_ph, h_c = synth.histogram_phase(300, 4, side=4, alpha=0.2, seed=203)
    o = dict(maxIters=50, rhoCoeff=2.0, updatePerLoops=10)
    return [(e_ph, e_c, o), (n_ph, n_c, o), (h_ph, h_c, dict(o, maxIters=40))]


def _update_twice(d2g, ph, c, o):
    P = d2g.Phase(ph, 0)
    try:
        P.run(c, o)          # first run: launch shapes configured, loop captured
        return P.run(c, o)   # graph replay
    finally:
        P.close()


def _three_threads(d2g):
    cases = _cases()
    out, errs = [None] * len(cases), []

    def work(i):
        try:
            out[i] = _update_twice(d2g, *cases[i])
        except Exception as e:  # reported below, on the main thread
            errs.append(e)

    threads = [threading.Thread(target=work, args=(i,)) for i in range(len(cases))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errs, errs
    return out


FRESH = r"""
import os, sys, numpy as np
sys.path.insert(0, {root!r}); sys.path.insert(0, os.path.join({root!r}, "tests"))
from d2_kmeans_gb300 import badmm
badmm.set_config(verbose=0, precision=0, use_graph=1, profile=0, sync_scratch=0, cost_gemm=0)
import test_gpu_threads as T
out = T._three_threads(badmm)
np.savez({path!r}, **{{f"{{i}}_{{k}}": v for i, r in enumerate(out) for k, v in r.items()
                      if k in ("c_w", "c_supp", "c_sym", "trace") and v is not None}})
"""


def test_phases_on_three_threads_match_runs_alone(d2g, tmp_path):
    """The threads run first, in a fresh process: the launch shapes,
    shared-memory attributes and graphs are all configured for the first time
    while three phases race for them; then the same updates run alone."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    path = str(tmp_path / "threads.npz")
    subprocess.run([sys.executable, "-c", FRESH.format(root=root, path=path)], check=True, timeout=600)
    z = np.load(path)
    out = []
    for i in range(len(_cases())):
        out.append({k: z[f"{i}_{k}"] for k in ("c_w", "c_supp", "c_sym", "trace") if f"{i}_{k}" in z.files})
    alone = [_update_twice(d2g, *cs) for cs in _cases()]
    for a, b in zip(out, alone):
        np.testing.assert_array_equal(a["c_w"], b["c_w"])
        np.testing.assert_array_equal(a["trace"], b["trace"])
        for key in ("c_supp", "c_sym"):
            if b.get(key) is not None:
                np.testing.assert_array_equal(a[key], b[key])


def test_three_threads_in_this_process(d2g):
    """The same with the caches already configured (after the tests above)."""
    out = _three_threads(d2g)
    alone = [_update_twice(d2g, *cs) for cs in _cases()]
    for a, b in zip(out, alone):
        np.testing.assert_array_equal(a["c_w"], b["c_w"])
        np.testing.assert_array_equal(a["trace"], b["trace"])
