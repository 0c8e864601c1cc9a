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


def test_phases_on_three_threads_match_runs_alone(d2g):
    cases = _cases()
    alone = [_update_twice(d2g, *cs) for cs in cases]
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
    for a, b in zip(out, alone):
        np.testing.assert_array_equal(a["c_w"], b["c_w"])
        np.testing.assert_array_equal(a["trace"], b["trace"])
        for key in ("c_supp", "c_sym"):
            if b.get(key) is not None:
                np.testing.assert_array_equal(a[key], b[key])
