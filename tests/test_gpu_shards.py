"""The instance-sharded centroid update on the GPU (d2g_badmm_run_shards:
several phases, each one shard of the instances, on one device, exchanging
the cluster sums between their streams at the reference's MPI_Allreduce
sites, src/d2/centroid_Bregman.c:142,188,215-217,308-310).

* With rho taken over all shards, two or three shards give the one-phase
  result (the FP64 cross-shard sums only reassociate), and every shard ends
  with the same centroids, bit for bit.
* With each shard's own rho (the reference's MPI build), the shards match the
  oracle's restatement of that build run as two ranks.
Tolerances are those of the other parity tests: objective
1e-5 relative, c_w L1 1e-4 per cluster, supports 1e-4 relative.
"""
import threading

import numpy as np
import pytest

from d2_kmeans_gb300 import synth
from d2_kmeans_gb300._lib import D2GError, D2G_E_EMPTY_CLUSTER, D2G_E_INVAL, D2G_E_UNSUPPORTED
from test_gpu_badmm import assert_close

pytestmark = pytest.mark.gpu


def _case(name):
    if name == "batched":
        ph, c, o = synth.workload("batched", seed=21, scale=0.005)
        o = dict(o, maxIters=60)
    elif name == "plain":
        ph, c, o = synth.workload("plain", seed=22, scale=0.2)
    else:  # 256-bin histograms: plans wider than one CTA
        ph, c = synth.histogram_phase(40, 4, side=16, alpha=0.1, seed=23)
        o = dict(maxIters=40, rhoCoeff=2.0, updatePerLoops=10)
    return dict(ph, global_size=len(ph["p_str"])), c, o


def _bounds(n, nshard):
    return [(n * s // nshard, n * (s + 1) // nshard) for s in range(nshard)]


def _shards(d2g, oracle_mod, ph, nshard):
    n = len(ph["p_str"])
    return [d2g.Phase(oracle_mod.shard_phase(ph, lo, hi), 0) for lo, hi in _bounds(n, nshard)]


def _same_on_every_shard(res):
    for r in res[1:]:
        np.testing.assert_array_equal(r["c_w"], res[0]["c_w"])
        if r["c_supp"] is not None:
            np.testing.assert_array_equal(r["c_supp"], res[0]["c_supp"])
        np.testing.assert_array_equal(r["trace"][:, 1:], res[0]["trace"][:, 1:])


@pytest.mark.parametrize("name", ["batched", "plain", "hist"])
@pytest.mark.parametrize("nshard", [2, 3])
def test_shards_equal_one_phase_with_rho_over_all_shards(d2g, oracle_mod, name, nshard):
    ph, c, opts = _case(name)
    P = d2g.Phase(ph, 0)
    one = P.run(c, opts)
    P.close()
    Ps = _shards(d2g, oracle_mod, ph, nshard)
    try:
        res = d2g.run_shards(Ps, c, opts, global_rho=True)
    finally:
        for p in Ps:
            p.close()
    _same_on_every_shard(res)
    assert res[0]["stats"]["iterations"] == opts["maxIters"] + 1
    assert_close(res[0], one, ph["num_of_labels"], ph["str"])


def _oracle_ranks(oracle_mod, ph, c, opts, nshard):
    """The reference's MPI build restated by the oracle, one thread per rank."""
    n = len(ph["p_str"])
    shards = [oracle_mod.shard_phase(ph, lo, hi) for lo, hi in _bounds(n, nshard)]
    bar = threading.Barrier(nshard)
    slots = [None] * nshard
    out = [None] * nshard

    def rank(r):
        def ex(buf):
            slots[r] = buf.copy()
            bar.wait()
            tot = slots[0].copy()
            for q in range(1, nshard):
                tot += slots[q]
            buf[:] = tot
            bar.wait()
        out[r] = oracle_mod.badmm_mpi(shards[r], c, opts, ex, False)
    ts = [threading.Thread(target=rank, args=(r,)) for r in range(nshard)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return out


@pytest.mark.parametrize("name", ["plain", "hist"])
def test_shards_follow_the_reference_mpi_build(d2g, oracle_mod, name):
    ph, c, opts = _case(name)
    ref = _oracle_ranks(oracle_mod, ph, c, opts, 2)
    assert ref[0]["rc"] == 0 and ref[1]["rc"] == 0
    if name != "hist":  # (every dense 256-bin histogram has the same mean cost)
        assert ref[0]["rho"] != ref[1]["rho"]  # each rank's own rho, as in the reference
    Ps = _shards(d2g, oracle_mod, ph, 2)
    try:
        res = d2g.run_shards(Ps, c, opts, global_rho=False)
    finally:
        for p in Ps:
            p.close()
    for r in range(2):
        assert_close(res[r], ref[r], ph["num_of_labels"], ph["str"])
        np.testing.assert_allclose(res[r]["stats"]["rho"], ref[r]["rho"], rtol=1e-6)


def test_pair_passes_in_shards(d2g, oracle_mod):
    """Shards whose plans all fit one CTA take two iterations per pass, like
    the one-phase update; one iteration per pass gives the same result."""
    ph, c, opts = _case("batched")
    P = d2g.Phase(ph, 0)
    one = P.run(c, opts)
    P.close()
    out = {}
    for pairs in (1, 0):
        # (profile mode counts the passes over the plans)
        old = d2g.set_config(pair_iterations=pairs, profile=1)
        Ps = _shards(d2g, oracle_mod, ph, 2)
        try:
            out[pairs] = d2g.run_shards(Ps, c, opts, global_rho=True)
        finally:
            for p in Ps:
                p.close()
            d2g.set_config(pair_iterations=old["pair_iterations"], profile=old["profile"])
    assert out[0][0]["stats"]["plan_launches"] == opts["maxIters"] + 1
    assert out[1][0]["stats"]["plan_launches"] < opts["maxIters"] // 2 + 5
    for pairs in (1, 0):
        assert_close(out[pairs][0], one, ph["num_of_labels"], ph["str"])


def test_a_cluster_may_be_missing_from_one_shard(d2g, oracle_mod):
    ph, c, opts = _case("plain")
    n = len(ph["p_str"])
    label = np.array(ph["label"], np.int32)
    label[: n // 2][label[: n // 2] == 3] = 4  # cluster 3 only in the second half
    ph = dict(ph, label=label)
    P = d2g.Phase(ph, 0)
    one = P.run(c, opts)
    P.close()
    Ps = _shards(d2g, oracle_mod, ph, 2)
    try:
        with pytest.raises(D2GError) as e:  # the first shard alone lacks cluster 3
            Ps[0].run(c, opts)
        assert e.value.code == D2G_E_EMPTY_CLUSTER
        res = d2g.run_shards(Ps, c, opts, global_rho=True)
    finally:
        for p in Ps:
            p.close()
    assert_close(res[0], one, ph["num_of_labels"], ph["str"])


def test_refusals(d2g, oracle_mod):
    ph, c, opts = _case("plain")
    Ps = _shards(d2g, oracle_mod, ph, 2)
    try:
        with pytest.raises(D2GError) as e:  # every shard must run every iteration
            d2g.run_shards(Ps, c, dict(opts, time_budget=5.0))
        assert e.value.code == D2G_E_INVAL
        label = np.array(ph["label"], np.int32)
        label[label == 2] = 1  # cluster 2 on no shard at all
        Qs = _shards(d2g, oracle_mod, dict(ph, label=label), 2)
        try:
            with pytest.raises(D2GError) as e:
                d2g.run_shards(Qs, c, opts)
            assert e.value.code == D2G_E_EMPTY_CLUSTER
        finally:
            for q in Qs:
                q.close()
        # the phases are usable alone again after a sharded run
        assert_close(Ps[0].run(c, opts), oracle_mod.badmm(oracle_mod.shard_phase(ph, 0, len(ph["p_str"]) // 2),
                                                          c, opts, "port", want=()),
                     ph["num_of_labels"], ph["str"])
    finally:
        for p in Ps:
            p.close()
    pe, ce = synth.embed_phase(40, 2, 8, V=100, dim=8, sizes=(3, 12), seed=24)
    pe = dict(pe, global_size=len(pe["p_str"]))
    Es = _shards(d2g, oracle_mod, pe, 2)
    try:
        with pytest.raises(D2GError) as e:
            d2g.run_shards(Es, ce, opts)
        assert e.value.code == D2G_E_UNSUPPORTED
    finally:
        for p in Es:
            p.close()
