"""Instance-sharded centroid update on the CPU: the oracle's restatement of
the reference's MPI build (src/d2/centroid_Bregman.c with __USE_MPI__: SUM
all-reduces of the label counts :142, cluster weights :188, support
numerators and X row sums :215-217 / :250-252, n-gram symbol counts :282 and
the three residuals :308-310) run as two gloo ranks, each on its shard of
the instances.

* One rank with an identity exchange is the serial update, bit for bit.
* Two gloo ranks give both ranks the same centroids, equal bit for bit to two
  threads of one process exchanging by a plain sum (a + b is the same in
  either order), so the exchange is what the reference's MPI_Allreduce does.
* Like the reference, each rank takes rho from its own instances; with rho
  taken over all ranks instead, two shards equal one shard up to the order of
  the FP64 sums: c_w L1 <= 1e-12 per cluster, objective 1e-12 relative.
"""
import os
import socket
import threading

import numpy as np
import pytest

from d2_kmeans_gb300 import synth

torch = pytest.importorskip("torch")

OPTS = dict(maxIters=40, rhoCoeff=2.0, updatePerLoops=10)


def _case(metric):
    if metric == "euclid":
        ph, c = synth.euclidean_phase(120, 4, 8, 3, (3, 20), False, 6, 1.0, seed=71)
    elif metric == "hist":
        ph, c = synth.histogram_phase(80, 3, side=4, alpha=0.3, seed=72)
    elif metric == "embed":
        ph, c = synth.embed_phase(60, 3, 8, V=200, dim=12, sizes=(3, 20), seed=73)
    else:
        ph, c = synth.ngram_phase(80, 3, 8, 2, 10, (10, 40), 4, seed=74)
    ph = dict(ph, global_size=len(ph["p_str"]))
    return ph, c


def _split(ph, k):
    """Two shards, each holding every cluster (the reference asserts that no
    cluster is empty across all ranks; here each shard has all of them too)."""
    n = len(ph["p_str"])
    return [(0, n // 2), (n // 2, n)]


@pytest.mark.parametrize("metric", ["euclid", "hist", "embed", "ngram"])
def test_one_rank_is_the_serial_update(oracle_mod, metric):
    ph, c = _case(metric)
    ser = oracle_mod.badmm(ph, c, OPTS, "port", want=())
    one = oracle_mod.badmm_mpi(ph, c, OPTS, lambda buf: None)
    assert ser["rc"] == 0 and one["rc"] == 0
    for key in ("c_w", "Z", "trace"):
        np.testing.assert_array_equal(one[key], ser[key])
    if c.get("c_supp") is not None:
        np.testing.assert_array_equal(one["c_supp"], ser["c_supp"])
    if c.get("c_sym") is not None:
        np.testing.assert_array_equal(one["c_sym"], ser["c_sym"])


def _threads(oracle_mod, ph, c, global_rho):
    """Two ranks as two threads of this process, exchanging by a plain sum."""
    shards = [oracle_mod.shard_phase(ph, lo, hi) for lo, hi in _split(ph, None)]
    bar = threading.Barrier(2)
    slots = [None, None]
    out = [None, None]

    def rank(r):
        def ex(buf):
            slots[r] = buf.copy()
            bar.wait()
            buf[:] = slots[0] + slots[1]
            bar.wait()
        out[r] = oracle_mod.badmm_mpi(shards[r], c, OPTS, ex, global_rho)
    ts = [threading.Thread(target=rank, args=(r,)) for r in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return out


def _gloo_rank(rank, port, metric, global_rho, outdir):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    import oracle
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=2)
    ph, c = _case(metric)
    lo, hi = _split(ph, None)[rank]

    def ex(buf):
        t = torch.from_numpy(buf)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
    r = oracle.badmm_mpi(oracle.shard_phase(ph, lo, hi), c, OPTS, ex, global_rho)
    np.savez(os.path.join(outdir, f"rank{rank}.npz"), c_w=r["c_w"], c_supp=r["c_supp"],
             trace=r["trace"], rc=r["rc"], rho=r["rho"])
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("metric", ["euclid", "ngram"])
@pytest.mark.parametrize("global_rho", [False, True])
def test_two_gloo_ranks(oracle_mod, tmp_path, metric, global_rho):
    import torch.multiprocessing as tmp
    tmp.spawn(_gloo_rank, args=(_free_port(), metric, global_rho, str(tmp_path)), nprocs=2, join=True)
    got = [np.load(tmp_path / f"rank{r}.npz") for r in range(2)]
    assert int(got[0]["rc"]) == 0 and int(got[1]["rc"]) == 0
    np.testing.assert_array_equal(got[0]["c_w"], got[1]["c_w"])
    np.testing.assert_array_equal(got[0]["c_supp"], got[1]["c_supp"])
    ph, c = _case(metric)
    th = _threads(oracle_mod, ph, c, global_rho)
    for r in range(2):
        np.testing.assert_array_equal(got[r]["c_w"], th[r]["c_w"])
        np.testing.assert_array_equal(got[r]["trace"], th[r]["trace"])


@pytest.mark.parametrize("metric", ["euclid", "hist", "embed", "ngram"])
def test_two_shards_equal_one_with_rho_over_all_ranks(oracle_mod, metric):
    ph, c = _case(metric)
    one = oracle_mod.badmm(ph, c, OPTS, "port", want=())
    two = _threads(oracle_mod, ph, c, True)
    k, m = ph["num_of_labels"], ph["str"]
    for r in range(2):
        assert two[r]["rc"] == 0
        l1 = np.abs(two[r]["c_w"].reshape(k, m) - one["c_w"].reshape(k, m)).sum(1).max()
        assert l1 <= 1e-12, l1
        obj = np.abs(two[r]["trace"][:, 1] - one["trace"][:, 1]) / np.abs(one["trace"][:, 1])
        assert obj.max() <= 1e-12, obj
        if c.get("c_sym") is not None:
            np.testing.assert_array_equal(two[r]["c_sym"], one["c_sym"])


def test_rank_local_rho_differs_like_the_reference(oracle_mod):
    """The reference's MPI build takes rho from each rank's own instances
    (:109 sits outside any #ifdef __USE_MPI__), so the ranks' rho differ."""
    ph, c = _case("euclid")
    two = _threads(oracle_mod, ph, c, False)
    assert two[0]["rho"] != two[1]["rho"]
    np.testing.assert_array_equal(two[0]["c_w"], two[1]["c_w"])
