"""The shard files of a sharded run: d2g_write_split (host code in libd2g.so)
against the reference's own d2_write_split (src/d2/clustering_io.c:329-480,
compiled from the reference tree into oracle/_ref), byte for byte on every
file it writes (<name>.ind and <name>.0 ... <name>.<splits-1>), as written
and pre-processed, on multi-phase Euclidean data, word embeddings, dense
and sparse histograms.  The files read back through d2g_read hold the
shuffled instances.  CPU only: no device work."""
import ctypes as C

import numpy as np
import pytest

from d2_kmeans_gb300 import _lib as L
from d2_kmeans_gb300 import d2io, synth
from d2_kmeans_gb300.assign import Mph


@pytest.fixture(scope="module")
def libs(oracle_mod):
    if not oracle_mod.available("ref"):
        pytest.skip("the reference tree is not present (its d2_write_split is built from it)")
    from d2_kmeans_gb300.build import build
    build()
    ref = oracle_mod._lib("ref").d2_write_split
    ref.restype = C.c_int
    ref.argtypes = [C.c_char_p, C.c_void_p, C.c_int, C.c_char]
    return L.load(), ref


def _data(kind):
    if kind == "euclid2":  # two Euclidean phases, supports larger than str to merge
        a, _ = synth.euclidean_phase(37, 3, 6, 3, (2, 14), False, 4, 1.0, seed=81)
        b, _ = synth.euclidean_phase(37, 3, 5, 2, (1, 9), False, 4, 1.0, seed=82)
        return [dict(a, str=6), dict(b, str=5)], 37
    if kind == "embed":
        e, _ = synth.embed_phase(25, 2, 6, V=40, dim=5, sizes=(3, 12), seed=83)
        return [dict(e, str=6)], 25
    if kind == "hist":
        h, _ = synth.histogram_phase(30, 2, side=3, alpha=0.3, seed=84)
        return [dict(h, str=9)], 30
    rng = np.random.default_rng(85)  # sparse histograms over 12 bins
    p_str = rng.integers(1, 8, size=20).astype(np.int32)
    sym = np.concatenate([np.sort(rng.choice(12, size=k, replace=False)) for k in p_str]).astype(np.int32)
    w = np.concatenate([rng.dirichlet(np.ones(k)) for k in p_str])
    return [dict(metric=12, dim=0, str=12, p_str=p_str, p_w=w, p_supp_sym=sym, vocab_size=12,
                 dist_mat=synth.grid_cost(4)[:12, :12].reshape(-1))], 20


@pytest.mark.parametrize("kind", ["euclid2", "embed", "hist", "sparse"])
@pytest.mark.parametrize("pre", [0, 1])
@pytest.mark.parametrize("splits", [1, 3])
def test_files_equal_the_reference(libs, tmp_path, kind, pre, splits):
    ours, ref = libs
    phases, n = _data(kind)
    if pre and kind == "sparse":
        pytest.skip("the reference reads through a null pointer here")
    data = Mph(phases, n, label=np.zeros(n, np.int32), num_of_labels=1)
    a, b = str(tmp_path / "ref"), str(tmp_path / "ours")
    assert ref(a.encode(), C.addressof(data.mph), splits, bytes([pre])) == 0
    assert ours.d2g_write_split(b.encode(), C.byref(data.mph), splits, bytes([pre])) == 0
    for suffix in [".ind"] + [f".{k}" for k in range(splits)]:
        assert open(a + suffix, "rb").read() == open(b + suffix, "rb").read(), suffix


def test_shards_read_back(libs, tmp_path):
    """The shards read back with d2g_read hold the instances in the order of
    the .ind file (weights to the files' 6 decimals, renormalised on reading)."""
    ours, _ = libs
    phases, n = _data("euclid2")
    data = Mph(phases, n, label=np.zeros(n, np.int32), num_of_labels=1)
    base = str(tmp_path / "d")
    assert ours.d2g_write_split(base.encode(), C.byref(data.mph), 3, b"\x00") == 0
    order = np.loadtxt(base + ".ind", dtype=np.int64)
    assert sorted(order.tolist()) == list(range(n))
    batch = 1 + (n - 1) // 3
    got = []
    for k in range(3):
        cnt = len(order[k * batch:(k + 1) * batch])
        got.append(d2io.read(f"{base}.{k}", cnt, [3, 2], [0, 0], avg_strides=[6, 5]))
    p_str = np.concatenate([g["phases"][0]["p_str"] for g in got])
    np.testing.assert_array_equal(p_str, np.asarray(phases[0]["p_str"])[order])
    w = np.concatenate([g["phases"][0]["p_w"] for g in got])
    cum = np.concatenate([[0], np.cumsum(phases[0]["p_str"])])
    w_ref = np.concatenate([phases[0]["p_w"][cum[i]:cum[i + 1]] for i in order])
    np.testing.assert_allclose(w, w_ref, atol=2e-6)


def test_refusals(libs, tmp_path):
    ours, _ = libs
    phases, n = _data("sparse")
    data = Mph(phases, n, label=np.zeros(n, np.int32), num_of_labels=1)
    rc = ours.d2g_write_split(str(tmp_path / "s").encode(), C.byref(data.mph), 2, b"\x01")
    assert rc == L.D2G_E_UNSUPPORTED
    assert ours.d2g_write_split(str(tmp_path / "s").encode(), C.byref(data.mph), 0, b"\x00") == L.D2G_E_INVAL
