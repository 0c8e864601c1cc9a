"""d2 input files: d2g_read (parallel parser in libd2g.so, host code) against
the reference's own d2_allocate + d2_read (src/d2/clustering_io.c:14-201,
compiled from the reference tree into oracle/_ref) and the oracle's fscanf
restatement, bit for bit on every array they fill.  CPU only.

Files are written by d2_kmeans_gb300.d2io.write (17 significant digits) from
seeded data in every format: multi-phase Euclidean (.d2), dense histograms
with a .hist0 cost file, symbolic supports with a .vocab0 embedding file
(including the id-0 boundary case), sparse histograms; plus early end of
file, capacity growth, empty objects, number spellings fscanf accepts
('+1.5', '1E+2', subnormals), and malformed input, which d2g_read refuses
with D2G_E_INVAL where the reference asserts."""
import os

import numpy as np
import pytest

from d2_kmeans_gb300 import d2io
from d2_kmeans_gb300._lib import D2G_E_INVAL, D2GError

import oracle  # noqa: E402

REF_DATA = os.path.join(oracle.REF_TREE, "data", "mountaindat.d2")


@pytest.fixture(scope="module")
def readers(oracle_mod):
    if not oracle_mod.available("ref"):
        pytest.skip("the reference tree is not present (its d2_read is built from it)")
    from d2_kmeans_gb300.build import build
    build()
    return oracle_mod


def assert_same(a, b):
    assert a["size"] == b["size"] and a["global_size"] == b["global_size"]
    assert len(a["phases"]) == len(b["phases"])
    for pa, pb in zip(a["phases"], b["phases"]):
        for k in ("metric", "dim", "str", "max_str", "col"):
            assert pa[k] == pb[k], (k, pa[k], pb[k])
        if pa["metric"] != d2io.EUCLIDEAN:  # (d2_allocate leaves it unset for Euclidean phases)
            assert pa["vocab_size"] == pb["vocab_size"]
        assert set(pa) == set(pb)
        for k in pa:
            if isinstance(pa[k], np.ndarray):
                assert pa[k].dtype == pb[k].dtype and np.array_equal(pa[k], pb[k]), k


def three_way(readers, path, size, dims, types, avg=None, meta=None):
    ours = d2io.read(path, size, dims, types, avg_strides=avg, meta_filename=meta)
    rc, ref = readers.read("ref", path, size, dims, types, avg_strides=avg, meta_filename=meta)
    assert rc == 0
    rc, port = readers.read("port", path, size, dims, types, avg_strides=avg, meta_filename=meta)
    assert rc == 0
    assert_same(ours, ref)
    assert_same(port, ref)
    return ours


def euclid_phase(rng, n, dim, lo, hi):
    p_str = rng.integers(lo, hi + 1, size=n).astype(np.int32)
    col = int(p_str.sum())
    w = rng.gamma(1.0, 1.0, size=col) + 1e-3   # not normalised: the reader renormalises
    return dict(metric=d2io.EUCLIDEAN, dim=dim, p_str=p_str, p_w=w,
                p_supp=rng.normal(size=col * dim) * 10.0)


def test_two_phase_euclidean(readers, tmp_path):
    rng = np.random.default_rng(1)
    phases = [euclid_phase(rng, 300, 3, 1, 20), euclid_phase(rng, 300, 2, 1, 9)]
    f = str(tmp_path / "two.d2")
    d2io.write(f, phases)
    out = three_way(readers, f, 300, [3, 2], [0, 0], avg=[6, 4])
    assert out["phases"][0]["col"] == int(phases[0]["p_str"].sum())
    w = out["phases"][0]["p_w"]
    cum = out["phases"][0]["p_str_cum"]
    np.testing.assert_allclose(w[cum[5]:cum[6]].sum(), 1.0, rtol=1e-15)


def test_capacity_growth_and_early_end(readers, tmp_path):
    rng = np.random.default_rng(2)
    phases = [euclid_phase(rng, 200, 3, 10, 40)]
    f = str(tmp_path / "grow.d2")
    d2io.write(f, phases)
    # avg_strides 1: the preallocated arrays are too small and grow; size 230 > 200 objects
    out = three_way(readers, f, 230, [3], [0], avg=[1])
    assert out["size"] == 200


def test_dense_histograms(readers, tmp_path):
    rng = np.random.default_rng(3)
    k, n = 16, 120
    p_str = np.full(n, k, np.int32)
    w = rng.dirichlet(np.full(k, 0.3), size=n).reshape(-1)
    w[rng.random(w.size) < 0.2] = 0.0   # dense histograms may hold empty bins
    w[::k] += 1e-3
    dm = np.abs(np.subtract.outer(np.arange(k), np.arange(k))).astype(float) ** 2
    f = str(tmp_path / "h.d2")
    d2io.write(f, [dict(metric=d2io.HISTOGRAM, dim=0, p_str=p_str, p_w=w)], dist_mats={0: dm})
    out = three_way(readers, f, n, [0], [d2io.HISTOGRAM], avg=[k])
    np.testing.assert_array_equal(out["phases"][0]["dist_mat"], dm.reshape(-1))
    # the cost file named explicitly (one phase)
    os.rename(f + ".hist0", str(tmp_path / "costs.txt"))
    three_way(readers, f, n, [0], [d2io.HISTOGRAM], avg=[k], meta=str(tmp_path / "costs.txt"))


def test_word_embedding_and_sparse_histograms(readers, tmp_path):
    rng = np.random.default_rng(4)
    V, dim, n = 50, 4, 150
    p_str = rng.integers(1, 12, size=n).astype(np.int32)
    col = int(p_str.sum())
    ids = rng.integers(0, V, size=col)
    ids[::17] = -1            # written as id 0: the reader maps it to the last vocabulary row
    w = rng.gamma(1.0, 1.0, size=col) + 1e-3
    vocab = rng.normal(size=(V, dim))
    f = str(tmp_path / "e.d2s")
    d2io.write(f, [dict(metric=d2io.WORD_EMBED, dim=dim, p_str=p_str, p_w=w, p_supp_sym=ids)],
               vocab={0: vocab})
    out = three_way(readers, f, n, [dim], [d2io.WORD_EMBED], avg=[5])
    sym = out["phases"][0]["p_supp_sym"]
    assert sym[0] == V - 1 and sym.max() == V - 1 and sym.min() >= 0
    # sparse histograms: the same ids over bins with a cost file; str becomes the bin count
    dm = rng.random((V, V))
    g = str(tmp_path / "s.d2")
    d2io.write(g, [dict(metric=d2io.SPARSE_HISTOGRAM, dim=0, p_str=p_str, p_w=w, p_supp_sym=ids)],
               dist_mats={0: dm})
    out = three_way(readers, g, n, [0], [d2io.SPARSE_HISTOGRAM], avg=[5])
    assert out["phases"][0]["str"] == V


def test_number_spellings_and_empty_objects(readers, tmp_path):
    f = tmp_path / "spell.d2"
    f.write_text("3 2\n+0.5 1E+2\n1 2 3\n-4.9e-324 +5 6e-1\n"
                 "3 0\n"                         # an empty object: skipped by every reader
                 "3 1 7\n0.1 0.2 0.3\n")
    out = three_way(readers, str(f), 3, [3], [0], avg=[2])
    ph = out["phases"][0]
    assert ph["col"] == 3 and list(ph["p_str"][:2]) == [2, 1]
    assert ph["p_supp"][3] == -5e-324


def test_malformed_input_is_refused(tmp_path):
    from d2_kmeans_gb300.build import build
    build()
    f = tmp_path / "bad.d2"
    for text in ("3 2 0.5 0.5 1 2 3 4 5 abc\n",      # not a number
                 "3 2 0.5 0.0 1 2 3 4 5 6\n",        # weight not above 1e-9 (reference: assert)
                 "2 1 1.0 1 2\n",                    # dimension differs from the phase's
                 "3 2 0.5 0.5 1 2 3\n"):             # cut off inside an object
        f.write_text(text)
        with pytest.raises(D2GError) as e:
            d2io.read(str(f), 1, [3], [0])
        assert e.value.code == D2G_E_INVAL


@pytest.mark.skipif(not os.path.exists(REF_DATA), reason="the reference's data files are not present")
def test_reference_data_file(readers):
    """The reference's own mountaindat.d2 (2 phases, d = 3 and 3), as its
    README reads it (-p 2 -n 1000 -d 3,3 -s 6,11)."""
    out = three_way(readers, REF_DATA, 1000, [3, 3], [0, 0], avg=[6, 11])
    assert out["size"] == 1000 and out["phases"][0]["col"] > 0
