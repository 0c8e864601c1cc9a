"""Exact transport on the GPU (d2g_emd_pairs, emd_kernel.cu) against the
oracle's successive-shortest-path solver (oracle/emd_oracle.c, itself checked
against scipy's HiGHS LP solver): the linear program of the reference's
d2_match_by_distmat (src/d2/solver_mosek.cc:61-226) on Euclidean supports,
dense and sparse histograms, with the degenerate cases a transportation
simplex meets (uniform weights, integer costs, repeated supports, empty bins,
one-support objects, identical distributions)."""
import numpy as np
import pytest

from d2_kmeans_gb300 import assign

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from d2_kmeans_gb300.build import build
    build()
    return assign


def euclid_set(rng, count, lo, hi, d, uniform=False, integer=False, fixed=None):
    p_str = np.full(count, fixed, np.int32) if fixed else rng.integers(lo, hi + 1, size=count).astype(np.int32)
    col = int(p_str.sum())
    supp = rng.normal(size=(col, d)) * 2.0
    if integer:
        supp = np.round(supp)
    w = []
    for s in p_str:
        w.append(np.full(s, 1.0 / s) if uniform else rng.dirichlet(np.full(s, 0.7)))
    return {"p_str": p_str, "p_w": np.concatenate(w), "p_supp": supp.reshape(-1)}


def oracle_costs(oracle_mod, rows, cols, pr, pc, d=None, dist_mat=None, rsym=None, csym=None):
    rc = np.concatenate([[0], np.cumsum(rows["p_str"])])
    cc = np.concatenate([[0], np.cumsum(cols["p_str"])])
    out = []
    for a, b in zip(pr, pc):
        ra, rb = rc[a], rc[a + 1]
        ca, cb = cc[b], cc[b + 1]
        if dist_mat is None:
            A = rows["p_supp"].reshape(-1, d)[ra:rb]
            B = cols["p_supp"].reshape(-1, d)[ca:cb]
            C = ((A[:, None, :] - B[None, :, :]) ** 2).sum(-1)
        else:
            ki = rsym[ra:rb] if rsym is not None else np.arange(rb - ra)
            kj = csym[ca:cb] if csym is not None else np.arange(cb - ca)
            C = dist_mat[np.ix_(ki, kj)]
        out.append(oracle_mod.emd(C, rows["p_w"][ra:rb], cols["p_w"][ca:cb]))
    return np.array(out)


def all_pairs(nr, nc):
    pr, pc = np.meshgrid(np.arange(nr), np.arange(nc), indexing="ij")
    return pr.reshape(-1), pc.reshape(-1)


@pytest.mark.parametrize("d,lo,hi,seed", [(3, 1, 40, 0), (1, 1, 12, 1), (2, 5, 70, 2), (5, 2, 30, 3),
                                          (7, 1, 9, 4), (3, 100, 300, 5)])
def test_euclidean_pairs_match_oracle(lib, oracle_mod, d, lo, hi, seed):
    rng = np.random.default_rng(seed)
    rows = euclid_set(rng, 6, lo, hi, d)
    cols = euclid_set(rng, 9, lo, hi, d)
    pr, pc = all_pairs(6, 9)
    got, piv = lib.emd_pairs(assign.EUCLIDEAN, rows, cols, pr, pc, dim=d, with_pivots=True)
    ref = oracle_costs(oracle_mod, rows, cols, pr, pc, d=d)
    np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-12)
    assert piv.min() >= 0


def test_centroid_rows_fixed_size(lib, oracle_mod):
    """Rows as the reference passes centroids: every object m = 32 supports."""
    rng = np.random.default_rng(7)
    rows = euclid_set(rng, 5, 0, 0, 3, fixed=32)
    rows_fixed = {"str": 32, "p_w": rows["p_w"], "p_supp": rows["p_supp"]}
    cols = euclid_set(rng, 40, 8, 128, 3)
    pr, pc = all_pairs(5, 40)
    got = lib.emd_pairs(assign.EUCLIDEAN, rows_fixed, cols, pr, pc, dim=3)
    ref = oracle_costs(oracle_mod, rows, cols, pr, pc, d=3)
    np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("case", ["uniform", "integer", "uniform_integer"])
def test_degenerate_pairs(lib, oracle_mod, case):
    rng = np.random.default_rng(11)
    uni, integer = "uniform" in case, "integer" in case
    rows = euclid_set(rng, 5, 1, 30, 2, uniform=uni, integer=integer)
    cols = euclid_set(rng, 8, 1, 30, 2, uniform=uni, integer=integer)
    pr, pc = all_pairs(5, 8)
    got = lib.emd_pairs(assign.EUCLIDEAN, rows, cols, pr, pc, dim=2)
    ref = oracle_costs(oracle_mod, rows, cols, pr, pc, d=2)
    np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-12)


def test_identical_and_single_support(lib):
    rng = np.random.default_rng(12)
    a = euclid_set(rng, 3, 1, 20, 3)
    got = lib.emd_pairs(assign.EUCLIDEAN, a, a, [0, 1, 2], [0, 1, 2], dim=3)
    assert np.all(np.abs(got) < 1e-10)
    one = {"p_str": np.array([1], np.int32), "p_w": np.array([1.0]), "p_supp": np.array([0.5, -1.0, 2.0])}
    got = lib.emd_pairs(assign.EUCLIDEAN, one, a, [0, 0, 0], [0, 1, 2], dim=3)
    cum = np.concatenate([[0], np.cumsum(a["p_str"])])
    S = a["p_supp"].reshape(-1, 3)
    for k in range(3):
        d2 = ((S[cum[k]:cum[k + 1]] - one["p_supp"]) ** 2).sum(1)
        assert abs(got[k] - (a["p_w"][cum[k]:cum[k + 1]] * d2).sum()) < 1e-12


def grid_costs(side):
    g = np.stack(np.meshgrid(np.arange(side), np.arange(side), indexing="ij"), -1).reshape(-1, 2)
    return ((g[:, None, :] - g[None, :, :]) ** 2).sum(-1).astype(float)


def test_dense_histograms(lib, oracle_mod):
    rng = np.random.default_rng(13)
    V = 64
    dm = grid_costs(8)
    def hists(k):
        w = rng.dirichlet(np.full(V, 0.2), size=k)
        w[w < 1e-3] = 0.0            # empty bins
        w /= w.sum(1, keepdims=True)
        return {"p_str": np.full(k, V, np.int32), "p_w": w.reshape(-1)}
    rows, cols = hists(4), hists(6)
    pr, pc = all_pairs(4, 6)
    got = lib.emd_pairs(assign.HISTOGRAM, rows, cols, pr, pc, dist_mat=dm)
    ref = oracle_costs(oracle_mod, rows, cols, pr, pc, dist_mat=dm)
    np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-12)


def test_sparse_histograms(lib, oracle_mod):
    rng = np.random.default_rng(14)
    V = 100
    dm = rng.random((V, V)) * 5
    dm = (dm + dm.T) / 2
    np.fill_diagonal(dm, 0)
    def sparse(k, lo, hi):
        p_str = rng.integers(lo, hi + 1, size=k).astype(np.int32)
        sym = np.concatenate([rng.choice(V, s, replace=False) for s in p_str]).astype(np.int32)
        w = np.concatenate([rng.dirichlet(np.ones(s)) for s in p_str])
        return {"p_str": p_str, "p_w": w, "p_supp_sym": sym}
    rows, cols = sparse(4, 3, 40), sparse(7, 1, 60)
    pr, pc = all_pairs(4, 7)
    got = lib.emd_pairs(assign.SPARSE_HISTOGRAM, rows, cols, pr, pc, dist_mat=dm)
    ref = oracle_costs(oracle_mod, rows, cols, pr, pc, dist_mat=dm, rsym=rows["p_supp_sym"],
                       csym=cols["p_supp_sym"])
    np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-12)


def test_many_pairs_spot_checked(lib, oracle_mod):
    """The assignment shape of the batched workload (m = 32 centroid supports,
    m_i 8-128, d = 3): 64 x 300 pairs, every 37th checked."""
    rng = np.random.default_rng(15)
    rows = euclid_set(rng, 64, 0, 0, 3, fixed=32)
    cols = euclid_set(rng, 300, 8, 128, 3)
    pr, pc = all_pairs(64, 300)
    got, piv = lib.emd_pairs(assign.EUCLIDEAN, rows, cols, pr, pc, dim=3, with_pivots=True)
    sel = np.arange(0, pr.size, 37)
    ref = oracle_costs(oracle_mod, rows, cols, pr[sel], pc[sel], d=3)
    np.testing.assert_allclose(got[sel], ref, rtol=1e-10, atol=1e-12)
    assert piv.min() >= 0


def test_bad_arguments_are_refused(lib):
    from d2_kmeans_gb300._lib import D2GError
    rng = np.random.default_rng(16)
    a = euclid_set(rng, 2, 1, 5, 3)
    with pytest.raises(D2GError):
        lib.emd_pairs(assign.EUCLIDEAN, a, a, [0, 2], [0, 0], dim=3)   # row index out of range
    with pytest.raises(D2GError):
        lib.emd_pairs(assign.EUCLIDEAN, a, a, [0], [0], dim=9)         # dimension beyond 7
