"""The oracle's exact transport solver (oracle/emd_oracle.c, successive
shortest paths) against scipy's HiGHS LP solver on the linear program of the
reference's d2_match_by_distmat (src/d2/solver_mosek.cc:61-226): row sums
fixed, column sums fixed except the last.  CPU only."""
import numpy as np
import pytest

scipy_opt = pytest.importorskip("scipy.optimize")


def lp_value(C, wX, wY):
    n, m = C.shape
    A, b = [], []
    for i in range(n):
        r = np.zeros((n, m)); r[i, :] = 1; A.append(r.reshape(-1)); b.append(wX[i])
    for j in range(m - 1):
        r = np.zeros((n, m)); r[:, j] = 1; A.append(r.reshape(-1)); b.append(wY[j])
    res = scipy_opt.linprog(C.reshape(-1), A_eq=np.array(A), b_eq=np.array(b), bounds=(0, None),
                            method="highs")
    assert res.status == 0
    return res.fun


def cases(seed, count):
    rng = np.random.default_rng(seed)
    for t in range(count):
        n = int(rng.integers(1, 40))
        m = int(rng.integers(1, 60))
        d = int(rng.integers(1, 6))
        A = rng.normal(size=(n, d)) * 2
        B = rng.normal(size=(m, d)) * 2
        C = ((A[:, None, :] - B[None, :, :]) ** 2).sum(-1)
        wX = rng.dirichlet(np.full(n, 0.7))
        wY = rng.dirichlet(np.full(m, 0.7))
        if t % 5 == 0:    # uniform weights: many ties, degenerate bases
            wX = np.full(n, 1.0 / n)
            wY = np.full(m, 1.0 / m)
        if t % 7 == 0:    # integer costs: ties between plans
            C = np.round(C)
        yield C, wX, wY


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_emd_matches_highs(oracle_mod, seed):
    for C, wX, wY in cases(seed, 25):
        v, x = oracle_mod.emd(C, wX, wY, want_plan=True)
        ref = lp_value(C, wX, wY)
        assert abs(v - ref) <= 1e-9 * max(1.0, abs(ref)), (C.shape, v, ref)
        # the plan is feasible: nonnegative, rows exact, columns but the last exact
        assert x.min() >= -1e-15
        np.testing.assert_allclose(x.sum(1), wX, atol=1e-12)
        np.testing.assert_allclose(x.sum(0)[:-1], wY[:-1], atol=1e-12)


def test_emd_identical_distributions_cost_zero(oracle_mod):
    rng = np.random.default_rng(5)
    A = rng.normal(size=(12, 3))
    C = ((A[:, None] - A[None]) ** 2).sum(-1)
    w = rng.dirichlet(np.ones(12))
    assert abs(oracle_mod.emd(C, w, w)) < 1e-14


def test_emd_single_support(oracle_mod):
    C = np.array([[1.0, 2.0, 3.0]])
    wY = np.array([0.2, 0.3, 0.5])
    assert abs(oracle_mod.emd(C, [1.0], wY) - (0.2 + 0.6 + 1.5)) < 1e-15
