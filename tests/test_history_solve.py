"""The host half of the history-projection guess (warm_start = 2): the m x m
Galerkin solve of history.cu (pdgb::hist_solve), called through the built
library without a GPU.  Given S = H^T H, G = H^T A H and c = H^T r1 it must
return y with H^T (r1 - A H y) = 0 over span H, drop columns that are
(numerically) in the span of the others, and give up cleanly on empty or
degenerate input."""
import ctypes as C

import numpy as np
import pytest

KMAX = 8
SYMBOL = "_ZN4pdgb10hist_solveEiPKdS1_S1_dPd"   # int hist_solve(int, const double*, const double*, const double*, double, double*)


@pytest.fixture(scope="module")
def hist_solve(pdgb):
    lib = pdgb.library()
    try:
        f = getattr(lib, SYMBOL)
    except AttributeError:
        pytest.fail("hist_solve not found in the library")
    dp = C.POINTER(C.c_double)
    f.argtypes = [C.c_int, dp, dp, dp, C.c_double, dp]
    f.restype = C.c_int

    def call(m, S, G, c, rel):
        su = np.zeros(KMAX * (KMAX + 1) // 2)
        gu = np.zeros_like(su)
        e = 0
        for a in range(KMAX):
            for b in range(a, KMAX):
                if a < m and b < m:
                    su[e], gu[e] = S[a, b], G[a, b]
                e += 1
        cc = np.zeros(KMAX)
        cc[:m] = c
        y = np.full(KMAX, np.nan)
        p = lambda x: x.ctypes.data_as(dp)
        used = f(m, p(su), p(gu), p(cc), rel, p(y))
        return used, y[:m]
    return call


def system(rng, n=300, m=6, dependent=False):
    B = rng.standard_normal((n, n)) / np.sqrt(n)
    A = B @ B.T + 2.0 * np.eye(n)                  # SPD
    base = rng.standard_normal(n)
    H = np.stack([base + 1e-3 * (j + 1) * rng.standard_normal(n) for j in range(m)], 1)
    if dependent:
        H[:, 3] = H[:, 1] - 0.5 * H[:, 2]
    r1 = rng.standard_normal(n)
    return A, H, r1


@pytest.mark.parametrize("dependent", [False, True])
def test_galerkin_condition(hist_solve, dependent):
    rng = np.random.default_rng(7 if dependent else 3)
    A, H, r1 = system(rng, dependent=dependent)
    m = H.shape[1]
    used, y = hist_solve(m, H.T @ H, H.T @ A @ H, H.T @ r1, 1e-24)
    assert used == (m - 1 if dependent else m)
    assert np.all(np.isfinite(y))
    if dependent:
        assert np.count_nonzero(y) == m - 1     # the dependent column is not used
    r0 = r1 - A @ (H @ y)
    # orthogonal to every history column, to the rounding of the Gram data
    assert np.abs(H.T @ r0).max() <= 1e-8 * np.abs(H.T @ r1).max()
    assert np.linalg.norm(r0) < np.linalg.norm(r1)


def test_dependent_column_after_the_first_pivot(hist_solve):
    """The largest column is chosen first (index 0) and a later column is a
    combination of it and another one: every row after the pivot must be
    downdated, so exactly one column is dropped."""
    rng = np.random.default_rng(5)
    n = 200
    B = rng.standard_normal((n, n)) / np.sqrt(n)
    A = B @ B.T + 2.0 * np.eye(n)
    h0 = 10.0 * rng.standard_normal(n)
    h1 = rng.standard_normal(n)
    h2 = rng.standard_normal(n)
    H = np.stack([h0, h1, h2, h0 + h1], 1)
    r1 = rng.standard_normal(n)
    used, y = hist_solve(4, H.T @ H, H.T @ A @ H, H.T @ r1, 1e-12)
    assert used == 3
    assert np.count_nonzero(y) == 3
    r0 = r1 - A @ (H @ y)
    assert np.abs(H.T @ r0).max() <= 1e-8 * np.abs(H.T @ r1).max()


def test_threshold_drops_noise_columns(hist_solve):
    """A column whose part outside the others' span is below sqrt(rel) of the
    largest norm is dropped."""
    rng = np.random.default_rng(11)
    A, H, r1 = system(rng, m=4)
    H[:, 2] = H[:, 0] + 1e-9 * rng.standard_normal(H.shape[0])   # 1e-9 relative remainder
    used, y = hist_solve(4, H.T @ H, H.T @ A @ H, H.T @ r1, 1e-12)   # keeps parts above 1e-6
    assert used == 3 and y[2] == 0.0 or used == 3 and y[0] == 0.0


def test_empty_and_degenerate(hist_solve):
    used, y = hist_solve(0, np.zeros((0, 0)), np.zeros((0, 0)), np.zeros(0), 1e-12)
    assert used == 0
    used, y = hist_solve(3, np.zeros((3, 3)), np.zeros((3, 3)), np.ones(3), 1e-12)
    assert used == 0 and np.all(y == 0.0)
