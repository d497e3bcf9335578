"""Composite-fermion matrices on the CPU: the library's host tables against
the oracle's, the oracle's vectorised builder against its entry-by-entry
restatement of the reference's calculateElement, and the C-ABI's argument
checks (which return before any device work)."""
import ctypes

import numpy as np
import pytest

import cf_oracle as co

K = (1.0, 0.5, 0.5, 1.0)   # k1, k2, r1, r2 (the reference's test values k1 = 1, k2 = 0.5)


@pytest.mark.parametrize("n", [3, 11, 25, 33, 63])
def test_tables_match_oracle(lufqhe_mod, n):
    phi, theta = co.random_config(2 * n, seed=n)
    uv, tab = lufqhe_mod.cf_tables(lufqhe_mod.CfConfig(phi, theta, *K, 0, 1), n)
    uvo, tabo = co.tables(phi, theta, n)
    assert np.array_equal(uv, uvo)
    # the recurrences multiply up to Q + 1 rounded factors
    assert np.all(np.abs(tab - tabo) <= 1e-13 * np.abs(tabo))


@pytest.mark.parametrize("n,mu,nu", [(11, 0, 1), (11, -2, 3), (25, 1, -1)])
def test_builder_matches_reference_order(lufqhe_mod, n, mu, nu):
    phi, theta = co.random_config(2 * n, seed=7)
    uv, tab = lufqhe_mod.cf_tables(lufqhe_mod.CfConfig(phi, theta, *K, mu, nu), n)
    perm = co.random_perms(4, n, 2 * n, seed=3)
    A = co.matrices(uv, tab, perm, n, *K, mu, nu)
    for b in range(perm.shape[0]):
        for r in range(n):
            for c in (0, n // 2, n - 3, n - 2, n - 1):
                e = co.entry_loop(uv, tab, perm[b], n, r, c, *K, mu, nu)
                assert abs(A[b, r, c] - e) <= 1e-13 * abs(e), (b, r, c)


def test_cf_det_argument_checks(lufqhe_mod):
    lib = lufqhe_mod.lib()
    phi = np.zeros(130)
    theta = np.full(130, 0.5)
    perm = np.ones((1, 11), dtype=np.int16)
    out = np.zeros(4)
    p = ctypes.c_void_p

    def call(n=11, np_=22, mu=0, nu=1, stride=11, mode=0):
        return lib.lufqhe_cf_det(phi.ctypes.data, theta.ctypes.data, np_, n, *K, mu, nu,
                                 perm.ctypes.data, stride, 1, mode, out.ctypes.data,
                                 out.ctypes.data, out.ctypes.data, out.ctypes.data, p(0))

    INVALID, UNSUPPORTED_N, UNSUPPORTED_MODE = -1, -2, -4
    assert call(n=10) == INVALID            # n even
    assert call(n=1) == INVALID
    assert call(np_=10) == INVALID          # fewer particles than rows
    assert call(stride=10) == INVALID
    assert call(mu=6) == INVALID            # Q + 1 + mu = 11 is outside the table
    assert call(nu=-6) == INVALID
    assert call(n=65, np_=22) == INVALID    # np < n
    assert call(n=65, np_=130, stride=65) == UNSUPPORTED_N
    assert call(mode=9) == UNSUPPORTED_MODE
    assert lib.lufqhe_cf_tables(phi.ctypes.data, theta.ctypes.data, 22, 10, out.ctypes.data,
                                out.ctypes.data) == INVALID
