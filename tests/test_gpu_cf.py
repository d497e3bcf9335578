"""Composite-fermion matrices built on the device: the builder's matrices equal
the oracle's restatement (from the same host tables) bit for bit; the
determinants taken with the matrices built inside the factorising kernels equal
the batched entry point's on the written-out matrices bit for bit in every
mode; mixed mode stays within 1e-10 of the double-double oracle; bad
permutations give NONFINITE for their matrix only."""
import numpy as np
import pytest

import cf_oracle as co

pytestmark = pytest.mark.gpu

K = (1.0, 0.5, 0.5, 1.0)


def setup(lufqhe_mod, cuda, n, batch, seed, mu=0, nu=1, stride=None, np_=None):
    np_ = 2 * n if np_ is None else np_
    phi, theta = co.random_config(np_, seed)
    cfg = lufqhe_mod.CfConfig(phi, theta, *K, mu, nu)
    perm = co.random_perms(batch, n, np_, seed + 1, stride)
    return cfg, perm, cuda.from_numpy(perm).cuda()


def results(out):
    return {k: getattr(out, k).cpu().numpy() for k in ("logabs", "phase", "parity", "status")}


def same(a, b):
    for k in ("logabs", "phase"):
        assert np.array_equal(a[k], b[k], equal_nan=True), k
    assert (a["parity"] == b["parity"]).all() and (a["status"] == b["status"]).all()


@pytest.mark.parametrize("n,mu,nu", [(3, 0, 1), (11, 0, 1), (11, -2, 3), (25, 1, -1), (33, 0, 1),
                                     (63, 0, 1)])
def test_builder_bits_equal_oracle(cuda, lufqhe_mod, n, mu, nu):
    cfg, perm, dperm = setup(lufqhe_mod, cuda, n, 64, seed=10 + n, mu=mu, nu=nu, stride=n + 3)
    uv, tab = lufqhe_mod.cf_tables(cfg, n)
    want = co.matrices(uv, tab, perm, n, *K, mu, nu)
    got = lufqhe_mod.gen_cf(cfg, dperm, n, lda=n + 1).cpu().numpy()[:, :, :n]
    assert np.array_equal(got.view(np.float64), want.view(np.float64))
    got32 = lufqhe_mod.gen_cf(cfg, dperm, n, dtype=cuda.complex64).cpu().numpy()
    assert np.array_equal(got32, want.astype(np.complex64))


@pytest.mark.parametrize("n,batch", [(3, 200), (11, 5000), (17, 700), (25, 2000), (31, 500),
                                     (33, 300), (45, 100), (63, 64)])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_cf_det_matches_written_matrices(cuda, lufqhe_mod, n, batch, mode):
    cfg, perm, dperm = setup(lufqhe_mod, cuda, n, batch, seed=100 + n, stride=n + 1)
    A = lufqhe_mod.gen_cf(cfg, dperm, n)
    want = results(lufqhe_mod.batch_lup_det(A, mode=mode))
    got = results(lufqhe_mod.cf_det(cfg, dperm, n, mode=mode))
    same(got, want)
    assert (got["status"] & ~(lufqhe_mod.ST_FALLBACK | lufqhe_mod.ST_FP64) == 0).all()


@pytest.mark.parametrize("n", [11, 17, 25, 31])
def test_cf_det_mixed_against_double_double(cuda, lufqhe_mod, oracle, n):
    """Every result within 1e-10 of the double-double determinant (log|det|
    relative to max(1, |log|det||), the phase likewise)."""
    cfg, perm, dperm = setup(lufqhe_mod, cuda, n, 1000, seed=300 + n)
    uv, tab = lufqhe_mod.cf_tables(cfg, n)
    A = co.matrices(uv, tab, perm, n, *K, 0, 1)
    la_dd, ph_dd = oracle.logdet_dd(A)[:2]
    got = results(lufqhe_mod.cf_det(cfg, dperm, n, mode=2))
    scale = np.maximum(1.0, np.abs(la_dd))
    err = np.abs(got["logabs"] - la_dd) / scale
    dph = np.abs(np.angle(np.exp(1j * (got["phase"] - ph_dd)))) / scale
    assert err.max() <= 1e-10 and dph.max() <= 1e-10, (err.max(), dph.max())


def test_bad_permutations_flag_their_matrix_only(cuda, lufqhe_mod):
    n = 11
    cfg, perm, _ = setup(lufqhe_mod, cuda, n, 64, seed=5)
    want = results(lufqhe_mod.cf_det(cfg, cuda.from_numpy(perm).cuda(), n, mode=1))
    perm[3, 4] = 0                       # outside 1..np
    perm[7, 0] = 2 * n + 1               # outside 1..np
    perm[9, 2] = -5
    perm[12, 5] = perm[12, 6]            # a repeated particle: 0/0 in its sums
    bad = [3, 7, 9, 12]
    for mode in (0, 1, 2):
        got = results(lufqhe_mod.cf_det(cfg, cuda.from_numpy(perm).cuda(), n, mode=mode))
        assert (got["status"][bad] & lufqhe_mod.ST_NONFINITE != 0).all()
        assert np.isnan(got["logabs"][bad]).all()
        ok = np.setdiff1d(np.arange(64), bad)
        if mode == 1:
            for k in ("logabs", "phase", "parity", "status"):
                assert np.array_equal(got[k][ok], want[k][ok]), k


@pytest.mark.parametrize("mode", [1, 2])
def test_cf_det_on_host_buffers(cuda, lufqhe_mod, mode):
    """Page-locked permutations and results, read and written over the host link."""
    n = 25
    cfg, perm, dperm = setup(lufqhe_mod, cuda, n, 3000, seed=9)
    want = results(lufqhe_mod.cf_det(cfg, dperm, n, mode=mode))
    hperm = cuda.from_numpy(perm).pin_memory()
    got = lufqhe_mod.cf_det(cfg, hperm, n, mode=mode)
    cuda.cuda.synchronize()
    same(results(got), want)


def test_cf_det_empty_batch(cuda, lufqhe_mod):
    cfg, _, dperm = setup(lufqhe_mod, cuda, 11, 1, seed=1)
    out = lufqhe_mod.cf_det(cfg, dperm[:0], 11, mode=2)
    assert out.logabs.numel() == 0
