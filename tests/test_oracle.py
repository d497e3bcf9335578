"""CPU tests of the oracle: known answers, numpy, the double-double truth, and
the golden vectors made with the reference's own float32 determinant."""
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_lup.npz"


def rel(a, b):
    return np.abs(a - b) / np.maximum(1.0, np.abs(b))


def dphase(a, b):
    return np.abs(np.angle(np.exp(1j * (a - b))))


def cgauss(rng, b, n):
    return (rng.standard_normal((b, n, n)) + 1j * rng.standard_normal((b, n, n))) / np.sqrt(2)


# ---------------------------------------------------------------- known answers
def test_identity(oracle):
    for n in (1, 2, 7, 64):
        r = oracle.lup_det(np.eye(n, dtype=np.complex128)[None])
        assert r["logabs"][0] == 0.0 and r["phase"][0] == 0.0
        assert r["parity"][0] == 0 and r["status"][0] == 0


def test_diagonal_and_triangular(oracle):
    rng = np.random.default_rng(5)
    d = rng.uniform(0.5, 2, 6) * np.exp(1j * rng.uniform(-3, 3, 6))
    D = np.diag(d)
    T = np.triu(cgauss(rng, 1, 6)[0], 1) + D
    for M in (D, T):
        r = oracle.lup_det(M[None])
        assert rel(r["logabs"][0], np.sum(np.log(np.abs(d)))) < 1e-14
        assert dphase(r["phase"][0], np.sum(np.angle(d))) < 1e-14
        assert r["parity"][0] == 0


@pytest.mark.parametrize("perm", [(1, 0), (2, 0, 1), (3, 1, 0, 2), (0, 2, 1, 3, 4)])
def test_permutation_parity(oracle, perm):
    n = len(perm)
    P = np.zeros((n, n), np.complex128)
    P[np.arange(n), perm] = 1
    sign = round(np.linalg.det(P.real))
    r = oracle.lup_det(P[None])
    assert r["status"][0] == 0
    assert r["parity"][0] == (sign < 0)
    assert r["logabs"][0] == 0.0
    assert dphase(r["phase"][0], 0.0 if sign > 0 else np.pi) < 1e-15


def test_2x2_closed_form(oracle):
    rng = np.random.default_rng(6)
    A = cgauss(rng, 50, 2)
    det = A[:, 0, 0] * A[:, 1, 1] - A[:, 0, 1] * A[:, 1, 0]
    r = oracle.lup_det(A)
    assert rel(r["logabs"], np.log(np.abs(det))).max() < 1e-13
    assert dphase(r["phase"], np.angle(det)).max() < 1e-13


def test_pivot_rule_ties_to_last_row(oracle):
    # column 0 quotients |Re|/scale are all 1: the reference keeps the last row
    A = np.array([[1, 0.5, 0.25], [2, 1, 0.5j], [-4, 1, 1]], np.complex128)
    r = oracle.lup_det(A[None])
    assert r["piv"][0, 0] == 2


def test_pivot_rule_uses_real_part_only(oracle):
    # row 0 has the larger modulus in column 0 but the smaller |Re|/scale
    A = np.array([[0.1 + 5j, 1.0], [0.5, 1.0]], np.complex128)
    r = oracle.lup_det(A[None])
    assert r["piv"][0, 0] == 1 and r["parity"][0] == 1


def test_singular_zero_pivot(oracle):
    A = np.array([[1, 2], [2, 4]], np.complex128)
    r = oracle.lup_det(A[None])
    assert r["status"][0] == 2 and r["logabs"][0] == -np.inf


def test_scale_tiny_row(oracle):
    A = np.eye(3, dtype=np.complex128)
    A[1] = 1e-25 + 1j  # |Re| below 1e-24 everywhere in row 1: the reference exits
    r = oracle.lup_det(A[None])
    assert r["status"][0] == 1 and np.isnan(r["logabs"][0])


def test_nonfinite(oracle):
    A = np.eye(3, dtype=np.complex128)
    A[2, 1] = np.nan
    r = oracle.lup_det(A[None])
    assert r["status"][0] == 4


def test_empty_batch(oracle):
    r = oracle.lup_det(np.zeros((0, 4, 4), np.complex128))
    assert r["logabs"].shape == (0,)


def test_lda_padding(oracle):
    rng = np.random.default_rng(7)
    A = cgauss(rng, 20, 24)
    P = np.zeros((20, 24, 32), np.complex128)
    P[:, :, :24] = A
    P[:, :, 24:] = 1e30  # padding must be ignored
    a = oracle.lup_det(A)
    b = oracle.lup_det(P)
    assert (a["logabs"] == b["logabs"]).all() and (a["piv"] == b["piv"]).all()


# ---------------------------------------------------------------- numpy / dd
@pytest.mark.parametrize("n", [1, 3, 8, 16, 24, 33, 64])
def test_vs_numpy_and_dd(oracle, n):
    rng = np.random.default_rng(n)
    A = cgauss(rng, 200, n)
    s, ld = np.linalg.slogdet(A)
    r = oracle.lup_det(A)
    la_dd, ph_dd, st = oracle.logdet_dd(A)
    assert (st == 0).all()
    assert rel(la_dd, ld).max() < 1e-11
    assert dphase(ph_dd, np.angle(s)).max() < 1e-11
    assert rel(r["logabs"], la_dd).max() < 1e-11
    assert dphase(r["phase"], ph_dd).max() < 1e-11


def test_literal_vs_kernel_arith_same_pivots(oracle):
    rng = np.random.default_rng(11)
    A = cgauss(rng, 500, 16)
    a = oracle.lup_det(A, arith=oracle.ARITH_LITERAL)
    b = oracle.lup_det(A, arith=oracle.ARITH_KERNEL)
    assert (a["piv"] == b["piv"]).all()
    assert rel(a["logabs"], b["logabs"]).max() < 1e-12
    assert dphase(a["phase"], b["phase"]).max() < 1e-12


def test_factors_reconstruct(oracle):
    rng = np.random.default_rng(12)
    n = 12
    A = cgauss(rng, 10, n)
    r = oracle.lup_det(A, want_factors=True)
    for b in range(10):
        F = r["factors"][b]
        L = np.tril(F, -1) + np.eye(n)
        U = np.triu(F)
        PA = A[b].copy()
        for j, p in enumerate(r["piv"][b]):
            PA[[j, p]] = PA[[p, j]]
        assert np.abs(L @ U - PA).max() < 1e-12


def test_pair_sum(oracle):
    rng = np.random.default_rng(13)
    A = cgauss(rng, 9, 5)  # odd count: the last matrix is dropped (LUCoreCPU.cu:83)
    d = np.linalg.det(A)
    want = np.sum(d[0:8:2] * d[1:8:2])
    la, ar = oracle.pair_sum(A)
    assert abs(la - np.log(abs(want))) < 1e-12
    assert dphase(ar, np.angle(want)) < 1e-12


# ---------------------------------------------------------------- golden vectors
def golden_sets():
    """The sets stored as complex128 inputs (the full fixture is complex64 only)."""
    g = np.load(GOLDEN)
    return sorted({k.split("/")[0] for k in g.files if k.endswith("/A")})


def golden_input32(g, name):
    return g[f"{name}/A32"] if f"{name}/A32" in g.files else g[f"{name}/A"].astype(np.complex64)


@pytest.mark.parametrize("name", golden_sets())
def test_golden_fp64_restatement(oracle, name):
    g = np.load(GOLDEN)
    A = g[f"{name}/A"]
    r = oracle.lup_det(A)
    assert (r["piv"] == g[f"{name}/piv"]).all()
    assert (r["parity"] == g[f"{name}/parity"]).all()
    assert rel(r["logabs"], g[f"{name}/logabs"]).max() < 1e-14
    assert dphase(r["phase"], g[f"{name}/phase"]).max() < 1e-14


@pytest.mark.parametrize("name", golden_sets())
def test_golden_vs_reference_float32(oracle, name):
    """The FP64 restatement agrees with the reference's own float32 Crout to
    float32 accuracy (the reference has no FP64 build)."""
    g = np.load(GOLDEN)
    d32 = g[f"{name}/ref_det_f32"].astype(np.complex128)
    la = g[f"{name}/logabs"]
    ph = g[f"{name}/phase"]
    if np.abs(la).min() > 88.0:
        # |det| beyond float32 range: the reference's direct product of the
        # diagonal (LUCoreCPU.cu:256-265) cannot represent it
        assert not np.isfinite(d32).any()
        return
    assert np.isfinite(d32).all()
    tol = 2e-5
    assert np.abs(np.log(np.abs(d32)) - la).max() < tol * max(1.0, np.abs(la).max())
    assert dphase(np.angle(d32), ph).max() < tol * 10


@pytest.mark.parametrize("name", golden_sets() + ["ref_fixture_all"])
def test_float32_restatement_bit_exact(oracle, name):
    """The restatement instantiated in float32 reproduces the reference's own
    compiled LUCoreCPU::determinant bit for bit: the complex64 determinant and
    the factors it leaves in place (so every pivot and every row swap), on all
    1000 matrices of the reference's fixture file and on the seeded sets."""
    g = np.load(GOLDEN)
    r = oracle.lup_det_f32(golden_input32(g, name))
    want = g[f"{name}/ref_det_f32"]
    assert np.array_equal(r["det"].view(np.uint32), want.view(np.uint32))
    assert np.array_equal(oracle.factor_digests(r["factors"]), g[f"{name}/ref_factor_digest"])


def test_fixture_fp64_restatement_pivots(oracle):
    """On the reference's fixture the FP64 restatement takes the float32
    restatement's (hence the reference's) pivots, and its log-determinants are
    the committed ones bit for bit."""
    g = np.load(GOLDEN)
    A32 = g["ref_fixture_all/A32"]
    r32 = oracle.lup_det_f32(A32)
    r64 = oracle.lup_det(A32.astype(np.complex128))
    assert (r64["piv"] == r32["piv"]).all()
    assert (r64["piv"] == g["ref_fixture_all/piv"]).all()
    assert np.array_equal(r64["logabs"], g["ref_fixture_all/logabs"])
    assert np.array_equal(r64["phase"], g["ref_fixture_all/phase"])
    la, ph, _ = oracle.logdet_dd(A32.astype(np.complex128))
    assert rel(r64["logabs"], la).max() < 1e-12
    assert dphase(r64["phase"], ph).max() < 1e-12


def test_float32_restatement_live(oracle):
    """Where the reference was compiled here: bit-identical on fresh seeded
    Gaussian and lowest-Landau-level inputs of several sizes."""
    if not oracle.ref_available():
        pytest.skip("reference CPU determinant not built on this machine")
    rng = np.random.default_rng(15)
    sets = [cgauss(rng, 500, n) for n in (1, 3, 8, 17)]
    sets += [oracle.gen_lll(500, n, seed=40 + n)[0] for n in (6, 12, 24)]
    for A in sets:
        A32 = A.astype(np.complex64)
        r = oracle.lup_det_f32(A32)
        det, fac = oracle.ref_factor_f32(A32)
        assert np.array_equal(r["det"].view(np.uint32), det.view(np.uint32))
        assert np.array_equal(r["factors"].view(np.uint32), fac.view(np.uint32))


@pytest.mark.parametrize("name", golden_sets())
def test_golden_dd(oracle, name):
    g = np.load(GOLDEN)
    la, ph, _ = oracle.logdet_dd(g[f"{name}/A"])
    assert rel(la, g[f"{name}/logabs_dd"]).max() < 1e-14
    assert dphase(ph, g[f"{name}/phase_dd"]).max() < 1e-13
    assert rel(g[f"{name}/logabs"], la).max() < 1e-9


def test_reference_float32_live(oracle):
    """When the reference was compiled here, it agrees with the restatement."""
    if not oracle.ref_available():
        pytest.skip("reference CPU determinant not built on this machine")
    rng = np.random.default_rng(14)
    A = cgauss(rng, 64, 16).astype(np.complex64)
    d32 = oracle.ref_det_f32(A).astype(np.complex128)
    r = oracle.lup_det(A.astype(np.complex128))
    assert np.abs(np.log(np.abs(d32)) - r["logabs"]).max() < 1e-4
