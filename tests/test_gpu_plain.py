"""GPU parity of the plain FP64 kernels against the CPU oracle, through the C-ABI.

ARITH reference mode must reproduce the FP64 restatement of the reference's
CPU Crout bit for bit (factors, pivots); the fused mode must reproduce the
oracle's fused arithmetic bit for bit. log|det| and phase must agree to
1e-12 (relative to max(1, |log|det||)) and 1e-12 rad, parity exactly.
"""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12
GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_lup.npz"


def rel(a, b):
    return np.abs(a - b) / np.maximum(1.0, np.abs(b))


def dphase(a, b):
    return np.abs(np.angle(np.exp(1j * (a - b))))


def run(lufqhe, torch, A_np, mode, lda=None):
    batch, n, _ = A_np.shape
    lda = n if lda is None else lda
    buf = np.zeros((batch, n, lda), np.complex128)
    buf[:, :, :n] = A_np
    A = torch.from_numpy(buf).cuda()
    out = lufqhe.batch_lup_det(A, mode=mode)
    torch.cuda.synchronize()
    return {k: getattr(out, k).cpu().numpy() for k in ("logabs", "phase", "parity", "status")}


def assert_parity(got, want, tol=TOL):
    ok = want["status"] == 0
    assert (got["status"] == want["status"]).all()
    assert (got["parity"][ok] == want["parity"][ok]).all()
    assert rel(got["logabs"][ok], want["logabs"][ok]).max(initial=0) < tol
    assert dphase(got["phase"][ok], want["phase"][ok]).max(initial=0) < tol


def test_config1_gaussian_n8(cuda, lufqhe_mod, oracle):
    """4096 complex Gaussian matrices, n=8, seed 0 (Re, Im ~ N(0, 1/2))."""
    A = lufqhe_mod.gen_gaussian(4096, 8, seed=0)
    for mode in (lufqhe_mod.MODE_PLAIN_FP64, lufqhe_mod.MODE_PLAIN_FP64_FUSED):
        out = lufqhe_mod.batch_lup_det(A, mode=mode)
        cuda.cuda.synchronize()
        got = {k: getattr(out, k).cpu().numpy() for k in ("logabs", "phase", "parity", "status")}
        want = oracle.lup_det(A.cpu().numpy(), arith=mode)
        assert_parity(got, want)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 13, 16, 24, 31, 32, 33, 48, 64])
@pytest.mark.parametrize("mode", [0, 1])
def test_inplace_factors_bit_exact(cuda, lufqhe_mod, oracle, n, mode):
    rng = np.random.default_rng(100 + n)
    batch = 37
    A_np = (rng.standard_normal((batch, n, n)) + 1j * rng.standard_normal((batch, n, n))) / np.sqrt(2)
    A = cuda.from_numpy(A_np.copy()).cuda()
    out = lufqhe_mod.factor_inplace(A, mode=mode)
    cuda.cuda.synchronize()
    want = oracle.lup_det(A_np, arith=mode, want_factors=True)
    F = A.cpu().numpy()
    assert (F.view(np.uint64) == want["factors"].view(np.uint64)).all(), "factors differ"
    got = {k: getattr(out, k).cpu().numpy() for k in ("logabs", "phase", "parity", "status")}
    assert_parity(got, want)


@pytest.mark.parametrize("mode", [0, 1])
def test_lll_n24_bit_exact(cuda, lufqhe_mod, oracle, mode):
    """Ill-conditioned lowest-Landau-level matrices: identical arithmetic gives
    identical factors, so parity holds to rounding of the final logs."""
    A, _ = lufqhe_mod.gen_lll(1024, 24, seed=2)
    A_np = A.cpu().numpy()
    Ac = A.clone()
    out = lufqhe_mod.factor_inplace(Ac, mode=mode)
    cuda.cuda.synchronize()
    want = oracle.lup_det(A_np, arith=mode, want_factors=True)
    assert (Ac.cpu().numpy().view(np.uint64) == want["factors"].view(np.uint64)).all()
    got = {k: getattr(out, k).cpu().numpy() for k in ("logabs", "phase", "parity", "status")}
    assert_parity(got, want)


def test_reference_mode_within_tolerance_of_reference_on_lll(cuda, lufqhe_mod, oracle):
    A, _ = lufqhe_mod.gen_lll(2048, 24, seed=2)
    got = run(lufqhe_mod, cuda, A.cpu().numpy(), lufqhe_mod.MODE_PLAIN_FP64)
    want = oracle.lup_det(A.cpu().numpy(), arith=0)
    assert_parity(got, want)


def test_padded_lda(cuda, lufqhe_mod, oracle):
    """loadSize = p2Above(n) as with the reference's __PADDED__ build."""
    rng = np.random.default_rng(3)
    A_np = (rng.standard_normal((300, 24, 24)) + 1j * rng.standard_normal((300, 24, 24))) / np.sqrt(2)
    got = run(lufqhe_mod, cuda, A_np, 0, lda=32)
    want = oracle.lup_det(A_np, arith=0)
    assert_parity(got, want)


def test_known_answers_and_status(cuda, lufqhe_mod, oracle):
    mats = []
    mats.append(np.eye(4, dtype=np.complex128))
    P = np.zeros((4, 4), np.complex128)
    P[np.arange(4), (2, 0, 3, 1)] = 1
    mats.append(P)
    S = np.zeros((4, 4), np.complex128)
    S[:2, :2] = [[1, 2], [2, 4]]
    S[2, 2] = S[3, 3] = 1
    mats.append(S)                           # exact zero pivot
    T = np.eye(4, dtype=np.complex128)
    T[1] = 1e-25 + 1j
    mats.append(T)                           # scale below 1e-24
    N = np.eye(4, dtype=np.complex128)
    N[3, 0] = np.inf
    mats.append(N)                           # non-finite
    A_np = np.stack(mats)
    for mode in (0, 1):
        got = run(lufqhe_mod, cuda, A_np, mode)
        want = oracle.lup_det(A_np, arith=mode)
        assert list(got["status"]) == [0, 0, 2, 1, 4]
        assert list(got["status"]) == list(want["status"])
        assert got["logabs"][0] == 0.0 and got["parity"][0] == 0
        assert got["parity"][1] == want["parity"][1]
        assert got["logabs"][2] == -np.inf
        assert np.isnan(got["logabs"][3]) and np.isnan(got["logabs"][4])


@pytest.mark.parametrize("name", ["gauss_n2", "gauss_n3", "gauss_n4", "gauss_n8", "gauss_n16",
                                  "lll_n24", "ref_fixture"])
def test_golden_vectors(cuda, lufqhe_mod, name):
    """Committed golden outputs of the FP64 restatement (made beside the
    reference's own float32 determinant)."""
    g = np.load(GOLDEN)
    got = run(lufqhe_mod, cuda, g[f"{name}/A"], 0)
    want = {"logabs": g[f"{name}/logabs"], "phase": g[f"{name}/phase"],
            "parity": g[f"{name}/parity"], "status": np.zeros(len(g[f"{name}/A"]), np.int32)}
    assert_parity(got, want)


def test_empty_and_ragged_batches(cuda, lufqhe_mod, oracle):
    A = cuda.zeros(0, 8, 8, dtype=cuda.complex128, device="cuda")
    out = lufqhe_mod.batch_lup_det(A)
    assert out.logabs.numel() == 0
    for batch in (1, 3, 33, 257):
        A = lufqhe_mod.gen_gaussian(batch, 11, seed=batch)
        got = run(lufqhe_mod, cuda, A.cpu().numpy(), 0)
        want = oracle.lup_det(A.cpu().numpy(), arith=0)
        assert_parity(got, want)


def test_compat_call_writes_det(cuda, lufqhe_mod, oracle):
    """Reference-shaped LUCoreGPU::CALL with WRITE_DET / PERFORM_PROD."""
    A = lufqhe_mod.gen_gaussian(10, 16, seed=4)
    A_np = A.cpu().numpy()
    want = oracle.lup_det(A_np, arith=0)
    det = np.exp(want["logabs"] + 1j * want["phase"])
    B = A.clone()
    lufqhe_mod.lucoregpu_call(B, pair_product=False)
    cuda.cuda.synchronize()
    d00 = B.cpu().numpy()[:, 0, 0]
    assert (np.abs(d00 - det) / np.abs(det)).max() < 1e-12
    C = A.clone()
    lufqhe_mod.lucoregpu_call(C, pair_product=True)
    cuda.cuda.synchronize()
    d00 = C.cpu().numpy()[:, 0, 0]
    prod = det[0::2] * det[1::2]
    assert (np.abs(d00[0::2] - prod) / np.abs(prod)).max() < 1e-12
    assert (np.abs(d00[1::2] - det[1::2]) / np.abs(det[1::2])).max() < 1e-12


def test_device_generators_match_host(cuda, lufqhe_mod):
    A = lufqhe_mod.gen_gaussian(50, 9, seed=7).cpu().numpy()
    H = lufqhe_mod.gen_gaussian_host(50, 9, seed=7)
    assert np.abs(A - H).max() < 1e-13
    A, z = lufqhe_mod.gen_lll(20, 16, seed=8)
    H, zh = lufqhe_mod.gen_lll_host(20, 16, seed=8)
    assert np.abs(z.cpu().numpy() - zh).max() < 1e-12
    assert (np.abs(A.cpu().numpy() - H) / np.abs(H).max(axis=2, keepdims=True)).max() < 1e-12


def test_concurrent_streams_different_n(cuda, lufqhe_mod, oracle):
    """Geometry travels in kernel arguments: two sizes in flight at once."""
    s1, s2 = cuda.cuda.Stream(), cuda.cuda.Stream()
    A1 = lufqhe_mod.gen_gaussian(2000, 8, seed=11)
    A2 = lufqhe_mod.gen_gaussian(2000, 20, seed=12)
    cuda.cuda.synchronize()
    o1 = lufqhe_mod.batch_lup_det(A1, stream=s1)
    o2 = lufqhe_mod.batch_lup_det(A2, stream=s2)
    cuda.cuda.synchronize()
    for A, o in ((A1, o1), (A2, o2)):
        want = oracle.lup_det(A.cpu().numpy(), arith=0)
        got = {k: getattr(o, k).cpu().numpy() for k in ("logabs", "phase", "parity", "status")}
        assert_parity(got, want)


@pytest.mark.parametrize("batch", [1, 2, 9, 1000, 4097])
def test_pair_sum_matches_oracle(cuda, lufqhe_mod, oracle, batch):
    """Wavefunction pair sum (LUCoreCPU::CALL / globalReduction) on the GPU."""
    A = lufqhe_mod.gen_gaussian(batch, 8, seed=batch)
    out = lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_PLAIN_FP64)
    res = lufqhe_mod.pair_sum(out).cpu().numpy()
    cuda.cuda.synchronize()
    if batch < 2:
        assert res[0] == -np.inf
        return
    la, ar = oracle.pair_sum(A.cpu().numpy())
    assert abs(res[0] - la) < 1e-12 * max(1.0, abs(la))
    assert dphase(res[1], ar) < 1e-11
