"""The wavefunction sum S = sum_i det(A_2i) det(A_2i+1) straight from the
matrices (lufqhe_batch_pair_sum): in the plain modes one kernel that fuses the
pair product and the sum into the factorisation, against the oracle's
restatement of LUCoreCPU::CALL (LU-fqhe/src/LUCoreCPU.cu:82-98) and against the
two-step path (per-matrix determinants, then lufqhe_pair_sum)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dphase(a, b):
    return abs(np.angle(np.exp(1j * (a - b))))


@pytest.mark.parametrize("n,batch,kind", [(8, 4096, "gauss"), (16, 2001, "gauss"),
                                          (24, 6000, "lll"), (32, 1000, "lll"),
                                          (48, 400, "lll")])
@pytest.mark.parametrize("mode", [0, 1])
def test_fused_pair_sum_plain(cuda, lufqhe_mod, oracle, n, batch, kind, mode):
    if kind == "lll":
        A, _ = lufqhe_mod.gen_lll(batch, n, seed=200 + n)
    else:
        A = lufqhe_mod.gen_gaussian(batch, n, seed=200 + n)
    got = lufqhe_mod.batch_pair_sum(A, mode=mode).cpu().numpy()
    la, ar = oracle.pair_sum(A.cpu().numpy())
    # the terms have random phases: the sum's relative error is the terms'
    # (1e-12 relative log-determinants in the reference's arithmetic) times
    # sum|terms| / |S| (about sqrt(pairs)); fused arithmetic differs from the
    # reference's by FP64's own error on these matrices (up to ~1e-9 relative)
    tol = (1e-12 * np.sqrt(batch) if mode == 0 else 1e-9) * max(1.0, abs(la))
    assert abs(got[0] - la) < tol and dphase(got[1], ar) < tol
    # the two-step path on the same determinants
    out = lufqhe_mod.batch_lup_det(A, mode=mode)
    two = lufqhe_mod.pair_sum(out).cpu().numpy()
    assert abs(got[0] - two[0]) < tol and dphase(got[1], two[1]) < tol
    # reproducible bit for bit
    again = lufqhe_mod.batch_pair_sum(A, mode=mode).cpu().numpy()
    assert np.array_equal(got, again)


def test_pair_sum_mixed_and_c64(cuda, lufqhe_mod):
    """Mixed mode (determinants, then the log-sum-exp pass) equals the two-step
    call on the mixed results; a complex64 batch equals its complex128 copy."""
    A, _ = lufqhe_mod.gen_lll(4097, 24, seed=230)    # odd: the last matrix is dropped
    got = lufqhe_mod.batch_pair_sum(A, mode=2).cpu().numpy()
    two = lufqhe_mod.pair_sum(lufqhe_mod.batch_lup_det(A, mode=2)).cpu().numpy()
    assert np.array_equal(got, two)
    A32 = A.to(cuda.complex64)
    for mode in (0, 1, 2):
        a = lufqhe_mod.batch_pair_sum(A32, mode=mode).cpu().numpy()
        b = lufqhe_mod.batch_pair_sum(A32.to(cuda.complex128), mode=mode).cpu().numpy()
        assert np.array_equal(a, b)


def test_pair_sum_edge_cases(cuda, lufqhe_mod):
    """Fewer than two matrices: the empty sum (-inf, 0). A singular pair (a
    zero column: an exact zero pivot) adds nothing; a non-finite matrix makes
    the sum NaN."""
    A = lufqhe_mod.gen_gaussian(1, 8, seed=1)
    assert lufqhe_mod.batch_pair_sum(A, mode=1).cpu().numpy().tolist() == [-np.inf, 0.0]
    A = lufqhe_mod.gen_gaussian(6, 8, seed=2)
    ref = lufqhe_mod.batch_pair_sum(A[2:].contiguous(), mode=1).cpu().numpy()
    A[0, :, 0] = 0
    got = lufqhe_mod.batch_pair_sum(A, mode=1).cpu().numpy()
    assert abs(got[0] - ref[0]) < 1e-12 and dphase(got[1], ref[1]) < 1e-12
    A[3, 1, 1] = float("nan")
    assert np.isnan(lufqhe_mod.batch_pair_sum(A, mode=1).cpu().numpy()[0])
