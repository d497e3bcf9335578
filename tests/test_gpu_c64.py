"""complex64 at the boundary: the reference's own float2 buffers.

LUCoreGPU::CALL takes float2 matrices (LU-fqhe/inc/LUCoreGPU.h:47) and its
Monte Carlo loop copies float32 matrices to the device
(LU-fqhe/src/MonteCarloLoop.cu:316-325); the reference's input files are
float32 (LU-fqhe/src/PermHandler.cpp:91-170). A complex64 batch is widened to
FP64 as it is loaded (exact), so every mode must give the bits of the batch's
complex128 copy, and the plain mode must meet the 1e-12 bar against the FP64
restatement on all 1000 matrices of the reference's fixture file.
"""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_lup.npz"


def host(out):
    return {k: getattr(out, k).cpu().numpy() for k in ("logabs", "phase", "parity", "status")}


def same(a, b):
    assert np.array_equal(a["logabs"], b["logabs"], equal_nan=True)
    assert np.array_equal(a["phase"], b["phase"], equal_nan=True)
    assert (a["parity"] == b["parity"]).all() and (a["status"] == b["status"]).all()


@pytest.mark.parametrize("n", [3, 8, 16, 24, 32, 48])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_c64_equals_c128_copy(cuda, lufqhe_mod, n, mode):
    A, _ = lufqhe_mod.gen_lll(700, n, seed=120 + n)
    A32 = A.to(cuda.complex64)
    want = host(lufqhe_mod.batch_lup_det(A32.to(cuda.complex128), mode=mode))
    same(host(lufqhe_mod.batch_lup_det(A32, mode=mode)), want)


@pytest.mark.parametrize("mode", [0, 2])
def test_c64_host_entry(cuda, lufqhe_mod, mode):
    """Host complex64 batches, page-locked (mixed: read over the host link)
    and pageable (staged), give the device call's bits."""
    A, _ = lufqhe_mod.gen_lll(3000, 24, seed=130)
    A32 = A.to(cuda.complex64)
    want = host(lufqhe_mod.batch_lup_det(A32, mode=mode))
    h = A32.cpu()
    for Ah in (h.pin_memory(), h):
        o = lufqhe_mod.batch_lup_det_host(Ah, mode=mode)
        cuda.cuda.synchronize()
        same({k: getattr(o, k).numpy() for k in ("logabs", "phase", "parity", "status")}, want)


def test_reference_fixture_through_file_reader(cuda, lufqhe_mod, oracle, tmp_path):
    """All 1000 matrices of the reference's fixture, written in its raw float32
    format and read back through lufqhe_read_matrices_f32, against the FP64
    restatement: log|det| and phase within 1e-12, parity identical, in the
    complex128 and the complex64 form of the plain call."""
    g = np.load(GOLDEN)
    A32 = g["ref_fixture_all/A32"]
    path = tmp_path / "1000_16x16.bin"
    A32.tofile(path)
    A = lufqhe_mod.read_matrices_f32(path, 16)
    assert A.shape == (1000, 16, 16) and np.array_equal(A, A32.astype(np.complex128))
    ref = oracle.lup_det(A)
    assert (ref["piv"] == g["ref_fixture_all/piv"]).all()
    for dev in (cuda.from_numpy(A).cuda(), cuda.from_numpy(A32).cuda()):
        out = host(lufqhe_mod.batch_lup_det(dev, mode=lufqhe_mod.MODE_PLAIN_FP64))
        assert (out["status"] == 0).all()
        assert (out["parity"] == ref["parity"]).all()
        err = np.abs(out["logabs"] - ref["logabs"]) / np.maximum(1.0, np.abs(ref["logabs"]))
        assert err.max() < 1e-12
        assert np.abs(np.angle(np.exp(1j * (out["phase"] - ref["phase"])))).max() < 1e-12
    # the in-place factors of the complex64 call are the restatement's rounded to float
    dev = cuda.from_numpy(A32.copy()).cuda()
    lufqhe_mod.lucoregpu_call(dev, pair_product=False)
    got = dev.cpu().numpy()
    fac = oracle.lup_det(A, want_factors=True)["factors"].astype(np.complex64)
    assert np.array_equal(got[:, 1:, :], fac[:, 1:, :])
    assert np.array_equal(got[:, 0, 1:], fac[:, 0, 1:])


@pytest.mark.parametrize("pair", [False, True])
def test_c64_reference_shaped_call(cuda, lufqhe_mod, oracle, pair):
    """lufqhe_lucoregpu_call_c64 writes each complex64 determinant (or pair
    product) into element (0,0), as LUCoreGPU::CALL does with WRITE_DET and
    PERFORM_PROD: the FP64 value rounded to float, and the reference's own
    float32 determinant agrees to float32 accuracy."""
    g = np.load(GOLDEN)
    A32 = g["ref_fixture_all/A32"][:200].copy()
    ref = oracle.lup_det(A32.astype(np.complex128))
    det = np.exp(ref["logabs"] + 1j * ref["phase"])
    if pair:
        want = det.copy()
        want[0::2] = det[0::2] * det[1::2]
    else:
        want = det
    dev = cuda.from_numpy(A32).cuda()
    lufqhe_mod.lucoregpu_call(dev, pair_product=pair)
    got = dev[:, 0, 0].cpu().numpy()
    idx = np.arange(0, 200, 2) if pair else np.arange(200)
    # the FP64 value rounded once to complex64: within 2^-23 of it per component
    w = want[idx]
    assert (np.abs(got[idx] - w) <= 2.0 ** -23 * np.abs(w)).all()
    if not pair:
        d32 = g["ref_fixture_all/ref_det_f32"][:200]
        assert (np.abs(got - d32) / np.abs(d32)).max() < 1e-4
