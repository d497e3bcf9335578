"""LLL orbital matrices built inside the factorising kernels from particle
coordinates give bit for bit what the generated matrices give through the
batched entry point, in every mode."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev_dict(out):
    return {k: getattr(out, k).cpu().numpy() for k in ("logabs", "phase", "parity", "status")}


@pytest.mark.parametrize("n,batch", [(6, 500), (8, 3000), (12, 700), (16, 2000), (17, 300),
                                     (24, 5000), (32, 800), (48, 200), (64, 100)])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_lll_det_matches_generated_matrices(cuda, lufqhe_mod, n, batch, mode):
    A, z = lufqhe_mod.gen_lll(batch, n, seed=400 + n)
    want = dev_dict(lufqhe_mod.batch_lup_det(A, mode=mode))
    got = dev_dict(lufqhe_mod.lll_det(z.contiguous(), mode=mode))
    for k in ("logabs", "phase"):
        assert np.array_equal(got[k], want[k], equal_nan=True), k
    assert (got["parity"] == want["parity"]).all() and (got["status"] == want["status"]).all()


def test_lll_det_fp64_share_and_nonfinite(cuda, lufqhe_mod):
    """The routed share hashes the built (0,0) entry exactly as the dense path
    does, and a non-finite coordinate gives the dense path's non-finite result."""
    lib = lufqhe_mod.lib()
    old = lib.lufqhe_get_option(3)
    lib.lufqhe_set_option(3, 0.5)
    try:
        A, z = lufqhe_mod.gen_lll(3000, 24, seed=77)
        z = z.contiguous()
        z[5, 3] = complex(float("nan"), 0.0)
        A[5, 3] = complex(float("nan"), float("nan"))
        want = dev_dict(lufqhe_mod.batch_lup_det(A, mode=2))
        got = dev_dict(lufqhe_mod.lll_det(z, mode=2))
    finally:
        lib.lufqhe_set_option(3, old)
    # row 3 of matrix 5 is all NaN in both forms; the route depends on entry (0,0)
    assert np.isnan(got["logabs"][5]) and got["status"][5] != 0
    assert (got["status"] == want["status"]).all()
    assert np.array_equal(got["logabs"], want["logabs"], equal_nan=True)
    assert ((got["status"] & lufqhe_mod.ST_FP64) != 0).mean() > 0.3


@pytest.mark.parametrize("mode", [1, 2])
def test_lll_det_on_host_buffers(cuda, lufqhe_mod, mode):
    """Page-locked host coordinates and results (read and written over the
    host link) give the device call's results bit for bit."""
    A, z = lufqhe_mod.gen_lll(5000, 24, seed=77)
    z = z.contiguous()
    want = lufqhe_mod.lll_det(z, mode=mode)
    zh = z.cpu().pin_memory()
    got = lufqhe_mod.lll_det(zh, mode=mode)
    cuda.cuda.synchronize()
    for k in ("logabs", "phase", "parity", "status"):
        a, b = getattr(got, k).numpy(), getattr(want, k).cpu().numpy()
        assert (((a == b) | (np.isnan(a) & np.isnan(b))) if a.dtype.kind == "f" else a == b).all(), k
