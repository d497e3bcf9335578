"""The host-buffer entry point: chunked copy / factorise / copy pipeline gives
the device entry point's results bit for bit, pinned or pageable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def host_dict(out):
    return {k: getattr(out, k).numpy().copy() for k in ("logabs", "phase", "parity", "status")}


def dev_dict(out):
    return {k: getattr(out, k).cpu().numpy() for k in ("logabs", "phase", "parity", "status")}


@pytest.mark.parametrize("n,batch", [(8, 3000), (24, 10000), (17, 4001)])
@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("pinned", [True, False])
def test_host_entry_matches_device_entry(cuda, lufqhe_mod, n, batch, mode, pinned):
    A, _ = lufqhe_mod.gen_lll(batch, n, seed=300 + n)
    want = dev_dict(lufqhe_mod.batch_lup_det(A, mode=mode))
    A_host = A.cpu()
    if pinned:
        A_host = A_host.pin_memory()
    s = cuda.cuda.Stream()
    out = lufqhe_mod.batch_lup_det_host(A_host, mode=mode, stream=s)
    s.synchronize()
    got = host_dict(out)
    for k in ("logabs", "phase"):
        assert np.array_equal(got[k], want[k], equal_nan=True), k
    assert (got["parity"] == want["parity"]).all() and (got["status"] == want["status"]).all()


def test_host_entry_repeated_calls_share_nothing(cuda, lufqhe_mod):
    """Back-to-back calls on one stream, outputs read only at the end."""
    A, _ = lufqhe_mod.gen_lll(9000, 24, seed=5)
    A_host = A.cpu().pin_memory()
    want = dev_dict(lufqhe_mod.batch_lup_det(A, mode=2))
    s = cuda.cuda.Stream()
    outs = [lufqhe_mod.batch_lup_det_host(A_host, mode=2, stream=s) for _ in range(3)]
    s.synchronize()
    for o in outs:
        assert np.array_equal(host_dict(o)["logabs"], want["logabs"], equal_nan=True)


@pytest.mark.parametrize("n,batch", [(24, 6000), (16, 5000), (32, 3000), (8, 4000), (48, 700)])
@pytest.mark.parametrize("out_pinned", [True, False])
def test_mixed_over_host_link(cuda, lufqhe_mod, n, batch, out_pinned):
    """Mixed mode on a pinned batch: the kernels read the matrices over the
    host link and refactorise rejected ones in place; results equal the device
    entry point's (FP32 pass + separate FP64 pass) bit for bit, with pinned or
    pageable result arrays."""
    import torch
    A, _ = lufqhe_mod.gen_lll(batch, n, seed=400 + n)
    want = dev_dict(lufqhe_mod.batch_lup_det(A, mode=2))
    A_host = A.cpu().pin_memory()
    out = lufqhe_mod.DetResult(*(torch.empty(batch, dtype=d, pin_memory=out_pinned)
                                 for d in (torch.float64, torch.float64, torch.int8, torch.int32)))
    s = cuda.cuda.Stream()
    lufqhe_mod.batch_lup_det_host(A_host, mode=2, stream=s, out=out)
    s.synchronize()
    got = host_dict(out)
    for k in ("logabs", "phase"):
        assert np.array_equal(got[k], want[k], equal_nan=True), k
    assert (got["parity"] == want["parity"]).all() and (got["status"] == want["status"]).all()
    assert ((got["status"] & lufqhe_mod.ST_FALLBACK) != 0).any() or n < 24 or n > 32


def test_mixed_over_host_link_special_matrices(cuda, lufqhe_mod):
    """Zero, singular, non-finite and tiny-scaled matrices in a pinned batch
    read over the host link: the same results and status flags as the device
    entry point."""
    import torch
    A, _ = lufqhe_mod.gen_lll(2000, 24, seed=31)
    A[3] = 0                                  # zero matrix
    A[10, 5] = A[10, 7]                       # two equal rows: singular
    A[20, 2, 2] = float("nan")                # non-finite
    A[30] *= 1e-30                            # rows below the reference's 1e-24 scale test
    A[40, :, 4] = 0                           # a zero column
    want = dev_dict(lufqhe_mod.batch_lup_det(A, mode=2))
    out = lufqhe_mod.batch_lup_det_host(A.cpu().pin_memory(), mode=2)
    cuda.cuda.synchronize()
    got = host_dict(out)
    for k in ("logabs", "phase"):
        assert np.array_equal(got[k], want[k], equal_nan=True), k
    assert (got["parity"] == want["parity"]).all() and (got["status"] == want["status"]).all()
    assert got["status"][20] == lufqhe_mod.ST_NONFINITE


@pytest.mark.parametrize("n", [24, 32])
def test_mixed_over_host_link_every_matrix_refactorised(cuda, lufqhe_mod, oracle, n):
    """Every matrix rejected (threshold 0): the factor lists of both paths
    (room for a quarter of the batch) overflow, and the rest are corrected in
    place by the warp that refactorised them; host-link results equal the
    device entry point's bit for bit, and every one is within 1e-10 of the
    double-double oracle."""
    lib = lufqhe_mod.lib()
    old = lib.lufqhe_get_option(1)
    lib.lufqhe_set_option(1, 0.0)
    try:
        A, _ = lufqhe_mod.gen_lll(3000, n, seed=500 + n)
        want = dev_dict(lufqhe_mod.batch_lup_det(A, mode=2))
        out = lufqhe_mod.batch_lup_det_host(A.cpu().pin_memory(), mode=2)
        cuda.cuda.synchronize()
    finally:
        lib.lufqhe_set_option(1, old)
    got = host_dict(out)
    for k in ("logabs", "phase"):
        assert np.array_equal(got[k], want[k], equal_nan=True), k
    assert (got["status"] == want["status"]).all()
    assert ((got["status"] & lufqhe_mod.ST_FALLBACK) != 0).all()
    la, ph, _ = oracle.logdet_dd(A.cpu().numpy())
    scale = np.maximum(1.0, np.abs(la))
    assert (np.abs(got["logabs"] - la) / scale).max() < 1e-10
    assert (np.abs(np.angle(np.exp(1j * (got["phase"] - ph)))) / scale).max() < 1e-10
