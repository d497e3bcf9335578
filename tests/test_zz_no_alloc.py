"""The no-allocation form of the reference-shaped determinant call.

Callers that may not allocate device memory while they run (a Monte Carlo
driver whose device budget is fixed at start-up, a server admitting work
against an HBM figure, a host whose buffers belong to its own pool) use
lufqhe_lucoregpu_call_noalloc, which keeps its temporaries in a fixed device
array instead of stream-ordered allocations. Its results must equal the
allocating call's: determinants within 1e-12 relative, L\\U factors bit for
bit, on two calls in a row. This file is collected last so a
stop-at-first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def run_pair(cuda, lufqhe_mod, A, n, lda, pair):
    lib = lufqhe_mod.lib()
    stream = cuda.cuda.current_stream().cuda_stream
    batch = A.shape[0]
    ref = A.clone()
    got = A.clone()
    assert lib.lufqhe_lucoregpu_call(ref.data_ptr(), batch, n, lda, int(pair), stream) == 0
    rc = lib.lufqhe_lucoregpu_call_noalloc(got.data_ptr(), batch, n, lda, int(pair), stream)
    assert rc == 0, lib.lufqhe_last_error().decode()
    cuda.cuda.synchronize()
    r = ref.cpu().numpy()
    g = got.cpu().numpy()
    d_ref, d_got = r[:, 0, 0], g[:, 0, 0]
    assert (np.abs(d_got - d_ref) / np.abs(d_ref)).max() < TOL
    # the L\U factors left in the rest of each matrix (and the padding) are the same
    mask = np.ones(r.shape[1:], bool)
    mask[0, 0] = False
    gm = np.ascontiguousarray(g[:, mask])
    rm = np.ascontiguousarray(r[:, mask])
    assert (gm.view(np.uint64) == rm.view(np.uint64)).all()


def test_noalloc_matches_allocating_call_twice(cuda, lufqhe_mod):
    """Two calls in a row (the second sees the first's contents in the shared
    array), then the warp-group path (n = 48) and a padded row stride."""
    for batch, n, pair, seed in [(1000, 16, False, 41), (777, 24, True, 42)]:
        A = lufqhe_mod.gen_gaussian(batch, n, seed=seed)
        run_pair(cuda, lufqhe_mod, A, n, n, pair)
    A = lufqhe_mod.gen_gaussian(300, 48, seed=43)
    run_pair(cuda, lufqhe_mod, A, 48, 48, True)
    A = lufqhe_mod.gen_gaussian(500, 13, seed=44, lda=16)
    run_pair(cuda, lufqhe_mod, A, 13, 16, False)


def test_noalloc_at_capacity_allocates_nothing(cuda, lufqhe_mod):
    """A batch of exactly LUFQHE_NOALLOC_MAX_MATRICES small matrices works, and
    neither it nor a second call changes the device's free memory."""
    from lufqhe import _native
    lib = lufqhe_mod.lib()
    cap = _native.header_constants()["LUFQHE_NOALLOC_MAX_MATRICES"]
    stream = cuda.cuda.current_stream().cuda_stream
    A = lufqhe_mod.gen_gaussian(cap, 4, seed=45)
    want = A.clone()
    assert lib.lufqhe_lucoregpu_call(want.data_ptr(), cap, 4, 4, 0, stream) == 0
    warm = A[:8].clone()
    assert lib.lufqhe_lucoregpu_call_noalloc(warm.data_ptr(), 8, 4, 4, 0, stream) == 0
    cuda.cuda.synchronize()
    free0 = cuda.cuda.mem_get_info()[0]
    got = A.clone()
    cuda.cuda.synchronize()
    free1 = cuda.cuda.mem_get_info()[0]
    for _ in range(2):
        got.copy_(A)
        rc = lib.lufqhe_lucoregpu_call_noalloc(got.data_ptr(), cap, 4, 4, 0, stream)
        assert rc == 0, lib.lufqhe_last_error().decode()
        cuda.cuda.synchronize()
        assert cuda.cuda.mem_get_info()[0] == free1
        assert np.array_equal(got.cpu().numpy().view(np.uint64), want.cpu().numpy().view(np.uint64))
    assert free1 <= free0


def test_noalloc_rejects_batches_beyond_its_scratch(cuda, lufqhe_mod):
    lib = lufqhe_mod.lib()
    from lufqhe import _native
    cap = _native.header_constants()["LUFQHE_NOALLOC_MAX_MATRICES"]
    fake = ctypes.c_void_p(0x1000)   # never dereferenced: the size check comes first
    rc = lib.lufqhe_lucoregpu_call_noalloc(fake, cap + 1, 8, 8, 0, None)
    assert rc == -1
    assert b"capacity" in lib.lufqhe_last_error()
