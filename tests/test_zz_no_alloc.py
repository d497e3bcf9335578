"""The no-allocation form of the reference-shaped determinant call.

Callers that may not allocate device memory while they run (a fixed budget set
at start-up, an HBM admission figure, a pool the caller owns) use
lufqhe_lucoregpu_call_noalloc, which keeps its temporaries in a fixed device
array instead of stream-ordered allocations. This file is collected last so a
stop-at-first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def test_noalloc_matches_allocating_call_twice(cuda, lufqhe_mod):
    lib = lufqhe_mod.lib()
    stream = cuda.cuda.current_stream().cuda_stream
    cases = [(1000, 16, False, 41), (777, 24, True, 42)]   # two calls in a row
    for batch, n, pair, seed in cases:
        A = lufqhe_mod.gen_gaussian(batch, n, seed=seed)
        ref = A.clone()
        got = A.clone()
        assert lib.lufqhe_lucoregpu_call(ref.data_ptr(), batch, n, n, int(pair), stream) == 0
        rc = lib.lufqhe_lucoregpu_call_noalloc(got.data_ptr(), batch, n, n, int(pair), stream)
        assert rc == 0, lib.lufqhe_last_error().decode()
        cuda.cuda.synchronize()
        r = ref.cpu().numpy()
        g = got.cpu().numpy()
        d_ref, d_got = r[:, 0, 0], g[:, 0, 0]
        assert (np.abs(d_got - d_ref) / np.abs(d_ref)).max() < TOL
        # the L\U factors left in the rest of each matrix are the same
        mask = np.ones((n, n), bool)
        mask[0, 0] = False
        gm = np.ascontiguousarray(g[:, mask])
        rm = np.ascontiguousarray(r[:, mask])
        assert (gm.view(np.uint64) == rm.view(np.uint64)).all()


def test_noalloc_rejects_batches_beyond_its_scratch(cuda, lufqhe_mod):
    lib = lufqhe_mod.lib()
    from lufqhe import _native
    cap = _native.header_constants()["LUFQHE_NOALLOC_MAX_MATRICES"]
    fake = ctypes.c_void_p(0x1000)   # never dereferenced: the size check comes first
    rc = lib.lufqhe_lucoregpu_call_noalloc(fake, cap + 1, 8, 8, 0, None)
    assert rc == -1
    assert b"capacity" in lib.lufqhe_last_error()
