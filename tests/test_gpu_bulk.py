"""Copy-engine staging of the matrices (LUFQHE_OPT_BULK_LOADS): the plain FP64
warp kernel and the n >= 24 mixed FP32 pass load each complex128 matrix from
device memory by bulk copies (one per row, completing on an mbarrier) and
prefetch the next one into L2. The results must be the bits of the per-lane
loads, including padded row strides, non-finite entries (which the staged path
detects in the exponent pass) and the reference-shaped in-place call."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def host(out):
    return {k: getattr(out, k).cpu().numpy() for k in ("logabs", "phase", "parity", "status")}


def same(a, b):
    assert np.array_equal(a["logabs"], b["logabs"], equal_nan=True)
    assert np.array_equal(a["phase"], b["phase"], equal_nan=True)
    assert (a["parity"] == b["parity"]).all() and (a["status"] == b["status"]).all()


@pytest.fixture
def bulk(lufqhe_mod):
    lib = lufqhe_mod.lib()
    old = lib.lufqhe_get_option(7)
    yield lambda v: lib.lufqhe_set_option(7, v)
    lib.lufqhe_set_option(7, old)


@pytest.mark.parametrize("n,lda", [(5, 5), (8, 8), (16, 16), (24, 24), (24, 32), (32, 32),
                                   (32, 33)])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_bulk_equals_lane_loads(cuda, lufqhe_mod, bulk, n, lda, mode):
    A, _ = lufqhe_mod.gen_lll(3000, n, seed=400 + n)
    buf = cuda.zeros((3000, n, lda), dtype=cuda.complex128, device="cuda")
    buf[:, :, :n] = A
    buf[7, 2, 3] = float("nan")       # non-finite entries, in the staged path too
    buf[2999, n - 1, n - 1] = float("inf")
    bulk(0.0)
    want = host(lufqhe_mod.batch_lup_det(buf, mode=mode))
    bulk(1.0)
    got = host(lufqhe_mod.batch_lup_det(buf, mode=mode))
    same(got, want)
    assert got["status"][7] & lufqhe_mod.ST_NONFINITE and got["status"][2999] & lufqhe_mod.ST_NONFINITE
    assert ((got["status"] & 32) == 0).all()   # no bounded wait ran out


def test_bulk_reference_shaped_call(cuda, lufqhe_mod, bulk):
    """The in-place call (factors written back over the matrices) with staged
    loads leaves the same bits in every matrix."""
    A = lufqhe_mod.gen_gaussian(2000, 16, seed=410)
    a, b = A.clone(), A.clone()
    bulk(0.0)
    lufqhe_mod.lucoregpu_call(a, pair_product=True)
    bulk(1.0)
    lufqhe_mod.lucoregpu_call(b, pair_product=True)
    assert np.array_equal(a.cpu().numpy().view(np.uint64), b.cpu().numpy().view(np.uint64))
