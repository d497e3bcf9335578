"""GPU accuracy of the mixed-precision mode (FP32 LUP + FP64-accurate
correction + FP64 fallback) against the double-double truth oracle.

Tolerance: the error of the complex log-determinant log|det| + i*phase,
relative to max(1, |log|det||), is <= 1e-10 in both parts for every matrix the
mixed path accepts and, for 17 <= n <= 32, for every matrix of the FP64 route
too (the FP64 factorisation plus its extended-precision correction). Outside
that range the FP64 route carries the fused FP64 kernel's result bit for bit.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-10
CORRECT_MIN_N, CORRECT_MAX_N = 17, 40   # sizes whose FP64 route is corrected


def rel(a, b):
    return np.abs(a - b) / np.maximum(1.0, np.abs(b))


def dphase(a, b):
    return np.abs(np.angle(np.exp(1j * (a - b))))


def host(out):
    return {k: getattr(out, k).cpu().numpy() for k in ("logabs", "phase", "parity", "status")}


@pytest.fixture
def fp64_share(lufqhe_mod):
    """Set the FP64-pipe routing share for one test (negative: per-size default)."""
    lib = lufqhe_mod.lib()
    old = lib.lufqhe_get_option(3)
    yield lambda v: lib.lufqhe_set_option(3, v)
    lib.lufqhe_set_option(3, old)


@pytest.fixture
def threshold(lufqhe_mod):
    lib = lufqhe_mod.lib()
    old = lib.lufqhe_get_option(1)
    yield lambda v: lib.lufqhe_set_option(1, v)
    lib.lufqhe_set_option(1, old)


def check_mixed(lufqhe_mod, oracle, A, max_fallback_frac):
    out = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED))
    A_np = A.cpu().numpy()
    la, ph, st = oracle.logdet_dd(A_np)
    ok = out["status"] == 0
    fb = (out["status"] & lufqhe_mod.ST_FALLBACK) != 0
    routed = (out["status"] & lufqhe_mod.ST_FP64) != 0   # FP64 pipe share, by design
    assert (ok | fb | routed).all(), f"unexpected status {np.unique(out['status'])}"
    mixed_path = ~routed
    n_mixed = int(mixed_path.sum())
    assert fb[mixed_path].sum() <= max_fallback_frac * max(1, n_mixed), \
        f"fallback fraction {fb[mixed_path].sum()} / {n_mixed}"
    assert rel(out["logabs"][ok], la[ok]).max(initial=0) < TOL_MIXED
    assert (dphase(out["phase"][ok], ph[ok]) / np.maximum(1.0, np.abs(la[ok]))).max(
        initial=0) < TOL_MIXED
    fp = fb | routed
    if fp.any():
        # the FP64 route carries the fused FP64 kernel's status bits (including
        # its scale-below-1e-24 rule, whose result is NaN) and its result:
        # bit for bit outside the corrected sizes, within the bound inside them
        fused = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_PLAIN_FP64_FUSED))
        flags = lufqhe_mod.ST_FALLBACK | lufqhe_mod.ST_FP64
        assert ((out["status"][fp] & ~flags) == fused["status"][fp]).all()
        n = A.shape[1]
        if CORRECT_MIN_N <= n <= CORRECT_MAX_N:
            good = fp & (out["status"] & ~flags == 0)
            assert rel(out["logabs"][good], la[good]).max(initial=0) < TOL_MIXED
            assert (dphase(out["phase"][good], ph[good]) /
                    np.maximum(1.0, np.abs(la[good]))).max(initial=0) < TOL_MIXED
            # the correction is of rounding size next to the fused result
            assert rel(out["logabs"][good], fused["logabs"][good]).max(initial=0) < 1e-6
            bad = fp & ~good
            assert np.array_equal(out["logabs"][bad], fused["logabs"][bad], equal_nan=True)
        else:
            assert np.array_equal(out["logabs"][fp], fused["logabs"][fp], equal_nan=True)
            assert np.array_equal(out["phase"][fp], fused["phase"][fp], equal_nan=True)
    return out


def test_config2_gaussian_n16(cuda, lufqhe_mod, oracle):
    """Complex Gaussian n=16, seed 1 (a 8192-matrix slice of the 65536 batch)."""
    A = lufqhe_mod.gen_gaussian(8192, 16, seed=1)
    out = check_mixed(lufqhe_mod, oracle, A, max_fallback_frac=0.001)
    assert ((out["status"] & ~lufqhe_mod.ST_FP64) == 0).mean() > 0.999


def test_config3_lll_n24(cuda, lufqhe_mod, oracle):
    """Lowest-Landau-level orbital matrices n=24, z ~ CN(0, 24)."""
    A, _ = lufqhe_mod.gen_lll(4096, 24, seed=2)
    check_mixed(lufqhe_mod, oracle, A, max_fallback_frac=0.15)


@pytest.mark.parametrize("n", [1, 2, 3, 6, 8, 12, 17, 31, 32, 33, 48, 64])
def test_sizes_gaussian(cuda, lufqhe_mod, oracle, fp64_share, n):
    fp64_share(0.0)     # every matrix through the FP32 arithmetic
    A = lufqhe_mod.gen_gaussian(300, n, seed=50 + n)
    check_mixed(lufqhe_mod, oracle, A, max_fallback_frac=0.02)


@pytest.mark.parametrize("n,max_fb", [(6, 0.02), (8, 0.02), (12, 0.05), (16, 0.05), (32, 0.3),
                                      (48, 0.8)])
def test_sizes_lll(cuda, lufqhe_mod, oracle, fp64_share, n, max_fb):
    fp64_share(0.0)
    A, _ = lufqhe_mod.gen_lll(512, n, seed=70 + n)
    check_mixed(lufqhe_mod, oracle, A, max_fallback_frac=max_fb)


def test_wide_dynamic_range_equilibration(cuda, lufqhe_mod, oracle):
    """Rows and columns scaled by 2^+-300: FP32 alone would overflow/underflow."""
    rng = np.random.default_rng(9)
    n, b = 20, 200
    G = (rng.standard_normal((b, n, n)) + 1j * rng.standard_normal((b, n, n))) / math.sqrt(2)
    r = 2.0 ** rng.integers(-300, 300, (b, n, 1))
    c = 2.0 ** rng.integers(-300, 300, (b, 1, n))
    A_np = G * r * c
    A = cuda.from_numpy(A_np).cuda()
    check_mixed(lufqhe_mod, oracle, A, max_fallback_frac=0.02)


def test_zero_threshold_sends_all_to_fp64(cuda, lufqhe_mod, threshold):
    A, _ = lufqhe_mod.gen_lll(1000, 16, seed=5)
    threshold(0.0)
    out = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED))
    fused = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_PLAIN_FP64_FUSED))
    assert np.isin(out["status"], [lufqhe_mod.ST_FALLBACK, lufqhe_mod.ST_FP64]).all()
    assert (out["logabs"] == fused["logabs"]).all() and (out["phase"] == fused["phase"]).all()
    assert (out["parity"] == fused["parity"]).all()


def test_singular_and_nonfinite(cuda, lufqhe_mod):
    n = 6
    A_np = np.tile(np.eye(n, dtype=np.complex128), (3, 1, 1))
    A_np[0, 2] = A_np[0, 1]          # duplicate rows: singular in FP32 and FP64
    A_np[1, 3, 3] = np.nan
    A = cuda.from_numpy(A_np).cuda()
    out = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED))
    assert out["status"][0] == (lufqhe_mod.ST_SINGULAR | lufqhe_mod.ST_FALLBACK)
    assert out["logabs"][0] == -np.inf
    assert out["status"][1] == lufqhe_mod.ST_NONFINITE
    assert out["status"][2] == 0 and abs(out["logabs"][2]) < 1e-14


@pytest.mark.parametrize("n", [8, 24, 28, 32, 48])
def test_default_precision_policy(cuda, lufqhe_mod, oracle, fp64_share, n):
    """Per-size defaults: n <= 32 all through the FP32 path, n > 32 (here 48)
    all FP64; accuracy holds whatever the route."""
    fp64_share(-1.0)
    A, _ = lufqhe_mod.gen_lll(1024, n, seed=90 + n)
    out = check_mixed(lufqhe_mod, oracle, A, max_fallback_frac=0.3)
    routed = ((out["status"] & lufqhe_mod.ST_FP64) != 0).mean()
    want = {8: 0.0, 24: 0.0, 28: 0.0, 32: 0.0, 48: 1.0}[n]
    assert abs(routed - want) < 0.06


@pytest.mark.parametrize("share", [0.0, 0.5, 1.0])
def test_fp64_share_routes_by_content(cuda, lufqhe_mod, share):
    """The FP64-pipe share: routed matrices carry the fused FP64 result and a
    given matrix takes the same route in any batch."""
    lib = lufqhe_mod.lib()
    old = lib.lufqhe_get_option(3)
    lib.lufqhe_set_option(3, share)
    try:
        A, _ = lufqhe_mod.gen_lll(2000, 24, seed=12)
        out = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED))
        routed = (out["status"] & lufqhe_mod.ST_FP64) != 0
        assert abs(routed.mean() - share) < 0.05
        half = host(lufqhe_mod.batch_lup_det(A[1000:].contiguous(), mode=lufqhe_mod.MODE_MIXED))
        assert (half["status"] == out["status"][1000:]).all()
        assert (half["logabs"] == out["logabs"][1000:]).all()
    finally:
        lib.lufqhe_set_option(3, old)


def test_mixed_deterministic_across_batch_positions(cuda, lufqhe_mod):
    """The same matrix gives the same result wherever it sits in the batch."""
    A, _ = lufqhe_mod.gen_lll(97, 24, seed=6)
    full = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED))
    for idx in (0, 31, 32, 96):
        one = host(lufqhe_mod.batch_lup_det(A[idx:idx + 1].contiguous(),
                                            mode=lufqhe_mod.MODE_MIXED))
        assert one["logabs"][0] == full["logabs"][idx]
        assert one["phase"][0] == full["phase"][idx]


@pytest.mark.parametrize("share", [0.0, 0.5])
def test_fp64_pass_every_matrix_listed(cuda, lufqhe_mod, oracle, threshold, fp64_share, share):
    """n = 24 hands every FP64 factorisation to the second pass through the
    call's pending list, which has room for the whole batch: with every matrix
    rejected (threshold 0), or half of them routed, all are refactorised, and
    every (corrected) FP64 result is within 1e-10 of the double-double oracle."""
    threshold(0.0)
    fp64_share(share)
    batch = 16384 + 1028
    A, _ = lufqhe_mod.gen_lll(batch, 24, seed=13)
    out = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED))
    fused = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_PLAIN_FP64_FUSED))
    flags = lufqhe_mod.ST_FALLBACK | lufqhe_mod.ST_FP64
    assert np.isin(out["status"] & flags, [lufqhe_mod.ST_FALLBACK, lufqhe_mod.ST_FP64]).all()
    routed = ((out["status"] & lufqhe_mod.ST_FP64) != 0).mean()
    assert abs(routed - share) < 0.02
    assert ((out["status"] & ~flags) == fused["status"]).all()
    la, ph, _ = oracle.logdet_dd(A.cpu().numpy())
    assert rel(out["logabs"], la).max() < TOL_MIXED
    assert (dphase(out["phase"], ph) / np.maximum(1.0, np.abs(la))).max() < TOL_MIXED
    assert rel(out["logabs"], fused["logabs"]).max() < 1e-6
    del A
    cuda.cuda.empty_cache()


def test_concurrent_calls_on_two_streams(cuda, lufqhe_mod):
    """Mixed calls in flight together on two streams (n = 24, with FP64
    refactorisations, and n = 32) each take their own work counters and
    pending lists and give the results of calls made one at a time."""
    A1, _ = lufqhe_mod.gen_lll(6000, 24, seed=31)
    A2, _ = lufqhe_mod.gen_lll(3000, 32, seed=32)
    A3, _ = lufqhe_mod.gen_lll(5000, 24, seed=33)
    want = [host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED)) for A in (A1, A2, A3)]
    cuda.cuda.synchronize()
    s1, s2 = cuda.cuda.Stream(), cuda.cuda.Stream()
    outs = []
    for rep in range(3):
        outs.append(lufqhe_mod.batch_lup_det(A1, mode=lufqhe_mod.MODE_MIXED, stream=s1))
        outs.append(lufqhe_mod.batch_lup_det(A2, mode=lufqhe_mod.MODE_MIXED, stream=s2))
        outs.append(lufqhe_mod.batch_lup_det(A3, mode=lufqhe_mod.MODE_MIXED, stream=s2 if rep % 2 else s1))
    cuda.cuda.synchronize()
    assert ((want[0]["status"] & lufqhe_mod.ST_FALLBACK) != 0).sum() > 100
    for i, o in enumerate(outs):
        got, w = host(o), want[i % 3]
        assert np.array_equal(got["logabs"], w["logabs"], equal_nan=True)
        assert (got["status"] == w["status"]).all() and (got["parity"] == w["parity"]).all()


@pytest.mark.parametrize("n", [24, 32])
def test_refinement_pass(cuda, lufqhe_mod, oracle, n):
    """n = 24 and 32: matrices whose correction the FP32 solves cannot carry to
    1e-10 get their back substitution refined in a pass of their own; far
    fewer then need the FP64 kernel, and every accepted result stays within
    1e-10 of the double-double oracle. Option 5 = 0 restores the two-pass
    behaviour."""
    lib = lufqhe_mod.lib()
    A, _ = lufqhe_mod.gen_lll(3000, n, seed=90 + n)
    old = lib.lufqhe_get_option(5)
    try:
        lib.lufqhe_set_option(5, 0.0)
        off = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED))
        lib.lufqhe_set_option(5, 1.0)
        on = check_mixed(lufqhe_mod, oracle, A, max_fallback_frac=0.5)
    finally:
        lib.lufqhe_set_option(5, old)
    fb_off = int(((off["status"] & lufqhe_mod.ST_FALLBACK) != 0).sum())
    fb_on = int(((on["status"] & lufqhe_mod.ST_FALLBACK) != 0).sum())
    assert fb_on < 0.7 * fb_off, (fb_on, fb_off)


@pytest.mark.parametrize("n,batch,seed", [(24, 32768, 2), (32, 16384, 3), (16, 32768, 4),
                                          (36, 8192, 5)])
def test_full_size_lll_against_double_double(cuda, lufqhe_mod, oracle, n, batch, seed):
    """The full config-3 batch (and full-size n = 16, 32, 36 LLL batches):
    every result, accepted (refined ones included) or from the corrected FP64
    route (all of them at n = 36), is within 1e-10 (relative to
    max(1, |log|det||)) of the double-double oracle in log|det| and phase."""
    A, _ = lufqhe_mod.gen_lll(batch, n, seed=seed)
    check_mixed(lufqhe_mod, oracle, A, max_fallback_frac=0.2)


def test_release_workspace(cuda, lufqhe_mod):
    """The pool keeps an n = 24 call's refinement buffer after the stream is
    synchronised; lufqhe_release_workspace hands it back to the driver, and
    the next call allocates again and gives the same bits."""
    lib = lufqhe_mod.lib()
    A, _ = lufqhe_mod.gen_lll(16384, 24, seed=41)
    ws = lib.lufqhe_workspace_bytes(24, 16384, lufqhe_mod.MODE_MIXED)
    assert ws > 30 << 20
    first = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED))
    cuda.cuda.synchronize()
    free_before = cuda.cuda.mem_get_info()[0]
    assert lib.lufqhe_release_workspace() == 0
    free_after = cuda.cuda.mem_get_info()[0]
    assert free_after - free_before >= 0.9 * ws, (free_after - free_before, ws)
    again = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED))
    assert np.array_equal(first["logabs"], again["logabs"], equal_nan=True)
    assert (first["status"] == again["status"]).all()


@pytest.mark.parametrize("n,lda", [(12, 16), (24, 32), (32, 33), (48, 64)])
def test_padded_lda(cuda, lufqhe_mod, n, lda):
    """A batch with row stride lda > n (the reference's padded loadSize) gives
    the bits of the same matrices packed at lda = n, through the device entry
    point and the host one (page-locked: read over the host link; pageable:
    staged). n = 48 takes the FP64 route."""
    A, _ = lufqhe_mod.gen_lll(1500, n, seed=70 + n)
    want = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED))
    buf = cuda.zeros((1500, n, lda), dtype=cuda.complex128, device="cuda")
    buf[:, :, :n] = A
    got = host(lufqhe_mod.batch_lup_det(buf, mode=lufqhe_mod.MODE_MIXED))
    hb = buf.cpu()
    outs = [got]
    for Ah in (hb.pin_memory(), hb):
        o = lufqhe_mod.batch_lup_det_host(Ah, mode=lufqhe_mod.MODE_MIXED)
        cuda.cuda.synchronize()
        outs.append({k: getattr(o, k).numpy() for k in ("logabs", "phase", "parity", "status")})
    for o in outs:
        assert np.array_equal(o["logabs"], want["logabs"], equal_nan=True)
        assert np.array_equal(o["phase"], want["phase"], equal_nan=True)
        assert (o["status"] == want["status"]).all() and (o["parity"] == want["parity"]).all()


@pytest.mark.parametrize("n", [8, 24, 48])
def test_empty_batches(cuda, lufqhe_mod, n):
    """An empty mixed-mode batch is a successful call with empty results
    through every entry point (device, host, coordinates)."""
    A = cuda.zeros(0, n, n, dtype=cuda.complex128, device="cuda")
    assert lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED).logabs.numel() == 0
    out = lufqhe_mod.batch_lup_det_host(A.cpu(), mode=lufqhe_mod.MODE_MIXED)
    cuda.cuda.synchronize()
    assert out.logabs.numel() == 0
    z = cuda.zeros(0, n, dtype=cuda.complex128, device="cuda")
    assert lufqhe_mod.lll_det(z, mode=lufqhe_mod.MODE_MIXED).logabs.numel() == 0
    cuda.cuda.synchronize()
