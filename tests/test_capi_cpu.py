"""CPU checks of the C-ABI library: it loads, exports every declared symbol,
rejects bad arguments before touching a device, and its host generators are
deterministic. No compute call runs here."""
import ctypes

import numpy as np
import pytest


def test_exports_match_header(lufqhe_mod):
    from lufqhe import _native
    lib = lufqhe_mod.lib()
    declared = _native.header_functions()
    assert len(declared) >= 10
    for name in declared:
        assert hasattr(lib, name), f"{name} declared in include/lufqhe.h but not exported"
        assert name in _native.SIGNATURES, f"{name} has no ctypes signature"
    for name in _native.SIGNATURES:
        assert name in declared, f"{name} bound but not declared"


def test_header_constants_match_python(lufqhe_mod):
    from lufqhe import _native
    c = _native.header_constants()
    assert c["LUFQHE_MODE_PLAIN_FP64"] == lufqhe_mod.MODE_PLAIN_FP64
    assert c["LUFQHE_MODE_PLAIN_FP64_FUSED"] == lufqhe_mod.MODE_PLAIN_FP64_FUSED
    assert c["LUFQHE_MODE_MIXED"] == lufqhe_mod.MODE_MIXED
    assert c["LUFQHE_ST_SINGULAR"] == lufqhe_mod.ST_SINGULAR
    assert c["LUFQHE_ST_FALLBACK"] == lufqhe_mod.ST_FALLBACK
    assert c["LUFQHE_MAX_N"] == lufqhe_mod.MAX_N


def test_version_and_error_string(lufqhe_mod):
    lib = lufqhe_mod.lib()
    assert lib.lufqhe_version().decode().count(".") == 2
    assert isinstance(lib.lufqhe_last_error(), bytes)


FAKE = ctypes.c_void_p(0x1000)   # never dereferenced: validation fails first
FAKE_ODD = ctypes.c_void_p(0x1008)


@pytest.mark.parametrize("args,code", [
    ((None, 8, 8, 4, 0, 0, FAKE, None, None, None, None), -1),     # null A
    ((None, 8, 8, 0, 0, 0, None, None, None, None, None), 0),      # empty batch: no-op
    ((FAKE, 8, 8, 4, 0, 0, None, None, None, None, None), -1),     # null logabs
    ((FAKE, 0, 8, 4, 0, 0, FAKE, None, None, None, None), -1),     # n < 1
    ((FAKE, 8, 7, 4, 0, 0, FAKE, None, None, None, None), -1),     # lda < n
    ((FAKE, 8, 8, -1, 0, 0, FAKE, None, None, None, None), -1),    # batch < 0
    ((FAKE, 65, 65, 4, 0, 0, FAKE, None, None, None, None), -2),   # n too large
    ((FAKE_ODD, 8, 8, 4, 0, 0, FAKE, None, None, None, None), -1),  # misaligned
    ((FAKE, 8, 8, 4, 7, 0, FAKE, None, None, None, None), -4),     # unknown dtype
    ((ctypes.c_void_p(0x1004), 8, 8, 4, 1, 0, FAKE, None, None, None, None), -1),  # c64 misaligned
    ((FAKE, 8, 8, 4, 0, 9, FAKE, None, None, None, None), -4),     # unknown mode
])
def test_argument_validation(lufqhe_mod, args, code):
    lib = lufqhe_mod.lib()
    assert lib.lufqhe_batch_lup_det(*args) == code
    if code != 0:
        assert len(lib.lufqhe_last_error()) > 0


@pytest.mark.parametrize("args,code", [
    ((None, 8, 8, 4, 0, 0, FAKE, None, None, None, None), -1),     # null A
    ((None, 8, 8, 0, 0, 0, None, None, None, None, None), 0),      # empty batch: no-op
    ((FAKE, 8, 8, 4, 0, 0, None, None, None, None, None), -1),     # null logabs
    ((FAKE, 8, 7, 4, 0, 0, FAKE, None, None, None, None), -1),     # lda < n
    ((FAKE, 8, 8, -1, 0, 0, FAKE, None, None, None, None), -1),    # batch < 0
    ((FAKE, 65, 65, 4, 0, 0, FAKE, None, None, None, None), -2),   # n too large
    ((FAKE, 8, 8, 4, 7, 0, FAKE, None, None, None, None), -4),     # unknown dtype
    ((FAKE, 8, 8, 4, 0, 9, FAKE, None, None, None, None), -4),     # unknown mode
])
def test_host_entry_argument_validation(lufqhe_mod, args, code):
    """The host-buffer entry point checks its arguments before any CUDA call."""
    lib = lufqhe_mod.lib()
    assert lib.lufqhe_batch_lup_det_host(*args) == code
    if code != 0:
        assert len(lib.lufqhe_last_error()) > 0


@pytest.mark.parametrize("args,code", [
    ((None, 8, 4, 0, FAKE, None, None, None, None), -1),     # null z
    ((None, 8, 0, 0, None, None, None, None, None), 0),      # empty batch: no-op
    ((FAKE, 8, 4, 0, None, None, None, None, None), -1),     # null logabs
    ((FAKE, 0, 4, 0, FAKE, None, None, None, None), -1),     # n < 1
    ((FAKE, 65, 4, 0, FAKE, None, None, None, None), -2),    # n too large
    ((FAKE_ODD, 8, 4, 0, FAKE, None, None, None, None), -1),  # misaligned
    ((FAKE, 8, 4, 9, FAKE, None, None, None, None), -4),     # unknown mode
])
def test_lll_entry_argument_validation(lufqhe_mod, args, code):
    lib = lufqhe_mod.lib()
    assert lib.lufqhe_lll_det(*args) == code
    if code != 0:
        assert len(lib.lufqhe_last_error()) > 0


def test_inplace_rejects_mixed(lufqhe_mod):
    lib = lufqhe_mod.lib()
    rc = lib.lufqhe_batch_lup_factor_inplace(FAKE, 8, 8, 4, 2, FAKE, None, None, None, None)
    assert rc == -4


def test_host_generators_deterministic(lufqhe_mod):
    a = lufqhe_mod.gen_gaussian_host(64, 8, seed=0)
    b = lufqhe_mod.gen_gaussian_host(64, 8, seed=0)
    c = lufqhe_mod.gen_gaussian_host(64, 8, seed=1)
    assert (a == b).all() and not (a == c).all()
    # Re, Im ~ N(0, 1/2)
    assert abs(a.real.var() - 0.5) < 0.05 and abs(a.imag.var() - 0.5) < 0.05
    assert abs(a.mean()) < 0.05


def test_host_lll_structure(lufqhe_mod):
    n = 12
    A, z = lufqhe_mod.gen_lll_host(16, n, seed=3)
    w = np.exp(-np.abs(z) ** 2 / 4)
    want = z[:, :, None] ** np.arange(n)[None, None, :] * w[:, :, None]
    assert np.abs(A - want).max() / np.abs(want).max() < 1e-12
    assert abs((np.abs(z) ** 2).mean() - n) < 0.25 * n


def test_read_reference_file_format(lufqhe_mod, tmp_path):
    """Raw interleaved complex64, row-major, back to back (PermHandler's format)."""
    rng = np.random.default_rng(4)
    M = (rng.random((7, 16, 16)) + 1j * rng.random((7, 16, 16))).astype(np.complex64)
    p = tmp_path / "mats.bin"
    M.tofile(p)
    A = lufqhe_mod.read_matrices_f32(p, 16)
    assert A.shape == (7, 16, 16) and (A == M.astype(np.complex128)).all()
    B = lufqhe_mod.read_matrices_f32(p, 16, first=5, count=10, lda=32)   # short tail
    assert B.shape == (2, 16, 32) and (B[:, :, :16] == M[5:].astype(np.complex128)).all()
    assert (B[:, :, 16:] == 0).all()


def test_workspace_bytes(lufqhe_mod):
    """A mixed call's state block from the library's pool: a 256-byte head (its
    work counter), for n >= 24 a pending list of one 4-byte entry per matrix,
    and at n = 24 and 32 room for a quarter of the batch of saved matrices
    (header 40 B + L\\U and Y at row stride n + 1, 16-byte aligned), each part
    rounded up to 256 bytes. The plain modes take nothing."""
    lib = lufqhe_mod.lib()
    up = lambda v: (v + 255) // 256 * 256  # noqa: E731
    entry24 = (40 + 2 * 24 * 25 * 8 + 15) // 16 * 16
    assert lib.lufqhe_workspace_bytes(24, 32768, 2) == 256 + up(4 * 32768) + up(8192 * entry24)
    entry32 = (40 + 2 * 32 * 33 * 8 + 15) // 16 * 16
    assert lib.lufqhe_workspace_bytes(32, 1000, 2) == 256 + up(4 * 1000) + up(256 * entry32)
    assert lib.lufqhe_workspace_bytes(16, 32768, 2) == 256
    assert lib.lufqhe_workspace_bytes(24, 32768, 1) == 0
    assert lib.lufqhe_workspace_bytes(24, 0, 2) == 0


def test_release_workspace_without_pool(lufqhe_mod):
    """Before any call has made the library's memory pool there is nothing to
    trim: the call succeeds without touching a device."""
    assert lufqhe_mod.lib().lufqhe_release_workspace() == 0


def test_oracle_generators_match_library(lufqhe_mod, oracle):
    """The oracle's seeded generators (used by the CPU reference arm, which must
    not load the product library) draw the library's host matrices bit for bit."""
    for n, seed in ((8, 0), (16, 1)):
        assert np.array_equal(oracle.gen_gaussian(64, n, seed=seed),
                              lufqhe_mod.gen_gaussian_host(64, n, seed=seed))
    for n, seed in ((6, 3), (24, 2), (48, 4)):
        A, z = oracle.gen_lll(64, n, seed=seed)
        B, zb = lufqhe_mod.gen_lll_host(64, n, seed=seed)
        assert np.array_equal(z, zb) and np.array_equal(A, B)


@pytest.mark.parametrize("fn", ["lufqhe_lucoregpu_call", "lufqhe_lucoregpu_call_c64",
                                "lufqhe_lucoregpu_call_noalloc"])
def test_reference_shaped_call_validation(lufqhe_mod, fn):
    """The reference-shaped calls reject bad geometry before any CUDA call and
    treat an empty batch as a no-op (the complex64 form also checks alignment)."""
    lib = lufqhe_mod.lib()
    f = getattr(lib, fn)
    assert f(None, 4, 8, 8, 0, None) == -1
    assert f(FAKE, -1, 8, 8, 0, None) == -1
    assert f(FAKE, 4, 8, 7, 0, None) == -1
    assert f(FAKE, 4, 65, 65, 0, None) == -2
    assert f(FAKE, 0, 8, 8, 0, None) == 0
    if fn.endswith("_c64"):
        assert f(ctypes.c_void_p(0x1004), 4, 8, 8, 0, None) == -1


def test_combine_log_sums_c(lufqhe_mod):
    """lufqhe_combine_log_sums: the complex log-sum-exp of (log|S_r|, arg S_r)
    parts, against the direct sum where it does not overflow; -inf parts add
    nothing, NaN poisons, no part gives -inf."""
    rng = np.random.default_rng(8)
    parts = list(zip(rng.uniform(-5, 5, 9), rng.uniform(-3, 3, 9)))
    s = sum(np.exp(a + 1j * b) for a, b in parts)
    la, ar = lufqhe_mod.combine_log_sums(parts)
    assert abs(la - np.log(abs(s))) < 1e-13 and abs(ar - np.angle(s)) < 1e-13
    big = [(a + 700.0, b) for a, b in parts] + [(-np.inf, 0.3)]
    la2, ar2 = lufqhe_mod.combine_log_sums(big)
    assert abs(la2 - (la + 700.0)) < 1e-12 and abs(ar2 - ar) < 1e-12
    assert lufqhe_mod.combine_log_sums([]) == (-np.inf, 0.0)
    assert np.isnan(lufqhe_mod.combine_log_sums(parts + [(np.nan, 0.0)])[0])


@pytest.mark.parametrize("groups,nshards", [
    ([(24, 32768)], 4), ([(6, 1000), (8, 999), (48, 3001), (64, 10)], 3),
    ([(16, 5)], 8), ([(8, 0), (32, 100), (8, 0)], 2), ([], 3)])
def test_shard_by_cost(lufqhe_mod, groups, nshards):
    """Shards cover every matrix exactly once, in order, boundaries inside a
    group fall on even indices, and the shards' LUP costs differ by at most
    two matrices of the largest size."""
    import bench
    shards = lufqhe_mod.shard_by_cost(groups, nshards, pair_aligned=True)
    assert len(shards) == nshards
    cost = []
    for g, (n, count) in enumerate(groups):
        pos = 0
        for s in range(nshards):
            b, e = shards[s][g]
            assert b == pos and b <= e <= count
            if 0 < e < count:
                assert e % 2 == 0
            pos = e
        assert pos == count
    for s in range(nshards):
        cost.append(sum((e - b) * max(1.0, bench.flops_per_matrix(groups[g][0]))
                        for g, (b, e) in enumerate(shards[s])))
    if groups and sum(c for _, c in groups) > 4 * nshards:
        biggest = max(bench.flops_per_matrix(n) for n, c in groups if c)
        assert max(cost) - min(cost) <= 4 * biggest


def test_shard_by_cost_rejects(lufqhe_mod):
    lib = lufqhe_mod.lib()
    n = (ctypes.c_int * 1)(8)
    c = (ctypes.c_longlong * 1)(10)
    b = (ctypes.c_longlong * 2)()
    e = (ctypes.c_longlong * 2)()
    assert lib.lufqhe_shard_by_cost(n, c, 1, 0, 1, b, e) == -1
    bad = (ctypes.c_int * 1)(0)
    assert lib.lufqhe_shard_by_cost(bad, c, 1, 2, 1, b, e) == -1


@pytest.mark.parametrize("opt,good,bad", [
    (1, [0.0, 0.3], [-1.0]),             # mixed threshold
    (5, [0.0, 1.0], [0.5, 2.0]),         # refinement on/off
    (6, [0.0, 1.0], [2.0]),              # kernel timing
    (7, [0.0, 1.0], [3.0]),              # bulk loads
    (8, [0.0, 1.0, 2.0], [0.5, 3.0]),    # serving moves (0: off, 2: by size)
    (9, [1e-12, 1e-8], [0.0, 1.0, -1e-12]),  # move error bound
])
def test_options_round_trip_and_validation(lufqhe_mod, opt, good, bad):
    """Options are host-side settings: set/get round-trips and out-of-range
    values are rejected (the previous value kept), without a GPU."""
    lib = lufqhe_mod.lib()
    invalid = lufqhe_mod._native.header_constants()["LUFQHE_ERR_INVALID_ARG"]
    old = lib.lufqhe_get_option(opt)
    try:
        for v in good:
            assert lib.lufqhe_set_option(opt, v) == 0
            assert lib.lufqhe_get_option(opt) == pytest.approx(v)
        for v in bad:
            before = lib.lufqhe_get_option(opt)
            assert lib.lufqhe_set_option(opt, v) == invalid
            assert lib.lufqhe_get_option(opt) == before
    finally:
        lib.lufqhe_set_option(opt, old)
    assert lib.lufqhe_set_option(99, 1.0) == invalid
