"""Mixed-size batches in one persistent, graph-captured launch: results equal
the per-size batched calls bit for bit, replays are deterministic, and new
inputs at the same addresses are picked up."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = (6, 8, 12, 16, 24, 32, 48)


def make_groups(lufqhe, torch, counts, seed0=300):
    groups, off = [], 0
    for n, c in zip(SIZES, counts):
        A, _ = lufqhe.gen_lll(c, n, seed=seed0 + n, sigma=math.sqrt(n))
        groups.append((A, off))
        off += c
    return groups, off


def alloc(lufqhe, torch, total):
    dev = "cuda"
    return lufqhe.DetResult(torch.empty(total, dtype=torch.float64, device=dev),
                            torch.empty(total, dtype=torch.float64, device=dev),
                            torch.empty(total, dtype=torch.int8, device=dev),
                            torch.empty(total, dtype=torch.int32, device=dev))


def host(out):
    return {k: getattr(out, k).cpu().numpy() for k in ("logabs", "phase", "parity", "status")}


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("autotune", [False, True])
def test_plan_matches_batched_calls(cuda, lufqhe_mod, mode, autotune):
    groups, total = make_groups(lufqhe_mod, cuda, (97, 130, 64, 75, 50, 33, 21))
    out = alloc(lufqhe_mod, cuda, total)
    plan = lufqhe_mod.Plan(groups, out, mode=mode, autotune=autotune)
    plan.execute()
    cuda.cuda.synchronize()
    got = host(out)
    lib = lufqhe_mod.lib()
    old_share = lib.lufqhe_get_option(3)
    lib.lufqhe_set_option(3, 0.0)       # batched mixed results with no FP64 routing
    refs = [host(lufqhe_mod.batch_lup_det(A, mode=mode)) for A, _ in groups]
    lib.lufqhe_set_option(3, 1.0)       # and with every matrix routed to the FP64 routine
    routed_refs = [host(lufqhe_mod.batch_lup_det(A, mode=mode)) for A, _ in groups]
    lib.lufqhe_set_option(3, old_share)
    for (A, off), ref, rref in zip(groups, refs, routed_refs):
        sl = slice(off, off + A.shape[0])
        # the tuner may send a size to the FP64 routine (status FP64): those
        # results are the batched call's routed ones (the fused FP64 result,
        # corrected for 17 <= n <= 32); the rest match the batched call
        routed = (got["status"][sl] & lufqhe_mod.ST_FP64) != 0
        for k in ("logabs", "phase", "parity"):
            a = np.ascontiguousarray(got[k][sl])
            b = np.where(routed, rref[k], ref[k]) if mode == lufqhe_mod.MODE_MIXED else ref[k]
            same = (a == b) | (np.isnan(a) & np.isnan(b))
            assert same.all(), (k, A.shape[1])
    desc = plan.describe()
    assert desc["chosen_warps"] >= 1
    plan.close()


def test_plan_replay_and_new_inputs(cuda, lufqhe_mod):
    groups, total = make_groups(lufqhe_mod, cuda, (40, 40, 40, 40, 40, 40, 10))
    out = alloc(lufqhe_mod, cuda, total)
    plan = lufqhe_mod.Plan(groups, out, mode=lufqhe_mod.MODE_MIXED, autotune=False)
    plan.execute()
    plan.execute()
    cuda.cuda.synchronize()
    first = host(out)
    # same addresses, new matrices
    for (A, _), n in zip(groups, SIZES):
        B, _ = lufqhe_mod.gen_lll(A.shape[0], n, seed=900 + n)
        A.copy_(B)
    plan.execute()
    cuda.cuda.synchronize()
    second = host(out)
    assert not np.array_equal(first["logabs"], second["logabs"])
    for A, off in groups:
        ref = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED))
        sl = slice(off, off + A.shape[0])
        assert (second["logabs"][sl] == ref["logabs"]).all()
    # a direct launch gives the same results as the graph replay
    plan.execute(graph=False)
    cuda.cuda.synchronize()
    assert (host(out)["logabs"] == second["logabs"]).all()
    plan.close()


def test_plan_empty_and_invalid(cuda, lufqhe_mod):
    out = alloc(lufqhe_mod, cuda, 1)
    plan = lufqhe_mod.Plan([], out, autotune=False)
    plan.execute()
    cuda.cuda.synchronize()
    plan.close()
    A = lufqhe_mod.gen_gaussian(4, 16, seed=1)
    with pytest.raises(RuntimeError):
        lufqhe_mod.Plan([(A, 0)], out, mode=7)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_plan_large_sizes(cuda, lufqhe_mod, mode):
    """Sizes above 32 only (the warp-group pass), with a size-33 edge group, in
    one plan: results equal the batched calls bit for bit."""
    sizes, counts = (33, 40, 64), (29, 11, 7)
    groups, off = [], 0
    for n, c in zip(sizes, counts):
        A, _ = lufqhe_mod.gen_lll(c, n, seed=700 + n, sigma=math.sqrt(n))
        groups.append((A, off))
        off += c
    out = alloc(lufqhe_mod, cuda, off)
    plan = lufqhe_mod.Plan(groups, out, mode=mode, autotune=False)
    plan.execute()
    cuda.cuda.synchronize()
    got = host(out)
    for A, o in groups:
        ref = host(lufqhe_mod.batch_lup_det(A, mode=mode))
        sl = slice(o, o + A.shape[0])
        for k in ("logabs", "phase", "parity", "status"):
            a, b = np.ascontiguousarray(got[k][sl]), ref[k]
            same = (a == b) | (np.isnan(a) & np.isnan(b)) if a.dtype.kind == "f" else a == b
            assert same.all(), (k, A.shape[1])
    plan.close()


@pytest.mark.parametrize("autotune", [False, True])
def test_plan_on_host_buffers(cuda, lufqhe_mod, autotune):
    """A plan whose groups and outputs are page-locked host memory: the kernels
    read and write over the host link; results equal the device plan's bit
    for bit, and new host inputs at the same addresses are picked up."""
    torch = cuda
    groups, total = make_groups(lufqhe_mod, cuda, (40, 33, 21, 17, 30, 12, 9))
    out = alloc(lufqhe_mod, cuda, total)
    plan = lufqhe_mod.Plan(groups, out, mode=lufqhe_mod.MODE_MIXED, autotune=False)
    plan.execute()
    hosts = [(A.cpu().pin_memory(), o) for A, o in groups]
    out_h = lufqhe_mod.DetResult(*(torch.empty(total, dtype=d, pin_memory=True)
                                   for d in (torch.float64, torch.float64, torch.int8, torch.int32)))
    plan_h = lufqhe_mod.Plan(hosts, out_h, mode=lufqhe_mod.MODE_MIXED, autotune=autotune)
    plan_h.execute()
    torch.cuda.synchronize()
    want = host(out)
    if autotune:
        # the tuner may send a size to the FP64 routine (status FP64), so the
        # bits can differ from the untuned device plan: check accuracy instead
        la, ref = out_h.logabs.numpy(), want["logabs"]
        ok = np.isfinite(ref)
        assert (np.abs(la[ok] - ref[ok]) / np.maximum(1, np.abs(ref[ok]))).max() < 1e-9
        plan.close()
        plan_h.close()
        return
    for k in ("logabs", "phase", "parity", "status"):
        a, b = getattr(out_h, k).numpy(), want[k]
        assert (((a == b) | (np.isnan(a) & np.isnan(b))) if a.dtype.kind == "f" else a == b).all(), k
    # new matrices in the same host buffers
    for (H, o), n in zip(hosts, SIZES):
        B, _ = lufqhe_mod.gen_lll(H.shape[0], n, seed=950 + n)
        H.copy_(B.cpu())
    plan_h.execute()
    torch.cuda.synchronize()
    for (H, o) in hosts:
        ref = host(lufqhe_mod.batch_lup_det(H.cuda(), mode=lufqhe_mod.MODE_MIXED))
        assert np.array_equal(out_h.logabs.numpy()[o:o + H.shape[0]], ref["logabs"], equal_nan=True)
    plan.close()
    plan_h.close()


def test_config4_full_plan_against_double_double(cuda, lufqhe_mod, oracle):
    """The full config-4 batch (200000 LLL matrices, n uniform over 6..48,
    seed 4) through an autotuned mixed plan, every result against the
    double-double oracle: within 1e-10 (relative to max(1, |log|det||), in
    log|det| and phase) for every n <= 32, whatever route the tuner picks;
    n = 48, the FP64 route without a correction (FP64 LUP itself misses 1e-10
    on about 1% of these matrices), equal to the fused FP64 kernel bit for bit."""
    rng = np.random.default_rng(4)
    counts = rng.multinomial(200000, [1.0 / len(SIZES)] * len(SIZES))
    groups, off = [], 0
    for n, c in zip(SIZES, counts):
        A, _ = lufqhe_mod.gen_lll(int(c), n, seed=4 * 100 + n, sigma=math.sqrt(n))
        groups.append((A, off))
        off += int(c)
    out = alloc(lufqhe_mod, cuda, off)
    plan = lufqhe_mod.Plan(groups, out, mode=lufqhe_mod.MODE_MIXED, autotune=True)
    plan.execute()
    cuda.cuda.synchronize()
    got = host(out)
    plan.close()
    for (A, o), n in zip(groups, SIZES):
        sl = slice(o, o + A.shape[0])
        la, ph = got["logabs"][sl], got["phase"][sl]
        if n <= 32:
            want, wph, _ = oracle.logdet_dd(A.cpu().numpy())
            scale = np.maximum(1.0, np.abs(want))
            err = np.maximum(np.abs(la - want), np.abs(np.angle(np.exp(1j * (ph - wph))))) / scale
            assert err.max() < 1e-10, (n, float(err.max()), int((err > 1e-10).sum()))
        else:
            fused = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_PLAIN_FP64_FUSED))
            assert np.array_equal(la, fused["logabs"], equal_nan=True)
            assert np.array_equal(ph, fused["phase"], equal_nan=True)
        del A
