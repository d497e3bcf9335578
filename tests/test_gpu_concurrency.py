"""Mixed-mode calls in flight together: every call owns its work counter,
pending list and saved matrices (one block from the library's stream-ordered
pool), so many calls on many streams, and concurrent replays of captured
calls, give the bits of the same calls made one at a time."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def host(out):
    return {k: getattr(out, k).cpu().numpy() for k in ("logabs", "phase", "parity", "status")}


def same(a, b):
    assert np.array_equal(a["logabs"], b["logabs"], equal_nan=True)
    assert np.array_equal(a["phase"], b["phase"], equal_nan=True)
    assert (a["parity"] == b["parity"]).all() and (a["status"] == b["status"]).all()


def test_300_calls_over_8_streams(cuda, lufqhe_mod):
    """300 mixed n = 24 calls (each with FP64 refactorisations and refinements)
    issued over 8 streams without synchronising: far more than the 256 calls
    the former round-robin lists allowed in flight."""
    torch = cuda
    batches = [lufqhe_mod.gen_lll(1024 + 17 * (i % 5), 24, seed=300 + (i % 5))[0]
               for i in range(5)]
    want = [host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED)) for A in batches]
    assert sum(((w["status"] & lufqhe_mod.ST_FALLBACK) != 0).sum() for w in want) > 100
    torch.cuda.synchronize()
    streams = [torch.cuda.Stream() for _ in range(8)]
    outs = []
    for i in range(300):
        outs.append(lufqhe_mod.batch_lup_det(batches[i % 5], mode=lufqhe_mod.MODE_MIXED,
                                             stream=streams[i % 8]))
    torch.cuda.synchronize()
    for i, o in enumerate(outs):
        same(host(o), want[i % 5])


def test_concurrent_graph_replays(cuda, lufqhe_mod):
    """Two captures of a mixed n = 24 call (with FP64 refactorisations) replayed
    at the same time on two streams, each several times: both give the serial
    call's bits."""
    torch = cuda
    A, _ = lufqhe_mod.gen_lll(4096, 24, seed=310)
    B, _ = lufqhe_mod.gen_lll(3000, 24, seed=311)
    want_a = host(lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED))
    want_b = host(lufqhe_mod.batch_lup_det(B, mode=lufqhe_mod.MODE_MIXED))
    torch.cuda.synchronize()
    graphs, outs = [], []
    for X in (A, B):
        s = torch.cuda.Stream()
        out = lufqhe_mod.DetResult(*(torch.empty(X.shape[0], dtype=d, device="cuda")
                                     for d in (torch.float64, torch.float64, torch.int8,
                                               torch.int32)))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            lufqhe_mod.batch_lup_det(X, mode=lufqhe_mod.MODE_MIXED, stream=s, out=out)  # warm
            s.synchronize()
            with torch.cuda.graph(g, stream=s):
                lufqhe_mod.batch_lup_det(X, mode=lufqhe_mod.MODE_MIXED, stream=s, out=out)
        graphs.append(g)
        outs.append(out)
    torch.cuda.synchronize()
    for o in outs:
        o.logabs.fill_(0.0)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    for _ in range(5):
        with torch.cuda.stream(s1):
            graphs[0].replay()
        with torch.cuda.stream(s2):
            graphs[1].replay()
    torch.cuda.synchronize()
    same(host(outs[0]), want_a)
    same(host(outs[1]), want_b)


def test_kernel_timing(cuda, lufqhe_mod):
    """With kernel timing on, a mixed n = 24 call records its FP32 pass and its
    finish kernel on the launching stream; the record clears when read and
    nothing is recorded once the option is off again."""
    import json
    import ctypes
    lib = lufqhe_mod.lib()
    A, _ = lufqhe_mod.gen_lll(4096, 24, seed=320)
    buf = ctypes.create_string_buffer(4096)
    assert lib.lufqhe_set_option(6, 1.0) == 0
    try:
        for _ in range(3):
            lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED)
        assert lib.lufqhe_kernel_times(buf, len(buf)) == 0
    finally:
        lib.lufqhe_set_option(6, 0.0)
    t = json.loads(buf.value.decode())
    assert t["lup_mixed_tile_kernel<24>"]["launches"] == 3
    assert t["lup_mixed_finish_kernel<24>"]["launches"] == 3
    assert t["lup_mixed_tile_kernel<24>"]["ms"] > 0
    lufqhe_mod.batch_lup_det(A, mode=lufqhe_mod.MODE_MIXED)
    assert lib.lufqhe_kernel_times(buf, len(buf)) == 0
    assert json.loads(buf.value.decode()) == {}
