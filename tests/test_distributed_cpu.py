"""The replicas' only exchange, tested with two gloo ranks on CPU: each rank
holds its shard's partial wavefunction sum (log|S_r|, arg S_r); an all-gather
plus a complex log-sum-exp gives every rank the total, equal to summing the
whole batch in one process. Also a rank that dies before the exchange makes
the survivor fail with an error instead of hanging."""
import math
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def shard_sums(world, seed=0, total=1001):
    rng = np.random.default_rng(seed)
    la = rng.uniform(200, 320, total)          # log|det| of lowest-Landau-level size
    ph = rng.uniform(-math.pi, math.pi, total)
    bounds = np.linspace(0, total // 2, world + 1).astype(int)  # shard by pairs
    parts = []
    for r in range(world):
        i0, i1 = bounds[r], bounds[r + 1]
        l = la[2 * i0:2 * i1:2] + la[2 * i0 + 1:2 * i1:2]
        p = ph[2 * i0:2 * i1:2] + ph[2 * i0 + 1:2 * i1:2]
        m = l.max()
        s = np.sum(np.exp(l - m) * np.exp(1j * p))
        parts.append((m + math.log(abs(s)), math.atan2(s.imag, s.real)))
    npair = total // 2
    l = la[0:2 * npair:2] + la[1:2 * npair:2]
    p = ph[0:2 * npair:2] + ph[1:2 * npair:2]
    m = l.max()
    s = np.sum(np.exp(l - m) * np.exp(1j * p))
    return parts, (m + math.log(abs(s)), math.atan2(s.imag, s.real))


def _worker(rank, world, port, q):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root / "lion-codes_gb300"))
    import torch.distributed as dist

    import lufqhe
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    parts, _ = shard_sums(world)
    q.put((rank, lufqhe.allreduce_log_sum(parts[rank])))
    dist.destroy_process_group()


def test_two_rank_gloo_log_sum():
    world = 2
    port = free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    _, want = shard_sums(world)
    for r in range(world):
        la, ph = got[r]
        assert abs(la - want[0]) < 1e-12 * abs(want[0])
        assert abs(math.remainder(ph - want[1], 2 * math.pi)) < 1e-10


def _dying_worker(rank, world, port, q):
    import datetime
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root / "lion-codes_gb300"))
    import torch.distributed as dist

    import lufqhe
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=5))
    if rank == 1:
        os._exit(3)  # a replica lost between steps, before the exchange
    try:
        lufqhe.allreduce_log_sum((1.0, 0.0))
        q.put("no error")
    except Exception as e:  # the survivor must see an error, not hang
        q.put(type(e).__name__)


def test_lost_rank_is_an_error_not_a_hang():
    world = 2
    port = free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_dying_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    msg = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
    assert msg != "no error"


def test_combine_log_sums_matches_direct():
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "lion-codes_gb300"))
    import lufqhe
    parts, want = shard_sums(5, seed=3)
    la, ph = lufqhe.combine_log_sums(parts)
    assert abs(la - want[0]) < 1e-12 * abs(want[0])
    assert abs(math.remainder(ph - want[1], 2 * math.pi)) < 1e-10
    assert lufqhe.combine_log_sums([]) == (float("-inf"), 0.0)
