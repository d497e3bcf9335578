"""Serving: device-resident walkers, moves, HBM admission, and the same
result for a walker alone and inside a mix of concurrent requests."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def lll_host(z):
    """(k, n) particle coordinates -> (k, n, n) orbital matrices."""
    n = z.shape[1]
    return z[:, :, None] ** np.arange(n)[None, None, :] * np.exp(-np.abs(z) ** 2 / 4)[:, :, None]


def zdraw(rng, k, n):
    return (rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))) * math.sqrt(n / 2)


def znew_draw(rng, k, n):
    """One new coordinate per matrix for a move in a size-n walker (E|z|^2 = n)."""
    return zdraw(rng, k, n)[:, 0]


@pytest.fixture(params=[False, "auto"], ids=["refactor", "moves"])
def server(request, lufqhe_mod, cuda):
    """The default server (every move refactorises) and one taking O(n^2)
    moves for its classes n <= 16."""
    srv = lufqhe_mod.Server(1 << 30, mode=lufqhe_mod.MODE_MIXED, classes=(8, 16), max_k=256,
                            moves=request.param)
    yield srv
    srv.close()


def test_move_matches_direct_determinant(server, oracle):
    rng = np.random.default_rng(1)
    z = zdraw(rng, 50, 16)
    w = server.walker(z)
    # no move: determinants of the initial matrices
    la, ph, st = server.result(server.submit(w, -1), 50)
    want, wph, _ = oracle.logdet_dd(lll_host(z))
    ok = (st & 8) == 0
    assert ok.mean() > 0.9
    assert (np.abs(la - want) / np.maximum(1, np.abs(want))).max() < 1e-10
    # move particle 5
    znew = znew_draw(rng, 50, 16)
    la2, ph2, st2 = server.result(server.submit(w, 5, znew), 50)
    z[:, 5] = znew
    want2, wph2, _ = oracle.logdet_dd(lll_host(z))
    assert (np.abs(la2 - want2) / np.maximum(1, np.abs(want2))).max() < 1e-10
    d = np.abs(np.angle(np.exp(1j * (ph2 - wph2)))) / np.maximum(1, np.abs(want2))
    assert d.max() < 1e-10
    server.destroy_walker(w)


def test_alone_and_in_mix_give_the_same_bits(server):
    rng = np.random.default_rng(2)
    z = zdraw(rng, 120, 16)
    znew = znew_draw(rng, 120, 16)
    a = server.walker(z)
    alone = server.result(server.submit(a, 3, znew), 120)
    server.destroy_walker(a)
    # the same walker and move among many other walkers' moves in flight
    others = [server.walker(zdraw(rng, int(k), n)) for k, n in
              zip(rng.integers(1, 256, 12), [8, 16] * 6)]
    b = server.walker(z)
    tickets = []
    for i, w in enumerate(others[:6]):
        tickets.append((w, server.submit(w, i % 8, znew_draw(rng, 256, 16))))
    tb = server.submit(b, 3, znew)
    for i, w in enumerate(others[6:]):
        tickets.append((w, server.submit(w, i % 8, znew_draw(rng, 256, 16))))
    mixed = server.result(tb, 120)
    for w, t in tickets:
        server.result(t, 256)
    for x, y in zip(alone, mixed):
        assert (np.ascontiguousarray(x).view(np.uint8) == np.ascontiguousarray(y).view(np.uint8)).all()
    for w in others + [b]:
        server.destroy_walker(w)


def test_hbm_admission(lufqhe_mod, cuda):
    """Without moves a walker holds its matrices and coordinates only."""
    n, k = 16, 256
    per_walker = k * n * n * 16 + k * n * 16
    srv = lufqhe_mod.Server(3 * per_walker + 4096, classes=(16,), max_k=256, moves=False)
    rng = np.random.default_rng(3)
    ws = [srv.walker(zdraw(rng, k, n)) for _ in range(3)]
    assert all(w is not None for w in ws)
    assert srv.walker(zdraw(rng, k, n)) is None          # over budget
    srv.destroy_walker(ws[1])
    assert srv.walker(zdraw(rng, k, n)) is not None      # admitted once memory frees
    srv.close()


def test_walker_stream(server):
    lat, ns, ks, elapsed, mats = server.run_stream(rate_hz=5000, nrequests=400, moves=10,
                                                   k_min=1, k_max=256, seed=7)
    assert len(lat) == 400 and np.isfinite(lat).all() and (lat > 0).all()
    assert set(np.unique(ns)) <= {8, 16}
    assert ((ks >= 1) & (ks <= 256)).all() and ks.sum() == mats
    assert mats > 400 and elapsed > 0


@pytest.mark.timeout(300)
def test_closed_loop_with_more_tiles_than_the_ring(lufqhe_mod, cuda):
    """Walkers holding more tiles than a class ring (20 walkers of 4096 n = 64
    matrices at one matrix per tile, against 65536 tiles per ring): the closed
    loop completes every request. A submit refused for ring space waits while
    the other walkers' requests are polled, which returns their space."""
    srv = lufqhe_mod.Server(8 << 30, mode=lufqhe_mod.MODE_MIXED, classes=(64,), max_k=4096,
                            moves=False)
    try:
        done, elapsed, mats = srv.run_closed(walkers=20, nrequests=40, moves=3, k_min=4096,
                                             k_max=4096, seed=3)
    finally:
        srv.close()
    assert done == 40 and mats == 40 * 4096 and elapsed > 0


def test_max_k_beyond_a_class_ring_is_refused(lufqhe_mod, cuda):
    """At one matrix per tile (n = 64) a walker of 70000 matrices would need
    more tiles than the class ring holds: creation refuses it."""
    with pytest.raises(RuntimeError, match="ring"):
        lufqhe_mod.Server(1 << 30, mode=lufqhe_mod.MODE_MIXED, classes=(64,), max_k=70000)


def test_idle_exit_and_relaunch(server, oracle):
    """The class loops leave after 0.2 s without work; a later request
    relaunches them and completes with the right result."""
    import time
    rng = np.random.default_rng(4)
    z = zdraw(rng, 64, 8)
    w = server.walker(z)
    server.result(server.submit(w, -1), 64)
    time.sleep(0.6)                      # every class loop has gone idle and exited
    znew = znew_draw(rng, 64, 8)
    la, ph, st = server.result(server.submit(w, 2, znew), 64)
    z[:, 2] = znew
    want, _, _ = oracle.logdet_dd(lll_host(z))
    ok = (st & 8) == 0
    assert (np.abs(la[ok] - want[ok]) / np.maximum(1, np.abs(want[ok]))).max() < 1e-10
    server.destroy_walker(w)


def test_large_class_follows_precision_policy(lufqhe_mod, cuda, oracle):
    """n = 64 in mixed mode takes the FP64 kernel (status bit 16), as batched
    mixed mode does for n >= 32."""
    srv = lufqhe_mod.Server(1 << 28, mode=lufqhe_mod.MODE_MIXED, classes=(64,), max_k=64)
    try:
        rng = np.random.default_rng(5)
        z = zdraw(rng, 20, 64)
        w = srv.walker(z)
        la, ph, st = srv.result(srv.submit(w, -1), 20)
        assert (st == lufqhe_mod.ST_FP64).all()
        want, _, _ = oracle.logdet_dd(lll_host(z))
        # FP64 LUP on n = 64 orbital matrices: accurate to the FP64 rounding
        # error the condition number allows, well inside 1e-8 here
        assert (np.abs(la - want) / np.maximum(1, np.abs(want))).max() < 1e-8
    finally:
        srv.close()


@pytest.mark.parametrize("mode", [1, 2])
def test_large_class_matches_batched_fp64_bits(lufqhe_mod, cuda, mode):
    """The n = 64 class factorises each matrix with a warp group (one named
    barrier per group, several groups per CTA): results equal the batched FP64
    fused kernel's on the same matrices bit for bit, before and after a move
    (every move refactorising), with many tiles in flight at once."""
    import torch
    srv = lufqhe_mod.Server(1 << 30, mode=mode, classes=(64,), max_k=512, tile=8, moves=False)
    try:
        rng = np.random.default_rng(8)
        z = zdraw(rng, 300, 64)
        w = srv.walker(z)
        la, ph, st = srv.result(srv.submit(w, -1), 300)
        ref = lufqhe_mod.lll_det(torch.from_numpy(z).cuda(), mode=lufqhe_mod.MODE_PLAIN_FP64_FUSED)
        flag = lufqhe_mod.ST_FP64 if mode == lufqhe_mod.MODE_MIXED else 0
        assert np.array_equal(la, ref.logabs.cpu().numpy())
        assert np.array_equal(ph, ref.phase.cpu().numpy())
        assert (st == (ref.status.cpu().numpy() | flag)).all()
        znew = znew_draw(rng, 300, 64)
        la2, ph2, _ = srv.result(srv.submit(w, 11, znew), 300)
        z[:, 11] = znew
        ref2 = lufqhe_mod.lll_det(torch.from_numpy(z).cuda(), mode=lufqhe_mod.MODE_PLAIN_FP64_FUSED)
        assert np.array_equal(la2, ref2.logabs.cpu().numpy())
        assert np.array_equal(ph2, ref2.phase.cpu().numpy())
        srv.destroy_walker(w)
    finally:
        srv.close()


@pytest.mark.parametrize("n", [8, 16, 32])
def test_default_server_matches_batched_mixed_bits(lufqhe_mod, cuda, n):
    """The default server (every move refactorised in mixed mode; one matrix
    per tile at n = 32, eight below) gives the batched mixed path's bits on
    the same matrices, for a walker's first request and after a move: log|det|,
    phase and status, FP64 refactorisations and their corrections included."""
    import torch
    mixed = lufqhe_mod.MODE_MIXED
    srv = lufqhe_mod.Server(1 << 30, mode=mixed, classes=(n,), max_k=512)
    try:
        rng = np.random.default_rng(20 + n)
        z = zdraw(rng, 300, n)
        w = srv.walker(z)
        for particle in (-1, n // 2):
            if particle >= 0:
                znew = znew_draw(rng, 300, n)
                la, ph, st = srv.result(srv.submit(w, particle, znew), 300)
                z[:, particle] = znew
            else:
                la, ph, st = srv.result(srv.submit(w, -1), 300)
            ref = lufqhe_mod.lll_det(torch.from_numpy(z).cuda(), mode=mixed)
            assert np.array_equal(la, ref.logabs.cpu().numpy())
            assert np.array_equal(ph, ref.phase.cpu().numpy())
            assert (st == ref.status.cpu().numpy()).all()
        srv.destroy_walker(w)
    finally:
        srv.close()


@pytest.mark.parametrize("n,tol", [(8, 1e-10), (16, 1e-10), (32, None), (64, None)])
def test_moves_against_double_double(lufqhe_mod, cuda, oracle, n, tol):
    """O(n^2) moves (kept FP64 factors, determinant lemma, Woodbury over the
    moves since the last factorisation, checked before use): after 10 and 100
    single-particle moves every walker matrix's log-determinant against the
    double-double oracle. n = 8, 16: within 1e-10. n = 32, 64, where FP64 LU
    itself misses 1e-10 on a tail of these orbital matrices: no worse than a
    fresh FP64 factorisation of the same matrices, by more than a factor 10,
    above 1e-10."""
    import json
    import torch
    k = 128
    srv = lufqhe_mod.Server(4 << 30, mode=lufqhe_mod.MODE_MIXED, classes=(n,), max_k=k,
                            moves=True)
    rec = {}
    try:
        rng = np.random.default_rng(600 + n)
        z = zdraw(rng, k, n)
        w = srv.walker(z)
        la, ph, st = srv.result(srv.submit(w, -1), k)
        for move in range(1, 101):
            p = int(rng.integers(n))
            znew = znew_draw(rng, k, n)
            la, ph, st = srv.result(srv.submit(w, p, znew), k)
            z[:, p] = znew
            if move in (10, 100):
                want, wph, _ = oracle.logdet_dd(lll_host(z))
                scale = np.maximum(1, np.abs(want))
                err = np.maximum(np.abs(la - want),
                                 np.abs(np.angle(np.exp(1j * (ph - wph))))) / scale
                fresh = lufqhe_mod.lll_det(torch.from_numpy(z).cuda(),
                                           mode=lufqhe_mod.MODE_PLAIN_FP64_FUSED)
                fl = fresh.logabs.cpu().numpy()
                fp = fresh.phase.cpu().numpy()
                ferr = np.maximum(np.abs(fl - want),
                                  np.abs(np.angle(np.exp(1j * (fp - wph))))) / scale
                rec[move] = {"max": float(err.max()), "median": float(np.median(err)),
                             "above_1e-10": int((err > 1e-10).sum()),
                             "fresh_fp64_max": float(ferr.max()),
                             "fresh_fp64_above_1e-10": int((ferr > 1e-10).sum())}
                assert (st == lufqhe_mod.ST_FP64).all()
                if tol is not None:
                    assert err.max() < tol, rec
                else:
                    # as accurate as FP64 itself: no more results above 1e-10
                    # than a fresh factorisation has (plus two), and the worst
                    # within 10x of its worst
                    assert (err > 1e-10).sum() <= (ferr > 1e-10).sum() + 2, rec
                    assert err.max() <= max(1e-10, 10 * ferr.max()), rec
        srv.destroy_walker(w)
    finally:
        srv.close()
    print("moves accuracy", n, json.dumps(rec))


def test_moves_bits_after_build_match_batched(lufqhe_mod, cuda):
    """A walker's first request (with moves on) is an FP64 factorisation whose
    results equal the batched FP64 kernel's bit for bit (the factors it keeps
    are that factorisation's)."""
    import torch
    for n in (16, 64):
        srv = lufqhe_mod.Server(1 << 30, mode=lufqhe_mod.MODE_PLAIN_FP64_FUSED, classes=(n,),
                                max_k=256, moves=True)
        try:
            z = zdraw(np.random.default_rng(700 + n), 200, n)
            w = srv.walker(z)
            la, ph, st = srv.result(srv.submit(w, -1), 200)
            ref = lufqhe_mod.lll_det(torch.from_numpy(z).cuda(),
                                     mode=lufqhe_mod.MODE_PLAIN_FP64_FUSED)
            assert np.array_equal(la, ref.logabs.cpu().numpy())
            assert np.array_equal(ph, ref.phase.cpu().numpy())
            srv.destroy_walker(w)
        finally:
            srv.close()
