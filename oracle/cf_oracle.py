"""CPU restatement of the reference's composite-fermion matrix-element builder
(LU-fqhe/src/mkMatrixElements.cu, compiled out there under #if 0), in FP64.

TEST INFRASTRUCTURE ONLY: imported by tests/, never by the product path.

Parity is pinned by restatement only: the reference's builder is compiled out,
has no tests and no golden outputs, and its own kernel returns the sum of both
derivative terms in both last columns (its column masks are commented out,
:251 and :285), which makes every matrix singular. The restatement keeps one
term per column, as the masks intend.

- tables(): u, v (:91-101) and the orbital table of setupM_Matrix (:169-194),
  from numpy's cos/sin/pow.
- matrices(): calculateElement (:196-293) for every entry of every matrix,
  vectorised over the batch with one numpy operation per rounded step, in the
  device builder's order (one reciprocal of |d|^2 per particle pair for both
  sums), so that from the same tables it reproduces the device's bits.
- entry_loop(): one entry by plain Python complex arithmetic in the
  reference's own order (sum over j < r, then j > r), the independent check of
  matrices().
"""
from __future__ import annotations

import numpy as np


def tables(phi, theta, n: int):
    """(uv (2, np), tab (np, n)) complex128 for n = 2Q + 3."""
    phi = np.asarray(phi, dtype=np.float64)
    theta = np.asarray(theta, dtype=np.float64)
    q = (n - 3) // 2
    ct, st, cp, sp = np.cos(theta), np.sin(theta), np.cos(phi), np.sin(phi)
    u = ct * cp + 1j * (ct * sp)
    v = st * cp - 1j * (st * sp)
    tab = np.zeros((phi.size, n), dtype=np.complex128)
    tab[:, q + 1] = (ct * st) ** q
    zplus, zminus = u / v, v / u
    for j in range(1, q + 2):
        tab[:, q + 1 + j] = tab[:, q + j] * zplus
        tab[:, q + 1 - j] = tab[:, q + 2 - j] * zminus
    return np.stack([u, v]), tab


def _mul(ax, ay, bx, by):
    return ax * bx - ay * by, ax * by + ay * bx


def _columns(u, v, p, n, k1, k2, r1, r2):
    """The two sums of every row r of every matrix (p: (batch, n) 0-based
    particles), in the device's order: per pair (p, q) a = u_p v_q,
    c = u_q v_p, d = a - c, w = 1 / |d|^2 (one correctly rounded reciprocal),
    S1 += ((k1 a + k2 c) conj d) w, S2 += ((r1 a + r2 c) conj d) w."""
    ui, vi = u[p], v[p]
    uix, uiy, vix, viy = ui.real, ui.imag, vi.real, vi.imag
    s1x, s1y, s2x, s2y = (np.zeros(p.shape) for _ in range(4))
    rows = np.arange(n)[None, :]
    for s in range(n):
        q = p[:, s:s + 1]
        uq, vq = u[q], v[q]
        ax, ay = _mul(uix, uiy, vq.real, vq.imag)
        cx, cy = _mul(uq.real, uq.imag, vix, viy)
        dx, dy = ax - cx, ay - cy
        with np.errstate(invalid="ignore", divide="ignore"):
            w = 1.0 / (dx * dx + dy * dy)
            n1x, n1y = k1 * ax + k2 * cx, k1 * ay + k2 * cy
            n2x, n2y = r1 * ax + r2 * cx, r1 * ay + r2 * cy
            t1x, t1y = (n1x * dx + n1y * dy) * w, (n1y * dx - n1x * dy) * w
            t2x, t2y = (n2x * dx + n2y * dy) * w, (n2y * dx - n2x * dy) * w
        keep = rows != s                         # s == r is skipped
        s1x = np.where(keep, s1x + t1x, s1x)
        s1y = np.where(keep, s1y + t1y, s1y)
        s2x = np.where(keep, s2x + t2x, s2x)
        s2y = np.where(keep, s2y + t2y, s2y)
    return (s1x, s1y), (s2x, s2y)


def matrices(uv, tab, perm, n: int, k1, k2, r1, r2, mu: int, nu: int):
    """(batch, n, n) complex128 from the tables and 1-based perm[:, :n]."""
    u, v = uv[0], uv[1]
    p = np.asarray(perm)[:, :n].astype(np.int64) - 1
    if (p < 0).any() or (p >= u.size).any():
        raise ValueError("permutation entries must lie in 1..np")
    q1 = (n - 3) // 2 + 1
    A = np.empty((p.shape[0], n, n), dtype=np.complex128)
    A[:, :, :n - 2] = tab[p, :n - 2]
    sums = _columns(u, v, p, n, k1, k2, r1, r2)
    for col, (sx, sy), c in ((n - 2, sums[0], q1 + mu), (n - 1, sums[1], q1 + nu)):
        t = tab[p, c]
        ex, ey = _mul(sx, sy, t.real, t.imag)
        A[:, :, col] = ex + 1j * ey
    return A


def entry_loop(uv, tab, perm_row, n: int, r: int, c: int, k1, k2, r1, r2, mu: int, nu: int):
    """Entry (r, c) of one matrix in the reference's order (calculateElement)."""
    u, v = uv[0], uv[1]
    q1 = (n - 3) // 2 + 1
    i = int(perm_row[r]) - 1
    if c < n - 2:
        return complex(tab[i, c])
    ka, kb, col = (k1, k2, q1 + mu) if c == n - 2 else (r1, r2, q1 + nu)
    ret = 0j
    others = list(range(r)) + list(range(r + 1, n))
    for j in others:
        q = int(perm_row[j]) - 1
        ret += (ka * u[i] * v[q] + kb * u[q] * v[i]) / (u[i] * v[q] - u[q] * v[i])
    return ret * complex(tab[i, col])


def random_config(np_: int, seed: int):
    """Seeded angles: theta in (0.05, pi/2 - 0.05), phi in [0, 2 pi)."""
    rng = np.random.default_rng(seed)
    theta = rng.uniform(0.05, np.pi / 2 - 0.05, np_)
    phi = rng.uniform(0.0, 2 * np.pi, np_)
    return phi, theta


def random_perms(batch: int, n: int, np_: int, seed: int, stride: int | None = None):
    """(batch, stride) int16: each row n distinct 1-based particles, then zeros."""
    rng = np.random.default_rng(seed)
    stride = n if stride is None else stride
    perm = np.zeros((batch, stride), dtype=np.int16)
    keys = rng.random((batch, np_))
    perm[:, :n] = (np.argsort(keys, axis=1)[:, :n] + 1).astype(np.int16)
    return perm
