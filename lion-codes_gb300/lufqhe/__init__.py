"""Python host side of lufqhe: batched LUP determinants through the C-ABI.

The compute is liblufqhe.so (hand-written sm_103a CUDA). This module only
hands it device pointers; PyTorch supplies device memory and streams. There is
no CPU path here: if the library is missing every call raises.

Names follow the reference's GPU entry point LUCoreGPU::CALL
(LU-fqhe/inc/LUCoreGPU.h:47): a batch of matrices in device memory, the matrix
side n, the row stride (the reference's loadSize) and the batch count in; one
determinant per matrix out, as log|det|, phase, parity and status.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

from . import _native
from .build import build  # noqa: F401  (re-export)

MODE_PLAIN_FP64 = 0
MODE_PLAIN_FP64_FUSED = 1
MODE_MIXED = 2

ST_SCALE_TINY = 1
ST_SINGULAR = 2
ST_NONFINITE = 4
ST_FALLBACK = 8
ST_FP64 = 16

MAX_N = 64

DTYPE_C128 = 0
DTYPE_C64 = 1


def lib():
    return _native.load()


def _stream_ptr(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


@dataclass
class DetResult:
    """Per-matrix determinant in log-polar form (device tensors)."""
    logabs: "object"
    phase: "object"
    parity: "object"
    status: "object"


def _shape(A, lda):
    if A.dim() != 3:
        raise ValueError("A must be (batch, n, lda)")
    batch, n, cols = A.shape
    lda = cols if lda is None else lda
    if not A.is_contiguous():
        raise ValueError("A must be contiguous")
    return batch, n, lda


def _dtype_code(A):
    import torch
    if A.dtype == torch.complex128:
        return DTYPE_C128
    if A.dtype == torch.complex64:
        return DTYPE_C64
    raise TypeError("A must be complex128 or complex64")


def batch_lup_det(A, mode: int = MODE_PLAIN_FP64, stream=None, out: DetResult | None = None):
    """Determinants of a (batch, n, lda) complex128 or complex64 CUDA tensor
    (first n columns used); complex64 entries are widened exactly."""
    import torch
    batch, n, lda = _shape(A, None)
    dtype = _dtype_code(A)
    if not A.is_cuda:
        raise TypeError("A must be a CUDA tensor")
    if out is None:
        dev = A.device
        out = DetResult(torch.empty(batch, dtype=torch.float64, device=dev),
                        torch.empty(batch, dtype=torch.float64, device=dev),
                        torch.empty(batch, dtype=torch.int8, device=dev),
                        torch.empty(batch, dtype=torch.int32, device=dev))
    rc = lib().lufqhe_batch_lup_det(A.data_ptr(), n, lda, batch, dtype, mode, out.logabs.data_ptr(),
                                    out.phase.data_ptr(), out.parity.data_ptr(),
                                    out.status.data_ptr(), _stream_ptr(stream))
    _native.check(rc, "lufqhe_batch_lup_det")
    return out


def lll_det(z, mode: int = MODE_PLAIN_FP64, stream=None, out: DetResult | None = None):
    """Determinants of the LLL orbital matrices of (batch, n) complex128
    coordinates z, built inside the factorising kernels. z and out may be CUDA
    tensors or page-locked host tensors (read and written over the host link)."""
    import torch
    if z.dim() != 2 or z.dtype != torch.complex128 or not z.is_contiguous() or \
            not (z.is_cuda or z.is_pinned()):
        raise TypeError("z must be a contiguous (batch, n) complex128 CUDA or pinned tensor")
    batch, n = z.shape
    if out is None:
        dev = z.device
        pin = not z.is_cuda
        out = DetResult(*(torch.empty(batch, dtype=d, device=dev, pin_memory=pin)
                          for d in (torch.float64, torch.float64, torch.int8, torch.int32)))
    rc = lib().lufqhe_lll_det(z.data_ptr(), n, batch, mode, out.logabs.data_ptr(),
                              out.phase.data_ptr(), out.parity.data_ptr(), out.status.data_ptr(),
                              _stream_ptr(stream))
    _native.check(rc, "lufqhe_lll_det")
    return out


@dataclass
class CfConfig:
    """One composite-fermion configuration: np particle angles and the
    parameters of the last two columns (the arguments of the reference's
    mkMatrixElements, LU-fqhe/src/mkMatrixElements.cu:46-50)."""
    phi: "object"
    theta: "object"
    k1: float
    k2: float
    r1: float
    r2: float
    mu: int
    nu: int

    def angles(self):
        import numpy as np
        phi = np.ascontiguousarray(self.phi, dtype=np.float64)
        theta = np.ascontiguousarray(self.theta, dtype=np.float64)
        if phi.ndim != 1 or phi.shape != theta.shape:
            raise ValueError("phi and theta must be 1-D arrays of the same length")
        return phi, theta


def _perm_shape(perm, n):
    import torch
    if perm.dim() != 2 or perm.dtype != torch.int16 or not perm.is_contiguous() or \
            not (perm.is_cuda or perm.is_pinned()):
        raise TypeError("perm must be a contiguous (batch, stride) int16 CUDA or pinned tensor")
    if perm.shape[1] < n:
        raise ValueError("perm rows must hold at least n entries")
    return perm.shape[0], perm.shape[1]


def cf_det(cfg: CfConfig, perm, n: int, mode: int = MODE_PLAIN_FP64, stream=None,
           out: DetResult | None = None):
    """Determinants of the CF matrices of configuration cfg and the 1-based
    particle lists perm[:, :n], built inside the factorising kernels."""
    import torch
    phi, theta = cfg.angles()
    batch, stride = _perm_shape(perm, n)
    if out is None:
        dev = perm.device
        pin = not perm.is_cuda
        out = DetResult(*(torch.empty(batch, dtype=d, device=dev, pin_memory=pin)
                          for d in (torch.float64, torch.float64, torch.int8, torch.int32)))
    rc = lib().lufqhe_cf_det(phi.ctypes.data, theta.ctypes.data, phi.size, n, cfg.k1, cfg.k2,
                             cfg.r1, cfg.r2, cfg.mu, cfg.nu, perm.data_ptr(), stride, batch, mode,
                             out.logabs.data_ptr(), out.phase.data_ptr(), out.parity.data_ptr(),
                             out.status.data_ptr(), _stream_ptr(stream))
    _native.check(rc, "lufqhe_cf_det")
    return out


def gen_cf(cfg: CfConfig, perm, n: int, lda: int | None = None, dtype=None, stream=None):
    """The CF matrices of cf_det written out: a (batch, n, lda) tensor."""
    import torch
    phi, theta = cfg.angles()
    batch, stride = _perm_shape(perm, n)
    lda = n if lda is None else lda
    dtype = torch.complex128 if dtype is None else dtype
    A = torch.zeros(batch, n, lda, dtype=dtype, device=perm.device)
    rc = lib().lufqhe_gen_cf(phi.ctypes.data, theta.ctypes.data, phi.size, n, cfg.k1, cfg.k2,
                             cfg.r1, cfg.r2, cfg.mu, cfg.nu, perm.data_ptr(), stride, batch,
                             A.data_ptr(), lda, _dtype_code(A), _stream_ptr(stream))
    _native.check(rc, "lufqhe_gen_cf")
    return A


def cf_tables(cfg: CfConfig, n: int):
    """The host tables the CF calls upload: (uv (2, np), tab (np, n)) complex128."""
    import numpy as np
    phi, theta = cfg.angles()
    uv = np.empty((2, phi.size), dtype=np.complex128)
    tab = np.empty((phi.size, n), dtype=np.complex128)
    rc = lib().lufqhe_cf_tables(phi.ctypes.data, theta.ctypes.data, phi.size, n, uv.ctypes.data,
                                tab.ctypes.data)
    _native.check(rc, "lufqhe_cf_tables")
    return uv, tab


def batch_lup_det_host(A, mode: int = MODE_PLAIN_FP64, stream=None,
                       out: DetResult | None = None) -> DetResult:
    """Determinants of a (batch, n, lda) complex128 tensor in HOST memory, results
    in host memory: the library pipelines the copies with the factorisation.
    Page-locked tensors (pin_memory) let the copies overlap. The call is
    asynchronous on `stream`; synchronise it before reading `out`."""
    import torch
    batch, n, lda = _shape(A, None)
    dtype = _dtype_code(A)
    if A.is_cuda or not A.is_contiguous():
        raise TypeError("A must be a contiguous complex128 / complex64 host tensor")
    if out is None:
        pin = A.is_pinned()
        out = DetResult(torch.empty(batch, dtype=torch.float64, pin_memory=pin),
                        torch.empty(batch, dtype=torch.float64, pin_memory=pin),
                        torch.empty(batch, dtype=torch.int8, pin_memory=pin),
                        torch.empty(batch, dtype=torch.int32, pin_memory=pin))
    rc = lib().lufqhe_batch_lup_det_host(A.data_ptr(), n, lda, batch, dtype, mode,
                                         out.logabs.data_ptr(), out.phase.data_ptr(),
                                         out.parity.data_ptr(), out.status.data_ptr(),
                                         _stream_ptr(stream))
    _native.check(rc, "lufqhe_batch_lup_det_host")
    return out


def factor_inplace(A, mode: int = MODE_PLAIN_FP64, stream=None) -> DetResult:
    """Overwrite A with its L\\U factors (pivoted row order); return the determinants."""
    import torch
    batch, n, lda = _shape(A, None)
    dev = A.device
    out = DetResult(torch.empty(batch, dtype=torch.float64, device=dev),
                    torch.empty(batch, dtype=torch.float64, device=dev),
                    torch.empty(batch, dtype=torch.int8, device=dev),
                    torch.empty(batch, dtype=torch.int32, device=dev))
    rc = lib().lufqhe_batch_lup_factor_inplace(A.data_ptr(), n, lda, batch, mode,
                                               out.logabs.data_ptr(), out.phase.data_ptr(),
                                               out.parity.data_ptr(), out.status.data_ptr(),
                                               _stream_ptr(stream))
    _native.check(rc, "lufqhe_batch_lup_factor_inplace")
    return out


def lucoregpu_call(A, pair_product: bool = False, stream=None) -> None:
    """Reference-shaped call: determinant written into element (0,0) of each
    matrix; complex64 tensors (the reference's float2 buffers) take the
    complex64 form of the call."""
    batch, n, lda = _shape(A, None)
    fn = lib().lufqhe_lucoregpu_call_c64 if _dtype_code(A) == DTYPE_C64 else \
        lib().lufqhe_lucoregpu_call
    rc = fn(A.data_ptr(), batch, n, lda, int(pair_product), _stream_ptr(stream))
    _native.check(rc, "lufqhe_lucoregpu_call")


def gen_gaussian(batch: int, n: int, seed: int, sigma: float = 1.0, lda: int | None = None,
                 device="cuda", stream=None):
    """Seeded i.i.d. complex Gaussian matrices (Re, Im ~ N(0, sigma^2/2)) on the device."""
    import torch
    lda = n if lda is None else lda
    A = torch.zeros(batch, n, lda, dtype=torch.complex128, device=device)
    rc = lib().lufqhe_gen_gaussian(A.data_ptr(), n, lda, batch, seed, sigma, _stream_ptr(stream))
    _native.check(rc, "lufqhe_gen_gaussian")
    return A


def gen_lll(batch: int, n: int, seed: int, sigma: float | None = None, lda: int | None = None,
            device="cuda", stream=None):
    """Seeded lowest-Landau-level orbital matrices; returns (A, z)."""
    import torch
    lda = n if lda is None else lda
    sigma = math.sqrt(n) if sigma is None else sigma
    A = torch.zeros(batch, n, lda, dtype=torch.complex128, device=device)
    z = torch.empty(batch, n, dtype=torch.complex128, device=device)
    rc = lib().lufqhe_gen_lll(A.data_ptr(), z.data_ptr(), n, lda, batch, seed, sigma,
                              _stream_ptr(stream))
    _native.check(rc, "lufqhe_gen_lll")
    return A, z


def gen_gaussian_host(batch: int, n: int, seed: int, sigma: float = 1.0):
    """Same draws as gen_gaussian, on the host (numpy complex128)."""
    import numpy as np
    A = np.empty((batch, n, n), dtype=np.complex128)
    rc = lib().lufqhe_gen_gaussian_host(A.ctypes.data, n, n, batch, seed, sigma)
    _native.check(rc, "lufqhe_gen_gaussian_host")
    return A


def gen_lll_host(batch: int, n: int, seed: int, sigma: float | None = None):
    """Same draws as gen_lll, on the host (numpy); returns (A, z)."""
    import numpy as np
    sigma = math.sqrt(n) if sigma is None else sigma
    A = np.empty((batch, n, n), dtype=np.complex128)
    z = np.empty((batch, n), dtype=np.complex128)
    rc = lib().lufqhe_gen_lll_host(A.ctypes.data, z.ctypes.data, n, n, batch, seed, sigma)
    _native.check(rc, "lufqhe_gen_lll_host")
    return A, z


class Plan:
    """A mixed-size batch (groups of same-size matrices) in one persistent,
    graph-captured launch: wraps lufqhe_plan_create/execute/destroy.

    groups: list of (A, out_offset) with A a (count, n, lda) complex128 CUDA
    tensor; results land in `out` at out_offset .. out_offset + count - 1.
    The tensors must stay alive (and at the same address) while the plan lives.
    """

    def __init__(self, groups, out: DetResult, mode: int = MODE_MIXED, autotune: bool = True,
                 stream=None):
        import ctypes
        self._h = None
        self._keep = [A for A, _ in groups]
        arr = (_native.Group * max(1, len(groups)))()
        for i, (A, off) in enumerate(groups):
            count, n, lda = _shape(A, None)
            arr[i].A = A.data_ptr()
            arr[i].n = n
            arr[i].lda = lda
            arr[i].count = count
            arr[i].out_offset = off
        self.out = out
        h = ctypes.c_void_p()
        rc = lib().lufqhe_plan_create(ctypes.byref(h), arr, len(groups), mode,
                                      out.logabs.data_ptr(), out.phase.data_ptr(),
                                      out.parity.data_ptr(), out.status.data_ptr(),
                                      1 if autotune else 0, _stream_ptr(stream))
        _native.check(rc, "lufqhe_plan_create")
        self._h = h

    def execute(self, stream=None, graph: bool = True):
        fn = lib().lufqhe_plan_execute if graph else lib().lufqhe_plan_launch_direct
        _native.check(fn(self._h, _stream_ptr(stream)), "lufqhe_plan_execute")

    def describe(self) -> dict:
        import ctypes
        import json
        buf = ctypes.create_string_buffer(8192)
        _native.check(lib().lufqhe_plan_describe(self._h, buf, len(buf)), "lufqhe_plan_describe")
        return json.loads(buf.value.decode())

    def kernels(self) -> int:
        """Kernels one execution of the plan launches."""
        return int(self.describe().get("kernels", 0))

    def close(self):
        if self._h:
            lib().lufqhe_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Device-resident walkers and the persistent request loop (lufqhe_server_*)."""

    def __init__(self, hbm_budget_bytes: int, mode: int = MODE_MIXED, classes=(8, 16, 32, 64),
                 class_sms=None, max_k: int = 4096, tile: int = 8,
                 moves: "bool | str | None" = None):
        """moves: O(n^2) determinant-ratio moves against kept FP64 factors
        (LUFQHE_OPT_SERVE_MOVES, read at creation): True for every class,
        False for none, "auto" for the classes n <= 16; None keeps the
        option's value (default False: every move refactorises)."""
        import ctypes
        self._h = None
        cn = (ctypes.c_int * len(classes))(*classes)
        cs = (ctypes.c_int * len(classes))(*class_sms) if class_sms else None
        h = ctypes.c_void_p()
        old = lib().lufqhe_get_option(8)
        if moves is not None:
            lib().lufqhe_set_option(8, 2.0 if moves == "auto" else (1.0 if moves else 0.0))
        try:
            rc = lib().lufqhe_server_create(ctypes.byref(h), int(hbm_budget_bytes), mode, cn, cs,
                                            len(classes), max_k, tile)
        finally:
            lib().lufqhe_set_option(8, old)
        _native.check(rc, "lufqhe_server_create")
        self._h = h
        self.max_k = max_k

    def walker(self, z):
        """z: (k, n) complex128 numpy array of particle coordinates -> walker id."""
        import ctypes

        import numpy as np
        z = np.ascontiguousarray(z, dtype=np.complex128)
        k, n = z.shape
        wid = ctypes.c_int()
        rc = lib().lufqhe_server_walker_create(self._h, n, k, z.ctypes.data, ctypes.byref(wid))
        if rc == -5:
            return None  # HBM budget exhausted
        _native.check(rc, "lufqhe_server_walker_create")
        return wid.value

    def destroy_walker(self, wid: int):
        _native.check(lib().lufqhe_server_walker_destroy(self._h, wid), "walker_destroy")

    def submit(self, wid: int, particle: int, znew=None):
        import ctypes

        import numpy as np
        t = ctypes.c_longlong()
        ptr = None
        if znew is not None:
            znew = np.ascontiguousarray(znew, dtype=np.complex128)
            ptr = znew.ctypes.data
        rc = lib().lufqhe_server_submit(self._h, wid, particle, ptr, ctypes.byref(t))
        _native.check(rc, "lufqhe_server_submit")
        return t.value

    def result(self, ticket: int, k: int, wait_us: int = 10_000_000):
        import numpy as np
        la = np.empty(k)
        ph = np.empty(k)
        st = np.empty(k, np.int32)
        rc = lib().lufqhe_server_poll(self._h, ticket, wait_us, la.ctypes.data, ph.ctypes.data,
                                      st.ctypes.data)
        _native.check(rc, "lufqhe_server_poll")
        return la, ph, st

    def run_stream(self, rate_hz: float, nrequests: int, moves: int = 100, k_min: int = 1,
                   k_max: int = 4096, seed: int = 5):
        import ctypes

        import numpy as np
        lat = np.empty(nrequests)
        ns = np.empty(nrequests, np.int32)
        ks = np.empty(nrequests, np.int32)
        el = ctypes.c_double()
        mats = ctypes.c_longlong()
        r = lib().lufqhe_server_run_stream(self._h, rate_hz, nrequests, moves, k_min, k_max, seed,
                                           lat.ctypes.data, ns.ctypes.data, ks.ctypes.data,
                                           nrequests, ctypes.byref(el), ctypes.byref(mats))
        if r < 0:
            _native.check(int(r), "lufqhe_server_run_stream")
        return lat[:r], ns[:r], ks[:r], el.value, mats.value

    def run_closed(self, walkers: int, nrequests: int, moves: int = 100, k_min: int = 1,
                   k_max: int = 4096, seed: int = 5):
        """Closed-loop capacity: (requests, elapsed_s, matrices)."""
        import ctypes
        el = ctypes.c_double()
        mats = ctypes.c_longlong()
        r = lib().lufqhe_server_run_closed(self._h, walkers, nrequests, moves, k_min, k_max, seed,
                                           ctypes.byref(el), ctypes.byref(mats))
        if r < 0:
            _native.check(int(r), "lufqhe_server_run_closed")
        return r, el.value, mats.value

    def stats(self, class_n: int = 0):
        """(moves taken by the O(n^2) path, moves that refactorised instead)."""
        import ctypes
        a = ctypes.c_longlong()
        b = ctypes.c_longlong()
        _native.check(lib().lufqhe_server_stats(self._h, class_n, ctypes.byref(a), ctypes.byref(b)),
                      "lufqhe_server_stats")
        return a.value, b.value

    def close(self):
        if self._h:
            lib().lufqhe_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pair_sum(out: DetResult, stream=None):
    """log|S| and arg S of S = sum_i det(A_2i) det(A_2i+1) (device computation)."""
    import torch
    res = torch.empty(2, dtype=torch.float64, device=out.logabs.device)
    rc = lib().lufqhe_pair_sum(out.logabs.data_ptr(), out.phase.data_ptr(), out.logabs.numel(),
                               res.data_ptr(), _stream_ptr(stream))
    _native.check(rc, "lufqhe_pair_sum")
    return res


def batch_pair_sum(A, mode: int = MODE_PLAIN_FP64, stream=None):
    """log|S| and arg S of S = sum_i det(A_2i) det(A_2i+1) straight from a
    (batch, n, lda) complex128 / complex64 CUDA tensor (a device tensor of 2)."""
    import torch
    batch, n, lda = _shape(A, None)
    res = torch.empty(2, dtype=torch.float64, device=A.device)
    rc = lib().lufqhe_batch_pair_sum(A.data_ptr(), n, lda, batch, _dtype_code(A), mode,
                                     res.data_ptr(), _stream_ptr(stream))
    _native.check(rc, "lufqhe_batch_pair_sum")
    return res


def combine_log_sums(parts):
    """Complex log-sum-exp of partial sums given as (log|S_r|, arg S_r) pairs:
    the host-side reduction of per-rank (or per-batch) wavefunction sums,
    computed by the library's C function (lufqhe_combine_log_sums)."""
    import ctypes
    flat = [float(v) for p in parts for v in p]
    arr = (ctypes.c_double * max(1, len(flat)))(*flat)
    out = (ctypes.c_double * 2)()
    _native.check(lib().lufqhe_combine_log_sums(arr, len(flat) // 2, out),
                  "lufqhe_combine_log_sums")
    return out[0], out[1]


def shard_by_cost(groups, nshards: int, pair_aligned: bool = True):
    """groups: [(n, count), ...] -> per shard, per group, (begin, end) index
    ranges of nearly equal LUP cost (lufqhe_shard_by_cost)."""
    import ctypes
    ng = len(groups)
    ns = (ctypes.c_int * max(1, ng))(*[g[0] for g in groups])
    cs = (ctypes.c_longlong * max(1, ng))(*[g[1] for g in groups])
    b = (ctypes.c_longlong * max(1, ng * nshards))()
    e = (ctypes.c_longlong * max(1, ng * nshards))()
    _native.check(lib().lufqhe_shard_by_cost(ns, cs, ng, nshards, int(pair_aligned), b, e),
                  "lufqhe_shard_by_cost")
    return [[(b[s * ng + g], e[s * ng + g]) for g in range(ng)] for s in range(nshards)]


def allreduce_log_sum(part, group=None):
    """Combine one (log|S|, arg S) per rank over torch.distributed (any
    backend): all-gather the pairs, then the same log-sum-exp on every rank.
    The replicas' only exchange (LU-fqhe/src/MonteCarloLoop.cu:373-392)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(part[0]), float(part[1])], dtype=torch.float64)
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    outs = [torch.empty_like(t) for _ in range(dist.get_world_size(group))]
    dist.all_gather(outs, t, group=group)
    return combine_log_sums([(o[0].item(), o[1].item()) for o in outs])


def read_matrices_f32(path, n: int, first: int = 0, count: int | None = None, lda: int | None = None):
    """Matrices of a raw float32 complex file (the reference's input format)
    as a (count, n, lda) complex128 numpy array."""
    import os

    import numpy as np
    lda = n if lda is None else lda
    if count is None:
        count = os.path.getsize(path) // (8 * n * n) - first
    out = np.zeros((max(0, count), n, lda), np.complex128)
    got = lib().lufqhe_read_matrices_f32(str(path).encode(), n, first, count, lda, out.ctypes.data)
    if got < 0:
        _native.check(int(got), "lufqhe_read_matrices_f32")
    return out[:got]
