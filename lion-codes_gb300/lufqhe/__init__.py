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

MAX_N = 64


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


def batch_lup_det(A, mode: int = MODE_PLAIN_FP64, stream=None, out: DetResult | None = None):
    """Determinants of a (batch, n, lda) complex128 CUDA tensor (first n columns used)."""
    import torch
    batch, n, lda = _shape(A, None)
    if A.dtype != torch.complex128 or not A.is_cuda:
        raise TypeError("A must be a complex128 CUDA tensor")
    if out is None:
        dev = A.device
        out = DetResult(torch.empty(batch, dtype=torch.float64, device=dev),
                        torch.empty(batch, dtype=torch.float64, device=dev),
                        torch.empty(batch, dtype=torch.int8, device=dev),
                        torch.empty(batch, dtype=torch.int32, device=dev))
    rc = lib().lufqhe_batch_lup_det(A.data_ptr(), n, lda, batch, 0, mode, out.logabs.data_ptr(),
                                    out.phase.data_ptr(), out.parity.data_ptr(),
                                    out.status.data_ptr(), _stream_ptr(stream))
    _native.check(rc, "lufqhe_batch_lup_det")
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
    """Reference-shaped call: determinant written into element (0,0) of each matrix."""
    batch, n, lda = _shape(A, None)
    rc = lib().lufqhe_lucoregpu_call(A.data_ptr(), batch, n, lda, int(pair_product),
                                     _stream_ptr(stream))
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
