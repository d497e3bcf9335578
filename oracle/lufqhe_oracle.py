"""ctypes wrapper of the CPU oracle (liblufqhe_oracle.so) and, when it was
built, of the reference's own float32 determinant (_ref/libref_lucorecpu.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the CPU
baseline leg of bench.py, never by the product path.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "liblufqhe_oracle.so"
REF_SO = HERE / "_ref" / "libref_lucorecpu.so"

ARITH_LITERAL = 0
ARITH_KERNEL = 1

_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_longlong
_lib = None
_ref = None


def build() -> None:
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not ORACLE_SO.exists():
            build()
        _lib = ctypes.CDLL(str(ORACLE_SO))
        _lib.lufqhe_oracle_lup_det_fp64.argtypes = [_P, _I, _I, _L, _I, _P, _P, _P, _P, _P, _P, _I]
        _lib.lufqhe_oracle_logdet_dd.argtypes = [_P, _I, _I, _L, _P, _P, _P, _I]
        _lib.lufqhe_oracle_pair_sum.argtypes = [_P, _I, _I, _L, _P, _P, _I]
        _lib.lufqhe_oracle_lup_det_f32.argtypes = [_P, _I, _I, _L, _P, _P, _P, _P, _I]
        _lib.lufqhe_oracle_gen_gaussian.argtypes = [_P, _I, _I, _L, ctypes.c_ulonglong,
                                                    ctypes.c_double]
        _lib.lufqhe_oracle_gen_lll.argtypes = [_P, _P, _I, _I, _L, ctypes.c_ulonglong,
                                               ctypes.c_double]
    return _lib


def ref_available() -> bool:
    return REF_SO.exists()


def ref_lib():
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(str(REF_SO))
        _ref.ref_lucorecpu_det_batch.argtypes = [_P, _I, _I, _L, _P, _I]
        _ref.ref_lucorecpu_factor_batch.argtypes = [_P, _I, _I, _L, _P, _P, _I]
    return _ref


def lup_det(A, arith: int = ARITH_LITERAL, lda: int | None = None, want_factors=False,
            nthreads: int = 0):
    """FP64 restatement of LUCoreCPU::determinant over a batch.

    A: complex128 array (batch, n, lda). Returns dict with logabs, phase,
    parity, status, piv (batch, n) and, if asked, factors (batch, n, n).
    """
    A = np.ascontiguousarray(A, dtype=np.complex128)
    batch, n, cols = A.shape
    lda = cols if lda is None else lda
    out = {
        "logabs": np.empty(batch), "phase": np.empty(batch),
        "parity": np.empty(batch, np.int8), "status": np.empty(batch, np.int32),
        "piv": np.empty((batch, n), np.int32),
    }
    fac = np.empty((batch, n, n), np.complex128) if want_factors else None
    rc = lib().lufqhe_oracle_lup_det_fp64(
        A.ctypes.data, n, lda, batch, arith, out["logabs"].ctypes.data, out["phase"].ctypes.data,
        out["parity"].ctypes.data, out["status"].ctypes.data, out["piv"].ctypes.data,
        fac.ctypes.data if fac is not None else None, nthreads)
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    if fac is not None:
        out["factors"] = fac
    return out


def logdet_dd(A, nthreads: int = 0):
    """Double-double truth: (logabs, phase, status)."""
    A = np.ascontiguousarray(A, dtype=np.complex128)
    batch, n, cols = A.shape
    la = np.empty(batch)
    ph = np.empty(batch)
    st = np.empty(batch, np.int32)
    rc = lib().lufqhe_oracle_logdet_dd(A.ctypes.data, n, cols, batch, la.ctypes.data,
                                       ph.ctypes.data, st.ctypes.data, nthreads)
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    return la, ph, st


def pair_sum(A, nthreads: int = 0):
    """log|sum| and arg of sum_i det(A_2i) det(A_2i+1) (LUCoreCPU::CALL)."""
    A = np.ascontiguousarray(A, dtype=np.complex128)
    batch, n, cols = A.shape
    la = ctypes.c_double()
    ar = ctypes.c_double()
    rc = lib().lufqhe_oracle_pair_sum(A.ctypes.data, n, cols, batch, ctypes.byref(la),
                                      ctypes.byref(ar), nthreads)
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    return la.value, ar.value


def ref_det_f32(A32, nthreads: int = 0):
    """The reference's own float32 determinant; A32 complex64 (batch, n, lda)."""
    A32 = np.ascontiguousarray(A32, dtype=np.complex64)
    batch, n, cols = A32.shape
    det = np.empty(batch, np.complex64)
    rc = ref_lib().ref_lucorecpu_det_batch(A32.ctypes.data, n, cols, batch, det.ctypes.data,
                                           nthreads)
    if rc != 0:
        raise ValueError("reference harness rejected the arguments")
    return det


def lup_det_f32(A32, nthreads: int = 0):
    """Float32 restatement of LUCoreCPU::determinant: complex64 det (direct
    product, as the reference returns it), factors (batch, n, n) complex64 in
    pivoted row order, piv (batch, n) and status."""
    A32 = np.ascontiguousarray(A32, dtype=np.complex64)
    batch, n, cols = A32.shape
    det = np.empty(batch, np.complex64)
    fac = np.empty((batch, n, n), np.complex64)
    piv = np.empty((batch, n), np.int32)
    st = np.empty(batch, np.int32)
    rc = lib().lufqhe_oracle_lup_det_f32(A32.ctypes.data, n, cols, batch, det.ctypes.data,
                                         fac.ctypes.data, piv.ctypes.data, st.ctypes.data,
                                         nthreads)
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    return {"det": det, "factors": fac, "piv": piv, "status": st}


def ref_factor_f32(A32, nthreads: int = 0):
    """The reference's own float32 determinant and the factors it leaves in place."""
    A32 = np.ascontiguousarray(A32, dtype=np.complex64)
    batch, n, cols = A32.shape
    det = np.empty(batch, np.complex64)
    fac = np.empty((batch, n, n), np.complex64)
    rc = ref_lib().ref_lucorecpu_factor_batch(A32.ctypes.data, n, cols, batch, det.ctypes.data,
                                              fac.ctypes.data, nthreads)
    if rc != 0:
        raise ValueError("reference harness rejected the arguments")
    return det, fac


def factor_digests(fac):
    """One 64-bit digest per matrix of its factor bytes (blake2b), for compact
    bit-for-bit comparison against committed golden values."""
    import hashlib
    fac = np.ascontiguousarray(fac)
    return np.array([int.from_bytes(hashlib.blake2b(m.tobytes(), digest_size=8).digest(), "little")
                     for m in fac], dtype=np.uint64)


def gen_gaussian(batch: int, n: int, seed: int, sigma: float = 1.0):
    """The library's seeded complex Gaussian matrices, generated here on the host."""
    A = np.empty((batch, n, n), np.complex128)
    if lib().lufqhe_oracle_gen_gaussian(A.ctypes.data, n, n, batch, seed, sigma) != 0:
        raise ValueError("oracle rejected the arguments")
    return A


def gen_lll(batch: int, n: int, seed: int, sigma: float | None = None):
    """The library's seeded lowest-Landau-level orbital matrices; returns (A, z)."""
    import math
    sigma = math.sqrt(n) if sigma is None else sigma
    A = np.empty((batch, n, n), np.complex128)
    z = np.empty((batch, n), np.complex128)
    if lib().lufqhe_oracle_gen_lll(A.ctypes.data, z.ctypes.data, n, n, batch, seed, sigma) != 0:
        raise ValueError("oracle rejected the arguments")
    return A, z
