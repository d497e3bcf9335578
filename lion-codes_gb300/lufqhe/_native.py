"""ctypes binding of liblufqhe.so (the C-ABI declared in include/lufqhe.h).

Loading fails loudly when the library has not been built: there is no CPU or
eager fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

from .build import INCLUDE, LIB_PATH

_c = ctypes
P = _c.c_void_p
I32 = _c.c_int
I64 = _c.c_longlong
U64 = _c.c_ulonglong
F64 = _c.c_double

# argtypes for every exported function; the header is parsed in tests to
# check that this table and include/lufqhe.h agree.
SIGNATURES = {
    "lufqhe_batch_lup_det": (I32, [P, I32, I32, I64, I32, I32, P, P, P, P, P]),
    "lufqhe_batch_lup_det_host": (I32, [P, I32, I32, I64, I32, I32, P, P, P, P, P]),
    "lufqhe_lll_det": (I32, [P, I32, I64, I32, P, P, P, P, P]),
    "lufqhe_cf_det": (I32, [P, P, I32, I32, F64, F64, F64, F64, I32, I32, P, I32, I64, I32, P, P,
                            P, P, P]),
    "lufqhe_batch_lup_factor_inplace": (I32, [P, I32, I32, I64, I32, P, P, P, P, P]),
    "lufqhe_lucoregpu_call": (I32, [P, I32, I32, I32, I32, P]),
    "lufqhe_lucoregpu_call_noalloc": (I32, [P, I32, I32, I32, I32, P]),
    "lufqhe_lucoregpu_call_c64": (I32, [P, I32, I32, I32, I32, P]),
    "lufqhe_pair_sum": (I32, [P, P, I64, P, P]),
    "lufqhe_batch_pair_sum": (I32, [P, I32, I32, I64, I32, I32, P, P]),
    "lufqhe_combine_log_sums": (I32, [P, I64, P]),
    "lufqhe_shard_by_cost": (I32, [P, P, I32, I32, I32, P, P]),
    "lufqhe_plan_create": (I32, [P, P, I32, I32, P, P, P, P, I32, P]),
    "lufqhe_plan_execute": (I32, [P, P]),
    "lufqhe_plan_launch_direct": (I32, [P, P]),
    "lufqhe_plan_describe": (I32, [P, P, _c.c_size_t]),
    "lufqhe_plan_destroy": (I32, [P]),
    "lufqhe_server_create": (I32, [P, _c.c_size_t, I32, P, P, I32, I32, I32]),
    "lufqhe_server_walker_create": (I32, [P, I32, I32, P, P]),
    "lufqhe_server_walker_destroy": (I32, [P, I32]),
    "lufqhe_server_submit": (I32, [P, I32, I32, P, P]),
    "lufqhe_server_poll": (I32, [P, I64, I32, P, P, P]),
    "lufqhe_server_destroy": (I32, [P]),
    "lufqhe_server_run_stream": (I64, [P, F64, I64, I32, I32, I32, U64, P, P, P, I64, P, P]),
    "lufqhe_server_run_closed": (I64, [P, I32, I64, I32, I32, I32, U64, P, P]),
    "lufqhe_server_stats": (I32, [P, I32, P, P]),
    "lufqhe_read_matrices_f32": (I64, [_c.c_char_p, I32, I64, I64, I32, P]),
    "lufqhe_gen_gaussian": (I32, [P, I32, I32, I64, U64, F64, P]),
    "lufqhe_gen_lll": (I32, [P, P, I32, I32, I64, U64, F64, P]),
    "lufqhe_gen_cf": (I32, [P, P, I32, I32, F64, F64, F64, F64, I32, I32, P, I32, I64, P, I32,
                            I32, P]),
    "lufqhe_cf_tables": (I32, [P, P, I32, I32, P, P]),
    "lufqhe_gen_gaussian_host": (I32, [P, I32, I32, I64, U64, F64]),
    "lufqhe_gen_lll_host": (I32, [P, P, I32, I32, I64, U64, F64]),
    "lufqhe_set_option": (I32, [I32, F64]),
    "lufqhe_get_option": (F64, [I32]),
    "lufqhe_probe_fma_peak": (I32, [I32, P, P]),
    "lufqhe_kernel_times": (I32, [P, _c.c_size_t]),
    "lufqhe_workspace_bytes": (_c.c_size_t, [I32, I64, I32]),
    "lufqhe_release_workspace": (I32, []),
    "lufqhe_last_error": (_c.c_char_p, []),
    "lufqhe_version": (_c.c_char_p, []),
}

_lib = None


class Group(ctypes.Structure):
    """lufqhe_group_t"""
    _fields_ = [("A", P), ("n", I32), ("lda", I32), ("count", I64), ("out_offset", I64)]


def header_constants() -> dict[str, int]:
    """#define NAME value pairs from include/lufqhe.h (integers only)."""
    out = {}
    for line in (INCLUDE / "lufqhe.h").read_text().splitlines():
        m = re.match(r"#define\s+(LUFQHE_\w+)\s+\(?(-?\d+)\)?", line)
        if m:
            out[m.group(1)] = int(m.group(2))
    return out


def header_functions() -> list[str]:
    text = (INCLUDE / "lufqhe.h").read_text()
    return re.findall(r"^\s*(?:const\s+)?(?:(?:unsigned|long)\s+)*[\w]+\s*\*?\s*(lufqhe_\w+)\s*\(",
                      text, re.M)


def load(path: Path | None = None) -> ctypes.CDLL:
    """Load liblufqhe.so once; raise if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"liblufqhe.so not built ({p}); run __graft_entry__.build()")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        msg = load().lufqhe_last_error().decode(errors="replace")
        raise RuntimeError(f"{what} failed with code {rc}: {msg}")
