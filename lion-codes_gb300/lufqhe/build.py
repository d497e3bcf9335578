"""Compile liblufqhe.so in-tree for sm_103a.

One nvcc invocation per translation unit, run in parallel, then a shared-library
link. Host code is portable C++ (no x86 intrinsics), so the same recipe builds
on x86-64 and on aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parents[1]          # lion-codes_gb300/
REPO_ROOT = PKG_ROOT.parent
CSRC = PKG_ROOT / "csrc"
INCLUDE = REPO_ROOT / "include"
BUILD_DIR = PKG_ROOT / "_build"
LIB_DIR = PKG_ROOT / "lib"
LIB_PATH = LIB_DIR / "liblufqhe.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code is compiled without floating-point contraction, so the host
# generators give the same bits on x86-64 and aarch64 (where FMA is baseline)
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]

SOURCES = ["capi.cu", "lup_plain.cu", "lup_mixed.cu", "lup_mixed_c64.cu", "gen.cu", "probe.cu", "noalloc.cu", "grouped.cu", "serve.cu", "pairsum.cu", "fileio.cu", "hostpipe.cu",
           "host_reduce.cu", "cf.cu"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n"
                           f"{proc.stdout}\n{proc.stderr}")


def build(verbose: bool = False, force: bool = False) -> Path:
    """Build liblufqhe.so if any source is newer than it; return its path."""
    BUILD_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    newest = max(p.stat().st_mtime for p in deps)
    if not force and LIB_PATH.exists() and LIB_PATH.stat().st_mtime >= newest:
        return LIB_PATH
    nvcc = _nvcc()
    objs = []
    cmds = []
    for src in SOURCES:
        obj = BUILD_DIR / (src + ".o")
        objs.append(obj)
        cmds.append([nvcc, *ARCH_FLAGS, *NVCC_FLAGS, "-I", str(INCLUDE), "-I", str(CSRC),
                     "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=min(len(cmds), os.cpu_count() or 4)) as ex:
        list(ex.map(_run, cmds))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    _run([nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs)])
    os.replace(tmp, LIB_PATH)
    if verbose:
        print(f"built {LIB_PATH}")
    return LIB_PATH


if __name__ == "__main__":
    build(verbose=True, force=True)
