"""CPU baseline legs of bench.py: the reference's CPU Crout path (its FP64
restatement in liblufqhe_oracle.so, literal arithmetic) timed on the host
cores with OpenMP over matrices, reported beside the GPU figures as a baseline only.

TEST INFRASTRUCTURE (the CPU-side checker and timing arm): imported by bench.py's cpu_baseline leg and its
`--impl reference` arm, nowhere else in the product.
"""
from __future__ import annotations

import os
import time

import lufqhe_oracle as orc


def _threads() -> int:
    env = os.environ.get("OMP_NUM_THREADS")
    if env and env.isdigit():
        return int(env)
    return os.cpu_count() or 1


def _time_passes(np, A, seconds: float, nthreads: int):
    """Repeat full passes over A until `seconds` elapse (at least one)."""
    orc.lup_det(A[: min(len(A), 64)], arith=orc.ARITH_LITERAL, nthreads=nthreads)  # warm
    t0 = time.perf_counter()
    done = 0
    passes = 0
    while True:
        orc.lup_det(A, arith=orc.ARITH_LITERAL, nthreads=nthreads)
        done += len(A)
        passes += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return done / el, passes, el


def cpu_baseline(np, A_host, n: int, seconds: float = 10.0, max_mats: int = 32768) -> dict:
    A = np.ascontiguousarray(A_host[:max_mats])
    nt = _threads()
    rate, passes, el = _time_passes(np, A, seconds, nt)
    return {"value": rate, "unit": "dets/s", "cores": nt, "kind": "port",
            "sample": f"{passes} passes over {len(A)} matrices n={n} ({el:.1f} s), FP64 "
                      f"restatement of LUCoreCPU::determinant, OpenMP {nt} threads"}


def reference_arm(np, args, kind: str, n: int, batch: int, seed: int, make_inputs,
                  config: dict) -> dict:
    """The `--impl reference` JSON line: K timed steps, each one pass over a
    bounded sample of the workload. `config` is the GPU arm's config object."""
    sample = min(batch, args.ref_sample)
    A = make_inputs(kind, n, sample, seed)
    nt = _threads()
    orc.lup_det(A[:64], arith=orc.ARITH_LITERAL, nthreads=nt)
    for _ in range(args.warmup):
        orc.lup_det(A, arith=orc.ARITH_LITERAL, nthreads=nt)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.lup_det(A, arith=orc.ARITH_LITERAL, nthreads=nt)
    el = time.perf_counter() - t0
    rate = sample * args.steps / el
    desc = (f"{sample} of {batch} matrices n={n} per step, FP64 restatement of the reference's "
            f"CPU Crout (LUCoreCPU::determinant), OpenMP {nt} threads")
    return {
        "impl": "reference",
        "metric": "determinants/s (mixed FP32+FP64-corrected, <=1e-10 rel log|det| err)",
        "value": rate, "unit": "dets/s", "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": config,
        "sample_per_step": sample,
        "cpu_baseline": {"value": rate, "unit": "dets/s", "cores": nt, "kind": "port",
                         "sample": desc},
        "e2e": {"value": rate, "unit": "dets/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
