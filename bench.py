"""Benchmark of the batched LUP determinant on GB300.

Default workload: 32768 lowest-Landau-level orbital matrices, n = 24, complex128
(M_ij = z_i^j exp(-|z_i|^2/4), z ~ CN(0, 24), seed 2), i.e. the precision-stress
configuration on which the mixed-vs-FP64 target is quoted. A "step" is one
batched determinant call over the whole batch. The batch is 302 MB, larger than
the 129 MB L2, so no flush is needed between steps.

Prints ONE JSON line (rank 0). `value` is mixed-precision determinants/s with
the batch resident in HBM; `e2e` is the same call through the C-ABI with the
batch copied from pinned host memory each step and the results copied back.
The plain FP64 kernels, accuracy against the double-double oracle, the
roofline of the dominant kernel and the CPU baseline ride along in the line.

`--impl reference` times the reference's CPU Crout path instead: the FP64
restatement of LUCoreCPU::determinant (the reference is float32-only and its
CPU code is not built on this machine), OpenMP over all host cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "lion-codes_gb300"))

WORKLOADS = {
    # name: (kind, n, batch, seed)
    "lll24": ("lll", 24, 32768, 2),
    "gauss16": ("gauss", 16, 65536, 1),
    "gauss8": ("gauss", 8, 4096, 0),
    # 200000 LLL matrices, n uniform over MIXED_SIZES, one persistent launch
    "mixedn": ("mixed", 0, 200000, 4),
    # Monte Carlo walker stream: Poisson moves, k log-uniform 1..4096, n in
    # SERVE_SIZES, 100 moves per walker, HBM-budgeted device-resident walkers
    "serving": ("serve", 0, 0, 5),
}
SERVE_SIZES = (8, 16, 32, 64)
MIXED_SIZES = (6, 8, 12, 16, 24, 32, 48)


def flops_per_matrix(n: int) -> float:
    """Algorithmic flops of one n x n complex LUP: trailing-update complex MACs
    at 8 real flops plus n(n-1)/2 multiplier scalings at 6 flops."""
    return 4.0 * (n - 1) * n * (2 * n - 1) / 3.0 + 3.0 * n * (n - 1)


def mixed_fp32_ops_per_matrix(n: int) -> float:
    """FP32 lane operations (an FMA counts once) of the mixed method on one
    n x n matrix, counting only entries that contribute:
      LUP trailing updates            4 per complex MAC, sum_m m^2 MACs
      float-float residual (Dot2)     38 per complex MAC, sum_ik (min(i,k)+1)
      forward + backward solves       4 per complex MAC, n^2 (n-1)/2 + n^2 (n+1)/2
      elimination of I + E            4 per complex MAC, sum_m m^2."""
    lu = sum(m * m for m in range(1, n))
    res = sum(min(i, k) + 1 for i in range(n) for k in range(n))
    solves = n * n * (n - 1) / 2 + n * n * (n + 1) / 2
    return 4.0 * lu + 38.0 * res + 4.0 * solves + 4.0 * lu


def mixed_launches_per_call(n: int) -> int:
    """Kernels one mixed-mode batched call launches: the FP32 pass, plus for
    n = 24 and n = 32 the kernel that refines the saved matrices and
    refactorises the rejected ones in FP64 (other n > 24 go straight to the
    FP64 kernel, n < 24 refines and refactorises inside the FP32 pass)."""
    return 2 if n in (24, 32) else 1


def host_chunks(n: int, lda: int, batch: int, chunk_mb: int = 32) -> int:
    """Chunks lufqhe_batch_lup_det_host cuts a batch into (chunk_mb MiB of input each)
    when it stages the batch through device memory (pageable input, plain modes)."""
    per = max(1, (chunk_mb << 20) // (n * lda * 16))
    return (batch + per - 1) // per


def host_launches_per_call(n: int, lda: int, batch: int, mode: int, pinned: bool) -> int:
    """Kernels one lufqhe_batch_lup_det_host call launches. Mixed mode on a
    pinned batch is one launch reading over the host link (FP64
    refactorisations in place, or the plain kernel when the policy sends the
    size to FP64); otherwise the staged pipeline runs the batched call per chunk."""
    if mode == 2 and pinned:
        return 1
    return host_chunks(n, lda, batch) * (mixed_launches_per_call(n) if mode == 2 else 1)


def bytes_per_matrix(n: int) -> float:
    """complex128 input + log|det| (8) + phase (8) + parity (1) + status (4)."""
    return 16.0 * n * n + 21.0


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            pass
    return {}


class ClockSampler:
    """nvidia-smi clock/throttle sampling while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl != "reference" else "gloo"
        if backend == "nccl":
            import torch
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, value: float) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64,
                     device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


ST_FALLBACK = 8
ST_FP64 = 16


def dd_accuracy(np, oracle, A_np, la, ph, st) -> tuple[dict, "object"]:
    """Error of EVERY result against the double-double oracle (complex LU in
    ~32 digits): max(|d log|det||, |d phase|) / max(1, |log|det||), overall and
    by route (accepted by the FP32 path, refactorised in FP64, routed to FP64)."""
    la_dd, ph_dd, _ = oracle.logdet_dd(A_np)
    scale = np.maximum(1.0, np.abs(la_dd))
    fin = np.isfinite(la_dd) & np.isfinite(la)
    e = np.zeros(len(la))
    dph = np.abs(np.angle(np.exp(1j * (ph[fin] - ph_dd[fin]))))
    e[fin] = np.maximum(np.abs(la[fin] - la_dd[fin]), dph) / scale[fin]
    # a non-finite result must match a non-finite truth (singular / NaN input)
    mismatch = int((np.isfinite(la_dd) != np.isfinite(la)).sum())
    routes = {"accepted": st == 0, "fp64_fallback": (st & ST_FALLBACK) != 0,
              "fp64_routed": (st & ST_FP64) != 0}
    out = {"vs": "double-double oracle, every result of the batch",
           "compared": int(fin.sum()), "nonfinite_mismatch": mismatch,
           "max_rel_err": float(e.max(initial=0.0)),
           "median_rel_err": float(np.median(e[fin])) if fin.any() else 0.0,
           "count_above_1e-10": int((e > 1e-10).sum()),
           "by_route": {k: {"count": int(m.sum()), "max_rel_err": float(e[m].max(initial=0.0)),
                            "count_above_1e-10": int((e[m] > 1e-10).sum())}
                        for k, m in routes.items()}}
    return out, (la_dd, ph_dd)


def rel_err_vs(np, la, ph, truth) -> "object":
    la_dd, ph_dd = truth
    scale = np.maximum(1.0, np.abs(la_dd))
    fin = np.isfinite(la_dd) & np.isfinite(la)
    e = np.zeros(len(la))
    e[fin] = np.maximum(np.abs(la[fin] - la_dd[fin]),
                        np.abs(np.angle(np.exp(1j * (ph[fin] - ph_dd[fin]))))) / scale[fin]
    return e


def ncu_traffic(kernel: str, workload: str):
    """dram bytes (read + write) per launch from the committed ncu summary."""
    p = ROOT / "profiles" / f"ncu_{kernel}_{workload}.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


# ---------------------------------------------------------------- GPU probes
def measure_pipe_peaks(torch, lufqhe) -> dict:
    """FP64 and FP32 FMA peaks of this GPU measured with the library's own
    probe kernels (TFLOP/s, 2 flops per FMA)."""
    import ctypes
    lib = lufqhe.lib()
    out = {}
    for name, kind in (("fp64_tflops", 0), ("fp32_tflops", 1)):
        v = ctypes.c_double()
        rc = lib.lufqhe_probe_fma_peak(kind, ctypes.byref(v), None)
        out[name] = v.value if rc == 0 else None
    return out


def kernel_times(torch, lufqhe, fn, steps: int) -> dict:
    """Per-kernel device time of `steps` calls of fn, from the CUDA events the
    library records around each launch on the launching stream
    (LUFQHE_OPT_KERNEL_TIMING): {name: {"launches", "ms", "ms_per_launch"}}."""
    import ctypes
    lib = lufqhe.lib()
    buf = ctypes.create_string_buffer(1 << 16)
    lib.lufqhe_kernel_times(buf, len(buf))  # drop anything recorded before
    lib.lufqhe_set_option(6, 1.0)
    try:
        for _ in range(steps):
            fn()
        torch.cuda.synchronize()
        rc = lib.lufqhe_kernel_times(buf, len(buf))
    finally:
        lib.lufqhe_set_option(6, 0.0)
    if rc != 0:
        return {}
    t = json.loads(buf.value.decode())
    for v in t.values():
        v["ms_per_launch"] = v["ms"] / max(1, v["launches"])
    return t


def make_inputs(torch, lufqhe, wl, want_z=False):
    kind, n, batch, seed = WORKLOADS[wl]
    z = None
    if kind == "lll":
        A, z = lufqhe.gen_lll(batch, n, seed=seed)
    else:
        A = lufqhe.gen_gaussian(batch, n, seed=seed)
    torch.cuda.synchronize()
    return (A, n, batch, z) if want_z else (A, n, batch)


def time_device(torch, lufqhe, A, mode, out, steps, warmup, stream):
    """ms per step with the batch resident; events on the launching stream."""
    for _ in range(warmup):
        lufqhe.batch_lup_det(A, mode=mode, stream=stream, out=out)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        lufqhe.batch_lup_det(A, mode=mode, stream=stream, out=out)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def hbm_peak_gbs():
    p = load_peaks().get("hbm_gbs")
    return (p, "MEASURED_PEAKS.json hbm_gbs (of measured)") if p else \
        (6800.0, "fallback 6.8 TB/s (of fallback)")


def run_batched(args, world, rank, local, workload, full=True):
    """One batched workload (configs 1-3): mixed determinants/s with the batch
    resident, the plain FP64 kernels on the same batch, every result against
    the double-double oracle, the dominant kernel's roofline from CUDA events
    around its own launches; with `full`, also e2e through the host-buffer
    C-ABI call, e2e from particle coordinates and the CPU baseline."""
    import numpy as np
    import torch

    import lufqhe
    import lufqhe_oracle

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(stream):
        A, n, batch, z_dev = make_inputs(torch, lufqhe, workload, want_z=True)
    torch.cuda.synchronize()
    res = lufqhe.DetResult(torch.empty(batch, dtype=torch.float64, device=dev),
                           torch.empty(batch, dtype=torch.float64, device=dev),
                           torch.empty(batch, dtype=torch.int8, device=dev),
                           torch.empty(batch, dtype=torch.int32, device=dev))
    steps = args.steps if full else max(5, args.steps // 2)
    mode = lufqhe.MODE_MIXED

    # ---- headline: mixed, device-resident --------------------------------
    for _ in range(args.warmup):
        lufqhe.batch_lup_det(A, mode=mode, stream=stream, out=res)
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    sampler = ClockSampler(local) if full else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        lufqhe.batch_lup_det(A, mode=mode, stream=stream, out=res)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_mixed = e0.elapsed_time(e1) / steps
    clocks = None
    if sampler:
        time.sleep(0.2)
        clocks = sampler.stop()
    barrier(world)
    ms_mixed_max = max_over_ranks(world, ms_mixed)
    launches = steps * mixed_launches_per_call(n)
    mixed_out = {k: getattr(res, k).cpu().numpy() for k in ("logabs", "phase", "status")}

    # ---- the dominant kernel alone: CUDA events around its own launches ----
    kt = kernel_times(torch, lufqhe,
                      lambda: lufqhe.batch_lup_det(A, mode=mode, stream=stream, out=res), steps)
    dom = f"lup_mixed_tile_kernel<{n}>"

    # ---- plain FP64 kernels (same batch) ---------------------------------
    ms_plain_ref = time_device(torch, lufqhe, A, lufqhe.MODE_PLAIN_FP64, res,
                               max(2, steps // 2), 2, stream)
    ms_plain_fused = time_device(torch, lufqhe, A, lufqhe.MODE_PLAIN_FP64_FUSED, res,
                                 max(2, steps // 2), 2, stream)
    fused_out = {k: getattr(res, k).cpu().numpy() for k in ("logabs", "phase", "status")}
    kt_plain = kernel_times(torch, lufqhe, lambda: lufqhe.batch_lup_det(
        A, mode=lufqhe.MODE_PLAIN_FP64_FUSED, stream=stream, out=res), max(2, steps // 2))

    dets_mixed = batch / (ms_mixed * 1e-3)
    dets_ref = batch / (ms_plain_ref * 1e-3)
    dets_fused = batch / (ms_plain_fused * 1e-3)
    F = flops_per_matrix(n)
    B = bytes_per_matrix(n)
    hbm_peak, hbm_src = hbm_peak_gbs()
    pipes = measure_pipe_peaks(torch, lufqhe)

    out = None
    if rank == 0:
        A_np = A.cpu().numpy()
        acc, truth = dd_accuracy(np, lufqhe_oracle, A_np, mixed_out["logabs"],
                                 mixed_out["phase"], mixed_out["status"])
        e_fp64 = rel_err_vs(np, fused_out["logabs"], fused_out["phase"], truth)
        acc["plain_fp64_fused_vs_dd"] = {"max_rel_err": float(e_fp64.max(initial=0.0)),
                                         "count_above_1e-10": int((e_fp64 > 1e-10).sum())}
        t_dom = kt.get(dom, {}).get("ms_per_launch")
        fp32_peak = pipes.get("fp32_tflops")
        fp64_peak = pipes.get("fp64_tflops")
        roof = {"kernel": dom, "bound": "hbm", "unit": "GB/s", "peak": hbm_peak,
                "peak_source": hbm_src,
                "algorithmic_bytes_per_launch": batch * B,
                "bytes_per_matrix": B,
                "traffic": ncu_traffic("lup_mixed_tile_kernel", workload)}
        if t_dom:
            ach = batch * B / (t_dom * 1e-3) * 1e-9
            roof.update({
                "achieved": ach, "frac": ach / hbm_peak,
                "kernel_ms_per_launch": t_dom, "launches_timed": kt[dom]["launches"],
                "share_of_step": t_dom / ms_mixed,
                "fp32": {"achieved_tflops": batch * F / (t_dom * 1e-3) * 1e-12,
                         "peak": fp32_peak,
                         "frac": (batch * F / (t_dom * 1e-3) * 1e-12 / fp32_peak)
                         if fp32_peak else None,
                         "peak_source": "library FMA probe kernel, this run (no FP32 figure in "
                                        "MEASURED_PEAKS.json)",
                         "flops_per_matrix": F},
                "method_fp32_lane_ops": {
                    "ops_per_matrix": mixed_fp32_ops_per_matrix(n),
                    "frac_of_half_fp32_peak": (mixed_fp32_ops_per_matrix(n) * batch /
                                               (t_dom * 1e-3) * 1e-12 / (fp32_peak / 2.0))
                    if fp32_peak else None},
            })
        t_pl = kt_plain.get(f"lup_plain_kernel<{n}>", kt_plain.get(
            f"lup_plain_group_kernel<{n}>", {})).get("ms_per_launch")
        roof["plain_fp64"] = {
            "kernel": f"lup_plain_kernel<{n}> (fused)", "bound": "fp64", "unit": "TFLOP/s",
            "peak": fp64_peak, "peak_source": "library FMA probe kernel, this run (no FP64 figure "
                                              "in MEASURED_PEAKS.json)",
            "kernel_ms_per_launch": t_pl,
            "achieved": batch * F / (t_pl * 1e-3) * 1e-12 if t_pl else None,
            "frac": (batch * F / (t_pl * 1e-3) * 1e-12 / fp64_peak) if t_pl and fp64_peak
            else None,
            "traffic": ncu_traffic("lup_plain_kernel", workload)}
        out = {
            "value": world * batch / (ms_mixed_max * 1e-3), "unit": "dets/s",
            "ms_per_step": ms_mixed_max, "steps": steps,
            "config": workload_config(workload, world),
            "plain_fp64": {"dets_per_s_reference_arith": dets_ref,
                           "dets_per_s_fused": dets_fused,
                           "mixed_over_plain_fused": dets_mixed / dets_fused,
                           "mixed_over_plain_reference_arith": dets_mixed / dets_ref},
            "accuracy": acc,
            "fallbacks": {"count": int(((mixed_out["status"] & ST_FALLBACK) != 0).sum()),
                          "of": batch},
            "hbm_gbs": B * dets_mixed * 1e-9,
            "kernel_times_ms": kt,
            "roofline": roof,
            "gpu_launches": launches,
        }
        if clocks is not None:
            out["clocks"] = clocks
    if not full:
        barrier(world)
        return out

    # ---- e2e through the C-ABI with host buffers ---------------------------
    # lufqhe_batch_lup_det_host: the batch and the results in page-locked host
    # memory (mixed mode: the kernels read the matrices over the host link)
    A_host = torch.empty(A.shape, dtype=A.dtype, pin_memory=True)
    A_host.copy_(A)
    out_host = lufqhe.DetResult(*(torch.empty(getattr(res, k).shape, dtype=getattr(res, k).dtype,
                                              pin_memory=True)
                                  for k in ("logabs", "phase", "parity", "status")))
    h2d = A_host.numel() * A_host.element_size()
    d2h = sum(getattr(out_host, k).numel() * getattr(out_host, k).element_size()
              for k in ("logabs", "phase", "parity", "status"))

    def e2e_step():
        lufqhe.batch_lup_det_host(A_host, mode=mode, stream=stream, out=out_host)

    for _ in range(max(3, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    barrier(world)
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e3.record(stream)
    torch.cuda.synchronize()
    ms_e2e = max_over_ranks(world, e2.elapsed_time(e3) / args.steps)

    # the host link this box gives a plain copy of the same pinned batch
    link_buf = torch.empty_like(A)
    link_ms = []
    for _ in range(3):
        l0 = torch.cuda.Event(enable_timing=True)
        l1 = torch.cuda.Event(enable_timing=True)
        l0.record(stream)
        with torch.cuda.stream(stream):
            link_buf.copy_(A_host, non_blocking=True)
        l1.record(stream)
        torch.cuda.synchronize()
        link_ms.append(l0.elapsed_time(l1))
    link_gbs = h2d / (min(link_ms) * 1e-3) * 1e-9
    del link_buf

    # ---- e2e from particle coordinates (LLL workloads) ---------------------
    e2e_coords = None
    if z_dev is not None:
        z_host = z_dev.contiguous().cpu().pin_memory()

        def coords_step():
            lufqhe.lll_det(z_host, mode=mode, stream=stream, out=out_host)

        for _ in range(max(3, args.warmup)):
            coords_step()
        torch.cuda.synchronize()
        barrier(world)
        e4 = torch.cuda.Event(enable_timing=True)
        e5 = torch.cuda.Event(enable_timing=True)
        e4.record(stream)
        for _ in range(args.steps):
            coords_step()
        e5.record(stream)
        torch.cuda.synchronize()
        ms_c = max_over_ranks(world, e4.elapsed_time(e5) / args.steps)
        e2e_coords = {"value": world * batch / (ms_c * 1e-3), "unit": "dets/s", "ms_per_step": ms_c,
                      "h2d_bytes_per_step": z_host.numel() * z_host.element_size(),
                      "d2h_bytes_per_step": d2h,
                      "call": "lufqhe_lll_det (orbital matrices built in the kernels from z)"}
    if rank == 0:
        import bench_cpu
        out["e2e"] = {"value": world * batch / (ms_e2e * 1e-3), "unit": "dets/s",
                      "ms_per_step": ms_e2e, "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": d2h,
                      "call": "lufqhe_batch_lup_det_host on page-locked host buffers (mixed mode: "
                              "the kernels read the matrices over the host link, no staging "
                              "copies)",
                      "host_link_copy_gbs": link_gbs,
                      "fraction_of_link": (h2d / (ms_e2e * 1e-3) * 1e-9) / link_gbs}
        out["e2e_from_coordinates"] = e2e_coords
        # cpu_baseline leg: the reference's CPU Crout path (FP64 restatement)
        out["cpu_baseline"] = bench_cpu.cpu_baseline(np, A.cpu().numpy(), n,
                                                     seconds=args.cpu_seconds)
    barrier(world)
    return out


def run_plan(args, world, rank, local, full=True):
    """Config 4: a mixed-size batch of LLL matrices as one plan (work list and
    CUDA graph, tiles, FP64 shares and CTA size from the autotuner), against the
    same plan in plain fused FP64; every result against the double-double
    oracle; per-n rates from batched calls; with `full`, e2e from page-locked
    host buffers."""
    import numpy as np
    import torch

    import lufqhe
    import lufqhe_oracle

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    _, _, total, seed = WORKLOADS["mixedn"]
    counts = np.random.default_rng(seed).multinomial(total, [1.0 / len(MIXED_SIZES)] * len(MIXED_SIZES))
    groups, off = [], 0
    with torch.cuda.stream(stream):
        for n, c in zip(MIXED_SIZES, counts):
            A, _ = lufqhe.gen_lll(int(c), n, seed=seed * 100 + n, sigma=math.sqrt(n))
            groups.append((A, off))
            off += int(c)
    torch.cuda.synchronize()
    steps = args.steps if full else max(5, args.steps // 2)

    def alloc():
        return lufqhe.DetResult(torch.empty(total, dtype=torch.float64, device=dev),
                                torch.empty(total, dtype=torch.float64, device=dev),
                                torch.empty(total, dtype=torch.int8, device=dev),
                                torch.empty(total, dtype=torch.int32, device=dev))

    out = alloc()
    plan = lufqhe.Plan(groups, out, mode=lufqhe.MODE_MIXED, autotune=True, stream=stream)
    tune = plan.describe()

    def timed(fn, nsteps):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(nsteps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / nsteps

    sampler = ClockSampler(local) if full else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    ms = timed(lambda: plan.execute(stream=stream), steps)
    clocks = None
    if sampler:
        time.sleep(0.2)
        clocks = sampler.stop()
    ms_max = max_over_ranks(world, ms)
    launches = steps * plan.kernels()
    mixed_st = out.status.cpu().numpy()
    mixed_la = out.logabs.cpu().numpy()
    mixed_ph = out.phase.cpu().numpy()
    kt = kernel_times(torch, lufqhe, lambda: plan.execute(stream=stream, graph=False), steps)

    # the same batch as one plain FP64 (fused) plan
    out_p = alloc()
    plan_p = lufqhe.Plan(groups, out_p, mode=lufqhe.MODE_PLAIN_FP64_FUSED, autotune=True,
                         stream=stream)
    ms_plain = timed(lambda: plan_p.execute(stream=stream), max(2, steps // 2))
    plain_la = out_p.logabs.cpu().numpy()
    plain_ph = out_p.phase.cpu().numpy()
    # per-size throughput: each group as its own batched call
    per_n = {}
    for (A, o), n in zip(groups, MIXED_SIZES):
        r = lufqhe.DetResult(out.logabs[o:o + A.shape[0]], out.phase[o:o + A.shape[0]],
                             out.parity[o:o + A.shape[0]], out.status[o:o + A.shape[0]])
        t = timed(lambda: lufqhe.batch_lup_det(A, mode=lufqhe.MODE_MIXED, stream=stream, out=r),
                  max(2, steps // 4))
        per_n[str(n)] = {"count": int(A.shape[0]), "dets_per_s": A.shape[0] / (t * 1e-3),
                         "fallbacks": int(((mixed_st[o:o + A.shape[0]] & ST_FALLBACK) != 0).sum())}
    F = sum(flops_per_matrix(n) * int(c) for n, c in zip(MIXED_SIZES, counts))
    B = sum(bytes_per_matrix(n) * int(c) for n, c in zip(MIXED_SIZES, counts))
    pipes = measure_pipe_peaks(torch, lufqhe)
    hbm_peak, hbm_src = hbm_peak_gbs()

    res = None
    if rank == 0:
        # every result of every group against the double-double oracle
        accs, e_all, e_fp64 = {}, [], []
        for (A, o), n in zip(groups, MIXED_SIZES):
            c = A.shape[0]
            a, truth = dd_accuracy(np, lufqhe_oracle, A.cpu().numpy(), mixed_la[o:o + c],
                                   mixed_ph[o:o + c], mixed_st[o:o + c])
            accs[str(n)] = a
            e_all.append(rel_err_vs(np, mixed_la[o:o + c], mixed_ph[o:o + c], truth))
            e_fp64.append(rel_err_vs(np, plain_la[o:o + c], plain_ph[o:o + c], truth))
        e_all = np.concatenate(e_all)
        e_fp64 = np.concatenate(e_fp64)
        acc = {"vs": "double-double oracle, every result of the 200000",
               "max_rel_err": float(e_all.max()), "count_above_1e-10": int((e_all > 1e-10).sum()),
               "plain_fp64_fused_vs_dd": {"max_rel_err": float(e_fp64.max()),
                                          "count_above_1e-10": int((e_fp64 > 1e-10).sum())},
               "per_n": accs}
        top = max(kt.items(), key=lambda kv: kv[1]["ms"]) if kt else None
        roof = None
        if top:
            name, v = top
            nn = int(name.split("<")[1].rstrip(">")) if "<" in name else MIXED_SIZES[-1]
            cnt = int(counts[MIXED_SIZES.index(nn)]) if nn in MIXED_SIZES else 0
            t_k = v["ms_per_launch"]
            fl = flops_per_matrix(nn) * cnt
            roof = {"kernel": name, "bound": "fp64", "unit": "TFLOP/s",
                    "kernel_ms_per_launch": t_k, "share_of_step": t_k / ms,
                    "achieved": fl / (t_k * 1e-3) * 1e-12,
                    "peak": pipes.get("fp64_tflops"),
                    "frac": (fl / (t_k * 1e-3) * 1e-12 / pipes["fp64_tflops"])
                    if pipes.get("fp64_tflops") else None,
                    "peak_source": "library FMA probe kernel, this run",
                    "traffic": None,
                    "hbm": {"achieved": B / (ms * 1e-3) * 1e-9, "peak": hbm_peak,
                            "unit": "GB/s", "frac": B / (ms * 1e-3) * 1e-9 / hbm_peak,
                            "peak_source": hbm_src}}
        res = {"value": world * total / (ms_max * 1e-3), "unit": "dets/s", "ms_per_step": ms_max,
               "steps": steps, "config": workload_config("mixedn", world)
               | {"counts": {str(n): int(c) for n, c in zip(MIXED_SIZES, counts)}},
               "plain_fp64_fused_plan_dets_per_s": total / (ms_plain * 1e-3),
               "mixed_over_plain_fused": ms_plain / ms, "per_n": per_n, "autotune": tune,
               "accuracy": acc,
               "fallbacks": {"count": int(((mixed_st & ST_FALLBACK) != 0).sum()), "of": total},
               "kernel_times_ms": kt, "roofline": roof, "gpu_launches": launches,
               "step_fp64_tflops": F / (ms * 1e-3) * 1e-12}
        if clocks is not None:
            res["clocks"] = clocks
    if full:
        # e2e: the same batch in page-locked host memory, results to page-locked
        # host memory: a plan on the host buffers (kernels read and write over
        # the host link), graph replay
        hosts = [torch.empty(A.shape, dtype=A.dtype, pin_memory=True) for A, _ in groups]
        for h, (A, _) in zip(hosts, groups):
            h.copy_(A)
        out_host = lufqhe.DetResult(*(torch.empty(total, dtype=getattr(out, k).dtype,
                                                  pin_memory=True)
                                      for k in ("logabs", "phase", "parity", "status")))
        plan_h = lufqhe.Plan([(h, o) for h, (_, o) in zip(hosts, groups)], out_host,
                             mode=lufqhe.MODE_MIXED, autotune=True, stream=stream)
        torch.cuda.synchronize()
        ms_e2e = max_over_ranks(world, timed(lambda: plan_h.execute(stream=stream), steps))
        h2d = sum(h.numel() * h.element_size() for h in hosts)
        d2h = sum(getattr(out_host, k).numel() * getattr(out_host, k).element_size()
                  for k in ("logabs", "phase", "parity", "status"))
        if res is not None:
            res["e2e"] = {"value": world * total / (ms_e2e * 1e-3), "unit": "dets/s",
                          "ms_per_step": ms_e2e, "h2d_bytes_per_step": h2d,
                          "d2h_bytes_per_step": d2h,
                          "call": "lufqhe_plan_execute on a plan over page-locked host buffers "
                                  "(the kernels read the matrices and write the results over the "
                                  "host link)"}
            import bench_cpu
            A0 = groups[MIXED_SIZES.index(24)][0][:4096].cpu().numpy()
            res["cpu_baseline"] = bench_cpu.cpu_baseline(np, A0, 24, seconds=args.cpu_seconds)
        plan_h.close()
    plan.close()
    plan_p.close()
    return res


def run_serve(args, world, rank, local, full=True):
    """Config 5: a Poisson stream of single-particle moves of device-resident
    walkers (k log-uniform 1..4096, n uniform over 8/16/32/64, 100 moves per
    walker). Three servers: the default (every move refactorised in mixed
    mode), one taking O(n^2) moves against kept FP64 factors for the classes
    n <= 16, and one refactorising every move in FP64. For
    each: its capacity (the determinants/s of a saturating stream), then the
    stream at 70% of that capacity and at the configured 20k requests/s, with
    p50/p99 latency (arrival to result on the host) and throughput. The
    batched factorisation rates of the size mix are reported beside them."""
    import numpy as np
    import torch

    import lufqhe

    torch.cuda.set_device(local)
    seed = WORKLOADS["serving"][3]
    rng = np.random.default_rng(seed)
    ks = np.maximum(1, np.minimum(4096, np.floor(np.exp(rng.uniform(0, np.log(4097), 200000)))))
    mean_k = float(ks.mean())
    # the same stream length in the default line's sub-result as in the full
    # run: with k up to 4096, a short window is dominated by the drain of its
    # last large requests
    nreq = args.serve_requests

    def offline_rate(n, mode):
        count = max(512, min(32768, int(2e8 // (16 * n * n))))
        A, _ = lufqhe.gen_lll(count, n, seed=seed * 100 + n)
        out = lufqhe.batch_lup_det(A, mode=mode)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            lufqhe.batch_lup_det(A, mode=mode, out=out)
        e1.record()
        torch.cuda.synchronize()
        return count / (e0.elapsed_time(e1) / 3 * 1e-3)

    def summary(lat, ns, el, mats, rate, capacity):
        served_k = mats / max(1, len(lat))
        per = {}
        for n in SERVE_SIZES:
            m = ns == n
            if m.any():
                per[str(n)] = {"p50_ms": float(np.percentile(lat[m], 50) / 1e3),
                               "p99_ms": float(np.percentile(lat[m], 99) / 1e3),
                               "requests": int(m.sum())}
        return {"rate_req_s": rate, "requests": int(len(lat)),
                "mean_k_served": served_k, "offered_dets_s": rate * served_k,
                "p50_ms": float(np.percentile(lat, 50) / 1e3),
                "p99_ms": float(np.percentile(lat, 99) / 1e3),
                "throughput_dets_s": mats / el,
                "fraction_of_capacity": (mats / el) / capacity if capacity else None,
                "per_n": per}

    # the library's default server (mixed refactorisation of every move), one
    # taking O(n^2) moves for the classes n <= 16, and FP64 refactorisation
    variants = [("default", lufqhe.MODE_MIXED, None),
                ("moves_n_le_16", lufqhe.MODE_MIXED, "auto"),
                ("fp64_refactor", lufqhe.MODE_PLAIN_FP64_FUSED, False)]
    def class_rate(n, mode, moves):
        """Determinants/s of one class alone on the whole GPU, closed loop
        (the same walker mix restricted to size n)."""
        srv = lufqhe.Server(96 << 30, mode=mode, classes=(n,), class_sms=[nsm], max_k=4096,
                            tile=8, moves=moves)
        try:
            _, el, mats = srv.run_closed(walkers=args.serve_walkers, nrequests=1000, moves=100,
                                         k_min=1, k_max=4096, seed=seed + 2)
        finally:
            srv.close()
        return mats / el

    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    result = {}
    # determinants per request of the stream: its walkers' shapes are one fixed
    # sequence, and a window of nreq requests sees the first hundred or so of
    # them, whose mean k is not the population's; measured once by a stream at
    # the population's rate, then used to set every offered load in dets/s
    k_req = None
    # each class's share of the stream's determinants, from the same stream
    demand = None

    def shares(weight):
        sms = np.maximum(2, np.round(nsm * weight / weight.sum())).astype(int)
        sms[np.argmax(sms)] -= max(0, int(sms.sum()) - nsm)
        return list(map(int, sms))

    for label, mode, moves in (variants if full else variants[:2]):
        rates = {n: offline_rate(n, mode) for n in SERVE_SIZES}
        batched_mix = 1.0 / float(np.mean([1.0 / rates[n] for n in SERVE_SIZES]))
        # SM shares per class in proportion to the SM time its traffic needs:
        # its share of the stream's determinants times its measured cost per
        # determinant when served alone
        alone = {n: class_rate(n, mode, moves) for n in SERVE_SIZES}
        cost = np.array([1.0 / alone[n] for n in SERVE_SIZES])
        if demand is None:
            # one stream at the population's rate, on shares for equal demand
            srv = lufqhe.Server(96 << 30, mode=mode, classes=SERVE_SIZES,
                                class_sms=shares(cost), max_k=4096, tile=8, moves=moves)
            lat, ns, ks_rec, _, mats = srv.run_stream(rate_hz=0.7 * batched_mix / mean_k,
                                                      nrequests=nreq, moves=100, k_min=1,
                                                      k_max=4096, seed=seed)
            srv.close()
            k_req = mats / max(1, len(lat))
            demand = np.array([ks_rec[ns == n].sum() for n in SERVE_SIZES], dtype=np.float64)
            demand /= max(1.0, demand.sum())
        sms = shares(demand * cost)
        srv = lufqhe.Server(96 << 30, mode=mode, classes=SERVE_SIZES, class_sms=sms, max_k=4096,
                            tile=8, moves=moves)
        # capacity: a closed loop of walkers, each moving again as soon as its
        # last move completes (the open stream's work mix: 100 moves, then a
        # new walker whose first request builds its matrices)
        done, el, mats = srv.run_closed(walkers=args.serve_walkers, nrequests=max(1000, nreq),
                                        moves=100, k_min=1, k_max=4096, seed=seed + 1)
        capacity = mats / el
        moved, refac = srv.stats()
        runs = {"closed_loop_capacity": {"walkers": args.serve_walkers, "requests": done,
                                         "seconds": el, "dets_per_s": capacity,
                                         "requests_per_s": done / el}}
        # the offered loads, in requests/s of the stream's determinants per
        # request: 70% of the batched (offline) rate of the size mix; 70% of
        # the closed-loop capacity; the configured 20k requests/s
        for tag, rate, nr in (("at_70pct_offline", 0.7 * batched_mix / k_req, nreq),
                              ("at_70pct_capacity", 0.7 * capacity / k_req, nreq),
                              ("at_20k_req_s", 20000.0, max(200, nreq // 4))):
            lat, ns, _, el, mats = srv.run_stream(rate_hz=rate, nrequests=nr, moves=100,
                                                  k_min=1, k_max=4096, seed=seed)
            runs[tag] = summary(lat, ns, el, mats, rate, capacity) | \
                {"fraction_of_offline": (mats / el) / batched_mix}
        srv.close()
        # a floor under p99 that no scheduling removes: the 99th percentile of
        # each request's service time alone on the whole GPU, k / (its class's
        # closed-loop rate alone), over the request mix
        ns_mix = rng.choice(np.array(SERVE_SIZES), size=len(ks))
        service = ks / np.array([alone[int(n)] for n in ns_mix])
        p99_floor_ms = float(np.percentile(service, 99) * 1e3)
        result[label] = {"capacity_dets_per_s": capacity,
                         "batched_offline_dets_per_s": {str(n): rates[n] for n in SERVE_SIZES},
                         "batched_offline_mix_dets_per_s": batched_mix,
                         "class_alone_dets_per_s": {str(n): alone[n] for n in SERVE_SIZES},
                         "class_sms": sms,
                         "class_demand_share": {str(n): float(d)
                                                for n, d in zip(SERVE_SIZES, demand)},
                         "runs": runs,
                         "p99_floor_ms_whole_gpu": p99_floor_ms,
                         "moves_o_n2": moved, "moves_refactorised": refac}
    if rank != 0:
        return None
    r70 = result["default"]["runs"]["at_70pct_offline"]
    return {"value": r70["throughput_dets_s"], "unit": "dets/s",
            "p50_ms": r70["p50_ms"], "p99_ms": r70["p99_ms"],
            "fraction_of_offline": r70["fraction_of_offline"],
            "fraction_of_capacity": r70["fraction_of_capacity"],
            "p99_floor_ms_whole_gpu": result["default"]["p99_floor_ms_whole_gpu"],
            "config": workload_config("serving", world) | {"mean_k": mean_k,
                                                           "stream_k_per_request": k_req},
            "serving": result}


METRIC = "determinants/s (mixed FP32+FP64-corrected, <=1e-10 rel log|det| err)"


def base_line(args, world) -> dict:
    return {"metric": METRIC, "n_gpus": world, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "c128 in / fp32+float-float compute / f64 out",
            "data": "synthetic (seeded, generated on device)"}


def run_ours(args):
    world, rank, local = dist_setup(args)
    if args.workload == "mixedn":
        r = run_plan(args, world, rank, local, full=True)
    elif args.workload == "serving":
        r = run_serve(args, world, rank, local, full=True)
        if r is not None:
            r |= {"steps": 1, "ms_per_step": None, "gpu_launches": None,
                  "metric": "serving: determinants/s at 70% of offline load, with p50/p99 latency",
                  "data": "synthetic (seeded Poisson walker stream)"}
    else:
        r = run_batched(args, world, rank, local, args.workload, full=True)
        if args.workload == "lll24" and not args.no_subconfigs:
            # compact results of the other configurations, in the same line
            subs = {
                "config1_gauss8": run_batched(args, world, rank, local, "gauss8", full=False),
                "config2_gauss16": run_batched(args, world, rank, local, "gauss16", full=False),
                "config4_mixedn": run_plan(args, world, rank, local, full=False),
                "config5_serving": run_serve(args, world, rank, local, full=False),
            }
            if r is not None:
                r["configs"] = subs
    if rank == 0 and r is not None:
        line = base_line(args, world) | r
        print(json.dumps(line), flush=True)


def workload_config(workload: str, world: int) -> dict:
    """The `config` object of the JSON line, identical in both arms."""
    kind, n, batch, seed = WORKLOADS[workload]
    if kind in ("lll", "gauss"):
        what = "LLL orbital" if kind == "lll" else "complex Gaussian"
        return {"workload": f"{workload}: {batch} x n={n} {what} complex128, seed {seed}",
                "batch": batch, "n": n, "l2": "inputs larger than L2 (no flush)",
                "parallelism": f"replicas x{world}"}
    if kind == "mixed":
        return {"workload": f"mixedn: {batch} LLL matrices, n uniform over {list(MIXED_SIZES)}, "
                            "one persistent launch in a CUDA graph",
                "batch": batch, "l2": "inputs larger than L2 (no flush)",
                "parallelism": f"replicas x{world}"}
    return {"workload": "serving: Poisson move requests, k log-uniform 1..4096, n in "
                        f"{SERVE_SIZES}, 100 moves per walker, walkers resident in HBM",
            "parallelism": f"replicas x{world}"}


def run_reference(args):
    """The reference's CPU Crout path (FP64 restatement, OpenMP over host cores).
    Inputs come from the oracle's own generators (the same seeded draws as the
    library's), so this arm loads nothing of the product."""
    import numpy as np

    import lufqhe_oracle

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import bench_cpu

    def make_inputs(kind, n, count, seed):
        if kind == "lll":
            return lufqhe_oracle.gen_lll(count, n, seed=seed)[0]
        return lufqhe_oracle.gen_gaussian(count, n, seed=seed)

    kind, n, batch, seed = WORKLOADS[args.workload]
    if kind in ("mixed", "serve"):  # the reference factorises one size at a time; n=24
        kind, n, batch = "lll", 24, 32768
    line = bench_cpu.reference_arm(np, args, kind, n, batch, seed, make_inputs,
                                   workload_config(args.workload, world))
    line["n_gpus"] = world
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="lll24", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    # the reference arm factorises the whole batch every step (about 15 ms on
    # 16 cores at n = 24): short steps let OpenMP start-up and box noise skew it
    ap.add_argument("--ref-sample", type=int, default=32768)
    ap.add_argument("--serve-requests", type=int, default=6000)
    ap.add_argument("--serve-walkers", type=int, default=128,
                    help="live walkers of the closed loop that measures a server's capacity")
    ap.add_argument("--no-subconfigs", action="store_true",
                    help="default workload only: leave out the compact config 1/2/4/5 results")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    sys.path.insert(0, str(ROOT / "oracle"))
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
