"""Benchmark: relaxed pixel·z points/s of the MechAFM scan hot path on GB300.

Workload: the 60-atom C/N/O/H planar cluster (LJ for C/N/H, Morse for the
tip-O pair, Coulomb on), 20x20 A at 0.05 A (401x401 pixels) x 41 z-levels
(10 -> 6 A, dz 0.1) = 6,592,841 relaxed points per step, FIRE + midpoint,
etol = ftol = 0.01, maxsteps 5000.  Seeded synthetic input written in the
reference's own file formats (mechafm_gb300.synth.cluster_60).

One step = one relaxation of the whole scan by the FP32-compensated
persistent kernel (mafm_run, MAFM_FP32C), output in HBM.  `value` is points/s
with inputs resident; `e2e` is the same through the C ABI from host memory
(scan creation with the H2D upload + relaxation + D2H of every point).
The plain FP64 GPU kernel runs on a column subset for the FP32/FP64 speed-up
and for the tip/Fz error of FP32C against it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "relaxed pixel·z points/s, FP32 batched vs FP64 GPU at ≤1e-3 Å tip error"
UNIT = "points/s"
WORKLOAD = "cluster_60: 60-atom C/N/O/H cluster, LJ+Morse+Coulomb, 401x401 px x 41 z"
L2_FLUSH_BYTES = 512 << 20
# Algorithmic flops per tip–atom term (counted from interactions.cpp:15-51):
# LJ 25, Morse 29, Coulomb 20.
FLOPS_LJ, FLOPS_MORSE, FLOPS_COUL = 25, 29, 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-columns", type=int, default=0,
                    help="columns of the bounded CPU sample (0 = sized to ~15 s)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--lanes", type=int, default=0, help="lanes per column (0 = default)")
    ap.add_argument("--sweep", action="store_true",
                    help="also time every lanes-per-column value and print one line each")
    ap.add_argument("--pixels", type=int, default=401,
                    help="pixels per side (401 = the benchmark workload; smaller for profiling)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_workload(tmp, pixels=401):
    from mechafm_gb300 import synth
    from mechafm_gb300.scan import Input
    inp = synth.cluster_60(area=0.05 * (pixels - 1)).write(tmp)
    I = Input(inp)
    return I, I.desc()


def term_flops(desc):
    """Algorithmic flops of one force evaluation over all tip–atom terms."""
    from mechafm_gb300 import _abi
    a = desc.atoms()
    kinds = np.array([desc.c.tip_pair[int(t)].kind for t in a["type"]])
    n_lj = int((kinds == _abi.PAIR_LJ).sum())
    n_mo = int((kinds == _abi.PAIR_MORSE).sum())
    n_co = int(((a["charge"] != 0) & bool(desc.c.coulomb) & (desc.c.tip_charge != 0)).sum())
    return n_lj * FLOPS_LJ + n_mo * FLOPS_MORSE + n_co * FLOPS_COUL


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_rate(desc, columns: int, threads: int):
    """Points/s of the oracle port over `columns` contiguous columns from the scan centre."""
    import oracle
    n_cols = desc.n_columns
    c0 = max(0, n_cols // 2 - columns // 2)
    t0 = time.perf_counter()
    out, _ = oracle.run(desc, c0, c0 + columns, threads=threads)
    t = time.perf_counter() - t0
    return len(out) / t, t, (c0, c0 + columns)


def reference_arm(args, rank):
    """--impl reference: the reference's CPU path (oracle port of its FP64 OpenMP code)."""
    if rank != 0:
        return
    tmp = tempfile.mkdtemp()
    I, desc = make_workload(tmp)
    threads = cpu_threads()
    cols = args.cpu_columns or 1200
    rates = []
    for _ in range(args.warmup):
        cpu_rate(desc, max(cols // 8, 16), threads)
    for _ in range(args.steps):
        r, t, rng = cpu_rate(desc, cols, threads)
        rates.append(r)
    value = float(np.mean(rates))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * 6592841 / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "precision": "FP64 CPU (oracle port, OpenMP)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{cols} contiguous columns x 41 z of the workload per step, "
                                   "points/s extrapolated to the full scan"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def ours(args, rank, world, local):
    import torch
    from mechafm_gb300 import _abi
    from mechafm_gb300.scan import Scan, Input

    dev = local
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    tmp = tempfile.mkdtemp()
    I, desc = make_workload(tmp, args.pixels)
    n_pts = desc.n_points
    scan = Scan(desc, device=dev)
    out = torch.empty(n_pts * 64, dtype=torch.uint8, device=f"cuda:{dev}")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{dev}")
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def one_step():
        return scan.run_device(out.data_ptr(), precision=_abi.FP32C, stream=sptr,
                               lanes=args.lanes)

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    st = scan.run_device(out.data_ptr(), precision=_abi.FP32C, stream=sptr, stats=True,
                         lanes=args.lanes)
    steps_per_scan = int(st.total_steps)
    evals_per_scan = int(st.force_evals)
    pairs_per_scan = int(st.pair_evals)

    times = []
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            one_step()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
    if world > 1:
        torch.distributed.barrier()
    ms = float(np.mean(times))
    if world > 1:
        t = torch.tensor([ms], device=f"cuda:{dev}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * n_pts / (ms / 1000.0)

    # e2e through the C ABI from host memory: scan creation (H2D) + run + D2H.
    host_out = np.zeros(n_pts, dtype=_abi.POINT_DTYPE)
    e2e_times = []
    h2d = desc.c.n_atoms * (3 * 8 + 8 + 4) + desc.c.n_types * 32
    for i in range(max(2, min(args.steps, 3)) + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s2 = Scan(desc, device=dev)
        s2.run(_abi.FP32C, out=host_out)
        s2.close()
        t1 = time.perf_counter()
        if i > 0:
            e2e_times.append(t1 - t0)
    e2e_value = world * n_pts / float(np.mean(e2e_times))

    if args.sweep and rank == 0:
        for lanes in (1, 2, 4, 8, 16, 32):
            best = 1e30
            for _ in range(2):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                scan.run_device(out.data_ptr(), precision=_abi.FP32C, stream=sptr, lanes=lanes)
                e1.record(stream)
                torch.cuda.synchronize()
                best = min(best, e0.elapsed_time(e1))
            print(json.dumps({"sweep_lanes": lanes, "ms": best, "points_per_s": n_pts / best * 1e3}),
                  file=sys.stderr)

    line = None
    if rank == 0:
        # FP64 plain kernel on a column subset: speed and the FP32C error against it.
        fp64 = None
        if not args.no_fp64:
            # enough columns for two FP64 blocks of 128 threads on every SM
            props = torch.cuda.get_device_properties(dev)
            cols = min(desc.n_columns, props.multi_processor_count * 256)
            c0 = desc.n_columns // 2 - cols // 2
            p64, s64 = scan.run(_abi.FP64, col_begin=c0, col_end=c0 + cols)
            p32, s32 = scan.run(_abi.FP32C, col_begin=c0, col_end=c0 + cols)
            tip_err = np.abs(p32["tip"] - p64["tip"]).max(axis=1)
            fz = np.abs(p32["force"][:, 2] - p64["force"][:, 2]) / np.maximum(
                np.abs(p64["force"][:, 2]), 0.01)
            rate64 = len(p64) / (s64.kernel_ms / 1000.0)
            fp64 = {
                "points_per_s": rate64, "columns": cols, "kernel_ms": s64.kernel_ms,
                "fp32c_speedup": value / world / rate64,
                "tip_err_A": {"max": float(tip_err.max()), "p99_9": float(np.percentile(tip_err, 99.9)),
                              "median": float(np.median(tip_err)),
                              "frac_le_1e-3": float((tip_err <= 1e-3).mean())},
                "fz_rel_err": {"max": float(fz.max()), "p99_9": float(np.percentile(fz, 99.9)),
                               "frac_le_1e-3": float((fz <= 1e-3).mean())},
                "step_count_match": float((p32["steps"] == p64["steps"]).mean()),
            }
        # roofline: FP32-pipe bound; peak = cuBLAS FP32 (non-tensor) GEMM, measured here
        torch.backends.cuda.matmul.allow_tf32 = False
        a = torch.randn(8192, 8192, device=f"cuda:{dev}")
        b = torch.randn(8192, 8192, device=f"cuda:{dev}")
        for _ in range(2):
            a @ b
        torch.cuda.synchronize()
        best = 1e9
        for _ in range(5):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            a @ b
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        peak_tflops = 2 * 8192 ** 3 / (best / 1000.0) / 1e12
        fl_eval = term_flops(desc)
        alg_flops = evals_per_scan * fl_eval
        achieved = alg_flops / (ms / 1000.0) / 1e12
        threads = cpu_threads()
        cpu_cols = args.cpu_columns or 1200
        cpu_value, cpu_t, _ = cpu_rate(desc, cpu_cols, threads)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (compensated; FP64 energy check and spring)", "data": "synthetic",
            "config": {"workload": WORKLOAD, "points_per_step": n_pts, "precision": "FP32C",
                       "l2": f"{L2_FLUSH_BYTES >> 20} MiB buffer written between timed steps",
                       "fire_steps_per_scan": steps_per_scan,
                       "pair_terms_per_scan": pairs_per_scan,
                       "parallelism": f"replica per GPU x{world}"},
            "pair_terms_per_s": pairs_per_scan * world / (ms / 1000.0),
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_tflops,
                         "unit": "TFLOP/s", "frac": achieved / peak_tflops, "traffic": None,
                         "peak_source": "cuBLAS FP32 SGEMM 8192^3 measured in this run "
                                        "(no FP32 figure in MEASURED_PEAKS.json)",
                         "flops_per_eval": fl_eval, "force_evals": evals_per_scan},
            "fp64_gpu": fp64,
            "cpu_baseline": {"value": cpu_value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{cpu_cols} contiguous columns x 41 z from the scan "
                                       f"centre, {cpu_t:.1f} s"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(n_pts * 64)},
            "gpu_launches": 2 * args.steps,
            "clocks": clk.summary(),
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        reference_arm(args, rank)
        return
    ours(args, rank, world, local)


if __name__ == "__main__":
    main()
