"""Benchmark: relaxed pixel·z points/s of the MechAFM scan hot path on GB300.

Default workload (the headline): the 60-atom C/N/O/H planar cluster (LJ for
C/N/H, Morse for the tip-O pair, Coulomb on), 20x20 A at 0.05 A (401x401
pixels) x 41 z-levels (10 -> 6 A, dz 0.1) = 6,592,841 relaxed points per
step, FIRE + midpoint, etol = ftol = 0.01, maxsteps 5000.  Seeded synthetic
input written in the reference's own file formats (mechafm_gb300.synth).

Other workloads (--workload): graphene_72 (101x101x41, LJ), molecule_batch
(256 scans, 20-400 atoms, 64^2..256^2 pixels, one persistent launch),
slab_2048 (512x512x41 over the rigid grid + FFT external field).

One step = one relaxation of every point by the FP32-compensated persistent
kernel, launched from a prepared plan (mafm_plan_launch) captured in a CUDA
graph; launch shape (lanes per column, block, tile) from mafm_autotune.
`value` = points/s with inputs resident and outputs in HBM; `e2e` = the same
through the C ABI from host memory (scan creation with the upload, relax, D2H
of every point).  The plain FP64 kernel runs on a subset for the FP32/FP64
speed-up and the FP32C error against it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--workload NAME]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
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
L2_FLUSH_BYTES = 512 << 20
# Algorithmic flops per tip–atom term (counted from interactions.cpp:15-51):
# LJ 25, Morse 29, Coulomb 20.
FLOPS_LJ, FLOPS_MORSE, FLOPS_COUL = 25, 29, 20

WORKLOADS = {
    "cluster_60": "60-atom C/N/O/H cluster, LJ+Morse+Coulomb, 401x401 px x 41 z",
    "graphene_72": "72-C graphene, LJ, 101x101 px x 41 z",
    "molecule_batch": "256 planar molecules (20-400 atoms, LJ+Coulomb), 64^2/128^2/256^2 px x 41 z",
    "slab_2048": "2048-atom periodic slab, rigid grid + FFT external field, 512x512 px x 41 z",
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cluster_60", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-columns", type=int, default=0,
                    help="columns of the bounded CPU sample (0 = 1200)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="default launch shape, no autotuner")
    ap.add_argument("--lanes", type=int, default=0, help="force lanes per column")
    ap.add_argument("--pixels", type=int, default=0, help="pixels per side (profiling)")
    ap.add_argument("--sweep", action="store_true",
                    help="also time every lanes-per-column value (stderr)")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def make_inputs(name, tmp, pixels=0):
    """Input files of a workload; returns (list of Input, description)."""
    from mechafm_gb300 import synth
    from mechafm_gb300.scan import Input
    if name == "cluster_60":
        px = pixels or 401
        specs = [synth.cluster_60(area=0.05 * (px - 1))]
    elif name == "graphene_72":
        px = pixels or 101
        specs = [synth.graphene_72(area=0.1 * (px - 1))]
    elif name == "slab_2048":
        specs = [synth.slab(pixels=pixels or 512)]
    else:
        specs = synth.molecule_batch()
    inputs = [Input(s.write(os.path.join(tmp, f"s{i:03d}"))) for i, s in enumerate(specs)]
    return inputs, WORKLOADS[name]


def term_flops(desc):
    """Algorithmic flops of one force evaluation over a scan's tip–atom terms."""
    from mechafm_gb300 import _abi
    if desc.c.rigidgrid:
        return 0
    a = desc.atoms()
    kinds = np.array([desc.c.tip_pair[int(t)].kind for t in a["type"]])
    images = 9 if desc.c.vdw_pbc else 1
    n_lj = int((kinds == _abi.PAIR_LJ).sum()) * images
    n_mo = int((kinds == _abi.PAIR_MORSE).sum()) * images
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


def cpu_rate(descs, columns: int, threads: int):
    """Points/s of the oracle port (FP64, OpenMP) on `columns` contiguous columns
    from the centre of each of up to 4 scans."""
    import oracle
    pts = 0
    t0 = time.perf_counter()
    for d in descs[:4]:
        n = min(columns, d.n_columns)
        c0 = max(0, d.n_columns // 2 - n // 2)
        out, _ = oracle.run(d, c0, c0 + n, threads=threads)
        pts += len(out)
    t = time.perf_counter() - t0
    return pts / t, t


def reference_arm(args, rank):
    """--impl reference: the reference's CPU path (the oracle port of its FP64
    OpenMP code; the reference's own build needs its sources, absent on the GPU
    host), on all host threads, over a bounded sample of the same workload."""
    if rank != 0:
        return
    tmp = tempfile.mkdtemp()
    inputs, desc_text = make_inputs(args.workload, tmp, args.pixels)
    descs = [i.desc() for i in inputs]
    threads = cpu_threads()
    cols = args.cpu_columns or 1200
    for _ in range(args.warmup):
        cpu_rate(descs, max(cols // 16, 8), threads)
    rates = [cpu_rate(descs, cols, threads)[0] for _ in range(args.steps)]
    value = float(np.mean(rates))
    n_pts = sum(d.n_points for d in descs)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * n_pts / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc_text, "precision": "FP64 CPU (oracle port, OpenMP)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{cols} contiguous columns x all z from the centre of "
                                   f"up to 4 scans per step; points/s of the sample"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def fp64_compare(scans, descs, value, dev):
    """Plain FP64 kernel on a subset: points/s, and the FP32C error against it."""
    import torch
    from mechafm_gb300 import _abi
    props = torch.cuda.get_device_properties(dev)
    if len(scans) == 1:
        d = descs[0]
        cols = min(d.n_columns, props.multi_processor_count * 256)
        c0 = d.n_columns // 2 - cols // 2
        jobs = [(scans[0], c0, c0 + cols)]
    else:
        jobs = [(s, 0, 0) for s in scans[:3]]
    p64s, p32s, ms64, npts = [], [], 0.0, 0
    for s, a, b in jobs:
        p64, s64 = s.run(_abi.FP64, col_begin=a, col_end=b)
        p32, _ = s.run(_abi.FP32C, col_begin=a, col_end=b)
        p64s.append(p64)
        p32s.append(p32)
        ms64 += s64.kernel_ms
        npts += len(p64)
    p64 = np.concatenate(p64s)
    p32 = np.concatenate(p32s)
    tip_err = np.abs(p32["tip"] - p64["tip"]).max(axis=1)
    fz = np.abs(p32["force"][:, 2] - p64["force"][:, 2]) / np.maximum(np.abs(p64["force"][:, 2]), 0.01)
    rate64 = npts / (ms64 / 1000.0)
    return {
        "points_per_s": rate64, "points": npts, "kernel_ms": ms64,
        "fp32c_speedup": value / rate64,
        "tip_err_A": {"max": float(tip_err.max()), "p99_9": float(np.percentile(tip_err, 99.9)),
                      "median": float(np.median(tip_err)),
                      "frac_le_1e-3": float((tip_err <= 1e-3).mean())},
        "fz_rel_err": {"max": float(fz.max()), "p99_9": float(np.percentile(fz, 99.9)),
                       "frac_le_1e-3": float((fz <= 1e-3).mean())},
        "step_count_match": float((p32["steps"] == p64["steps"]).mean()),
    }


def fp32_peak(dev):
    """FP32 CUDA-core throughput: best of 5 FP32 GEMMs with TF32 disabled."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
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
    torch.backends.cuda.matmul.allow_tf32 = prev
    return 2 * 8192 ** 3 / (best / 1000.0) / 1e12


def ours(args, rank, world, local):
    import torch
    from mechafm_gb300 import _abi
    from mechafm_gb300.scan import Scan

    L = _abi.lib()
    dev = local
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    tmp = tempfile.mkdtemp()
    inputs, desc_text = make_inputs(args.workload, tmp, args.pixels)
    descs = [i.desc() for i in inputs]
    t_create = time.perf_counter()
    scans = [Scan(d, device=dev) for d in descs]
    torch.cuda.synchronize()
    t_create = time.perf_counter() - t_create
    n_pts = sum(d.n_points for d in descs)
    outs = [torch.empty(d.n_points * 64, dtype=torch.uint8, device=f"cuda:{dev}") for d in descs]
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{dev}")
    stream = torch.cuda.Stream(device=dev)
    sptr = C.c_void_p(stream.cuda_stream)
    n = len(scans)
    handles = (C.c_void_p * n)(*[s.handle for s in scans])
    optrs = (C.c_void_p * n)(*[o.data_ptr() for o in outs])

    # FP32 rigid grids are built on first use: build them outside the timing.
    t_grid = 0.0
    if any(d.c.rigidgrid for d in descs):
        t0 = time.perf_counter()
        for s in scans:
            if s.desc.c.rigidgrid:
                s.sample(np.array([[0.0, 0.0, 10.0]]), precision=_abi.FP32C)
        torch.cuda.synchronize()
        t_grid = time.perf_counter() - t0

    # launch shape: the autotuner (on at most 32 scans of a batch)
    opts = _abi.RunOpts(_abi.FP32C, args.lanes, 0, 0, 0, 0)
    tune_ms = None
    if not args.no_tune and not args.lanes:
        best = _abi.RunOpts()
        tms = C.c_double()
        _abi.check(L.mafm_autotune(handles, min(n, 32), C.byref(best), C.byref(tms), sptr))
        opts, tune_ms = best, tms.value
    plan = C.c_void_p()
    _abi.check(L.mafm_plan_create(handles, n, C.byref(opts), optrs, C.byref(plan)))
    used = _abi.RunOpts()
    _abi.check(L.mafm_plan_config(plan, C.byref(used)))

    for _ in range(args.warmup):
        _abi.check(L.mafm_plan_launch(plan, sptr))
    st = _abi.RunStats()
    _abi.check(L.mafm_plan_stats(plan, C.byref(st), sptr))
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        _abi.check(L.mafm_plan_launch(plan, sptr))
    torch.cuda.synchronize()

    times = []
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                graph.replay()
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
    _abi.check(L.mafm_plan_stats(plan, C.byref(st), sptr))   # the last replay ended cleanly

    if args.sweep and rank == 0:
        for lanes in (1, 2, 4, 8, 16, 32):
            o = _abi.RunOpts(_abi.FP32C, lanes, 0, 0, 0, 0)
            p2 = C.c_void_p()
            _abi.check(L.mafm_plan_create(handles, n, C.byref(o), optrs, C.byref(p2)))
            _abi.check(L.mafm_plan_launch(p2, sptr))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _abi.check(L.mafm_plan_launch(p2, sptr))
            e1.record(stream)
            torch.cuda.synchronize()
            L.mafm_plan_destroy(p2)
            t = e0.elapsed_time(e1)
            print(json.dumps({"sweep_lanes": lanes, "ms": t, "points_per_s": n_pts / t * 1e3}),
                  file=sys.stderr)

    # e2e through the C ABI from host memory: scan creation (H2D), relax, D2H.
    host = [np.zeros(d.n_points, dtype=_abi.POINT_DTYPE) for d in descs]
    h2d = 0
    for d in descs:
        h2d += d.c.n_atoms * (3 * 8 + 8 + 4) + d.c.n_types * 32
        if d.c.use_external_potential:
            h2d += 8 * d.c.epot_n[0] * d.c.epot_n[1] * d.c.epot_n[2]
    e2e_opts = _abi.RunOpts(_abi.FP32C, used.lanes_per_column, used.block_threads,
                            used.columns_per_tile, 0, 0)
    e2e_times = []
    reps = 2 if n == 1 else 1
    for i in range(reps + 1):   # the first pass warms up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s2 = [Scan(d, device=dev) for d in descs]
        hh = (C.c_void_p * n)(*[s.handle for s in s2])
        ho = (C.c_void_p * n)(*[h.ctypes.data for h in host])
        est = _abi.RunStats()
        _abi.check(L.mafm_run_batch(hh, n, C.byref(e2e_opts), ho, C.byref(est), None))
        for s in s2:
            s.close()
        if i > 0:
            e2e_times.append(time.perf_counter() - t0)
    e2e_value = world * n_pts / float(np.mean(e2e_times))

    if rank == 0:
        fp64 = None if args.no_fp64 else fp64_compare(scans, descs, value / world, dev)
        peak_tflops = fp32_peak(dev)
        fl = float(np.mean([term_flops(d) for d in descs]))
        achieved = st.force_evals * fl / (ms / 1000.0) / 1e12
        threads = cpu_threads()
        cpu_cols = args.cpu_columns or 1200
        cpu_value, cpu_t = cpu_rate(descs, cpu_cols, threads)
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (compensated sums, double-float positions and energy)",
            "data": "synthetic",
            "config": {"workload": desc_text, "scans": n, "points_per_step": n_pts,
                       "precision": "FP32C",
                       "launch": {"lanes_per_column": used.lanes_per_column,
                                  "block_threads": used.block_threads,
                                  "columns_per_tile": used.columns_per_tile,
                                  "chosen_by": "autotuner" if tune_ms is not None else "default",
                                  "column_order": "expected cost, descending",
                                  "cuda_graph": True},
                       "l2": f"{L2_FLUSH_BYTES >> 20} MiB buffer written between timed steps",
                       "fire_steps_per_step": int(st.total_steps),
                       "pair_terms_per_step": int(st.pair_evals),
                       "scan_create_s": t_create, "rigid_grid_build_s": t_grid,
                       "parallelism": f"replica per GPU x{world}"},
            "pair_terms_per_s": st.pair_evals * world / (ms / 1000.0),
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_tflops,
                         "unit": "TFLOP/s", "frac": achieved / peak_tflops, "traffic": None,
                         "peak_source": "FP32 CUDA-core SGEMM (cuBLAS, 8192^3) measured in this "
                                        "run; MEASURED_PEAKS.json has no FP32 figure",
                         "flops_per_force_eval": fl, "force_evals": int(st.force_evals)},
            "fp64_gpu": fp64,
            "cpu_baseline": {"value": cpu_value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{cpu_cols} contiguous columns x all z from the centre of "
                                       f"up to 4 scans, {cpu_t:.1f} s"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(n_pts * 64)},
            "gpu_launches": args.steps,
            "clocks": clk.summary(),
        }))
    L.mafm_plan_destroy(plan)
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
