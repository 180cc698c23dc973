"""Benchmark: relaxed pixel·z points/s of the MechAFM scan hot path on GB300.

Default workload (the headline): the 60-atom C/N/O/H planar cluster (LJ for
C/N/H, Morse for the tip-O pair, Coulomb on), 20x20 A at 0.05 A (401x401
pixels) x 41 z-levels (10 -> 6 A, dz 0.1) = 6,592,841 relaxed points per
step, FIRE + midpoint, etol = ftol = 0.01, maxsteps 5000.  Seeded synthetic
input written in the reference's own file formats (mechafm_gb300.synth).

Other workloads (--workload): graphene_72 (101x101x41, LJ), molecule_batch
(256 scans, 20-400 atoms, 64^2..256^2 pixels, one persistent launch),
slab_2048 (512x512x41 over the rigid grid + FFT external field; a step
rebuilds the rigid grid and relaxes, as the reference does per scan) and
adjoint_128 (the cluster at 128x128x41: forward relax + the implicit-
differentiation adjoint of an MSE loss on the Fz image).

One step = one relaxation of every point by the FP32-compensated persistent
kernel, launched from a prepared plan (mafm_plan_launch) captured in a CUDA
graph; launch shape (lanes per column, block, tile) from mafm_autotune.
`value` = points/s with inputs resident and outputs in HBM; `e2e` = the same
through the C ABI from host memory (scan creation with the upload, relax, and
every point record delivered into pinned host memory).  The plain FP64 kernel runs on a subset for the FP32/FP64
speed-up and the FP32C error against it.  The CPU baseline is the oracle port
(FP64, OpenMP on every host thread) on a sample of about ten seconds: centre
column blocks of every scan, or for rigid-grid scans a centre crop whose
set-up, grid build and relaxation are timed apart and scaled to the full scan.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--workload NAME]
  profiling knobs: --pixels P (a smaller scan), --lanes/--block/--tile
  (a forced launch shape instead of the autotuner), --no-tune (the default
  shape), --sweep (times lanes x block x tile shapes, to stderr),
  --no-fp64 and --cpu-seconds 0 (skip the comparison legs).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "relaxed pixel·z points/s, FP32 batched vs FP64 GPU at ≤1e-3 Å tip error"
UNIT = "points/s"
L2_FLUSH_BYTES = 512 << 20
# Algorithmic flops per tip–atom term (counted from interactions.cpp:15-51):
# LJ 25, Morse 29, Coulomb 20.
FLOPS_LJ, FLOPS_MORSE, FLOPS_COUL = 25, 29, 20
# Algorithmic bytes of one trilinear lookup: 8 FP32 {F, E} nodes.
BYTES_LOOKUP = 8 * 16
# DRAM bytes per trilinear lookup of the rigid-grid relax: ncu dram__bytes
# (20.13 GB/s x 17.454 ms = 351.3 MB) over the 190,890,530 lookups of one
# 200 x 200 px slab launch: the grid nodes read once and the output records
# written (gathers within a column are served by L1 and L2).
DRAM_BYTES_PER_LOOKUP = 351.3e6 / 190890530
# DRAM bytes (read + write) per relaxed point of relax32_kernel, from one ncu
# capture of the cluster at 285 x 285 px x 41 z (171.9 MB for 3,330,225
# points); the traffic is the 64 B output record per point, so it scales with
# the points.
DRAM_BYTES_PER_POINT = 171.9e6 / 3330225
CPU_TARGET_S = 10.0        # CPU sample length
RIGID_CROP = 16            # pixels per side of the rigid-grid CPU sample
FP64_RIGID_CROP = 64       # pixels per side of the rigid-grid FP64 comparison
ADJ_CROP = 64              # pixels per side of the adjoint CPU sample

WORKLOADS = {
    "cluster_60": "60-atom C/N/O/H cluster, LJ+Morse+Coulomb, 401x401 px x 41 z",
    "graphene_72": "72-C graphene, LJ, 101x101 px x 41 z",
    "molecule_batch": "256 planar molecules (20-400 atoms, LJ+Coulomb), 64^2/128^2/256^2 px x 41 z",
    "slab_2048": "2048-atom periodic slab, rigid grid + FFT external field, 512x512 px x 41 z "
                 "(dummy 18 -> 14 A, top layer at 6 A, tip charge -0.02 e)",
    "adjoint_128": "60-atom C/N/O/H cluster at 128x128 px x 41 z, forward + adjoint of an "
                   "MSE loss on the Fz image",
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cluster_60", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=CPU_TARGET_S,
                    help="length of the CPU sample (0 = skip the CPU baseline)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="default launch shape, no autotuner")
    ap.add_argument("--lanes", type=int, default=0, help="force lanes per column")
    ap.add_argument("--tile", type=int, default=0, help="force columns per tile")
    ap.add_argument("--block", type=int, default=0, help="force threads per block")
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
    elif name == "adjoint_128":
        px = pixels or 128
        specs = [synth.cluster_60(area=20.0, step=20.0 / (px - 1))]
    elif name == "graphene_72":
        px = pixels or 101
        specs = [synth.graphene_72(area=0.1 * (px - 1))]
    elif name == "slab_2048":
        # tip 4-8 A above the top layer, tip charge -0.02 e: the lateral
        # deflection stays inside the rigid grid's 1.5 A margin (the synthetic
        # Hartree field of random charges is strong; at -0.1 e or 2 A closer
        # the tip leaves the grid and the reference stops)
        specs = [synth.slab(pixels=pixels or 512, zhigh=18.0, zlow=14.0, tip_charge=-0.02)]
    else:
        specs = synth.molecule_batch()
    inputs = [Input(s.write(os.path.join(tmp, f"s{i:03d}"))) for i, s in enumerate(specs)]
    return inputs, WORKLOADS[name]


def term_flops(desc, direct: bool = False):
    """Algorithmic flops of one force evaluation over a scan's tip–atom terms
    (direct=True: the terms a rigid-grid node samples)."""
    from mechafm_gb300 import _abi
    if desc.c.rigidgrid and not direct:
        return 0
    a = desc.atoms()
    kinds = np.array([desc.c.tip_pair[int(t)].kind for t in a["type"]])
    images = 9 if desc.c.vdw_pbc else 1
    n_lj = int((kinds == _abi.PAIR_LJ).sum()) * images
    n_mo = int((kinds == _abi.PAIR_MORSE).sum()) * images
    n_co = int(((a["charge"] != 0) & bool(desc.c.coulomb) & (desc.c.tip_charge != 0)).sum())
    return n_lj * FLOPS_LJ + n_mo * FLOPS_MORSE + n_co * FLOPS_COUL


def rigid_nodes(d) -> int:
    """Nodes of a scan's rigid grid (buildTipGridInteractions, simulation.cpp:426-436)."""
    sp = (d.dx / 2, d.dy / 2, d.dz / 2)
    border = [math.ceil(1.5 / s) for s in sp]
    n0 = math.floor(d.area[0] / sp[0]) + 2 * border[0] + 1
    n1 = math.floor(d.area[1] / sp[1]) + 2 * border[1] + 1
    n2 = math.floor((d.zhigh - d.zlow) / sp[2]) + 2 * border[2] + 1
    return n0 * n1 * n2


def centre_crop(desc, n: int):
    d = desc.c
    ni, nj = min(n, d.nx), min(n, d.ny)
    return desc.crop((d.nx - ni) // 2, (d.ny - nj) // 2, ni, nj)


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


# ------------------------------------------------------------ CPU baseline ----

def _cpu_columns(descs, frac, threads):
    """Relax the same centre fraction of every scan with the oracle port."""
    import oracle
    jobs = []
    for d in descs:
        n = max(1, min(d.n_columns, int(round(frac * d.n_columns))))
        c0 = max(0, d.n_columns // 2 - n // 2)
        jobs.append((d, c0, c0 + n))
    t0 = time.perf_counter()
    if len(jobs) == 1:
        d, a, b = jobs[0]
        pts = len(oracle.run(d, a, b, threads=threads)[0])
    else:
        # many scans: one scan per host thread (the port releases the GIL)
        with ThreadPoolExecutor(threads) as ex:
            pts = sum(ex.map(lambda j: len(oracle.run(j[0], j[1], j[2], threads=1)[0]), jobs))
    return pts, time.perf_counter() - t0, sum(b - a for _, a, b in jobs)


def cpu_direct(descs, threads, target_s):
    """Points/s of the oracle over centre column blocks of every scan, sized to
    about target_s seconds after a short pilot."""
    total = sum(d.n_columns for d in descs)
    frac = min(1.0, 400.0 / total)
    pts, t, cols = _cpu_columns(descs, frac, threads)
    if t < target_s and frac < 1.0:
        frac = min(1.0, frac * target_s / max(t, 1e-3))
        pts, t, cols = _cpu_columns(descs, frac, threads)
    return pts / t, (f"{cols} centre columns x all z ({100 * frac:.2f}% of every scan), "
                     f"{t:.1f} s")


def cpu_rigid(descs, threads, crop_n):
    """Points/s of the oracle on rigid-grid scans, from a centre crop: the
    set-up (external field), the grid build and the relaxation are timed apart
    and scaled to the full scan by grid nodes and by points."""
    import oracle
    from mechafm_gb300 import _abi
    from mechafm_gb300.scan import Desc
    est, pts, wall = 0.0, 0, 0.0
    for desc in descs:
        crop = centre_crop(desc, crop_n)
        es = _abi.ScanDesc()
        C.pointer(es)[0] = crop.c
        es.rigidgrid = 0
        _, _, t_es, _ = oracle.run_split(Desc(es, keep=crop), 0, 0, threads)
        out, _, t_setup, t_relax = oracle.run_split(crop, threads=threads)
        t_grid = max(t_setup - t_es, 0.0)
        est += (t_es + t_grid * rigid_nodes(desc.c) / rigid_nodes(crop.c)
                + t_relax * desc.n_points / len(out))
        pts += desc.n_points
        wall += t_es + t_setup + t_relax
    return pts / est, (f"{crop_n}x{crop_n} centre crop of every scan ({wall:.1f} s): external "
                       f"field, grid build (scaled by grid nodes) and relaxation (scaled by "
                       f"points) timed apart")


def cpu_adjoint(descs, threads, crop_n):
    """Points/s of the oracle's forward relaxation + adjoint on a centre crop."""
    import oracle
    rate, wall = [], 0.0
    for desc in descs:
        crop = centre_crop(desc, crop_n)
        t0 = time.perf_counter()
        pts, _ = oracle.run(crop, threads=threads)
        w = np.random.default_rng(0).normal(size=len(pts))
        oracle.adjoint(crop, pts, w)
        t = time.perf_counter() - t0
        rate.append(len(pts) / t)
        wall += t
    return float(np.mean(rate)), (f"{crop_n}x{crop_n} centre crop, forward FP64 relaxation + "
                                  f"adjoint, {wall:.1f} s")


def cpu_rate(kind, descs, threads, target_s):
    if kind == "adjoint":
        return cpu_adjoint(descs, threads, ADJ_CROP)
    if any(d.c.rigidgrid for d in descs):
        return cpu_rigid(descs, threads, RIGID_CROP)
    return cpu_direct(descs, threads, target_s)


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
    kind = "adjoint" if args.workload == "adjoint_128" else "forward"
    for _ in range(args.warmup):
        cpu_rate(kind, descs, threads, 0.5)
    rates, sample = [], ""
    for _ in range(args.steps):
        r, sample = cpu_rate(kind, descs, threads, args.cpu_seconds or CPU_TARGET_S)
        rates.append(r)
    value = float(np.mean(rates))
    n_pts = sum(d.n_points for d in descs)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * n_pts / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc_text, "precision": "FP64 CPU (oracle port, OpenMP)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample + " per step; points/s of the sample"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ------------------------------------------------------------- GPU helpers ----

def fp64_compare(scans, descs, value, dev):
    """Plain FP64 kernel on a subset: points/s, and the FP32C error against it.
    Rigid-grid scans are compared on a centre crop (both precisions build
    their own grid of the crop; the FP64 time is the relaxation only)."""
    import torch
    from mechafm_gb300 import _abi
    from mechafm_gb300.scan import Scan
    props = torch.cuda.get_device_properties(dev)
    owned = []
    if len(scans) == 1 and descs[0].c.rigidgrid:
        s = Scan(centre_crop(descs[0], FP64_RIGID_CROP), device=dev)
        owned.append(s)
        jobs = [(s, 0, 0)]
        subset = f"{FP64_RIGID_CROP}x{FP64_RIGID_CROP} centre crop"
    elif len(scans) == 1:
        d = descs[0]
        cols = min(d.n_columns, props.multi_processor_count * 256)
        c0 = d.n_columns // 2 - cols // 2
        jobs = [(scans[0], c0, c0 + cols)]
        subset = f"{cols} centre columns"
    else:
        jobs = [(s, 0, 0) for s in scans[:3]]
        subset = "the first 3 scans"
    p64s, p32s, ms64, npts = [], [], 0.0, 0
    ms_build64 = 0.0
    for s, a, b in jobs:
        if s.desc.c.rigidgrid:
            # the FP64 grid build of the crop, timed on its own
            stream = torch.cuda.current_stream(dev)
            sp = C.c_void_p(stream.cuda_stream)
            _abi.check(_abi.lib().mafm_scan_build_grid(s.handle, _abi.FP64, sp))
            ms_build64 = time_events(stream, lambda: _abi.check(
                _abi.lib().mafm_scan_build_grid(s.handle, _abi.FP64, sp)))
        p64, s64 = s.run(_abi.FP64, col_begin=a, col_end=b)
        p32, _ = s.run(_abi.FP32C, col_begin=a, col_end=b)
        p64s.append(p64)
        p32s.append(p32)
        ms64 += s64.kernel_ms
        npts += len(p64)
    crop_nodes = rigid_nodes(owned[0].desc.c) if owned else 0
    for s in owned:
        s.close()
    p64 = np.concatenate(p64s)
    p32 = np.concatenate(p32s)
    tip_err = np.abs(p32["tip"] - p64["tip"]).max(axis=1)
    fz = np.abs(p32["force"][:, 2] - p64["force"][:, 2]) / np.maximum(np.abs(p64["force"][:, 2]), 0.01)
    rate64 = npts / (ms64 / 1000.0)
    extra = {}
    if owned:
        # a rigid-grid step is grid build + relax: scale the crop's FP64 build
        # by grid nodes and its relax by points, as the FP32C step does both
        d = descs[0]
        t64 = (ms_build64 * rigid_nodes(d.c) / crop_nodes + ms64 * d.n_points / npts) / 1000.0
        rate64 = d.n_points / t64
        extra = {"grid_build_ms_crop": ms_build64, "relax_ms_crop": ms64,
                 "scaled_to": "full scan: build by grid nodes, relax by points"}
    return {
        "points_per_s": rate64, "points": npts, "subset": subset, "kernel_ms": ms64, **extra,
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


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (copy, measured)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s"


def time_events(stream, fn, reps=1):
    """Mean ms of fn() on the stream, CUDA events around each call."""
    import torch
    ts = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.mean(ts))


def job_ms(times, world, device):
    """Mean step time of this rank, then the maximum over ranks (every rank
    relaxes its own replica; the job ends with the slowest)."""
    import torch
    ms = float(np.mean(times))
    if world > 1:
        torch.distributed.barrier()
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms


def replica_throughput(points_per_rank, world, ms):
    """Whole-job points/s: every rank relaxes points_per_rank in ms."""
    return world * points_per_rank / (ms / 1000.0)


def fp32_roofline(achieved, peak, extra):
    r = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
         "frac": achieved / peak, "traffic": None,
         "peak_source": "FP32 CUDA-core SGEMM (cuBLAS, 8192^3, TF32 off) measured in this run; "
                        "MEASURED_PEAKS.json has no FP32 figure"}
    r.update(extra)
    return r


# --------------------------------------------------------------- our arm -----

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
    adjoint = args.workload == "adjoint_128"
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
    rigid = [s for s in scans if s.desc.c.rigidgrid]

    # Rigid grids: the first build allocates (outside the timing); a step rebuilds.
    t_grid = 0.0
    if rigid:
        t0 = time.perf_counter()
        for s in rigid:
            _abi.check(L.mafm_scan_build_grid(s.handle, _abi.FP32C, sptr))
        torch.cuda.synchronize()
        t_grid = time.perf_counter() - t0

    # launch shape: the autotuner (its sweep on the first 32 scans of a batch,
    # then the winner against the default shape on all of them)
    opts = _abi.RunOpts(_abi.FP32C, args.lanes, args.block, args.tile, 0, 0)
    tune_ms = None
    if not args.no_tune and not (args.lanes or args.block or args.tile):
        best = _abi.RunOpts()
        tms = C.c_double()
        _abi.check(L.mafm_autotune(handles, n, C.byref(best), C.byref(tms), sptr))
        opts, tune_ms = best, tms.value
    plan = C.c_void_p()
    _abi.check(L.mafm_plan_create(handles, n, C.byref(opts), optrs, C.byref(plan)))
    used = _abi.RunOpts()
    _abi.check(L.mafm_plan_config(plan, C.byref(used)))

    def relax():
        _abi.check(L.mafm_plan_launch(plan, sptr))

    def build():
        for s in rigid:
            _abi.check(L.mafm_scan_build_grid(s.handle, _abi.FP32C, sptr))

    # adjoint workload: the target image comes from a perturbed molecule
    target = grads = None
    if adjoint:
        d0 = descs[0]
        rng = np.random.default_rng(11)
        a = d0.atoms()
        pair = d0.pair_params().copy()
        kinds = d0.pair_kinds()
        ue = rng.uniform(0.9, 1.1, size=len(pair))
        us = rng.uniform(0.9, 1.1, size=len(pair))
        for t in range(len(pair)):
            if kinds[t] == _abi.PAIR_LJ:
                pair[t, 0] *= ue[t] * us[t] ** 6
                pair[t, 1] *= ue[t] * us[t] ** 12
            else:
                pair[t, 0] *= ue[t]
                pair[t, 2] *= us[t]
        dt_ = d0.with_terms(a["pos"] + rng.normal(0, 0.05, size=a["pos"].shape), a["charge"], pair)
        st_ = Scan(dt_, device=dev)
        tp, _ = st_.run(_abi.FP32C)
        st_.close()
        target = torch.from_numpy(tp["force"][:, 2].copy()).to(f"cuda:{dev}")
        fz_view = outs[0].view(torch.float64).view(-1, 8)[:, 5]
        wbuf = torch.empty(n_pts, dtype=torch.float64, device=f"cuda:{dev}")
        dpos = np.zeros((d0.c.n_atoms, 3))
        dq = np.zeros(d0.c.n_atoms)
        dpair = np.zeros((d0.c.n_types, 3))
        grads = _abi.Grad(dpos.ctypes.data_as(C.POINTER(C.c_double)),
                          dq.ctypes.data_as(C.POINTER(C.c_double)),
                          dpair.ctypes.data_as(C.POINTER(C.c_double)))

        def adj():
            with torch.cuda.stream(stream):
                torch.sub(fz_view, target, out=wbuf)
                wbuf.mul_(2.0 / n_pts)
            _abi.check(L.mafm_adjoint_ex(scans[0].handle, _abi.FP32C, C.c_void_p(outs[0].data_ptr()),
                                         C.c_void_p(wbuf.data_ptr()), C.byref(grads), sptr))

    for _ in range(args.warmup):
        build()
        relax()
        if adjoint:
            adj()
    st = _abi.RunStats()
    _abi.check(L.mafm_plan_stats(plan, C.byref(st), sptr))
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        build()
        relax()
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
                if adjoint:
                    adj()
                e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
    ms = job_ms(times, world, f"cuda:{dev}")
    value = replica_throughput(n_pts, world, ms)
    _abi.check(L.mafm_plan_stats(plan, C.byref(st), sptr))   # the last replay ended cleanly

    # the kernels apart, for the rooflines
    ms_relax = time_events(stream, relax, 2)
    ms_build = time_events(stream, build, 2) if rigid else 0.0
    ms_adj = time_events(stream, adj, 2) if adjoint else 0.0

    if args.sweep and rank == 0:
        for lanes in (1, 2, 4, 8):
            for block in (128, 256):
                for tile in sorted({1, 2, 4, 8, 32 // lanes, 128 // lanes}):
                    o = _abi.RunOpts(_abi.FP32C, lanes, block, tile, 0, 0)
                    p2 = C.c_void_p()
                    _abi.check(L.mafm_plan_create(handles, n, C.byref(o), optrs, C.byref(p2)))
                    _abi.check(L.mafm_plan_launch(p2, sptr))
                    t = time_events(stream, lambda: _abi.check(L.mafm_plan_launch(p2, sptr)), 2)
                    L.mafm_plan_destroy(p2)
                    print(json.dumps({"sweep_lanes": lanes, "block": block, "tile": tile, "ms": t,
                                      "points_per_s": n_pts / t * 1e3}), file=sys.stderr)

    # e2e through the public API from host memory
    h2d = 0
    for d in descs:
        h2d += d.c.n_atoms * (3 * 8 + 8 + 4) + d.c.n_types * 32
        if d.c.use_external_potential:
            h2d += 8 * d.c.epot_n[0] * d.c.epot_n[1] * d.c.epot_n[2]
    e2e_times = []
    reps = 2 if n == 1 else 1
    if adjoint:
        # torch.autograd through fz_image: scan creation, FP32C relax, D2H of
        # the points, loss, backward = mafm_adjoint (points and dL/dFz uploaded)
        from mechafm_gb300.torch_ops import fz_image
        d0 = descs[0]
        a = d0.atoms()
        tgt = target.cpu().reshape(d0.shape)
        for i in range(reps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            pos = torch.tensor(a["pos"], requires_grad=True)
            chg = torch.tensor(a["charge"], requires_grad=True)
            pr = torch.tensor(d0.pair_params(), requires_grad=True)
            fz = fz_image(d0, pos, chg, pr, precision=_abi.FP32C, device=dev)
            loss = ((fz - tgt) ** 2).mean()
            loss.backward()
            if i > 0:
                e2e_times.append(time.perf_counter() - t0)
        h2d += n_pts * (64 + 8)
        d2h = n_pts * 64
    else:
        # pinned host buffers for the results (written by the kernel directly)
        pinned = [torch.empty(d.n_points * 64, dtype=torch.uint8, pin_memory=True) for d in descs]
        host = [p.numpy().view(_abi.POINT_DTYPE) for p in pinned]
        e2e_opts = _abi.RunOpts(_abi.FP32C, used.lanes_per_column, used.block_threads,
                                used.columns_per_tile, 0, 0)
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
        d2h = n_pts * 64
    e2e_value = world * n_pts / float(np.mean(e2e_times))

    if rank == 0:
        fp64 = None if args.no_fp64 else fp64_compare(scans, descs, value / world, dev)
        peak_tflops = fp32_peak(dev)
        # flops of the relax kernel: per-scan flops per pair term, weighted by
        # each scan's share of the pair terms (points x terms)
        wts = np.array([d.n_points * max(d.c.n_atoms, 1) for d in descs], dtype=float)
        fpe = np.array([term_flops(d) for d in descs], dtype=float)
        relax_flops = st.force_evals * float((wts * fpe).sum() / wts.sum()) if fpe.any() else 0.0
        relax_line = None
        if fpe.any():
            relax_line = fp32_roofline(relax_flops / (ms_relax / 1000.0) / 1e12, peak_tflops, {
                "traffic": DRAM_BYTES_PER_POINT * n_pts,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                  "285x285x41 cluster launch, scaled by points (the output "
                                  "records are the traffic)",
                "kernel": "relax32_kernel", "kernel_ms": ms_relax,
                "flops_per_force_eval": float((wts * fpe).sum() / wts.sum()),
                "force_evals": int(st.force_evals)})
        else:
            hp, src = hbm_peak()
            gbs = st.force_evals * BYTES_LOOKUP / (ms_relax / 1000.0) / 1e9
            relax_line = {"bound": "gather latency (L1-resident), not HBM", "achieved": gbs,
                          "peak": hp, "unit": "GB/s", "frac": gbs / hp,
                          "traffic": DRAM_BYTES_PER_LOOKUP * st.force_evals, "peak_source": src,
                          "traffic_source": "ncu dram__bytes of one 200x200 px slab launch "
                                            "(190.9 M lookups), scaled by lookups",
                          "kernel": "relax32_kernel (trilinear lookups)", "kernel_ms": ms_relax,
                          "bytes_per_lookup": BYTES_LOOKUP, "lookups": int(st.force_evals),
                          "note": "achieved = algorithmic bytes of the gathers; ncu: L1 hit 91 %, "
                                  "L2 hit 83 % at 3 % L2 throughput, DRAM 20 GB/s, issue 43 %"}
        rooflines = [(ms_relax, relax_line)]
        if rigid:
            nodes = sum(rigid_nodes(s.desc.c) for s in rigid)
            gflops = sum(rigid_nodes(s.desc.c) * term_flops(s.desc, direct=True) for s in rigid)
            rooflines.append((ms_build, fp32_roofline(gflops / (ms_build / 1000.0) / 1e12,
                                                      peak_tflops, {
                "kernel": "grid_build32_kernel", "kernel_ms": ms_build, "nodes": nodes,
                "flops_per_node": float(gflops / nodes)})))
        if adjoint:
            rooflines.append((ms_adj, {"kernel": "adjoint32_kernel (FP32C)", "kernel_ms": ms_adj,
                                       "bound": "fp32", "note": "FP32 per-term Jacobians and "
                                       "parameter derivatives, FP64 3x3 solve per point"}))
        rooflines.sort(key=lambda r: -r[0])
        threads = cpu_threads()
        if args.cpu_seconds > 0:
            cpu_value, cpu_sample = cpu_rate("adjoint" if adjoint else "forward", descs, threads,
                                             args.cpu_seconds)
            cpu = {"value": cpu_value, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": cpu_sample}
        else:
            cpu = None
        launches = args.steps * (1 + len(rigid) + (1 if adjoint else 0))
        step_text = ("rigid grid rebuild + relax" if rigid else
                     "relax + adjoint" if adjoint else "relax")
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (compensated sums, double-float positions and energy)",
            "data": "synthetic",
            "config": {"workload": desc_text, "scans": n, "points_per_step": n_pts,
                       "precision": "FP32C", "step": step_text,
                       "launch": {"lanes_per_column": used.lanes_per_column,
                                  "block_threads": used.block_threads,
                                  "columns_per_tile": used.columns_per_tile,
                                  "chosen_by": ("autotuner" if tune_ms is not None else
                                                "forced" if (args.lanes or args.block or args.tile)
                                                else "default"),
                                  "column_order": ("natural (rigid grid: no pair terms to cost)"
                                                   if rigid else "expected cost, descending"),
                                  "cuda_graph": True},
                       "l2": f"{L2_FLUSH_BYTES >> 20} MiB buffer written between timed steps",
                       "fire_steps_per_step": int(st.total_steps),
                       "pair_terms_per_step": int(st.pair_evals),
                       "scan_create_s": t_create, "first_grid_build_s": t_grid,
                       "parallelism": f"replica per GPU x{world}"},
            "pair_terms_per_s": st.pair_evals * world / (ms / 1000.0),
            "roofline": rooflines[0][1],
            "roofline_other": [r[1] for r in rooflines[1:]],
            "fp64_gpu": fp64,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": launches,
            "clocks": clk.summary(),
        }
        if adjoint:
            line["adjoint"] = {"loss_grad_norms": {"dpos": float(np.linalg.norm(dpos)),
                                                   "dcharge": float(np.linalg.norm(dq)),
                                                   "dpair": float(np.linalg.norm(dpair))},
                               "forward_ms": ms_relax, "adjoint_ms": ms_adj}
        print(json.dumps(line))
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
