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

One step = one relaxation of every point, launched from a prepared plan
(mafm_plan_launch) captured in a CUDA graph.  The headline precision is
MAFM_DF (double-float on the FP32 pipes, FP64's FIRE decisions, near-tie
columns re-relaxed in FP64 inside the same step): its points meet the metric's
1e-3 A / 1e-3 bar against FP64 on every point, which the run checks on all
points of the scan (or a seeded uniform sample of columns of every scan when
the scans hold more than FP64_FULL_POINTS; rigid-grid scans: a centre crop,
each precision over its own grid, the double-float one built in double-float).
MAFM_FP32C is also timed as the fast path, with
its own error against FP64.  `value` = points/s with inputs resident and
outputs in HBM; `e2e` = the same through the C ABI from host memory (scan
creation with the upload, relax, every point record delivered into pinned host
memory).  kernel_ms of the rooflines comes from events recorded inside the same
graph replays that give ms_per_step.  The CPU baseline is the reference's own
relaxation (oracle/_ref, where it was built) or the oracle port (FP64, OpenMP
on every host thread) on a seeded uniform sample of pixel columns of about ten
seconds.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--workload NAME] [--precision df|fp32c]
  profiling knobs: --pixels P (a smaller scan), --lanes/--block/--tile
  (a forced FP32C launch shape instead of the autotuner), --no-tune (the
  default shape), --no-fp64 and --cpu-seconds 0 (skip the comparison legs).
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
# FP32 operations (FMA = 2) of one term in the double-float kernel, counted
# from its source (pair_df2 and the dfloat2 operations it calls): the work of
# the double-float algorithms that compute the FP64-faithful term.
# A Coulomb term costs less beside an LJ term (their 1/r^2 factors merge).
DF_FLOPS_LJ, DF_FLOPS_MORSE, DF_FLOPS_COUL_LJ, DF_FLOPS_COUL_MORSE = 201, 475, 23, 30
DF_TABLE = (DF_FLOPS_LJ, DF_FLOPS_MORSE, DF_FLOPS_COUL_LJ, DF_FLOPS_COUL_MORSE)
DF_TABLE_TEXT = (f"double-float FP32 operations (FMA = 2) per term, counted from the kernel source: "
                 f"LJ {DF_FLOPS_LJ}, Morse {DF_FLOPS_MORSE}, Coulomb {DF_FLOPS_COUL_LJ} beside LJ "
                 f"and {DF_FLOPS_COUL_MORSE} beside Morse")
# GB300's nominal FP64 rate (MEASURED_PEAKS.json measures HBM and bf16 only).
FP64_PEAK_NOMINAL_TFLOPS = 1.25
# Algorithmic bytes of one trilinear lookup: 8 FP32 {F, E} nodes.
BYTES_LOOKUP = 8 * 16
# DRAM bytes per trilinear lookup of the rigid-grid relax: ncu dram__bytes
# (20.13 GB/s x 17.454 ms = 351.3 MB) over the 190,890,530 lookups of one
# 200 x 200 px slab launch: the grid nodes read once and the output records
# written (gathers within a column are served by L1 and L2).
DRAM_BYTES_PER_LOOKUP = 351.3e6 / 190890530
# Output bytes of one relaxed point (the 64 B mafm_point record), written once.
POINT_BYTES = 64
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per relaxed point of
# the relax kernels, from ncu captures of one 285 x 285 x 41 cluster launch
# (3,330,225 points): relaxdf_kernel 13.0 + 180.4 MB, relax32_kernel 6.0 +
# 165.9 MB.  The output records are the traffic; the last of them can still
# sit in the 126 MB L2 when the capture ends, so these are lower bounds.
DRAM_BYTES_PER_POINT_DF = 193.4e6 / 3330225
DRAM_BYTES_PER_POINT_32 = 171.9e6 / 3330225
# DRAM bytes per node of grid_builddf_kernel: ncu of one 64 x 64 px slab grid
# (3,475,509 nodes): 9.5 + 57.1 MB (a lower bound, as above).
DRAM_BYTES_PER_NODE_DF = 66.6e6 / 3475509
CPU_TARGET_S = 10.0        # CPU sample length
RIGID_CROP = 16            # pixels per side of the rigid-grid CPU sample
FP64_RIGID_CROP = 64       # pixels per side of the rigid-grid FP64 comparison
ADJ_CROP = 64              # pixels per side of the adjoint CPU sample
FP64_FULL_POINTS = 8_000_000   # up to this many points FP64 relaxes every point
FP64_SAMPLE_COLUMNS = 96       # else this many seeded columns per scan
FP64_RATE_SCANS, FP64_RATE_COLUMNS = 8, 2048   # the FP64 rate of a batch (see fp64_reference)

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
    ap.add_argument("--precision", default="df", choices=["df", "fp32c"],
                    help="headline precision")
    ap.add_argument("--cpu-seconds", type=float, default=CPU_TARGET_S,
                    help="length of the CPU sample (0 = skip the CPU baseline)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="default launch shape, no autotuner")
    ap.add_argument("--lanes", type=int, default=0, help="force FP32C lanes per column")
    ap.add_argument("--tile", type=int, default=0, help="force FP32C columns per tile")
    ap.add_argument("--block", type=int, default=0, help="force FP32C threads per block")
    ap.add_argument("--pixels", type=int, default=0, help="pixels per side (profiling)")
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


def term_flops(desc, direct: bool = False, table=(FLOPS_LJ, FLOPS_MORSE, FLOPS_COUL, FLOPS_COUL)):
    """Algorithmic flops of one force evaluation over a scan's tip–atom terms
    (direct=True: the terms a rigid-grid node samples); table = flops of an
    LJ term, a Morse term, and a Coulomb term beside an LJ or a Morse term
    (the FP64 expressions' by default)."""
    from mechafm_gb300 import _abi
    if desc.c.rigidgrid and not direct:
        return 0
    a = desc.atoms()
    kinds = np.array([desc.c.tip_pair[int(t)].kind for t in a["type"]])
    images = 9 if desc.c.vdw_pbc else 1
    n_lj = int((kinds == _abi.PAIR_LJ).sum()) * images
    n_mo = int((kinds == _abi.PAIR_MORSE).sum()) * images
    charged = (a["charge"] != 0) & bool(desc.c.coulomb) & (desc.c.tip_charge != 0)
    n_co_lj = int((charged & (kinds == _abi.PAIR_LJ)).sum())
    n_co_mo = int((charged & (kinds == _abi.PAIR_MORSE)).sum())
    return n_lj * table[0] + n_mo * table[1] + n_co_lj * table[2] + n_co_mo * table[3]


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


def sample_columns(n_columns: int, n: int, seed: int) -> np.ndarray:
    """A seeded uniform sample of n pixel columns (i * ny + j) of a scan, sorted."""
    rng = np.random.default_rng(seed)
    n = min(n, n_columns)
    return np.sort(rng.choice(n_columns, size=n, replace=False)).astype(np.int32)


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

def _cpu_sample(inputs, descs, frac, threads, tmp):
    """Relax a seeded uniform fraction of every scan's pixel columns on the
    host: with the reference's own code (oracle/_ref/ref_dump, timed inside
    it) where that was built, else with the oracle port.  Returns (points,
    seconds, columns, kind)."""
    import oracle
    use_ref = oracle.ref_available()
    jobs = []
    for i, (inp, d) in enumerate(zip(inputs, descs)):
        n = max(1, min(d.n_columns, int(round(frac * d.n_columns))))
        jobs.append((inp, d, sample_columns(d.n_columns, n, 1000 + i)))
    pts, wall = 0, 0.0
    if use_ref:
        for k, (inp, d, cols) in enumerate(jobs):
            p, t, _ = oracle.ref_time_columns(inp.path, cols, os.path.join(tmp, f"cpu{k}"), threads)
            pts += p
            wall += t
    elif len(jobs) == 1:
        inp, d, cols = jobs[0]
        t0 = time.perf_counter()
        pts = len(oracle.run_columns(d, cols, threads=threads)[0])
        wall = time.perf_counter() - t0
    else:
        # many scans: one scan per host thread (the port releases the GIL)
        t0 = time.perf_counter()
        with ThreadPoolExecutor(threads) as ex:
            pts = sum(ex.map(lambda j: len(oracle.run_columns(j[1], j[2], threads=1)[0]), jobs))
        wall = time.perf_counter() - t0
    return pts, wall, sum(len(c) for _, _, c in jobs), ("reference" if use_ref else "port")


def cpu_direct(inputs, descs, threads, target_s, tmp):
    """Points/s over a seeded uniform sample of the columns of every scan, sized
    to about target_s seconds after a short pilot.  Returns (rate, text,
    kind, seconds, points)."""
    total = sum(d.n_columns for d in descs)
    frac = min(1.0, 400.0 / total)
    pts, t, cols, kind = _cpu_sample(inputs, descs, frac, threads, tmp)
    if t < target_s and frac < 1.0:
        frac = min(1.0, frac * target_s / max(t, 1e-3))
        pts, t, cols, kind = _cpu_sample(inputs, descs, frac, threads, tmp)
    return pts / t, (f"{cols} seeded uniform columns x all z ({100 * frac:.2f}% of the columns "
                     f"of every scan), {pts} points in {t:.1f} s"), kind, t, pts


def cpu_rigid(descs, threads, crop_n):
    """Points/s of the oracle on rigid-grid scans, from a centre crop: the
    set-up (external field), the grid build and the relaxation are timed apart
    and scaled to the full scan by grid nodes and by points (a rigid grid spans
    the whole scan area, so a sample of scattered columns would build it all)."""
    import oracle
    from mechafm_gb300 import _abi
    from mechafm_gb300.scan import Desc
    est, pts, wall, n_crop = 0.0, 0, 0.0, 0
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
        n_crop += len(out)
        wall += t_es + t_setup + t_relax
    return pts / est, (f"{crop_n}x{crop_n} centre crop of every scan ({n_crop} points, "
                       f"{wall:.1f} s): external field, grid build (scaled by grid nodes) and "
                       f"relaxation (scaled by points) timed apart"), "port", wall, n_crop


def cpu_adjoint(descs, threads, crop_n):
    """Points/s of the oracle's forward relaxation + adjoint on a centre crop."""
    import oracle
    rate, wall, n_pts = [], 0.0, 0
    for desc in descs:
        crop = centre_crop(desc, crop_n)
        t0 = time.perf_counter()
        pts, _ = oracle.run(crop, threads=threads)
        w = np.random.default_rng(0).normal(size=len(pts))
        oracle.adjoint(crop, pts, w)
        t = time.perf_counter() - t0
        rate.append(len(pts) / t)
        wall += t
        n_pts += len(pts)
    return float(np.mean(rate)), (f"{crop_n}x{crop_n} centre crop, forward FP64 relaxation + "
                                  f"adjoint, {wall:.1f} s"), "port", wall, n_pts


def cpu_rate(kind, inputs, descs, threads, target_s, tmp):
    if kind == "adjoint":
        return cpu_adjoint(descs, threads, ADJ_CROP)
    if any(d.c.rigidgrid for d in descs):
        return cpu_rigid(descs, threads, RIGID_CROP)
    return cpu_direct(inputs, descs, threads, target_s, tmp)


def reference_arm(args, rank):
    """--impl reference: the reference's CPU path on all host threads over a
    bounded sample of the same workload: the reference's own code
    (oracle/_ref, built from its sources where they were present) or else the
    oracle port of its FP64 OpenMP code.  ms_per_step is the time each step
    actually took for its sample; value is the sample's points/s."""
    if rank != 0:
        return
    tmp = tempfile.mkdtemp()
    inputs, desc_text = make_inputs(args.workload, tmp, args.pixels)
    descs = [i.desc() for i in inputs]
    threads = cpu_threads()
    kind = "adjoint" if args.workload == "adjoint_128" else "forward"
    for _ in range(args.warmup):
        cpu_rate(kind, inputs, descs, threads, 0.5, tmp)
    rates, secs, pts = [], [], []
    sample, arm = "", "port"
    for _ in range(args.steps):
        r, sample, arm, t, p = cpu_rate(kind, inputs, descs, threads,
                                        args.cpu_seconds or CPU_TARGET_S, tmp)
        rates.append(r)
        secs.append(t)
        pts.append(p)
    value = float(np.mean(rates))
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * float(np.mean(secs)), "points_per_step": int(np.mean(pts)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": desc_text,
                   "precision": ("FP64 CPU, the reference's own code built from its sources "
                                 "(oracle/_ref), OpenMP" if arm == "reference" else
                                 "FP64 CPU (oracle port of the reference's code, OpenMP)"),
                   "step": "a seeded sample of the workload (see cpu_baseline.sample)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": arm,
                         "sample": sample + " per step; points/s of the sample"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ------------------------------------------------------------- GPU helpers ----

def err_stats(pts, ref):
    """Tip and relative Fz error (denominator max(|Fz_ref|, 0.01 = ftol)) of
    pts against ref, over every point."""
    tip = np.abs(pts["tip"] - ref["tip"]).max(axis=1)
    fz = np.abs(pts["force"][:, 2] - ref["force"][:, 2]) / np.maximum(np.abs(ref["force"][:, 2]), 0.01)
    return {"tip_err_A": {"max": float(tip.max()), "p99_9": float(np.percentile(tip, 99.9)),
                          "median": float(np.median(tip)),
                          "frac_le_1e-3": float((tip <= 1e-3).mean())},
            "fz_rel_err": {"max": float(fz.max()), "p99_9": float(np.percentile(fz, 99.9)),
                           "frac_le_1e-3": float((fz <= 1e-3).mean())},
            "points_beyond_bar": int(((tip > 1e-3) | (fz > 1e-3)).sum()),
            "step_count_match": float((pts["steps"] == ref["steps"]).mean())}


def fp64_reference(scans, descs, dev):
    """FP64 points to check the other precisions against, and the FP64 GPU
    rate: every point of the scans when they hold at most FP64_FULL_POINTS
    (the plain FP64 kernel, mafm_run), else a seeded uniform sample of
    FP64_SAMPLE_COLUMNS columns of every scan (mafm_run_columns, same bits).
    Rigid-grid scans: a centre crop (every precision builds its own grid of
    the crop); the FP64 rate there is the crop's grid build scaled to the
    full grid by nodes plus its relaxation scaled by points.  Returns
    (list of (scan, columns or None, points), FP64 points/s, compared
    points, text)."""
    import torch
    from mechafm_gb300 import _abi
    from mechafm_gb300.scan import Scan
    total = sum(d.n_points for d in descs)
    refs, ms, npts = [], 0.0, 0
    if any(d.c.rigidgrid for d in descs):
        L = _abi.lib()
        stream = torch.cuda.Stream(device=dev)
        sp = C.c_void_p(stream.cuda_stream)
        est_s, full = 0.0, 0
        for s in scans:
            crop = Scan(centre_crop(s.desc, FP64_RIGID_CROP), device=dev)
            p64, st = crop.run(_abi.FP64)          # builds the crop's FP64 grid
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _abi.check(L.mafm_scan_build_grid(crop.handle, _abi.FP64, sp))
            e1.record(stream)
            torch.cuda.synchronize()
            build_ms = e0.elapsed_time(e1)
            refs.append((crop, None, p64))
            est_s += (build_ms * rigid_nodes(s.desc.c) / rigid_nodes(crop.desc.c)
                      + st.kernel_ms * s.desc.n_points / len(p64)) / 1000.0
            full += s.desc.n_points
            npts += len(p64)
        return refs, full / est_s, npts, (
            f"{FP64_RIGID_CROP}x{FP64_RIGID_CROP} centre crop, every point; FP64 rate = the crop's "
            f"FP64 grid build scaled by grid nodes + its relaxation scaled by points")
    if total <= FP64_FULL_POINTS:
        for s in scans:
            p64, st = s.run(_abi.FP64)
            refs.append((s, None, p64))
            ms += st.kernel_ms
            npts += len(p64)
        return refs, npts / (ms / 1000.0), npts, "every point of the scan (relax64_kernel)"
    for i, s in enumerate(scans):
        cols = sample_columns(s.desc.n_columns, FP64_SAMPLE_COLUMNS, 2000 + i)
        p64, _ = s.run_columns(cols)
        refs.append((s, cols, p64))
        npts += len(p64)
    # The rate: a few ordered columns per scan keep too few warps busy to
    # measure throughput, so FP64_RATE_SCANS seeded scans relax
    # FP64_RATE_COLUMNS seeded columns each (enough warps to fill the GPU);
    # the batch's FP64 time is their time per point and term, scaled by every
    # scan's points x terms.
    rng = np.random.default_rng(3000)
    pick_scans = rng.choice(len(scans), size=min(FP64_RATE_SCANS, len(scans)), replace=False)
    t_sample, w_sample = 0.0, 0.0
    for i in pick_scans:
        s = scans[int(i)]
        cols = sample_columns(s.desc.n_columns, FP64_RATE_COLUMNS, 4000 + int(i))
        p64, st = s.run_columns(cols)
        t_sample += st.kernel_ms / 1000.0
        w_sample += len(p64) * max(s.desc.c.n_atoms, 1)
    est = sum(s.desc.n_points * max(s.desc.c.n_atoms, 1) for s in scans) * t_sample / w_sample
    return refs, total / est, npts, (
        f"{FP64_SAMPLE_COLUMNS} seeded uniform columns x all z of each of the {len(scans)} scans "
        f"(mafm_run_columns, one warp per column, the bits of relax64_kernel); the FP64 rate from "
        f"{FP64_RATE_COLUMNS} seeded columns of {len(pick_scans)} seeded scans, scaled to the batch "
        f"by points x atoms")


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


def timing_event(external):
    import torch
    if external:
        return torch.cuda.Event(enable_timing=True, external=True)
    return torch.cuda.Event(enable_timing=True)


def external_events_work(stream) -> bool:
    """Whether this PyTorch records timing events inside a captured graph
    (external event-record nodes): probed on a throwaway graph."""
    import torch
    try:
        x = torch.zeros(16, device=stream.device)
        a, b = timing_event(True), timing_event(True)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            a.record(stream)
            x.add_(1.0)
            b.record(stream)
        g.replay()
        torch.cuda.synchronize()
        a.elapsed_time(b)
        return True
    except Exception:
        torch.cuda.synchronize()
        return False


class GraphStep:
    """One step captured in a CUDA graph, with events recorded inside the
    graph around each part (external event-record nodes), so that the parts'
    device times come from the same replays as the step time.  Where the
    PyTorch build lacks external events, the parts are timed by events around
    plain launches of the same replays instead."""

    def __init__(self, stream, parts):
        import torch
        self.stream = stream
        self.parts = parts          # [(name, fn)]
        self.graph = torch.cuda.CUDAGraph()
        self.external = external_events_work(stream)
        self.ev = [timing_event(self.external) for _ in range(len(parts) + 1)]
        with torch.cuda.graph(self.graph, stream=stream):
            if self.external:
                self.ev[0].record(stream)
            for k, (_, fn) in enumerate(self.parts):
                fn()
                if self.external:
                    self.ev[k + 1].record(stream)

    def replay(self):
        """Replay the step on the stream (the caller synchronises)."""
        if self.external:
            self.graph.replay()
        else:
            self.ev[0].record(self.stream)
            for k, (_, fn) in enumerate(self.parts):
                fn()
                self.ev[k + 1].record(self.stream)

    def part_ms(self):
        return {name: self.ev[k].elapsed_time(self.ev[k + 1]) for k, (name, _) in enumerate(self.parts)}


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
    nz = descs[0].c.nz
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{dev}")
    stream = torch.cuda.Stream(device=dev)
    sptr = C.c_void_p(stream.cuda_stream)
    n = len(scans)
    handles = (C.c_void_p * n)(*[s.handle for s in scans])
    rigid = [s for s in scans if s.desc.c.rigidgrid]
    head = _abi.DF if args.precision == "df" else _abi.FP32C
    head_name = "DF" if head == _abi.DF else "FP32C"

    def device_outs():
        bufs = [torch.empty(d.n_points * 64, dtype=torch.uint8, device=f"cuda:{dev}") for d in descs]
        return bufs, (C.c_void_p * n)(*[o.data_ptr() for o in bufs])

    def host_points(bufs, refs=None):
        """Point records of device buffers on the host: whole scans, or only the
        listed columns of each (gathered on the device first)."""
        got = []
        for k, b in enumerate(bufs):
            cols = refs[k][1] if refs is not None else None
            if cols is not None:
                nzk = descs[k].c.nz
                idx = torch.from_numpy((cols[:, None].astype(np.int64) * nzk +
                                        np.arange(nzk)[None, :]).reshape(-1)).to(b.device)
                b = b.view(-1, POINT_BYTES).index_select(0, idx).reshape(-1)
            got.append(np.frombuffer(b.cpu().numpy().tobytes(), dtype=_abi.POINT_DTYPE))
        return got

    def record_evals(bufs):
        """Force evaluations per scan from its point records: FIRE steps x the
        integrator's evaluations per step (SD, euler 1, midpoint 2, rk4 4),
        plus each point's output evaluation."""
        ev = []
        for b, d in zip(bufs, descs):
            steps = b.view(torch.int32).view(-1, POINT_BYTES // 4)[:, 14].to(torch.int64).sum().item()
            per = (1 if d.c.minimiser == _abi.MIN_SD else
                   {_abi.INT_EULER: 1, _abi.INT_MIDPOINT: 2, _abi.INT_RK4: 4}[d.c.integrator])
            ev.append(steps * per + d.n_points)
        return np.array(ev, dtype=float)

    # Rigid grids: the first build allocates (outside the timing); a step rebuilds.
    t_grid = 0.0
    if rigid:
        t0 = time.perf_counter()
        for s in rigid:
            _abi.check(L.mafm_scan_build_grid(s.handle, head, sptr))
            if head != _abi.FP32C:   # the fast path's grid
                _abi.check(L.mafm_scan_build_grid(s.handle, _abi.FP32C, sptr))
        torch.cuda.synchronize()
        t_grid = time.perf_counter() - t0

    # FP32C launch shape: the autotuner (its sweep on the first 32 scans of a
    # batch, then the winner against the default shape on all of them)
    opts32 = _abi.RunOpts(_abi.FP32C, args.lanes, args.block, args.tile, 0, 0)
    tune_ms = None
    if not args.no_tune and not (args.lanes or args.block or args.tile):
        best = _abi.RunOpts()
        tms = C.c_double()
        _abi.check(L.mafm_autotune(handles, n, C.byref(best), C.byref(tms), sptr))
        opts32, tune_ms = best, tms.value

    def make_plan(prec, bufs_ptrs):
        o = opts32 if prec == _abi.FP32C else _abi.RunOpts(prec, 0, 0, 0, 0, 0)
        plan = C.c_void_p()
        _abi.check(L.mafm_plan_create(handles, n, C.byref(o), bufs_ptrs, C.byref(plan)))
        return plan

    outs, optrs = device_outs()
    plan = make_plan(head, optrs)
    used = _abi.RunOpts()
    _abi.check(L.mafm_plan_config(plan, C.byref(used)))

    def relax():
        _abi.check(L.mafm_plan_launch(plan, sptr))

    def build():
        for s in rigid:
            _abi.check(L.mafm_scan_build_grid(s.handle, head, sptr))

    def build32():
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
        tp, _ = st_.run(head)
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

    parts = ([("grid_build", build)] if rigid else []) + [("relax", relax)]
    for _ in range(args.warmup):
        for _, fn in parts:
            fn()
        if adjoint:
            adj()
    st = _abi.RunStats()
    _abi.check(L.mafm_plan_stats(plan, C.byref(st), sptr))
    step = GraphStep(stream, parts)
    torch.cuda.synchronize()

    times, part_times = [], {name: [] for name, _ in parts}
    if adjoint:
        part_times["adjoint"] = []
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                ea = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                step.replay()
                ea.record(stream)
                if adjoint:
                    adj()
                e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
            for name, v in step.part_ms().items():
                part_times[name].append(v)
            if adjoint:
                part_times["adjoint"].append(ea.elapsed_time(e1))
    ms = job_ms(times, world, f"cuda:{dev}")
    value = replica_throughput(n_pts, world, ms)
    _abi.check(L.mafm_plan_stats(plan, C.byref(st), sptr))   # the last replay ended cleanly
    ms_part = {k: float(np.mean(v)) for k, v in part_times.items()}

    # the fast path (FP32C) timed the same way, when the headline is DF
    fast = None
    outs32 = None
    if head == _abi.DF:
        outs32, optrs32 = device_outs()
        plan32 = make_plan(_abi.FP32C, optrs32)

        def relax32():
            _abi.check(L.mafm_plan_launch(plan32, sptr))

        parts32 = ([("grid_build", build32)] if rigid else []) + [("relax", relax32)]
        for _ in range(args.warmup):
            for _, fn in parts32:
                fn()
        step32 = GraphStep(stream, parts32)
        t32, b32 = [], []
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                step32.replay()
                e1.record(stream)
            torch.cuda.synchronize()
            t32.append(e0.elapsed_time(e1))
            if rigid:
                b32.append(step32.part_ms()["grid_build"])
        st32 = _abi.RunStats()
        _abi.check(L.mafm_plan_stats(plan32, C.byref(st32), sptr))
        ms32 = job_ms(t32, world, f"cuda:{dev}")
        used32 = _abi.RunOpts()
        _abi.check(L.mafm_plan_config(plan32, C.byref(used32)))
        fast = {"precision": "FP32C", "points_per_s": replica_throughput(n_pts, world, ms32),
                "ms_per_step": ms32, "force_evals": int(st32.force_evals),
                "step": "rigid grid rebuild + relax" if rigid else "relax",
                **({"grid_build_ms": float(np.mean(b32))} if rigid else {}),
                "launch": {"lanes_per_column": used32.lanes_per_column,
                           "block_threads": used32.block_threads,
                           "columns_per_tile": used32.columns_per_tile}}
        L.mafm_plan_destroy(plan32)

    # e2e through the public API from host memory
    h2d = 0
    for d in descs:
        h2d += d.c.n_atoms * (3 * 8 + 8 + 4) + d.c.n_types * 32
        if d.c.use_external_potential:
            h2d += 8 * d.c.epot_n[0] * d.c.epot_n[1] * d.c.epot_n[2]
    e2e_times = []
    reps = 2 if n == 1 else 1
    if adjoint:
        # torch.autograd through fz_image: scan creation, relax, D2H of the
        # points, loss, backward = mafm_adjoint (points and dL/dFz uploaded)
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
            fz = fz_image(d0, pos, chg, pr, precision=head, device=dev)
            loss = ((fz - tgt) ** 2).mean()
            loss.backward()
            if i > 0:
                e2e_times.append(time.perf_counter() - t0)
        h2d += n_pts * (64 + 8)
        d2h = n_pts * 64
    else:
        # pinned host buffers for the results (written by the kernels directly)
        pinned = [torch.empty(d.n_points * 64, dtype=torch.uint8, pin_memory=True) for d in descs]
        host = [p.numpy().view(_abi.POINT_DTYPE) for p in pinned]
        e2e_opts = (_abi.RunOpts(_abi.FP32C, used.lanes_per_column, used.block_threads,
                                 used.columns_per_tile, 0, 0) if head == _abi.FP32C
                    else _abi.RunOpts(head, 0, 0, 0, 0, 0))
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
        # accuracy against FP64 (the oracle's arithmetic; bit-identical to the
        # reference on LJ/Coulomb terms)
        fp64 = None
        if not args.no_fp64:
            refs, rate64, npts64, subset = fp64_reference(scans, descs, dev)
            if not rigid:
                head_pts = host_points(outs, refs)
                fast_pts = host_points(outs32, refs) if outs32 is not None else None
            if rigid:
                # the crop's own relaxations (each precision over its own grid)
                cmp_head = np.concatenate([s.run(head)[0] for s, _, _ in refs])
                cmp_fast = (np.concatenate([s.run(_abi.FP32C)[0] for s, _, _ in refs])
                            if fast is not None else None)
            else:
                cmp_head = np.concatenate(head_pts)
                cmp_fast = np.concatenate(fast_pts) if fast_pts is not None else None
            p64 = np.concatenate([p for _, _, p in refs])
            fp64 = {"points_per_s": rate64, "points": npts64, "subset": subset,
                    "speedup_vs_fp64": {head_name: value / world / rate64},
                    head_name: err_stats(cmp_head, p64)}
            if cmp_fast is not None:
                fp64["FP32C"] = err_stats(cmp_fast, p64)
                fp64["speedup_vs_fp64"]["FP32C"] = fast["points_per_s"] / world / rate64
            if rigid:
                for s, _, _ in refs:
                    s.close()
        peak_tflops = fp32_peak(dev)
        # algorithmic flops of the relax: every scan's force evaluations (from
        # its point records) x its flops per evaluation
        evs = record_evals(outs)
        fpe = np.array([term_flops(d) for d in descs], dtype=float)
        ms_relax = ms_part["relax"]
        relax_flops = float((evs * fpe).sum())
        kname = "relaxdf_kernel + repair64_kernel" if head == _abi.DF else "relax32_kernel"
        if fpe.any():
            relax_line = fp32_roofline(relax_flops / (ms_relax / 1000.0) / 1e12, peak_tflops, {
                "traffic": (DRAM_BYTES_PER_POINT_DF if head == _abi.DF else DRAM_BYTES_PER_POINT_32) * n_pts,
                "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one 285x285x41 "
                                   "cluster launch, scaled by points; a lower bound (the capture's last "
                                   "output records can stay in L2); algorithmic bytes: the 64 B output "
                                   "record per point"),
                "algorithmic_bytes": POINT_BYTES * n_pts,
                "kernel": kname, "kernel_ms": ms_relax,
                "kernel_ms_source": ("events recorded inside the timed graph replays"
                                     if step.external else
                                     "events around the same launches (no external graph events)"),
                "flops_per_force_eval": relax_flops / evs.sum(),
                "force_evals": int(evs.sum()),
                "force_evals_source": "FIRE steps of every point record x evaluations per step, "
                                      "plus the output evaluation (the kernel's own counter, which "
                                      "also counts re-relaxed columns' evaluations: "
                                      f"{int(st.force_evals)})"})
            if head == _abi.DF:
                # the kernel computes in double-float: its algorithmic work is
                # the FP32 operations of the double-float term algorithms
                fpe_df = np.array([term_flops(d, table=DF_TABLE) for d in descs], dtype=float)
                df_flops = float((evs * fpe_df).sum())
                fp64_equiv = relax_flops / (ms_relax / 1000.0) / 1e12
                relax_line["achieved"] = df_flops / (ms_relax / 1000.0) / 1e12
                relax_line["frac"] = relax_line["achieved"] / peak_tflops
                relax_line["flops_per_force_eval"] = df_flops / evs.sum()
                relax_line["flops_source"] = DF_TABLE_TEXT
                relax_line["fp64_equivalent"] = {
                    "flops_per_force_eval": relax_flops / evs.sum(),
                    "achieved_tflops": fp64_equiv,
                    "vs_fp64_peak_nominal": fp64_equiv / FP64_PEAK_NOMINAL_TFLOPS,
                    "note": "the FP64 expressions' flops (LJ 25, Morse 29, Coulomb 20 per term) "
                            "per second, against GB300's nominal 1.25 TFLOP/s FP64 rate"}
        else:
            hp, src = hbm_peak()
            if head == _abi.DF:
                # double-float nodes: 8 x 32 B per lookup
                gbs = st.force_evals * 2 * BYTES_LOOKUP / (ms_relax / 1000.0) / 1e9
                relax_line = {"bound": "gather latency (L1-resident), not HBM", "achieved": gbs,
                              "peak": hp, "unit": "GB/s", "frac": gbs / hp, "traffic": None,
                              "peak_source": src,
                              "kernel": "relaxdf_kernel (trilinear lookups, double-float nodes)",
                              "kernel_ms": ms_relax, "bytes_per_lookup": 2 * BYTES_LOOKUP,
                              "lookups": int(st.force_evals)}
            else:
                gbs = st.force_evals * BYTES_LOOKUP / (ms_relax / 1000.0) / 1e9
                relax_line = {"bound": "gather latency (L1-resident), not HBM", "achieved": gbs,
                              "peak": hp, "unit": "GB/s", "frac": gbs / hp,
                              "traffic": DRAM_BYTES_PER_LOOKUP * st.force_evals, "peak_source": src,
                              "traffic_source": "ncu dram__bytes of one 200x200 px slab launch "
                                                "(190.9 M lookups), scaled by lookups",
                              "kernel": "relax32_kernel (trilinear lookups)", "kernel_ms": ms_relax,
                              "bytes_per_lookup": BYTES_LOOKUP, "lookups": int(st.force_evals),
                              "note": "achieved = algorithmic bytes of the gathers; ncu: L1 hit "
                                      "91 %, L2 hit 83 % at 3 % L2 throughput, DRAM 20 GB/s, "
                                      "issue 43 %"}
        rooflines = [(ms_relax, relax_line)]
        if rigid:
            nodes = sum(rigid_nodes(s.desc.c) for s in rigid)
            flops64 = sum(rigid_nodes(s.desc.c) * term_flops(s.desc, direct=True) for s in rigid)

            def build_line(ms_b, df):
                tbl = DF_TABLE if df else (FLOPS_LJ, FLOPS_MORSE, FLOPS_COUL, FLOPS_COUL)
                fl = sum(rigid_nodes(s.desc.c) * term_flops(s.desc, direct=True, table=tbl)
                         for s in rigid)
                extra = {"kernel": ("grid_builddf_kernel (+ its FP64 copy)" if df else
                                    "grid_build32_kernel" + ("" if head == _abi.FP32C else
                                                             " (MAFM_FP32C, the fast path)")),
                         "kernel_ms": ms_b, "nodes": nodes, "flops_per_node": float(fl / nodes)}
                if df:
                    extra["traffic"] = DRAM_BYTES_PER_NODE_DF * nodes
                    extra["traffic_source"] = ("ncu dram__bytes of one 64x64 px slab grid build "
                                               "(3,475,509 nodes), scaled by nodes; a lower bound")
                    f64 = flops64 / (ms_b / 1000.0) / 1e12
                    extra["flops_source"] = DF_TABLE_TEXT
                    extra["fp64_equivalent"] = {"achieved_tflops": f64,
                                                "vs_fp64_peak_nominal": f64 / FP64_PEAK_NOMINAL_TFLOPS}
                return fp32_roofline(fl / (ms_b / 1000.0) / 1e12, peak_tflops, extra)

            ms_build = ms_part["grid_build"]
            rooflines.append((ms_build, build_line(ms_build, head == _abi.DF)))
            if fast is not None and "grid_build_ms" in fast:
                rooflines.append((fast["grid_build_ms"], build_line(fast["grid_build_ms"], False)))
        if adjoint:
            rooflines.append((ms_part["adjoint"], {"kernel": "adjoint32_kernel (FP32C)",
                                                   "kernel_ms": ms_part["adjoint"], "bound": "fp32",
                                                   "note": "FP32 per-term Jacobians and parameter "
                                                           "derivatives, FP64 3x3 solve per point"}))
        if fast is not None and fpe.any():
            f32 = float((record_evals(outs32) * fpe).sum())
            rooflines.append((fast["ms_per_step"], fp32_roofline(
                f32 / (fast["ms_per_step"] / 1000.0) / 1e12, peak_tflops,
                {"kernel": "relax32_kernel (MAFM_FP32C, the fast path)",
                 "kernel_ms": fast["ms_per_step"]})))
        rooflines.sort(key=lambda r: -r[0])
        main_line = relax_line if not rigid else rooflines[0][1]
        threads = cpu_threads()
        if args.cpu_seconds > 0:
            cpu_value, cpu_sample, cpu_kind, _, _ = cpu_rate("adjoint" if adjoint else "forward",
                                                             inputs, descs, threads,
                                                             args.cpu_seconds, tmp)
            cpu = {"value": cpu_value, "unit": UNIT, "cores": threads, "kind": cpu_kind,
                   "sample": cpu_sample}
        else:
            cpu = None
        launches = args.steps * ((2 if head == _abi.DF else 1) + len(rigid) + (1 if adjoint else 0))
        step_text = ("rigid grid rebuild + relax" if rigid else
                     "relax + adjoint" if adjoint else "relax")
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": ("f32 double-float (pairs of FP32 numbers, 48-bit significand) on the FP32 "
                      "pipes; near-tie columns in f64" if head == _abi.DF else
                      "f32 (compensated sums, double-float positions and energy)"),
            "data": "synthetic",
            "config": {"workload": desc_text, "scans": n, "points_per_step": n_pts,
                       "precision": head_name, "step": step_text,
                       "launch": ({"kernel": "relaxdf_kernel: persistent, one column per lane, a lane "
                                             "takes the next column from the queue as soon as its "
                                             "own ends (columns in expected-cost order); "
                                             "repair64_kernel: one warp per listed column",
                                   "cuda_graph": True}
                                  if head == _abi.DF else
                                  {"lanes_per_column": used.lanes_per_column,
                                   "block_threads": used.block_threads,
                                   "columns_per_tile": used.columns_per_tile,
                                   "chosen_by": ("autotuner" if tune_ms is not None else
                                                 "forced" if (args.lanes or args.block or args.tile)
                                                 else "default"),
                                   "column_order": ("natural (rigid grid: no pair terms to cost)"
                                                    if rigid else "expected cost, descending"),
                                   "cuda_graph": True}),
                       "l2": f"{L2_FLUSH_BYTES >> 20} MiB buffer written between timed steps",
                       "fire_steps_per_step": int(st.total_steps),
                       "pair_terms_per_step": int(st.pair_evals),
                       "fp64_columns_per_step": int(st.fp64_columns),
                       "scan_create_s": t_create, "first_grid_build_s": t_grid,
                       "parallelism": f"replica per GPU x{world}"},
            "pair_terms_per_s": st.pair_evals * world / (ms / 1000.0),
            "roofline": main_line,
            "roofline_other": [r[1] for r in rooflines if r[1] is not main_line],
            "fp64_gpu": fp64,
            "fast_path": fast,
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
                               "forward_ms": ms_relax, "adjoint_ms": ms_part["adjoint"]}
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
