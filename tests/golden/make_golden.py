"""Generate the golden fixtures from the reference's own code.

Run where the reference sources exist:
    MAFM_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py
It builds oracle/_ref (the unmodified reference sources, compiled out of tree
by oracle/Makefile), writes each case's seeded synthetic input files into
tests/golden/<case>/ and stores the reference's full-precision results for a
block of pixel columns in tests/golden/<case>/ref.npz:

  i, j, k, steps            int32 per point
  tip (n,3), force (n,3), energy (n), angle (n), r (n)  float64
  block                     [i0, i1, j0, j1] pixel block
  sample_pts / sample_fe    optional tip positions and the reference's
                            tip-surface force+energy there (sample_ts / sample_es)

The GPU machine has no reference sources: tests read only these files.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from mechafm_gb300 import synth  # noqa: E402


def graphene_cell(n: int = 6, bond: float = 1.42):
    a = bond * np.sqrt(3.0)
    return (n * a, 0.0, 0.0), (n * a / 2, n * a * np.sqrt(3.0) / 2, 0.0), (0.0, 0.0, 20.0)


def _vec(v):
    return " ".join(repr(float(x)) for x in v)


def small_slab(rigidgrid: bool, voxels: int = 24, shear: float = 0.0, zlow: float = 9.0):
    """36-atom periodic slab, 6x6x10 A cell; 24 voxels = 0.25 A as the full-size slab.
    shear tilts the cell (a non-orthogonal cube basis)."""
    return synth.slab(seed=3, nlx=3, nly=6, layers=2, cell=(6.0, 6.0, 10.0),
                      cube_n=(voxels, voxels, voxels * 10 // 6), pixels=5, step=0.5,
                      zhigh=zlow + 1.0, zlow=zlow, dz=0.1, rigidgrid=rigidgrid, external=True,
                      shear=shear)


def cases():
    """(name, ScanInput, pixel block, sample mode or None)."""
    c = []
    c.append(("graphene_ef", synth.graphene_72(), (45, 50, 45, 50), None))
    c.append(("cluster_ef", synth.cluster_60(), (195, 200, 195, 200), None))
    c.append(("cluster_edge", synth.cluster_60(), (0, 3, 380, 384), None))
    c.append(("graphene_euler", synth.graphene_72(zlow=8.0, integrator="euler"),
              (40, 43, 60, 63), None))
    c.append(("cluster_rk4", synth.cluster_60(zlow=8.0, integrator="rk4"),
              (150, 153, 220, 223), None))
    c.append(("graphene_sd", synth.graphene_72(zlow=9.0, minimiser="SD", minterm="f",
                                              dt="0.01"), (30, 32, 70, 72), None))
    c.append(("cluster_e", synth.cluster_60(zlow=8.0, minterm="e"), (210, 213, 190, 193), None))
    c.append(("cluster_f", synth.cluster_60(zlow=8.0, minterm="f"), (170, 173, 240, 243), None))
    ca, cb, cc = graphene_cell()
    c.append(("graphene_pbc", synth.graphene_72(zlow=9.0, vdw_pbc="on",
                                               cell_a=_vec(ca), cell_b=_vec(cb), cell_c=_vec(cc)), (0, 4, 96, 101), None))
    c.append(("graphene_grid", synth.graphene_72(area=6.0, step=0.5, zlow=7.0, rigidgrid="on"),
              (0, 13, 0, 13), "sample_ts"))
    c.append(("slab_es", small_slab(False), (0, 5, 0, 5), "sample_es"))
    c.append(("slab_es_grid", small_slab(True), (0, 5, 0, 5), "sample_ts"))
    # 0.5 A voxels under-resolve the 0.5 A tip Gaussian: the reference stops with
    # "Imaginary part of inverse FFT exceeded threshold" (fft.cpp:79-83).
    c.append(("slab_es_coarse", small_slab(False, voxels=12), None, "error"))
    # non-orthogonal cube basis: b tilted by 30 % of its length (with a rigid
    # grid on top the reference stops: the tip leaves the grid at every shear
    # and height tried, so only the pair + field form is a fixture)
    c.append(("slab_es_tric", small_slab(False, shear=0.3), (0, 5, 0, 5), "sample_es"))
    c.append(("cluster_tdcoul_ev", synth.cluster_60(zlow=8.0, units="eV",
                                                    tip_dummy_coulomb="on"),
              (200, 203, 200, 203), None))
    ow = synth.graphene_72(zlow=8.0)
    ow.overwrites.append(("C", "O", "lj", 0.1, 3.3))
    c.append(("graphene_ovwrt", ow, (50, 53, 20, 23), None))
    c.append(("cluster_maxsteps", synth.cluster_60(zlow=9.0, maxsteps="40"),
              (180, 183, 180, 183), None))
    # kJ/mol units (qbase 1389.354563, parse.cpp:286-288), the molecule centred
    # away from the scan centre (center, system.cpp:119-136) and an XY spring
    # with a non-zero rest length (harm k r0, interactions.cpp:252-266)
    kj = synth.cluster_60(zlow=8.0, units="kJ/mol", center="1.5 -2.0")
    kj.harm = (0.5, 0.3)
    c.append(("cluster_kj_r0", kj, (190, 193, 205, 208), None))
    # surface normal along y or x: the file's axes are rotated into z
    # (rotateCoordAxes "ZXY" / "YZX", system.cpp:68-89), so the graphene is
    # written with (y, z, x) resp. (z, x, y) as its file coordinates
    gy = synth.graphene_72(zlow=8.0, surface_normal="y")
    gy.pos = gy.pos[:, [1, 2, 0]].copy()
    c.append(("graphene_normal_y", gy, (45, 48, 45, 48), None))
    gx = synth.graphene_72(zlow=8.0, surface_normal="x")
    gx.pos = gx.pos[:, [2, 0, 1]].copy()
    c.append(("graphene_normal_x", gx, (45, 48, 45, 48), None))
    # flexible molecule (bonds, angles, dihedrals, non-bonded pairs between
    # fragments, substrate, XY tethers); the middle column's atom states too
    c.append(("flex_naph", synth.flexible_naphthalene(), (0, 3, 0, 3), "states"))
    c.append(("flex_naph_rk4", synth.flexible_naphthalene(integrator="rk4", zlow=9.0),
              (0, 3, 0, 3), "states"))
    return c


def sample_points(inp_name: str, spec, n: int = 64, seed: int = 5):
    rng = np.random.default_rng(seed)
    area = [float(x) for x in spec.options["area"].split()]
    zlow, zhigh = float(spec.options["zlow"]), float(spec.options["zhigh"])
    x = rng.uniform(0, area[0], n)
    y = rng.uniform(0, area[1], n)
    z = rng.uniform(zlow - 4.2, zhigh - 3.8, n)
    return np.column_stack([x, y, z])


def cli_cases():
    """Tiny inputs run through the reference's own executable (oracle/_ref/mechafm-omp)."""
    ca, cb, cc = graphene_cell()
    return [
        ("cli_cluster", synth.cluster_60(area=0.2, step=0.1, zhigh=10.0, zlow=9.8, dz=0.1)),
        ("cli_pbc", synth.graphene_72(area=20.0, step=10.0, zhigh=10.0, zlow=9.8, dz=0.1,
                                      vdw_pbc="on", cell_a=_vec(ca), cell_b=_vec(cb),
                                      cell_c=_vec(cc))),
        ("cli_flex", synth.flexible_naphthalene(area=1.0, step=0.5, zhigh=10.0, zlow=9.6, dz=0.2)),
    ]


def mask_times(text: str) -> str:
    """Stdout of the executable with the numbers of its two timing lines
    (mechafm.cpp:140-152) replaced by '#'."""
    import re
    return re.sub(r"(wall time is|simulation took) [0-9.]+ seconds", r"\1 # seconds", text)


def make_cli_fixture(name, spec):
    """Sorted rows of every scan-*.dat file, and statistics.txt without its timing lines."""
    folder = os.path.join(HERE, name)
    if os.path.isdir(folder):
        shutil.rmtree(folder)
    inp = spec.write(folder)
    out = os.path.join(folder, "_out")
    r = subprocess.run([oracle.REF_CLI, os.path.abspath(inp), out], check=True, cwd=folder,
                       capture_output=True, text=True)
    # the executable's stdout with the two run times masked and the fixture
    # and output folders as {DIR} and {OUT}
    text = mask_times(r.stdout).replace(out, "{OUT}").replace(folder, "{DIR}")
    with open(os.path.join(folder, "cli_stdout.txt"), "w") as f:
        f.write(text)
    rows = []
    for fn in sorted(os.listdir(out)):
        if fn.startswith("scan-"):
            with open(os.path.join(out, fn)) as f:
                rows += [fn + "\t" + l.rstrip("\n") for l in f]
    with open(os.path.join(folder, "cli_rows.txt"), "w") as f:
        f.write("\n".join(sorted(rows)) + "\n")
    states = []
    for fn in sorted(os.listdir(out)):
        if fn.startswith("state_"):
            with open(os.path.join(out, fn)) as f:
                states += [fn + "\t" + l.rstrip("\n") for l in f]
    if states:
        with open(os.path.join(folder, "cli_states.txt"), "w") as f:
            f.write("\n".join(states) + "\n")
    with open(os.path.join(out, "statistics.txt")) as f:
        stats = f.readlines()[:4]
    with open(os.path.join(folder, "cli_statistics_head.txt"), "w") as f:
        f.writelines(stats)
    shutil.rmtree(out)
    return {"input": os.path.basename(inp), "cli": True, "rows": len(rows)}


def main(only=()):
    """Regenerate every fixture, or only the named cases (the manifest keeps the others)."""
    oracle.build()
    if not oracle.ref_available():
        raise SystemExit("reference build missing")
    manifest = {}
    mpath = os.path.join(HERE, "manifest.json")
    if only and os.path.exists(mpath):
        with open(mpath) as f:
            manifest = json.load(f)
    for name, spec, block, sample in cases():
        if only and name not in only:
            continue
        folder = os.path.join(HERE, name)
        if os.path.isdir(folder):
            shutil.rmtree(folder)
        inp = spec.write(folder)
        if sample == "error":
            r = subprocess.run([oracle.REF_DUMP, "scan", os.path.abspath(inp), "/dev/null"],
                               cwd=folder, capture_output=True, text=True)
            assert r.returncode != 0
            msg = [l for l in r.stderr.splitlines() if "what()" in l or "ERROR" in l][-1]
            msg = msg.split("what():", 1)[-1].strip()
            manifest[name] = {"input": os.path.basename(inp), "error": msg}
            print(name, "reference error:", msg)
            continue
        tmp = os.path.join(folder, "_ref.bin")
        rec = oracle.ref_scan(inp, tmp, block[:2], block[2:])
        os.remove(tmp)
        out = {
            "i": rec[:, 0].astype(np.int32), "j": rec[:, 1].astype(np.int32),
            "k": rec[:, 2].astype(np.int32), "steps": rec[:, 3].astype(np.int32),
            "tip": rec[:, 4:7], "force": rec[:, 13:16], "energy": rec[:, 16],
            "r": rec[:, 20], "angle": rec[:, 21], "block": np.array(block, dtype=np.int32),
        }
        sysinfo = oracle.ref_system(inp, os.path.join(folder, "_sys.txt"))
        os.remove(os.path.join(folder, "_sys.txt"))
        atoms = sysinfo["atoms"]
        out["sys_types"] = np.array([a[0] for a in atoms])
        out["sys_pos"] = np.array([a[1:4] for a in atoms])
        out["sys_charge"] = np.array([a[4] for a in atoms])
        out["sys_tip_dummy_d"] = np.array(sysinfo["tip_dummy_d"])
        out["sys_offset"] = np.array(sysinfo["offset"])
        out["sys_n_points"] = np.array(sysinfo["n_points"], dtype=np.int32)
        out["sys_xyz_charges"] = np.array(int(sysinfo["xyz_charges"]), dtype=np.int32)
        if sample == "states":
            n = out["sys_n_points"]
            i, j = (n[0] * n[1] // 2) // n[1], (n[0] * n[1] // 2) % n[1]
            sbin = os.path.join(folder, "_states.bin")
            subprocess.run([oracle.REF_DUMP, "states", os.path.abspath(inp), sbin, str(i), str(j)],
                           check=True, cwd=folder, stdout=subprocess.DEVNULL,
                           stderr=subprocess.DEVNULL)
            out["states"] = np.fromfile(sbin).reshape(int(n[2]), -1, 3)
            out["states_column"] = np.array([i, j], dtype=np.int32)
            os.remove(sbin)
        elif sample:
            pts = sample_points(name, spec)
            fe = oracle.ref_sample(inp, pts, sample, os.path.join(folder, "_s"))
            for ext in (".pts", ".fe"):
                os.remove(os.path.join(folder, "_s" + ext))
            out["sample_pts"] = pts
            out["sample_fe"] = fe
            out["sample_mode"] = np.array(0 if sample == "sample_ts" else 1, dtype=np.int32)
        np.savez_compressed(os.path.join(folder, "ref.npz"), **out)
        manifest[name] = {"input": os.path.basename(inp), "block": list(block),
                          "points": int(len(rec)), "sample": sample}
        print(name, len(rec), "points, mean steps", rec[:, 3].mean())
    for name, spec in cli_cases():
        if only and name not in only:
            continue
        manifest[name] = make_cli_fixture(name, spec)
        print(name, manifest[name]["rows"], "rows from the reference executable")
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
