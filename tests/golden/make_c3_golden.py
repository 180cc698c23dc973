"""Golden vectors of the full-size external field (the 2048-atom periodic slab
with its 160 x 160 x 120 Hartree cube), made by the reference's own code.

Run where the reference exists:
    MAFM_REFERENCE_DIR=<reference checkout> python tests/golden/make_c3_golden.py

The cube is 40 MB of text, too large to commit, but the seeded generator
(mechafm_gb300.synth.slab) writes it again bit for bit, so the fixture keeps
the generator's arguments and the SHA-256 of every file it writes; the tests
regenerate the files and check the hashes before they compare anything.

tests/golden/slab_c3/ref.npz holds
  es_pts, es_fe      4000 seeded tip positions over the periodic cell and the
                     scan's heights, and the reference's external-field force
                     and energy there: ElectrostaticPotentialInteraction
                     (interactions.cpp:53-242), whose field the reference
                     computes with kiss_fft (fft.cpp:11-94, kiss_fftnd.c).
                     Sampled on the same slab with rigidgrid off (field_spec):
                     with a rigid grid the reference folds the interaction
                     into the grid, and its tip–surface list holds no
                     ElectrostaticPotentialInteraction to evaluate
  steps, tip, force, energy
                     the reference's relaxed points of the 8 x 8 pixel block
                     at the origin of the same scan geometry (rigid grid of
                     the slab's 18,432 image terms plus the field,
                     simulation.cpp:420-501), i.e. the scan with pixels = 8
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from mechafm_gb300 import synth  # noqa: E402

FOLDER = os.path.join(HERE, "slab_c3")
# the bench's slab workload, cropped to its first 8 x 8 pixels
SPEC = {"pixels": 8, "zhigh": 18.0, "zlow": 14.0, "tip_charge": -0.02}
N_SAMPLES = 4000


def spec():
    return synth.slab(**SPEC)


def field_spec():
    """The same slab and cube without the rigid grid (the field samples)."""
    return synth.slab(**SPEC, rigidgrid=False)


def file_hashes(folder: str) -> dict:
    out = {}
    for fn in sorted(os.listdir(folder)):
        if fn.startswith("_") or fn.endswith(".npz") or fn.endswith(".json"):
            continue
        with open(os.path.join(folder, fn), "rb") as f:
            out[fn] = hashlib.sha256(f.read()).hexdigest()
    return out


def sample_points(n: int = N_SAMPLES, seed: int = 17) -> np.ndarray:
    """Tip positions over the whole 40 x 40 A periodic cell (the field repeats)
    at the heights the scan's tip visits (dummy 18 -> 14 A, tip ~4 A below)."""
    rng = np.random.default_rng(seed)
    return np.column_stack([rng.uniform(0, 40.0, n), rng.uniform(0, 40.0, n),
                            rng.uniform(9.5, 15.0, n)])


def main():
    oracle.build()
    if not oracle.ref_available():
        raise SystemExit("reference build missing")
    if os.path.isdir(FOLDER):
        shutil.rmtree(FOLDER)
    os.makedirs(FOLDER)
    work = os.path.join(FOLDER, "_work")
    inp = spec().write(work)
    fwork = os.path.join(FOLDER, "_field")
    finp = field_spec().write(fwork)
    pts = sample_points()
    fe = oracle.ref_sample(finp, pts, "sample_es", os.path.join(fwork, "_s"))
    if not np.abs(fe).max() > 0:
        raise SystemExit("the reference sampled no external field")
    rec = oracle.ref_scan(inp, os.path.join(work, "_ref.bin"), (0, 8), (0, 8))
    meta = {"spec": SPEC, "input": os.path.basename(inp), "sha256": file_hashes(work),
            "sha256_field": file_hashes(fwork), "points": int(len(rec))}
    np.savez_compressed(os.path.join(FOLDER, "ref.npz"), es_pts=pts, es_fe=fe,
                        steps=rec[:, 3].astype(np.int32), tip=rec[:, 4:7], force=rec[:, 13:16],
                        energy=rec[:, 16])
    with open(os.path.join(FOLDER, "meta.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    shutil.rmtree(work)
    shutil.rmtree(fwork)
    print("slab_c3:", N_SAMPLES, "field samples,", len(rec), "points, mean steps",
          rec[:, 3].mean())


if __name__ == "__main__":
    main()
