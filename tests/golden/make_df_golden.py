"""Golden vectors of the frequency-shift post-processing, made by the
reference's own script.

Run where the reference exists:
    MAFM_REFERENCE_DIR=<reference checkout> python tests/golden/make_df_golden.py

simple-vafm-image.py is a Python 2 script that plots with matplotlib and
writes only images.  This generator runs the script itself, read from the
reference tree at run time and never copied into this repository, under
Python 3:

* four mechanical source edits, none of which touches its arithmetic:
  `print x` statements become `print(x)`, `ur'...'` literals become
  `r'...'`, and execution stops at the "Creating animated gifs" line
  (ImageMagick calls follow);
* `map` and `filter` in the script's namespace return lists, as in Python 2;
* matplotlib is replaced by an inert stand-in whose `figure(0)`, called by
  the script right after each `DF = ...` line (simple-vafm-image.py:204-208),
  records a copy of each new DF.

Input: scan files written by the reference executable (oracle/_ref/mechafm-omp)
for a small cluster scan with 21 heights, so the script sees the reference's
own output format.  Stored in tests/golden/df_script/ref.npz:

  fz        (nx, ny, nz) Fz read from the scan files (k = 0 at zhigh)
  dz        height step
  df        (nshifts, nx, ny) the script's frequency-shift images
  W, fshiftfac, nosc, nshifts   the script's weights and window counts
  steps, sw, sfac               W and fshiftfac of the weight block
                                (simple-vafm-image.py:76-89) run alone for
                                each step in `steps` (sw padded with NaN)
"""
from __future__ import annotations

import builtins
import os
import re
import shutil
import subprocess
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from mechafm_gb300 import synth  # noqa: E402

# the reference checkout comes from $MAFM_REFERENCE_DIR (read-only)
SCRIPT = os.path.join(oracle.reference_dir() or "", "simple-vafm-image.py")
STEPS = [0.1, 0.05, 0.2, 0.25, 0.125, 0.3, 0.07, 0.5 / 3]


def py3_source(text: str) -> str:
    """The script's text with the Python 2 constructs it uses made valid Python 3."""
    stop = text.index("print 'Creating animated gifs'")
    text = text[:stop]
    text = re.sub(r"(?m)^(\s*)print\s+(.+?)\s*$", r"\1print(\2)", text)
    text = re.sub(r"\bur'", "r'", text)
    return text


class _Inert:
    """Accepts any attribute access and call (stands in for matplotlib)."""

    def __getattr__(self, name):
        return _Inert()

    def __call__(self, *a, **k):
        return _Inert()

    def __iter__(self):
        return iter(())


def _fake_matplotlib(record):
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    ticker = types.ModuleType("matplotlib.ticker")

    def figure(num=None, *a, **k):
        if num == 0:
            record()
        return _Inert()

    for name in ("contourf", "colorbar", "savefig", "get_cmap", "clf", "close", "subplots"):
        setattr(plt, name, _Inert())
    plt.figure = figure
    ticker.MultipleLocator = _Inert()
    ticker.FormatStrFormatter = _Inert()
    mpl.pyplot = plt
    mpl.ticker = ticker
    mpl.use = _Inert()
    return {"matplotlib": mpl, "matplotlib.pyplot": plt, "matplotlib.ticker": ticker}


def py2_namespace():
    ns = {"__name__": "__main__", "__builtins__": builtins}
    ns["map"] = lambda f, *s: list(builtins.map(f, *s))
    ns["filter"] = lambda f, s: list(builtins.filter(f, s))
    return ns


def run_script(src: str, inp: str, outdir: str):
    """Run the script on the scan files in outdir; returns (namespace, DF list)."""
    ns = py2_namespace()
    dfs, seen = [], []

    def record():   # figure(0) opens each of a step's three plots; DF is new once per step
        if not seen or ns["DF"] is not seen[-1]:
            seen.append(ns["DF"])
            dfs.append(np.array(ns["DF"], copy=True))

    fakes = _fake_matplotlib(record)
    saved = {k: sys.modules.get(k) for k in fakes}
    argv = sys.argv
    try:
        sys.modules.update(fakes)
        sys.argv = ["simple-vafm-image.py", "-i", inp, "-o", outdir]
        exec(compile(src, SCRIPT, "exec"), ns)
    finally:
        sys.argv = argv
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return ns, dfs


def weight_block(text: str, dz: float):
    """The script's weight lines (Nm2kcalAA ... W = W[1:-1]) run alone for dz."""
    a = text.index("Nm2kcalAA = 1.438978")
    b = text.index("W = W[1:-1]")
    b = text.index("\n", b)
    ns = py2_namespace()
    ns["numpy"] = np
    ns["dz"] = dz
    exec(compile(text[a:b], SCRIPT, "exec"), ns)
    return np.array(ns["W"]), float(ns["fshiftfac"])


def main():
    oracle.build()
    if not oracle.ref_available():
        raise SystemExit("reference build missing")
    with open(SCRIPT) as f:
        text = f.read()
    src = py3_source(text)

    # the script takes heights from the file names split at '-', so the
    # folder's path must hold none
    work = tempfile.mkdtemp(prefix="dfgold", dir="/tmp")
    assert "-" not in work
    try:
        spec = synth.cluster_60(area=1.0, step=0.25, zhigh=10.0, zlow=8.0, dz=0.1)
        inp = spec.write(work)
        out = os.path.join(work, "out")
        subprocess.run([oracle.REF_CLI, inp, out], check=True, cwd=work,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        ns, dfs = run_script(src, inp, out + "/")
        # Fz per point from the same files, k = 0 at zhigh
        files = sorted((f for f in os.listdir(out) if f.startswith("scan-")), reverse=True)
        nx, ny, nz = int(ns["nx"]), int(ns["ny"]), len(files)
        fz = np.zeros((nx, ny, nz))
        for k, fn in enumerate(files):
            with open(os.path.join(out, fn)) as f:
                for line in f:
                    if line.startswith("%"):
                        continue
                    c = line.split()
                    fz[int(c[1]), int(c[2]), k] = float(c[8])
        dz = float(ns["dz"])
    finally:
        shutil.rmtree(work)

    sw = np.full((len(STEPS), 64), np.nan)
    sfac = np.zeros(len(STEPS))
    for i, s in enumerate(STEPS):
        w, fac = weight_block(text, s)
        sw[i, :len(w)] = w
        sfac[i] = fac

    dest = os.path.join(HERE, "df_script")
    os.makedirs(dest, exist_ok=True)
    np.savez(os.path.join(dest, "ref.npz"), fz=fz, dz=dz, df=np.array(dfs),
             W=np.array(ns["W"]), fshiftfac=float(ns["fshiftfac"]), nosc=int(ns["nosc"]),
             nshifts=int(ns["nshifts"]), steps=np.array(STEPS), sw=sw, sfac=sfac)
    print(f"df_script: {len(dfs)} images of {nx}x{ny}, nosc {ns['nosc']}, dz {dz}")


if __name__ == "__main__":
    main()
