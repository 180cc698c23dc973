"""Golden finite differences of the reference's own relaxation, for the
gradients of libmafm's adjoint (the reference has no derivatives).

Run where the reference exists:
    MAFM_REFERENCE_DIR=<reference checkout> python tests/golden/make_grad_golden.py

The case is the 60-atom cluster over 3 x 3 pixels and 4 heights relaxed to
|F| < 1e-10 (minterm f, ftol 1e-10), so that a difference quotient measures
the derivative and not the stopping tolerance.  For a loss
L = sum_p w_p Fz_p (w seeded normal, points in (i, j, k) order) it perturbs
the reference's INPUT FILES by +-h, runs the reference's code
(oracle/_ref/ref_dump) on the whole scan each time, and stores the central
difference (L+ - L-) / 2h for:

  pos{a}.{k}   coordinate k of atom a in the xyz file (h = 1e-4 A)
  q{a}         the xyz charge of atom a (h = 1e-4 e)
  eps.{T}      the parameter-file epsilon of atom type T (h = 1e-4 relative)
  sig.{T}      the parameter-file sigma of atom type T (h = 1e-4 relative)
  morse.{m}    De, a, re of the pair_ovwrt Morse line (h = 1e-4 relative)

Stored in tests/golden/grad_ref/: the input files and ref.npz with w, the
unperturbed Fz, names, h and fd.  The tests map the adjoint's outputs
(gradients with respect to the prepared positions, charges and tip pair
parameters) to these file parameters by the chain rule of the reference's
set-up: centring on the mean x, y (system.cpp:119-136) and the mixing rules
eps = sqrt(eps1 eps2), sig = (sig1 + sig2) / 2, es6 = 4 eps sig^6,
es12 = 4 eps sig^12 (simulation.cpp:261-264, interactions.hpp:58-64).
"""
from __future__ import annotations

import copy
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from mechafm_gb300 import synth  # noqa: E402

ATOMS = (3, 17, 40)
CHARGES = (5, 22)
TYPES = ("C", "N", "H")          # not O: it is the tip type too


def spec0():
    return synth.cluster_60(area=0.3, step=0.1, zhigh=10.0, zlow=9.7, minterm="f",
                            ftol="1e-10", maxsteps="400000")


def fz_of(spec, work):
    folder = tempfile.mkdtemp(dir=work)
    inp = spec.write(folder)
    rec = oracle.ref_scan(inp, os.path.join(folder, "_r.bin"))
    shutil.rmtree(folder)
    order = np.lexsort((rec[:, 2], rec[:, 1], rec[:, 0]))
    rec = rec[order]
    assert (rec[:, 3] < 400000).all()
    return rec[:, 15]


def variants():
    """(name, h, function(spec, sign))."""
    out = []
    for a in ATOMS:
        for k in range(3):
            def f(s, sg, a=a, k=k):
                s.pos[a, k] += sg * 1e-4
            out.append((f"pos{a}.{k}", 1e-4, f))
    for a in CHARGES:
        def f(s, sg, a=a):
            s.charges[a] += sg * 1e-4
        out.append((f"q{a}", 1e-4, f))
    base = spec0()
    for t in TYPES:
        eps, sig = base.atom_params[t][0], base.atom_params[t][1]
        for m, (nm, v) in enumerate((("eps", eps), ("sig", sig))):
            def f(s, sg, t=t, m=m, v=v):
                p = list(s.atom_params[t])
                p[m] = v + sg * 1e-4 * v
                s.atom_params[t] = tuple(p)
            out.append((f"{nm}.{t}", 1e-4 * v, f))
    ow = base.overwrites[0]
    for m in range(3):
        v = ow[3 + m]

        def f(s, sg, m=m, v=v):
            o = list(s.overwrites[0])
            o[3 + m] = v + sg * 1e-4 * v
            s.overwrites[0] = tuple(o)
        out.append((f"morse.{m}", 1e-4 * v, f))
    return out


def main():
    oracle.build()
    if not oracle.ref_available():
        raise SystemExit("reference build missing")
    dest = os.path.join(HERE, "grad_ref")
    if os.path.isdir(dest):
        shutil.rmtree(dest)
    base = spec0()
    base.write(dest)
    work = tempfile.mkdtemp()
    try:
        fz0 = fz_of(base, work)
        w = np.random.default_rng(3).normal(size=len(fz0))
        names, hs, fds = [], [], []
        for name, h, f in variants():
            lo = []
            for sg in (+1, -1):
                s = copy.deepcopy(base)
                s.pos = base.pos.copy()
                s.charges = base.charges.copy()
                f(s, sg)
                lo.append(float((w * fz_of(s, work)).sum()))
            names.append(name)
            hs.append(h)
            fds.append((lo[0] - lo[1]) / (2 * h))
            print(name, fds[-1])
    finally:
        shutil.rmtree(work)
    np.savez(os.path.join(dest, "ref.npz"), w=w, fz0=fz0, names=np.array(names),
             h=np.array(hs), fd=np.array(fds))


if __name__ == "__main__":
    main()
