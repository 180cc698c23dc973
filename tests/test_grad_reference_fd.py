"""Adjoint gradients against finite differences of the reference's own
relaxation (the reference has no derivatives).

tests/golden/grad_ref was made by tests/golden/make_grad_golden.py: central
differences of L = sum_p w_p Fz_p over a tightly converged cluster scan,
with the reference's code run on perturbed input files (xyz positions and
charges, parameter-file epsilon / sigma per type, the Morse pair_ovwrt
line).  The adjoint gives dL with respect to the prepared positions,
charges and tip pair parameters; the chain rule of the reference's set-up
maps them to the file parameters:

  x, y of atom a   g[a] - mean_b g[b]   (centring on the mean x, y,
                                          system.cpp:119-136); z: g[a]
  epsilon of T     (g_es6 es6 + g_es12 es12) / (2 eps_T)
  sigma of T       (3 g_es6 es6 + 6 g_es12 es12) / sig_mix
                   (eps = sqrt(eps_tip eps_T), sig_mix = (sig_tip + sig_T) / 2,
                    es6 = 4 eps sig^6, es12 = 4 eps sig^12; simulation.cpp:261-264)
  Morse De, a, re  the tip pair's three parameters directly

Tolerance: 1e-4 relative (the adjoint bar) of max(|fd|, 1e-3 max|fd|).
"""
import os

import numpy as np
import pytest

import oracle
from mechafm_gb300 import _abi
from mechafm_gb300.scan import Input, Scan

DIR = os.path.join(os.path.dirname(__file__), "golden", "grad_ref")
REF = np.load(os.path.join(DIR, "ref.npz"))
REL = 1e-4


def _files():
    with open(os.path.join(DIR, "cluster_60.xyz")) as f:
        lines = f.read().splitlines()
    names = [l.split()[0] for l in lines[2:2 + int(lines[0])]]
    params = {}
    with open(os.path.join(DIR, "cluster_60.par")) as f:
        for l in f:
            c = l.split()
            if c and c[0] == "atom":
                params[c[1]] = (float(c[2]), float(c[3]))
    return names, params


def file_gradients(desc, g):
    """The adjoint's gradients mapped to the golden's file parameters."""
    names, params = _files()
    d = desc.c
    types = np.ctypeslib.as_array(d.type, shape=(d.n_atoms,))
    tidx = {n: int(types[names.index(n)]) for n in set(names)}
    dpos = g["dpos"]
    mean = dpos.mean(axis=0)
    eps_tip, sig_tip = params["O"]
    out = {}
    for name in REF["names"]:
        name = str(name)
        if name.startswith("pos"):
            a, k = map(int, name[3:].split("."))
            out[name] = dpos[a, k] - (mean[k] if k < 2 else 0.0)
        elif name.startswith("q"):
            out[name] = g["dcharge"][int(name[1:])]
        elif name.startswith("morse"):
            out[name] = g["dpair"][tidx["O"], int(name.split(".")[1])]
        else:
            kind, T = name.split(".")
            t = tidx[T]
            es6, es12 = d.tip_pair[t].p[0], d.tip_pair[t].p[1]
            g6, g12 = g["dpair"][t, 0], g["dpair"][t, 1]
            if kind == "eps":
                out[name] = (g6 * es6 + g12 * es12) / (2 * params[T][0])
            else:
                sig = 0.5 * (sig_tip + params[T][1])
                out[name] = (3 * g6 * es6 + 6 * g12 * es12) / sig
    return out


def check(got):
    fd = REF["fd"]
    floor = 1e-3 * np.abs(fd).max()
    bad = []
    for name, want in zip(REF["names"], fd):
        ad = got[str(name)]
        if abs(ad - want) > REL * max(abs(want), floor):
            bad.append((str(name), ad, want))
    assert not bad, bad


def test_oracle_relaxation_is_the_reference():
    desc = Input(os.path.join(DIR, "cluster_60.scan")).desc()
    pts, _ = oracle.run(desc)
    np.testing.assert_array_equal(pts["force"][:, 2], REF["fz0"])


def test_oracle_adjoint_matches_reference_differences():
    desc = Input(os.path.join(DIR, "cluster_60.scan")).desc()
    pts, _ = oracle.run(desc)
    check(file_gradients(desc, oracle.adjoint(desc, pts, REF["w"])))


@pytest.mark.gpu
def test_gpu_adjoint_matches_reference_differences():
    desc = Input(os.path.join(DIR, "cluster_60.scan")).desc()
    scan = Scan(desc, device=0)
    pts, _ = scan.run(_abi.FP64)
    np.testing.assert_array_equal(pts["force"][:, 2], REF["fz0"])
    check(file_gradients(desc, scan.adjoint(pts, REF["w"])))
    scan.close()
