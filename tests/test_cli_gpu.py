"""The drop-in executable `mechafm-gpu INPUT OUTPUT` on the GPU against the
reference executable's own output (tests/golden/cli_*): every scan-file row,
and for a flexible molecule the middle pixel's state_*.xyz files.  The
default (double-float) and the plain FP64 kernels match the reference to
rounding (FP64 bit for bit on LJ terms), so the printed numbers are compared
to within one unit of their last printed digit.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, MANIFEST, ROOT

CLI = os.path.join(ROOT, "mechafm_gb300", "bin", "mechafm-gpu")
CASES = sorted(k for k, v in MANIFEST.items() if v.get("cli"))


def _rows(path):
    out = {}
    for line in open(path).read().splitlines():
        name, row = line.split("\t", 1)
        if row.startswith("%") or not row.strip():
            continue
        t = row.split()
        out[(name, int(t[1]), int(t[2]))] = [float(x) for x in t[3:]]
    return out


def _run(name, tmp_path, precision=""):
    folder = os.path.join(GOLDEN, name)
    inp = os.path.join(folder, MANIFEST[name]["input"])
    out = str(tmp_path / "out") + "/"
    env = dict(os.environ)
    env.pop("MAFM_PRECISION", None)
    if precision:
        env["MAFM_PRECISION"] = precision
    r = subprocess.run([CLI, inp, out], cwd=folder, capture_output=True, text=True, timeout=600,
                       env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    return folder, out, r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["", "fp64"])
@pytest.mark.parametrize("name", CASES)
def test_cli_rows_match_reference_executable(name, precision, tmp_path):
    folder, out, stdout = _run(name, tmp_path, precision)
    got_lines = []
    for fn in sorted(os.listdir(out)):
        if fn.startswith("scan-"):
            got_lines += [fn + "\t" + l.rstrip("\n") for l in open(os.path.join(out, fn))]
    tmp = tmp_path / "rows.txt"
    tmp.write_text("\n".join(got_lines) + "\n")
    got, want = _rows(str(tmp)), _rows(os.path.join(folder, "cli_rows.txt"))
    assert got.keys() == want.keys()
    for key in want:
        # columns: x y z (3 dec), F (4), r_vec (3), r (3), angle (4), E (4), steps
        g, w = np.array(got[key]), np.array(want[key])
        tol = np.array([1e-3] * 3 + [1e-4] * 3 + [1e-3] * 4 + [1e-4] * 2 + [0])
        assert (np.abs(g[:-1] - w[:-1]) <= tol[:-1] + 1e-9).all(), (key, g, w)
    assert "Computed %d tip positions" % len(want) in stdout


@pytest.mark.gpu
def test_cli_flexible_state_files(tmp_path):
    folder, out, stdout = _run("cli_flex", tmp_path)
    want = open(os.path.join(folder, "cli_states.txt")).read().splitlines()
    got = []
    for fn in sorted(os.listdir(out)):
        if fn.startswith("state_"):
            got += [fn + "\t" + l.rstrip("\n") for l in open(os.path.join(out, fn))]
    assert len(got) == len(want)
    for g, w in zip(got, want):
        gn, gr = g.split("\t", 1)
        wn, wr = w.split("\t", 1)
        assert gn == wn
        gt, wt = gr.split(), wr.split()
        assert len(gt) == len(wt)
        if len(wt) == 4:
            assert gt[0] == wt[0]
            assert np.abs(np.array(gt[1:], float) - np.array(wt[1:], float)).max() <= 1e-4 + 1e-9
        else:
            assert gt == wt
    assert "+- Wrote" in stdout


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_cli_stdout_matches_reference_executable(name, tmp_path):
    """The whole stdout against the reference executable's: the same lines
    before the relaxation and after it (run times masked, step totals to
    1 %), the same state
    files reported, and the reference's progress lines a prefix of ours (its
    pixel counter is shared by OpenMP threads without synchronisation, so it
    can stop short of 100 %; ours prints all ten)."""
    import re
    from test_cli_args import cli_stdout
    ours, ref, rc = cli_stdout(name, tmp_path)
    assert rc == 0
    ours = [re.sub(r"(wall time is|simulation took) [0-9.]+ seconds", r"\1 # seconds", l) for l in ours]
    k, e = ref.index("+- Starting simulation"), ref.index("+- Simulation run finished")
    ko, eo = ours.index("+- Starting simulation"), ours.index("+- Simulation run finished")
    assert ours[:k + 1] == ref[:k + 1]
    # the step totals: FP64 kernels agree with the reference to rounding, so
    # a FIRE decision may flip on a near-tie (1 %); every other line exactly
    tail, tail_ref = ours[eo:], ref[e:]
    assert len(tail) == len(tail_ref)
    for a, b in zip(tail, tail_ref):
        if "minimization steps" in a:
            na, nb = float(re.findall(r"[0-9.]+", a)[0]), float(re.findall(r"[0-9.]+", b)[0])
            assert re.sub(r"[0-9.]+", "#", a) == re.sub(r"[0-9.]+", "#", b)
            assert abs(na - nb) <= 0.01 * nb, (a, b)
        else:
            assert a == b
    mid, mid_ref = ours[ko + 1:eo], ref[k + 1:e]
    wrote = sorted(l for l in mid if l.startswith("+- Wrote"))
    assert wrote == sorted(l for l in mid_ref if l.startswith("+- Wrote"))
    fin = [l for l in mid if l.startswith("+- Finished")]
    fin_ref = [l for l in mid_ref if l.startswith("+- Finished")]
    assert fin == ["+- Finished %4.1f %% of the simulation" % (10.0 * (i + 1)) for i in range(10)]
    assert fin[:len(fin_ref)] == fin_ref
    assert len(mid) == len(wrote) + len(fin)



@pytest.mark.gpu
def test_cli_rigid_grid_default_matches_fp64(tmp_path):
    """A rigid-grid scan through the executable: the default (double-float
    grid build and relaxation) against MAFM_PRECISION=fp64 (the FP64 grid
    and kernel), row for row, within one unit of the last printed digit and
    with equal step counts."""
    folder = os.path.join(GOLDEN, "graphene_grid")
    inp = os.path.join(folder, MANIFEST["graphene_grid"]["input"])
    rows = {}
    for prec in ("", "fp64"):
        out = str(tmp_path / f"out_{prec or 'df'}") + "/"
        env = dict(os.environ)
        env.pop("MAFM_PRECISION", None)
        if prec:
            env["MAFM_PRECISION"] = prec
        r = subprocess.run([CLI, inp, out], cwd=folder, capture_output=True, text=True, timeout=600,
                           env=env)
        assert r.returncode == 0, r.stderr[-2000:]
        lines = []
        for fn in sorted(os.listdir(out)):
            if fn.startswith("scan-"):
                lines += [fn + "\t" + l.rstrip("\n") for l in open(os.path.join(out, fn))]
        path = tmp_path / f"rows_{prec or 'df'}.txt"
        path.write_text("\n".join(lines) + "\n")
        rows[prec] = _rows(str(path))
    got, want = rows[""], rows["fp64"]
    assert got.keys() == want.keys() and len(want) == MANIFEST["graphene_grid"]["points"]
    tol = np.array([1e-3] * 3 + [1e-4] * 3 + [1e-3] * 4 + [1e-4] * 2)
    for key in want:
        g, w = np.array(got[key]), np.array(want[key])
        assert (np.abs(g[:-1] - w[:-1]) <= tol + 1e-9).all(), (key, g, w)
        assert g[-1] == w[-1], (key, g[-1], w[-1])
