"""The drop-in executable `mechafm-gpu INPUT OUTPUT` on the GPU against the
reference executable's own output (tests/golden/cli_*): every scan-file row,
and for a flexible molecule the middle pixel's state_*.xyz files.  The FP64
kernels match the reference to rounding (bit for bit on LJ terms), so the
printed numbers are compared to within one unit of their last printed digit.
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


def _run(name, tmp_path):
    folder = os.path.join(GOLDEN, name)
    inp = os.path.join(folder, MANIFEST[name]["input"])
    out = str(tmp_path / "out") + "/"
    r = subprocess.run([CLI, inp, out], cwd=folder, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return folder, out, r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_cli_rows_match_reference_executable(name, tmp_path):
    folder, out, stdout = _run(name, tmp_path)
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
