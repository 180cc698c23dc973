"""The scan-file writer formats numbers itself (no printf per field); its
output must equal printf's "%6.3f" / "%8.4f" / "%d" for every double,
including exact ties (rounded to even on the exact binary value), negative
values that round to zero ("-0.000"), signed zeros, subnormals, values
beyond 1e12 and infinities.  Python's %-formatting rounds the same way
(correctly rounded, ties to even), so it is the reference here.
"""
import os

import numpy as np

from mechafm_gb300 import _abi, synth
from mechafm_gb300.scan import Input


def _edge_values(rng, n):
    ties3 = (np.arange(-2000, 2000) + 0.5) / 1000.0        # near x.xxx5: inexact in binary
    exact = np.array([0.0625, -0.0625, 0.3125, 2.5e-4, 1.5, -1.5, 0.0005, -0.0005, 1e-4,
                      -1e-4, -0.0, 0.0, 5e-324, -5e-324, 1e-310, 123456.78905, 999999.99995,
                      1e11 + 0.00005, -1e11, 1e12, 3.3e13, -7.7e20, 1e300, np.inf, -np.inf,
                      2.0 ** -20, 0.00015, 0.00025, 0.00035, 12.34565, -12.34565])
    rnd = np.concatenate([rng.normal(0, 3, n), rng.normal(0, 1e-3, n), rng.uniform(-1e6, 1e6, n)])
    halves = np.round(rng.uniform(-50, 50, n) * 2 ** 12) / 2 ** 12       # exact binary ties
    return np.concatenate([ties3, exact, rnd, halves])


def test_writer_formats_like_printf(tmp_path):
    spec = synth.graphene_72(area=3.0, step=0.1, zhigh=10.0, zlow=9.0)
    inp = Input(spec.write(str(tmp_path / "in")))
    d = inp.desc()
    rng = np.random.default_rng(5)
    vals = _edge_values(rng, 4000)
    n = d.n_points
    pts = np.zeros(n, dtype=_abi.POINT_DTYPE)
    pick = lambda: vals[rng.integers(0, len(vals), n)]
    for c in range(3):
        pts["force"][:, c] = pick()
    pts["energy"] = pick()
    pts["tip"][:, 0] = pick()
    pts["tip"][:, 1] = pick()
    pts["tip"][:, 2] = rng.normal(6, 1, n)
    pts["steps"] = rng.integers(0, 100000, n)
    out = tmp_path / "out"
    out.mkdir()
    inp.write_output(pts, str(out), gzip=False)
    nx, ny, nz = d.shape
    rows = {}
    for fn in os.listdir(out):
        if not fn.startswith("scan-"):
            continue
        for line in open(out / fn):
            if line.startswith("%"):
                continue
            k, i, j = (int(t) for t in line.split()[:3])
            rows[(k, i, j)] = line.rstrip("\n")
    assert len(rows) == n
    zk = d.c.zhigh
    checked = 0
    for k in range(nz):
        for i in range(nx):
            for j in range(ny):
                p = pts[(i * ny + j) * nz + k]
                x, y = i * d.c.dx, j * d.c.dy
                rx, ry, rz = p["tip"][0] - x, p["tip"][1] - y, p["tip"][2] - zk
                with np.errstate(all="ignore"):
                    r = np.sqrt(rx * rx + ry * ry + rz * rz)
                line = rows[(k, i, j)]
                # every field but the angle, with printf's padding
                prefix = "%d %d %d %6.3f %6.3f %6.3f %8.4f %8.4f %8.4f %6.3f %6.3f %6.3f " % (
                    k, i, j, x, y, zk, p["force"][0], p["force"][1], p["force"][2], rx, ry, rz)
                assert line.startswith(prefix), (line, prefix)
                rest = line[len(prefix):]
                if np.isfinite(r):
                    assert rest.startswith("%6.3f " % r), (rest, r)
                suffix = " %8.4f %d" % (p["energy"], p["steps"])
                assert line.endswith(suffix), (line, suffix)
                checked += 1
        zk -= d.c.dz
    assert checked == n
