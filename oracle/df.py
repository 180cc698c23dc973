"""ORACLE — test infrastructure, not product.

numpy restatement of the reference's frequency-shift post-processing
(simple-vafm-image.py), used only by tests/ to check libmafm's mafm_df and
mafm_df_adjoint.  The script is Python 2 with matplotlib and file globbing;
this follows its arithmetic line by line, and is pinned to the script's own
results (tests/golden/df_script, made by running the script under Python 3
with its plotting stubbed on scan files written by the reference
executable): weights and images bit for bit.

* weights: simple-vafm-image.py:77-89 (Giessibl, Beilstein J. Nanotechnol.
  3:238, 2012) — fshiftfac, the ampcut precaution (Python float % and //),
  zosc from numpy.arange, the mirrored offsets without -zosc[1] and -zosc[0],
  W = z / sqrt(|A^2 - z^2|) with both ends dropped;
* windows: :116-199 — the scan files sorted by name (ascending height, the
  writer's %06.3f names), window pl holding heights pl .. pl+nosc-1;
* image: :204 — DF = -fshiftfac * sum_m(FZ * W) * dz.
"""
from __future__ import annotations

import numpy as np

NM2KCALAA = 1.438978


def weights(dz, amplitude=0.50, k_cantilever=1800 * NM2KCALAA, f0=25.000e3):
    fshiftfac = (f0 / (2 * k_cantilever)) * (2 / (np.pi * amplitude * amplitude))
    ampcut = (1 + (amplitude / dz)) % (1 + (amplitude // dz))
    if ampcut < 0.01:
        amplitude += dz / 2
    z = np.arange(0, amplitude + dz, dz)
    z = np.concatenate((-z[-1:1:-1], z))
    w = z / np.sqrt(abs((amplitude ** 2) - (z ** 2)))
    return w[1:-1], fshiftfac


def df_images(fz_levels, dz, **prm):
    """fz_levels (nx, ny, nz) with k = 0 at zhigh -> df (nshift, nx, ny)."""
    w, fac = weights(dz, **prm)
    asc = fz_levels[:, :, ::-1]                 # ascending heights, as the sorted files
    nosc = len(w)
    nshift = asc.shape[2] - nosc
    out = np.zeros((max(nshift, 0),) + asc.shape[:2])
    for pl in range(nshift):
        FZ = asc[:, :, pl:pl + nosc]
        out[pl] = -fac * (FZ * w).sum(axis=2) * dz
    return out


def df_adjoint(g_df, nz, dz, **prm):
    """Transpose of df_images: g_df (nshift, nx, ny) -> dL/dFz (nx, ny, nz), level order."""
    w, fac = weights(dz, **prm)
    nosc = len(w)
    nshift, nx, ny = g_df.shape
    asc = np.zeros((nx, ny, nz))
    for pl in range(nshift):
        asc[:, :, pl:pl + nosc] += (-fac * dz) * g_df[pl][:, :, None] * w
    return asc[:, :, ::-1]
