"""Desc.crop: a pixel block of a scan run as a scan of its own gives the same
points as that block of the full scan (oracle port, FP64, CPU).

The crop moves the surface, the cell offset and the external field's origin by
-(i0 dx, j0 dy); tip–surface separations then differ from the full scan's only
by the rounding of that shift, and the crop's rigid grid lies on the same
lattice, so points agree to 1e-9 A / 1e-9 relative.
"""
import numpy as np
import pytest

import oracle
from conftest import golden
from mechafm_gb300.scan import Input


def _block(desc, pts, i0, j0, ni, nj):
    d = desc.c
    p = pts.reshape(d.nx, d.ny, d.nz)
    return p[i0:i0 + ni, j0:j0 + nj].reshape(-1)


@pytest.mark.parametrize("case,block", [("graphene_ef", (3, 5, 4, 3)),
                                        ("graphene_pbc", (2, 1, 3, 4)),
                                        ("graphene_grid", (1, 2, 3, 3)),
                                        ("slab_es_grid", (1, 1, 2, 2))])
def test_crop_matches_full_scan(case, block):
    desc = Input(golden(case).input).desc()
    i0, j0, ni, nj = block
    full, _ = oracle.run(desc)
    crop = desc.crop(i0, j0, ni, nj)
    part, _ = oracle.run(crop)
    want = _block(desc, full, i0, j0, ni, nj)
    assert (part["steps"] == want["steps"]).mean() > 0.95
    tip = want["tip"].copy()
    tip[:, 0] -= i0 * desc.c.dx
    tip[:, 1] -= j0 * desc.c.dy
    np.testing.assert_allclose(part["tip"], tip, atol=1e-9)
    fz = want["force"][:, 2]
    np.testing.assert_allclose(part["force"][:, 2], fz, rtol=1e-9, atol=1e-9 * np.abs(fz).max())


def test_crop_rejects_outside_blocks():
    desc = Input(golden("graphene_ef").input).desc()
    with pytest.raises(ValueError):
        desc.crop(0, 0, desc.c.nx + 1, 1)
    with pytest.raises(ValueError):
        desc.crop(-1, 0, 2, 2)
