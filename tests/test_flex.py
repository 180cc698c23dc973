"""Flexible molecules (`flexible on`): the host topology, the oracle's
restatement and the GPU kernel against the reference's own results
(tests/golden/flex_*: naphthalene plus a separate H2, with bonds, angles,
dihedrals, non-bonded pairs between the fragments, the substrate wall, XY
tethers and one fixed atom; midpoint and RK4).

The oracle evaluates the reference's interaction list in order with the same
C library (exp, acos, sin, atan), so it is bit-identical to the reference
here.  The GPU kernel sums every atom's force in the same order but uses
CUDA's transcendental functions: within 1e-6 A of the reference's tip and atom
positions and 1e-6 relative in force where FIRE took the same steps (at least
95 % of the points).
"""
import numpy as np
import pytest

import oracle
from conftest import FLEX_CASES, golden
from mechafm_gb300 import _abi
from mechafm_gb300.scan import FlexScan, Input


def _load(name):
    case = golden(name)
    inp = Input(case.input)
    return case, inp, inp.desc(), inp.flex_desc()


def test_flexible_topology_counts():
    """naphthalene: 11 C-C + 8 C-H bonds; H2: 1 bond; no pairs inside a fragment."""
    _, inp, desc, flex = _load("flex_naph")
    f = flex.c
    assert desc.c.flexible == 1
    assert f.n_bonds == 20
    assert f.n_pairs == 18 * 2          # every ring atom with both H2 atoms
    fixed = np.ctypeslib.as_array(f.fixed, shape=(desc.c.n_atoms,))
    assert (fixed == 1).sum() == 1 and (fixed == 2).sum() == 2


def test_rigid_entry_points_refuse_flexible_molecules():
    _, inp, desc, _ = _load("flex_naph")
    from mechafm_gb300.scan import Scan
    with pytest.raises(_abi.MafmError) as e:
        Scan(desc, device=0)
    assert e.value.code == _abi.MAFM_E_UNSUPPORTED


@pytest.mark.parametrize("name", FLEX_CASES)
def test_oracle_matches_reference(name):
    case, inp, desc, flex = _load(name)
    ref = case.ref
    parts = [oracle.flex_run(desc, flex, c0, c1)[0] for c0, c1 in case.columns(desc.c.ny)]
    pts = np.concatenate(parts)
    np.testing.assert_array_equal(pts["steps"], ref["steps"])
    np.testing.assert_array_equal(pts["tip"], ref["tip"])
    np.testing.assert_array_equal(pts["force"], ref["force"])
    np.testing.assert_array_equal(pts["energy"], ref["energy"])
    i, j = ref["states_column"]
    col = int(i) * desc.c.ny + int(j)
    _, _, states = oracle.flex_run(desc, flex, col, col + 1, state_column=col)
    np.testing.assert_array_equal(states, ref["states"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", FLEX_CASES)
def test_gpu_matches_reference(name):
    case, inp, desc, flex = _load(name)
    ref = case.ref
    scan = FlexScan(desc, flex, device=0)
    parts = []
    for c0, c1 in case.columns(desc.c.ny):
        p, _, _ = scan.run(c0, c1)
        parts.append(p)
    pts = np.concatenate(parts)
    same = pts["steps"] == ref["steps"]
    assert same.mean() >= 0.95, same.mean()
    d = np.abs(pts["tip"] - ref["tip"]).max(axis=1)
    assert d[same].max() < 1e-6, d[same].max()
    scale = np.maximum(np.abs(ref["force"]), 1e-3)
    assert (np.abs(pts["force"] - ref["force"]) / scale)[same].max() < 1e-6
    i, j = ref["states_column"]
    col = int(i) * desc.c.ny + int(j)
    _, _, states = scan.run(col, col + 1, state_column=col)
    np.testing.assert_allclose(states, ref["states"], rtol=0, atol=1e-6)


@pytest.mark.gpu
def test_gpu_full_scan_matches_oracle():
    """Every column of the case through one launch, against the oracle."""
    _, inp, desc, flex = _load("flex_naph")
    pts, st, _ = FlexScan(desc, flex, device=0).run()
    want, steps, _ = oracle.flex_run(desc, flex)
    same = pts["steps"] == want["steps"]
    assert same.mean() >= 0.95
    assert np.abs(pts["tip"] - want["tip"]).max(axis=1)[same].max() < 1e-6
    assert st.total_steps > 0
