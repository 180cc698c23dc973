"""The input front-end (parse.cpp / cube_io.cpp / Simulation::initialize
restated in C++): prepared System state against the reference's own dump, and
error messages and status codes for malformed inputs.  Where the reference
build exists (oracle/_ref), each malformed input is also run through the
reference executable and its `+- ERROR` text compared live."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from conftest import POINT_CASES, golden
from mechafm_gb300 import _abi, synth
from mechafm_gb300.scan import Input


@pytest.mark.parametrize("name", POINT_CASES)
def test_prepared_system_matches_reference(name):
    case = golden(name)
    ref = case.ref
    desc = Input(case.input).desc()
    d = desc.c
    atoms = desc.atoms()
    np.testing.assert_array_equal(atoms["pos"], ref["sys_pos"][2:])
    assert d.tip_dummy_d == float(ref["sys_tip_dummy_d"])
    np.testing.assert_array_equal(np.array(d.offset[:]), ref["sys_offset"])
    assert [d.nx, d.ny, d.nz] == list(ref["sys_n_points"])
    if d.coulomb:
        np.testing.assert_array_equal(atoms["charge"], ref["sys_charge"][2:])
        assert d.tip_charge == ref["sys_charge"][1]


def base_input(tmp, **opt):
    spec = synth.cluster_60(area=0.2, step=0.1, zlow=9.9, **opt)
    return spec, spec.write(str(tmp))


def edit(path, drop=(), add=(), replace=None):
    lines = open(path).read().splitlines()
    lines = [l for l in lines if not any(l.split()[:1] == [k] for k in drop)]
    if replace:
        lines = [replace.get(l.split()[0], l) if l.split() else l for l in lines]
    lines += list(add)
    open(path, "w").write("\n".join(lines) + "\n")


def reference_error(inp):
    if not oracle.ref_available():
        return None
    r = subprocess.run([oracle.REF_CLI, inp], capture_output=True, text=True,
                       cwd=os.path.dirname(inp))
    err = [l for l in r.stderr.splitlines() if l.startswith("+- ERROR")]
    return err[-1].split(": ", 1)[1] if err else None


SCAN = "cluster_60.scan"
PAR = "cluster_60.par"
XYZ = "cluster_60.xyz"

CASES = [
    # (id, file, edit kwargs, expected message, code)
    ("unknown", SCAN, dict(add=["foo 1"]), "Unknown option foo!", _abi.MAFM_E_PARSE),
    ("gzip", SCAN, dict(add=["gzip maybe"]), "Option gzip must be either on or off!", _abi.MAFM_E_PARSE),
    ("minterm", SCAN, dict(add=["minterm x"]), "Option minterm must be either e, f or ef!", _abi.MAFM_E_PARSE),
    ("normal", SCAN, dict(add=["surface_normal w"]), "Option surface_normal must be either X, Y or Z!", _abi.MAFM_E_PARSE),
    ("units", SCAN, dict(add=["units furlong"]), "Option units must be either kcal/mol (default), kJ/mol or eV!", _abi.MAFM_E_PARSE),
    ("minimiser", SCAN, dict(add=["minimiser CG"]), "Unrecognised minimiser type!", _abi.MAFM_E_PARSE),
    ("integrator", SCAN, dict(add=["integrator verlet"]), "Unrecognised integrator type!", _abi.MAFM_E_PARSE),
    ("no_xyz", SCAN, dict(drop=["xyzfile"]), "Specify at least an xyzfile!", _abi.MAFM_E_PARSE),
    ("no_par", SCAN, dict(drop=["paramfile"]), "Specify at least a parameter file!", _abi.MAFM_E_PARSE),
    ("no_tip", SCAN, dict(drop=["tipatom"]), "Specify at least a tip atom!", _abi.MAFM_E_PARSE),
    ("no_dummy", SCAN, dict(drop=["dummyatom"]), "Specify at least a dummy atom!", _abi.MAFM_E_PARSE),
    ("onoff", SCAN, dict(replace={"coulomb": "coulomb maybe"}), "Option coulomb must be either on or off!",
     _abi.MAFM_E_PARSE),
    ("ext_flex", SCAN, dict(replace={"coulomb": "coulomb off", "flexible": "flexible on"},
                            add=["use_external_potential on", "e_potential_file x.cube"]),
     "External potential can be used only for non-flexible systems!", _abi.MAFM_E_PARSE),
    ("flex_bond", SCAN, dict(replace={"flexible": "flexible on"}),
     "No harmonic bond parameters found in parameter file!", _abi.MAFM_E_PARSE),
    ("no_minterm", SCAN, dict(drop=["minterm"]),
     "Specify at least a minimization termination criterion (e, f, or ef)!", _abi.MAFM_E_PARSE),
    ("grid_flex", SCAN, dict(add=["rigidgrid on", "flexible on"]),
     "Cannot use a flexible molecule with a static force grid!", _abi.MAFM_E_PARSE),
    ("coul_ext", SCAN, dict(add=["use_external_potential on"]),
     "Cannot use Coulomb interaction and external electrostatic potential at the same time!", _abi.MAFM_E_PARSE),
    ("pbc_coul", SCAN, dict(add=["vdw_pbc on"]),
     "Implementation of Coulomb interaction does not support any periodic boundary conditions! "
     "Use periodic external electrostatic potential instead.", _abi.MAFM_E_PARSE),
    ("pbc_cell", SCAN, dict(replace={"coulomb": "coulomb off"}, add=["vdw_pbc on"]),
     "The unit cell vectors must be given if periodic vdW is used.", _abi.MAFM_E_PARSE),
    ("ext_file", SCAN, dict(replace={"coulomb": "coulomb off"}, add=["use_external_potential on"]),
     "If you want to use external electrostatic potential, you must specify a file that contains it!",
     _abi.MAFM_E_PARSE),
    ("xyz_cols", XYZ, dict(replace={"C": "C 1.0 2.0"}), "Invalid number of columns in the xyz file.", _abi.MAFM_E_PARSE),
    ("no_harm", PAR, dict(drop=["harm"]), "No harmonic spring parameters found in parameter file!", _abi.MAFM_E_PARSE),
    ("two_harm", PAR, dict(add=["harm 1.0 0.0"]),
     "Parameters for harmonic spring can only be specified once!", _abi.MAFM_E_PARSE),
    ("ow_lj", PAR, dict(add=["pair_ovwrt C O lj 1 2 3"]), "Only two parameters (eps, sig) allowed for LJ", _abi.MAFM_E_PARSE),
    ("ow_morse", PAR, dict(add=["pair_ovwrt C O morse 1 2"]), "Only three parameters (De, a, re) allowed for Morse", _abi.MAFM_E_PARSE),
    ("ow_style", PAR, dict(add=["pair_ovwrt C O buck 1 2"]), "Unknown pair style overwrite 'buck'", _abi.MAFM_E_PARSE),
    ("no_type", PAR, dict(drop=["atom"], add=["atom C 0.086 3.4 12.0 0.0", "atom O 0.21 3.0 16.0 -0.1",
                                            "atom X 20.0 4.127 0.0 0.0", "atom H 0.03 2.42 1.0 0.0"]),
     "Parameters for atom type N not found in parameter file!", _abi.MAFM_E_PARSE),
]


@pytest.mark.parametrize("cid,fname,kw,message,code", CASES, ids=[c[0] for c in CASES])
def test_malformed_input_errors(cid, fname, kw, message, code, tmp_path):
    _, inp = base_input(tmp_path)
    edit(os.path.join(tmp_path, fname), **kw)
    with pytest.raises(_abi.MafmError) as e:
        Input(inp).desc()
    assert e.value.code == code
    assert e.value.msg == message
    ref = reference_error(inp)
    if ref is not None:
        assert ref == message


def test_missing_files(tmp_path):
    _, inp = base_input(tmp_path)
    with pytest.raises(_abi.MafmError) as e:
        Input(str(tmp_path / "nope.scan"))
    assert e.value.code == _abi.MAFM_E_IO and "does not exist" in e.value.msg
    os.remove(tmp_path / PAR)
    with pytest.raises(_abi.MafmError) as e:
        Input(inp)
    assert e.value.msg == f"No parameter file {tmp_path}/{PAR} found!"
    ref = reference_error(inp)
    if ref is not None:
        assert ref == e.value.msg
    os.remove(tmp_path / XYZ)
    with pytest.raises(_abi.MafmError) as e:
        Input(inp)
    assert e.value.msg == f"No such file: {tmp_path}/{XYZ}!"
    ref = reference_error(inp)
    if ref is not None:
        assert ref == e.value.msg


def test_xyz_formats_and_charge_source(tmp_path):
    """4-column xyz (no charges): charges come from the parameter file (parse.cpp:571-584)."""
    spec = synth.cluster_60(area=0.2, step=0.1, zlow=9.9)
    spec.charges = None
    spec.atom_params["C"] = (0.086, 3.4, 12.011, 0.05)
    inp = spec.write(str(tmp_path))
    d = Input(inp).desc()
    a = d.atoms()
    types = [spec.types[i] for i in range(len(spec.types))]
    want = np.array([spec.atom_params[t][3] for t in types])
    np.testing.assert_array_equal(a["charge"], want)
    assert d.c.tip_charge == -0.1


def test_surface_normal_rotation(tmp_path):
    """surface_normal y rotates coordinates ZXY (system.cpp:68-90)."""
    spec = synth.graphene_72(area=0.2, step=0.1, zlow=9.9)
    pos = spec.pos.copy()
    spec.pos = np.column_stack([pos[:, 1], pos[:, 2], pos[:, 0]])   # plane normal along y
    spec.options["surface_normal"] = "y"
    inp = spec.write(str(tmp_path))
    a = Input(inp).desc().atoms()
    assert np.ptp(a["pos"][:, 2]) < 1e-12   # flat in z after the rotation
