"""Output parity with the reference executable: scan-%06.3f.dat rows and
statistics.txt written by libmafm (mafm_write_output / mafm_write_statistics)
from oracle points are byte-identical to what `mechafm-omp` wrote (rows are
compared sorted: the reference writes them in thread order,
simulation.cpp:176)."""
import ctypes as C
import gzip
import os

import pytest

import oracle
from conftest import GOLDEN, MANIFEST
from mechafm_gb300 import _abi
from mechafm_gb300.scan import Input

CLI_CASES = sorted(k for k, v in MANIFEST.items() if v.get("cli"))


def rows_of(folder):
    rows = []
    for fn in sorted(os.listdir(folder)):
        if fn.startswith("scan-"):
            path = os.path.join(folder, fn)
            opener = gzip.open if fn.endswith(".gz") else open
            with opener(path, "rt") as f:
                name = fn[:-3] if fn.endswith(".gz") else fn
                rows += [name + "\t" + l.rstrip("\n") for l in f]
    return sorted(rows)


@pytest.mark.parametrize("name", CLI_CASES)
@pytest.mark.parametrize("use_gzip", [False, True])
def test_scan_files_match_reference_executable(name, use_gzip, tmp_path):
    folder = os.path.join(GOLDEN, name)
    inp = Input(os.path.join(folder, MANIFEST[name]["input"]))
    desc = inp.desc()
    if desc.c.flexible:
        pts, steps, _ = oracle.flex_run(desc, inp.flex_desc())
    else:
        pts, steps = oracle.run(desc)
    inp.write_output(pts, str(tmp_path), gzip=use_gzip)
    want = open(os.path.join(folder, "cli_rows.txt")).read().splitlines()
    assert rows_of(str(tmp_path)) == want
    out = str(tmp_path) + "/"
    _abi.check(_abi.lib().mafm_write_statistics(inp.handle, out.encode(), steps, 1.0, 1.0))
    head = open(os.path.join(tmp_path, "statistics.txt")).readlines()[:4]
    assert head == open(os.path.join(folder, "cli_statistics_head.txt")).readlines()


def test_state_files_match_reference_executable(tmp_path):
    """System::makeXYZFile's state_*.xyz files of the middle pixel of a
    flexible scan (simulation.cpp:114-116), written by mafm_write_states from
    the oracle's atom states, equal the reference executable's."""
    folder = os.path.join(GOLDEN, "cli_flex")
    inp = Input(os.path.join(folder, MANIFEST["cli_flex"]["input"]))
    desc = inp.desc()
    col = desc.c.nx * desc.c.ny // 2
    _, _, states = oracle.flex_run(desc, inp.flex_desc(), col, col + 1, state_column=col)
    out = str(tmp_path) + "/"
    _abi.check(_abi.lib().mafm_write_states(inp.handle, states.ctypes.data, col, out.encode()))
    got = []
    for fn in sorted(os.listdir(tmp_path)):
        if fn.startswith("state_"):
            got += [fn + "\t" + l.rstrip("\n") for l in open(os.path.join(tmp_path, fn))]
    want = open(os.path.join(folder, "cli_states.txt")).read().splitlines()
    assert got == want


@pytest.mark.parametrize("use_gzip", [False, True])
def test_chunked_writer_equals_one_shot_writer(use_gzip, tmp_path):
    """mafm_writer_append over uneven column chunks (some ending inside a
    pixel row) writes the same bytes as mafm_write_output, and refuses a
    chunk that does not continue the columns written so far."""
    import numpy as np
    folder = os.path.join(GOLDEN, "cli_cluster")
    inp = Input(os.path.join(folder, MANIFEST["cli_cluster"]["input"]))
    desc = inp.desc()
    pts, _ = oracle.run(desc)
    one = tmp_path / "one"
    chunked = tmp_path / "chunked"
    one.mkdir()
    chunked.mkdir()
    inp.write_output(pts, str(one), gzip=use_gzip)
    L = _abi.lib()
    w = C.c_void_p()
    _abi.check(L.mafm_writer_open(inp.handle, (str(chunked) + "/").encode(), int(use_gzip),
                                  C.byref(w)))
    n_cols, nz = desc.n_columns, desc.c.nz
    cuts = sorted({0, n_cols, 1, n_cols // 3, n_cols // 3 + desc.c.ny + 1, n_cols - 2})
    assert L.mafm_writer_append(w, pts.ctypes.data, 1, 2) == _abi.MAFM_E_INVALID
    for a, b in zip(cuts[:-1], cuts[1:]):
        chunk = np.ascontiguousarray(pts[a * nz:b * nz])
        _abi.check(L.mafm_writer_append(w, chunk.ctypes.data, a, b))
    L.mafm_writer_close(w)
    names = sorted(os.listdir(one))
    assert names == sorted(os.listdir(chunked)) and len(names) == nz
    for fn in names:
        opener = gzip.open if use_gzip else open
        with opener(os.path.join(one, fn), "rb") as f1, opener(os.path.join(chunked, fn), "rb") as f2:
            assert f1.read() == f2.read(), fn
