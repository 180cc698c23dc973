"""The C ABI library: loads without a GPU, exports every symbol include/mafm.h
declares, and its structures have the layout the Python mirror assumes."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from conftest import ROOT
from mechafm_gb300 import _abi

HEADER = os.path.join(ROOT, "include", "mafm.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mafm_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_expected_entry_points():
    names = declared_functions()
    for n in ("mafm_input_load", "mafm_scan_create", "mafm_run", "mafm_run_batch",
              "mafm_scan_sample", "mafm_write_output", "mafm_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(libmafm):
    missing = [n for n in declared_functions() if not hasattr(libmafm, n)]
    assert not missing, missing


def test_python_mirror_covers_every_symbol():
    assert set(declared_functions()) <= set(_abi.SIGNATURES)


def test_struct_layouts_match_header():
    """Compile a probe against the header and compare sizes and offsets with ctypes."""
    probe = r"""
#include <stdio.h>
#include <stddef.h>
#include "mafm.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(mafm_pair), sizeof(mafm_scan_desc), sizeof(mafm_point),
         sizeof(mafm_run_opts), sizeof(mafm_run_stats));
  printf("%zu %zu %zu %zu %zu\n", offsetof(mafm_scan_desc, dummy_pair), offsetof(mafm_scan_desc, nx),
         offsetof(mafm_scan_desc, minimiser), offsetof(mafm_scan_desc, epot),
         offsetof(mafm_scan_desc, epot_origin));
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "probe.c")
        exe = os.path.join(tmp, "probe")
        open(src, "w").write(probe)
        subprocess.run(["gcc", "-I" + os.path.dirname(HEADER), src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    sizes = [int(x) for x in out[:5]]
    offs = [int(x) for x in out[5:]]
    assert sizes == [C.sizeof(_abi.Pair), C.sizeof(_abi.ScanDesc), C.sizeof(_abi.Point),
                     C.sizeof(_abi.RunOpts), C.sizeof(_abi.RunStats)]
    D = _abi.ScanDesc
    assert offs == [D.dummy_pair.offset, D.nx.offset, D.minimiser.offset, D.epot.offset,
                    D.epot_origin.offset]


def test_abi_version_and_errors_without_gpu(libmafm):
    assert libmafm.mafm_abi_version() == 1
    h = C.c_void_p()
    code = libmafm.mafm_input_load(b"/nonexistent/input.scan", 0, C.byref(h))
    assert code == _abi.MAFM_E_IO
    assert b"does not exist" in libmafm.mafm_last_error()
    assert libmafm.mafm_run(None, None, None, None, None) == _abi.MAFM_E_INVALID


def test_product_path_refuses_to_run_without_the_library(tmp_path, monkeypatch):
    """No silent fallback: a missing libmafm.so is an error, never a CPU path."""
    monkeypatch.setattr(_abi, "_lib", None)
    with pytest.raises(OSError):
        _abi.lib(str(tmp_path / "libmafm.so"))
