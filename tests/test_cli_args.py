"""The mechafm-gpu executable's argument handling (parse.cpp:41-45, 136-140):
errors on stderr as `+- ERROR (on process 0): ...`, exit code 1, before any
GPU work, so these run on CPU.  Where the reference executable was built
here (oracle/_ref), its stdout and stderr must be the same."""
import os
import subprocess

import pytest

import oracle
from mechafm_gb300 import build

CASES = [
    ("no_args", [], "Specify an input file to be read!"),
    ("too_many", ["a.scan", "out", "extra"], "Too many command line arguments!"),
    ("missing_input", ["{tmp}/nope.scan"], "The file {tmp}/nope.scan does not exist!"),
]


def _run(exe, args, cwd):
    return subprocess.run([exe] + args, capture_output=True, text=True, cwd=cwd)


@pytest.mark.parametrize("cid,args,message", CASES, ids=[c[0] for c in CASES])
def test_cli_argument_errors(cid, args, message, tmp_path):
    if not os.path.exists(build.CLI):
        pytest.skip("mechafm-gpu not built")
    args = [a.format(tmp=tmp_path) for a in args]
    r = _run(build.CLI, args, tmp_path)
    assert r.returncode == 1
    assert r.stderr.splitlines()[-1] == "+- ERROR (on process 0): " + message.format(tmp=tmp_path)
    if oracle.ref_available() and os.path.exists(oracle.REF_CLI):
        ref = _run(oracle.REF_CLI, args, tmp_path)
        assert ref.returncode == r.returncode
        assert ref.stdout == r.stdout
        assert ref.stderr == r.stderr
