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


def _placeholders(text, folder, out):
    return text.replace(out, "{OUT}").replace(folder, "{DIR}")


def cli_stdout(name, tmp_path):
    """(our stdout lines with {DIR}/{OUT} placeholders, the reference's, exit code)."""
    from conftest import GOLDEN, MANIFEST
    folder = os.path.join(GOLDEN, name)
    out = str(tmp_path / "out")
    r = _run(build.CLI, [os.path.join(folder, MANIFEST[name]["input"]), out], folder)
    ours = _placeholders(r.stdout, folder, out).splitlines()
    with open(os.path.join(folder, "cli_stdout.txt")) as f:
        ref = f.read().splitlines()
    return ours, ref, r.returncode


@pytest.mark.parametrize("name", ["cli_cluster", "cli_pbc", "cli_flex"])
def test_cli_banner_and_settings_match_reference(name, tmp_path):
    """Everything the executable prints before the relaxation starts (banner,
    the echo of every input setting, the 3D data grid) equals the reference
    executable's stdout (tests/golden/cli_*/cli_stdout.txt).  Without a GPU
    the run stops right after these lines."""
    if not os.path.exists(build.CLI):
        pytest.skip("mechafm-gpu not built")
    ours, ref, _ = cli_stdout(name, tmp_path)
    k = ref.index("+- Starting simulation")
    assert ours[:k] == ref[:k]
