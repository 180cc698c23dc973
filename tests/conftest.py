import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a kernels")


def _manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


MANIFEST = _manifest()
POINT_CASES = sorted(k for k, v in MANIFEST.items()
                     if "error" not in v and not v.get("cli") and v.get("sample") != "states")
# flexible molecules: relaxed through mafm_flex_* with the atoms' states
FLEX_CASES = sorted(k for k, v in MANIFEST.items() if v.get("sample") == "states")
ERROR_CASES = sorted(k for k, v in MANIFEST.items() if "error" in v)


class GoldenCase:
    """One reference run: input files plus the reference's full-precision results."""

    def __init__(self, name):
        self.name = name
        self.meta = MANIFEST[name]
        self.folder = os.path.join(GOLDEN, name)
        self.input = os.path.join(self.folder, self.meta["input"])
        self.ref = dict(np.load(os.path.join(self.folder, "ref.npz"))) \
            if "error" not in self.meta else None

    def columns(self, ny):
        """Column ranges [c0, c1) covering the reference block, one per row i."""
        i0, i1, j0, j1 = self.meta["block"]
        return [(i * ny + j0, i * ny + j1) for i in range(i0, i1)]


@pytest.fixture(scope="session")
def libmafm():
    from mechafm_gb300 import _abi
    return _abi.lib()


def golden(name) -> GoldenCase:
    return GoldenCase(name)


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
