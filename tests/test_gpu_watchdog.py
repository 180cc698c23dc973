"""Time limits of the persistent relax kernels.

The reference stops a failed run with error() and exit(1)
(src/messages.cpp:12-27); the GPU kernels instead read %globaltimer and end
with a device error bit once a warp runs past MAFM_WATCHDOG_S seconds
(fractions allowed, 120 s by default).  The host reports that bit as
MAFM_E_DEVICE and the context stays usable: the kernel returns normally, it
never traps.  Each test sets a limit of one microsecond, which every warp
passes long before its first column is relaxed, expects MAFM_E_DEVICE, and
then relaxes the same scan again without the limit in the same process
(FP32C, FP32C batch, double-float and flexible kernels).
"""
import numpy as np
import pytest

from conftest import golden
from mechafm_gb300 import _abi
from mechafm_gb300.scan import FlexScan, Input, Scan, run_batch

pytestmark = pytest.mark.gpu

TINY = "0.000001"


def _same_points(a, b):
    for f in ("tip", "force", "energy", "steps", "status"):
        np.testing.assert_array_equal(a[f], b[f])


def test_fp32c_watchdog_ends_the_kernel_and_the_context_recovers(monkeypatch):
    case = golden("graphene_ef")
    scan = Scan(Input(case.input).desc(), device=0)
    before, _ = scan.run(_abi.FP32C)
    before64, _ = scan.run(_abi.FP64, col_begin=0, col_end=8)
    monkeypatch.setenv("MAFM_WATCHDOG_S", TINY)
    with pytest.raises(_abi.MafmError) as e:
        scan.run(_abi.FP32C)
    assert e.value.code == _abi.MAFM_E_DEVICE
    assert "watchdog" in e.value.msg
    with pytest.raises(_abi.MafmError) as e:
        run_batch([scan])
    assert e.value.code == _abi.MAFM_E_DEVICE
    monkeypatch.delenv("MAFM_WATCHDOG_S")
    after, _ = scan.run(_abi.FP32C)
    _same_points(after, before)
    after64, _ = scan.run(_abi.FP64, col_begin=0, col_end=8)
    _same_points(after64, before64)
    scan.close()


def test_df_watchdog_ends_the_kernel_and_the_context_recovers(monkeypatch):
    case = golden("graphene_ef")
    scan = Scan(Input(case.input).desc(), device=0)
    before, _ = scan.run(_abi.DF)
    monkeypatch.setenv("MAFM_WATCHDOG_S", TINY)
    with pytest.raises(_abi.MafmError) as e:
        scan.run(_abi.DF)
    assert e.value.code == _abi.MAFM_E_DEVICE
    assert "watchdog" in e.value.msg
    monkeypatch.delenv("MAFM_WATCHDOG_S")
    after, _ = scan.run(_abi.DF)
    _same_points(after, before)
    scan.close()


def test_flexible_watchdog_ends_the_kernel_and_the_context_recovers(monkeypatch):
    case = golden("flex_naph")
    src = Input(case.input)
    desc, flex = src.desc(), src.flex_desc()
    fs = FlexScan(desc, flex, device=0)
    before, _, _ = fs.run()
    monkeypatch.setenv("MAFM_WATCHDOG_S", TINY)
    with pytest.raises(_abi.MafmError) as e:
        fs.run()
    assert e.value.code == _abi.MAFM_E_DEVICE
    monkeypatch.delenv("MAFM_WATCHDOG_S")
    after, _, _ = fs.run()
    _same_points(after, before)
    fs.close()


@pytest.mark.parametrize("value", ["0", "-3", "junk"])
def test_invalid_limits_fall_back_to_the_default(monkeypatch, value):
    """Zero, negative and non-numeric limits mean the 120 s default, not 0 s."""
    case = golden("graphene_ef")
    scan = Scan(Input(case.input).desc(), device=0)
    monkeypatch.setenv("MAFM_WATCHDOG_S", value)
    scan.run(_abi.FP32C, col_begin=0, col_end=4)
    scan.close()
