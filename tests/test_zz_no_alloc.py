"""mafm_run_batch_noalloc, the entry point for callers that cannot let the
library allocate device memory (their own capped pool, no implicit
synchronisation from cudaFree, exact memory accounting on a shared GPU).

Its scratch sits in a fixed device array of the library, shared by every call
and keeping the last call's contents, so two calls in a row must each start
from cleared counters and give the same points as the allocating entry point
mafm_run_batch (same kernel, same launch shape: bit-identical, the tolerance
tests/test_gpu_parity.py uses for batch-versus-single runs).

This file is named to be collected last; the test also passes alone in a
fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden
from mechafm_gb300 import _abi
from mechafm_gb300.scan import Input, Scan, run_batch

pytestmark = pytest.mark.gpu

CASES = ["cluster_f", "graphene_euler", "graphene_pbc", "graphene_grid"]


def _noalloc(scans, outs, lanes=1):
    n = len(scans)
    handles = (C.c_void_p * n)(*[s.handle for s in scans])
    optrs = (C.c_void_p * n)(*[o.data_ptr() for o in outs])
    opts = _abi.RunOpts(_abi.FP32C, lanes, 0, 0, 0, 0)
    stats = _abi.RunStats()
    _abi.check(_abi.lib().mafm_run_batch_noalloc(handles, n, C.byref(opts), optrs,
                                                 C.byref(stats), None))
    return stats


def _points(t):
    return np.frombuffer(t.cpu().numpy().tobytes(), dtype=_abi.POINT_DTYPE)


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    scans = [Scan(Input(golden(n).input).desc(), device=0) for n in CASES]
    # The allocating entry point builds the rigid grid's FP32 copy on first use.
    want, want_stats = run_batch(scans, lanes=1)
    outs = [torch.zeros(s.desc.n_points * 64, dtype=torch.uint8, device="cuda:0") for s in scans]
    for call in range(2):
        for o in outs:
            o.fill_(0xFF)   # stale bytes must not survive into the result
        stats = _noalloc(scans, outs)
        torch.cuda.synchronize()
        assert stats.total_steps == want_stats.total_steps, call
        assert stats.force_evals == want_stats.force_evals, call
        for o, w in zip(outs, want):
            got = _points(o)
            np.testing.assert_array_equal(got["steps"], w["steps"])
            np.testing.assert_array_equal(got["tip"], w["tip"])
            np.testing.assert_array_equal(got["force"], w["force"])
            np.testing.assert_array_equal(got["energy"], w["energy"])


def test_noalloc_rejects_too_many_scans_and_host_outputs():
    import torch
    scan = Scan(Input(golden("graphene_euler").input).desc(), device=0)
    out = torch.zeros(scan.desc.n_points * 64, dtype=torch.uint8, device="cuda:0")
    n = _abi.NOALLOC_MAX_SCANS + 1
    handles = (C.c_void_p * n)(*([scan.handle] * n))
    optrs = (C.c_void_p * n)(*([out.data_ptr()] * n))
    opts = _abi.RunOpts(_abi.FP32C, 1, 0, 0, 0, 0)
    code = _abi.lib().mafm_run_batch_noalloc(handles, n, C.byref(opts), optrs, None, None)
    assert code == _abi.MAFM_E_RANGE
    assert b"at most 32 scans" in _abi.lib().mafm_last_error()
    host = np.zeros(scan.desc.n_points, dtype=_abi.POINT_DTYPE)
    h1 = (C.c_void_p * 1)(scan.handle)
    o1 = (C.c_void_p * 1)(host.ctypes.data)
    code = _abi.lib().mafm_run_batch_noalloc(h1, 1, C.byref(opts), o1, None, None)
    assert code == _abi.MAFM_E_INVALID
    assert b"not device memory" in _abi.lib().mafm_last_error()


def test_noalloc_leaves_free_device_memory_unchanged():
    """After one warm-up call (which may load the kernels' module), repeated
    calls change the device's free memory (cudaMemGetInfo) by not one byte,
    and a call without statistics still reports success only after the work
    is done."""
    import torch
    scans = [Scan(Input(golden(n).input).desc(), device=0) for n in CASES]
    run_batch(scans, lanes=1)   # FP32 rigid grid built by the allocating entry point
    outs = [torch.zeros(s.desc.n_points * 64, dtype=torch.uint8, device="cuda:0") for s in scans]
    _noalloc(scans, outs)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    n = len(scans)
    handles = (C.c_void_p * n)(*[s.handle for s in scans])
    optrs = (C.c_void_p * n)(*[o.data_ptr() for o in outs])
    opts = _abi.RunOpts(_abi.FP32C, 1, 0, 0, 0, 0)
    for _ in range(3):
        _noalloc(scans, outs)
        assert _abi.lib().mafm_run_batch_noalloc(handles, n, C.byref(opts), optrs, None, None) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)
