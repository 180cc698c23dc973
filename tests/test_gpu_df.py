"""MAFM_DF, the double-float relaxation, against the reference's own results.

Every quantity of the relaxation is an unevaluated sum of two FP32 numbers
(48-bit significand), so FIRE takes the FP64 decisions; columns in which a
decision came within the double-float error margin of its threshold are
re-relaxed in FP64.  The bars therefore hold on EVERY point, with no
step-matched filter and no fraction:

  step count            equal to the reference's
  tip position          within 1e-8 A of the reference's fixtures (the metric's bar
                        is 1e-3 A); within 1e-6 A on the random scans, whose long,
                        loosely converged trajectories (random tolerances, SD,
                        maxsteps) move that much even between two FP64 builds that
                        differ only in exp's last bit (tests/test_gpu_random.py
                        allows the FP64 kernel the same)
  Fz                    within 1e-8 relative (denominator max(|Fz_ref|, 0.01 = ftol);
                        the metric's bar is 1e-3); 1e-6 on the random scans

The FP64 re-relaxation itself (one warp per column, inside the double-float
kernel or in repair64_kernel after it) must reproduce the plain FP64 kernel
bit for bit: MAFM_DF_TIE_SCALE widens the near-tie margins until every column
is re-relaxed, and the result is compared with MAFM_FP64 on every field.
Over a rigid grid the grid is built in double-float and the re-relaxation
reads its FP64 copy, whose nodes agree with the FP64 build to about 1e-14:
there the re-relaxed points must equal FP64's steps and lie within 1e-9.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from conftest import POINT_CASES, golden
from mechafm_gb300 import _abi
from mechafm_gb300.scan import Input, Scan, run_batch

pytestmark = pytest.mark.gpu

TIP_TOL = 1e-8
FZ_TOL = 1e-8
FZ_FLOOR = 0.01
DF_CASES = list(POINT_CASES)
RIGID_CASES = ["graphene_grid", "slab_es_grid"]


def run_case(case, precision, **kw):
    desc = Input(case.input).desc()
    scan = Scan(desc, device=0)
    parts, fp64_cols = [], 0
    for c0, c1 in case.columns(desc.c.ny):
        p, st = scan.run(precision, col_begin=c0, col_end=c1, **kw)
        parts.append(p)
        fp64_cols += st.fp64_columns
    scan.close()
    return np.concatenate(parts), fp64_cols


def assert_faithful(pts, ref, tip_tol=TIP_TOL, fz_tol=FZ_TOL):
    """Every point: equal steps, tip within tip_tol, Fz within fz_tol relative."""
    tip = np.abs(pts["tip"] - ref["tip"]).max(axis=1)
    fz = np.abs(pts["force"][:, 2] - ref["force"][:, 2]) / np.maximum(np.abs(ref["force"][:, 2]), FZ_FLOOR)
    bad = np.nonzero(pts["steps"] != ref["steps"])[0]
    assert len(bad) == 0, ("step counts differ", bad[:10], pts["steps"][bad[:10]], ref["steps"][bad[:10]])
    assert tip.max() <= tip_tol, tip.max()
    assert fz.max() <= fz_tol, fz.max()


@pytest.mark.parametrize("name", DF_CASES)
def test_df_matches_reference_on_every_point(name):
    case = golden(name)
    pts, _ = run_case(case, _abi.DF)
    assert_faithful(pts, case.ref)


def test_df_matches_oracle_on_random_scans(tmp_path):
    """The seeded random molecules and periodic sheets of test_oracle_random
    (random integrators, minimisers, terminations, units, overrides): every
    point against the oracle, which is pinned to the reference on them."""
    from test_oracle_random import N_CASES, random_periodic_spec, random_spec
    specs = [random_spec(s, geometry=False) for s in range(N_CASES)]
    specs += [random_periodic_spec(s) for s in range(8)]
    for i, spec in enumerate(specs):
        desc = Input(spec.write(str(tmp_path / f"s{i}"))).desc()
        want, _ = oracle.run(desc)
        scan = Scan(desc, device=0)
        got, _ = scan.run(_abi.DF)
        scan.close()
        assert_faithful(got, want, tip_tol=1e-6, fz_tol=1e-6)


@pytest.mark.parametrize("name", ["graphene_ef", "graphene_euler", "graphene_sd", "cluster_rk4",
                                  "cluster_e", "slab_es", "graphene_pbc"])
def test_fp64_re_relaxation_is_bit_identical_to_the_fp64_kernel(name, monkeypatch):
    case = golden(name)
    want, _ = run_case(case, _abi.FP64)
    monkeypatch.setenv("MAFM_DF_TIE_SCALE", "1e20")
    got, n_fp64 = run_case(case, _abi.DF)
    assert n_fp64 == sum(c1 - c0 for c0, c1 in case.columns(Input(case.input).desc().c.ny))
    assert np.all(got["status"] & _abi.PT_FP64)
    assert np.all(got["status"] & _abi.PT_NEAR_TIE)
    for f in ("tip", "force", "energy", "steps"):
        np.testing.assert_array_equal(got[f], want[f])


def test_df_batch_equals_single_runs_and_plan_replays():
    import torch
    names = ["graphene_euler", "cluster_rk4", "cluster_f", "slab_es"]
    scans = [Scan(Input(golden(n).input).desc(), device=0) for n in names]
    # small sub-scans keep the test short: crop each to its golden block
    crops = []
    for n, s in zip(names, scans):
        i0, i1, j0, j1 = golden(n).meta["block"]
        crops.append(Scan(s.desc.crop(i0, j0, i1 - i0, j1 - j0), device=0))
    singles = [c.run(_abi.DF)[0] for c in crops]
    outs, st = run_batch(crops, precision=_abi.DF)
    for a, b in zip(outs, singles):
        np.testing.assert_array_equal(a, b)
    # a plan of the same scans, launched and replayed from a CUDA graph
    L = _abi.lib()
    n = len(crops)
    dev = [torch.zeros(c.desc.n_points * 64, dtype=torch.uint8, device="cuda:0") for c in crops]
    handles = (C.c_void_p * n)(*[c.handle for c in crops])
    optrs = (C.c_void_p * n)(*[o.data_ptr() for o in dev])
    opts = _abi.RunOpts(_abi.DF, 0, 0, 0, 0, 0)
    plan = C.c_void_p()
    _abi.check(L.mafm_plan_create(handles, n, C.byref(opts), optrs, C.byref(plan)))
    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)
    _abi.check(L.mafm_plan_launch(plan, sp))
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        _abi.check(L.mafm_plan_launch(plan, sp))
    for o in dev:
        o.fill_(0xFF)
    g.replay()
    torch.cuda.synchronize()
    rs = _abi.RunStats()
    _abi.check(L.mafm_plan_stats(plan, C.byref(rs), sp))
    for o, want in zip(dev, singles):
        got = np.frombuffer(o.cpu().numpy().tobytes(), dtype=_abi.POINT_DTYPE)
        np.testing.assert_array_equal(got, want)
    L.mafm_plan_destroy(plan)


@pytest.mark.parametrize("name", RIGID_CASES)
def test_fp64_re_relaxation_over_the_df_grid(name, monkeypatch):
    case = golden(name)
    want, _ = run_case(case, _abi.FP64)
    monkeypatch.setenv("MAFM_DF_TIE_SCALE", "1e20")
    got, n_fp64 = run_case(case, _abi.DF)
    assert n_fp64 == sum(c1 - c0 for c0, c1 in case.columns(Input(case.input).desc().c.ny))
    assert np.all(got["status"] & _abi.PT_FP64)
    assert_faithful(got, want, tip_tol=1e-9, fz_tol=1e-9)


def test_df_grid_rebuild_is_identical_and_captures_with_the_plan():
    """mafm_scan_build_grid(MAFM_DF) rebuilds the double-float grid bit for
    bit, and a CUDA graph of [grid build, plan launch] replays the run."""
    import torch
    case = golden("slab_es_grid")
    desc = Input(case.input).desc()
    i0, i1, j0, j1 = case.meta["block"]
    scan = Scan(desc.crop(i0, j0, i1 - i0, j1 - j0), device=0)
    first, _ = scan.run(_abi.DF)
    L = _abi.lib()
    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)
    _abi.check(L.mafm_scan_build_grid(scan.handle, _abi.DF, sp))
    again, _ = scan.run(_abi.DF)
    np.testing.assert_array_equal(again, first)
    dev = torch.zeros(scan.desc.n_points * 64, dtype=torch.uint8, device="cuda:0")
    handles = (C.c_void_p * 1)(scan.handle)
    optrs = (C.c_void_p * 1)(dev.data_ptr())
    opts = _abi.RunOpts(_abi.DF, 0, 0, 0, 0, 0)
    plan = C.c_void_p()
    _abi.check(L.mafm_plan_create(handles, 1, C.byref(opts), optrs, C.byref(plan)))
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        _abi.check(L.mafm_scan_build_grid(scan.handle, _abi.DF, sp))
        _abi.check(L.mafm_plan_launch(plan, sp))
    dev.fill_(0xFF)
    g.replay()
    torch.cuda.synchronize()
    got = np.frombuffer(dev.cpu().numpy().tobytes(), dtype=_abi.POINT_DTYPE)
    np.testing.assert_array_equal(got, first)
    L.mafm_plan_destroy(plan)
    scan.close()
