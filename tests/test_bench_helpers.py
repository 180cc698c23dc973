"""The measurement helpers of bench.py that need no GPU: the algorithmic flop
counts per force evaluation (FP64 expressions and double-float operations),
the seeded column samples of the CPU baseline and the FP64 comparison, and
the error statistics against FP64."""
import sys

import numpy as np

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402
from mechafm_gb300 import _abi, synth  # noqa: E402
from mechafm_gb300.scan import Input  # noqa: E402


def test_flops_per_evaluation_of_the_cluster(tmp_path):
    """The headline cluster: 54 LJ and 6 Morse terms, every atom charged:
    54 x 25 + 6 x 29 + 60 x 20 FP64-expression flops; in double-float
    operations 54 x 201 + 6 x 475 + 54 x 23 + 6 x 30."""
    desc = Input(synth.cluster_60(area=1.0).write(str(tmp_path))).desc()
    assert bench.term_flops(desc) == 54 * 25 + 6 * 29 + 60 * 20 == 2724
    assert bench.term_flops(desc, table=bench.DF_TABLE) == 54 * 201 + 6 * 475 + 54 * 23 + 6 * 30


def test_flops_of_rigid_grid_scans_count_only_the_grid_build(tmp_path):
    desc = Input(synth.slab(pixels=4, nlx=4, nly=4, layers=1, cube_n=(24, 24, 40)).write(str(tmp_path))).desc()
    assert desc.c.rigidgrid
    assert bench.term_flops(desc) == 0
    # every image term is LJ, no Coulomb beside the external field
    assert bench.term_flops(desc, direct=True) == 9 * desc.c.n_atoms * 25


def test_column_samples_are_seeded_uniform_and_distinct():
    a = bench.sample_columns(160801, 4096, 1000)
    b = bench.sample_columns(160801, 4096, 1000)
    np.testing.assert_array_equal(a, b)
    assert len(np.unique(a)) == 4096 and np.all(np.diff(a) > 0)
    assert a.min() >= 0 and a.max() < 160801
    # spread over the whole scan, not a band
    assert a.min() < 160801 * 0.05 and a.max() > 160801 * 0.95
    assert len(bench.sample_columns(100, 4096, 1)) == 100


def test_error_statistics_against_fp64():
    ref = np.zeros(4, dtype=_abi.POINT_DTYPE)
    ref["force"][:, 2] = [1.0, -0.5, 0.001, 2.0]
    ref["steps"] = [10, 20, 30, 40]
    pts = ref.copy()
    pts["tip"][1, 0] = 2e-3                  # beyond the tip bar
    pts["force"][2, 2] = 0.001 + 5e-6        # within the bar: 5e-6 / max(0.001, 0.01)
    pts["force"][3, 2] = 2.0 + 4e-3          # beyond the Fz bar: 2e-3 relative
    pts["steps"][3] = 41
    s = bench.err_stats(pts, ref)
    assert s["points_beyond_bar"] == 2
    assert s["tip_err_A"]["max"] == 2e-3
    assert abs(s["fz_rel_err"]["max"] - 2e-3) < 1e-12
    assert s["step_count_match"] == 0.75


def test_rigid_grid_node_count_follows_the_reference_geometry(tmp_path):
    """nodes = prod(floor(extent / (step / 2)) + 2 ceil(1.5 / (step / 2)) + 1)
    (simulation.cpp:426-436) for the bench's slab geometry."""
    desc = Input(synth.slab(pixels=8, nlx=4, nly=4, layers=1, cube_n=(24, 24, 40),
                            zhigh=18.0, zlow=14.0).write(str(tmp_path))).desc()
    d = desc.c
    sp = (d.dx / 2, d.dy / 2, d.dz / 2)
    border = [int(np.ceil(1.5 / s)) for s in sp]
    want = ((int(np.floor(d.area[0] / sp[0])) + 2 * border[0] + 1) *
            (int(np.floor(d.area[1] / sp[1])) + 2 * border[1] + 1) *
            (int(np.floor((d.zhigh - d.zlow) / sp[2])) + 2 * border[2] + 1))
    assert bench.rigid_nodes(d) == want
