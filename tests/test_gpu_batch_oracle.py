"""A batch of 32 seeded molecules of uneven sizes (20-400 atoms, LJ +
Coulomb, 8^2 to 16^2 pixels x 41 heights) relaxed in one persistent launch,
against the oracle scan by scan, every point (the per-scan loop of
Simulation::run, simulation.cpp:67-143, that a batch replaces):

  MAFM_DF     the oracle's step count on every point, tip within 1e-6 A,
              Fz within 1e-6 relative (floor 0.01)
  MAFM_FP32C  the metric's bar (tip 1e-3 A, Fz 1e-3 relative) on at least
              99.5 % of the points of every scan
"""
import numpy as np
import pytest

import oracle
from mechafm_gb300 import _abi, synth
from mechafm_gb300.scan import Input, Scan, run_batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("batch")
    specs = synth.molecule_batch(n_scans=32, seed=5, grids=(8, 12, 16))
    descs = [Input(s.write(str(tmp / f"m{i:02d}"))).desc() for i, s in enumerate(specs)]
    want = [oracle.run(d)[0] for d in descs]
    scans = [Scan(d, device=0) for d in descs]
    yield scans, want
    for s in scans:
        s.close()


def errors(got, ref):
    tip = np.abs(got["tip"] - ref["tip"]).max(axis=1)
    fz = np.abs(got["force"][:, 2] - ref["force"][:, 2]) / np.maximum(np.abs(ref["force"][:, 2]), 0.01)
    return tip, fz


def test_df_batch_matches_oracle_on_every_point(batch):
    scans, want = batch
    outs, _ = run_batch(scans, precision=_abi.DF)
    assert sum(len(w) for w in want) == sum(len(o) for o in outs)
    for i, (got, ref) in enumerate(zip(outs, want)):
        np.testing.assert_array_equal(got["steps"], ref["steps"], err_msg=f"scan {i}")
        tip, fz = errors(got, ref)
        assert tip.max() <= 1e-6 and fz.max() <= 1e-6, (i, tip.max(), fz.max())


def test_fp32c_batch_within_bar(batch):
    scans, want = batch
    outs, _ = run_batch(scans, precision=_abi.FP32C)
    for i, (got, ref) in enumerate(zip(outs, want)):
        tip, fz = errors(got, ref)
        ok = (tip <= 1e-3) & (fz <= 1e-3)
        assert ok.mean() >= 0.995, (i, ok.mean(), tip.max(), fz.max())
