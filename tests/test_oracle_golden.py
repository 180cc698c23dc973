"""Pin the oracle: the C restatement (oracle/mafm_oracle.c), fed by the product's
input front-end, must reproduce the reference's own results stored in
tests/golden (generated by running the unmodified reference sources).

Pair-force cases are bit-identical on the x86-64 host where the fixtures were
made; the external-field cases compare a direct 3-D DFT with kiss_fft, so they
are held to 1e-9 relative.
"""
import numpy as np
import pytest

import oracle
from conftest import ERROR_CASES, POINT_CASES, golden
from mechafm_gb300.scan import Input

FFT_CASES = {"slab_es", "slab_es_grid", "slab_es_tric"}


def run_block(case):
    desc = Input(case.input).desc()
    parts = [oracle.run(desc, c0, c1)[0] for c0, c1 in case.columns(desc.c.ny)]
    return desc, np.concatenate(parts)


@pytest.mark.parametrize("name", POINT_CASES)
def test_oracle_matches_reference(name):
    case = golden(name)
    _, pts = run_block(case)
    ref = case.ref
    assert len(pts) == len(ref["steps"])
    if name in FFT_CASES:
        # Different FFT algorithm: trajectories agree to rounding level.
        assert np.mean(pts["steps"] == ref["steps"]) > 0.99
        assert np.abs(pts["tip"] - ref["tip"]).max() < 1e-6
        scale = np.maximum(np.abs(ref["force"]), 1.0)
        assert (np.abs(pts["force"] - ref["force"]) / scale).max() < 1e-6
    else:
        np.testing.assert_array_equal(pts["steps"], ref["steps"])
        np.testing.assert_array_equal(pts["tip"], ref["tip"])
        np.testing.assert_array_equal(pts["force"], ref["force"])
        np.testing.assert_array_equal(pts["energy"], ref["energy"])


@pytest.mark.parametrize("name", [n for n in POINT_CASES if golden(n).meta["sample"]])
def test_oracle_samples_match_reference(name):
    case = golden(name)
    desc = Input(case.input).desc()
    what = int(case.ref["sample_mode"])
    fe = oracle.sample(desc, case.ref["sample_pts"], what=what)
    ref = case.ref["sample_fe"]
    scale = np.maximum(np.abs(ref), 1e-3)
    tol = 1e-9 if name in FFT_CASES else 1e-14
    assert (np.abs(fe - ref) / scale).max() < tol


@pytest.mark.parametrize("name", ERROR_CASES)
def test_oracle_reproduces_reference_error(name):
    case = golden(name)
    desc = Input(case.input).desc()
    with pytest.raises(RuntimeError) as e:
        oracle.run(desc, 0, 1)
    expected = case.meta["error"].split("Value:")[0].strip()
    assert expected in str(e.value)


def test_oracle_detects_planted_error():
    """A planted change of the FIRE constants in a copy of the descriptor must show."""
    case = golden("cluster_ef")
    desc = Input(case.input).desc()
    c0, c1 = case.columns(desc.c.ny)[0]
    good, _ = oracle.run(desc, c0, c1)
    desc.c.dt = desc.c.dt * 1.01
    bad, _ = oracle.run(desc, c0, c1)
    assert not np.array_equal(good["tip"], bad["tip"])
