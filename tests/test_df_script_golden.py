"""Frequency-shift post-processing against the reference script's own output.

tests/golden/df_script/ref.npz was made by tests/golden/make_df_golden.py,
which runs simple-vafm-image.py itself (under Python 3, plotting stubbed) on
scan files written by the reference executable: its weights W and factor
fshiftfac for several height steps (simple-vafm-image.py:76-89) and its
frequency-shift images DF (:204) for every window of a 21-height scan.

Oracle and product weights: bit for bit.  Oracle images: bit for bit (the
same numpy expression).  GPU images: the kernel sums each window in order in
FP64, numpy pairwise, so to 1e-13 of the image's magnitude.
"""
import os

import numpy as np
import pytest

from oracle import df as odf
from mechafm_gb300 import df

REF = np.load(os.path.join(os.path.dirname(__file__), "golden", "df_script", "ref.npz"))


def _script_weights(i):
    w = REF["sw"][i]
    return w[~np.isnan(w)], float(REF["sfac"][i])


@pytest.mark.parametrize("i", range(len(REF["steps"])))
def test_oracle_weights_equal_script(i):
    want, wfac = _script_weights(i)
    with np.errstate(divide="ignore", invalid="ignore"):
        w, fac = odf.weights(float(REF["steps"][i]))
    assert fac == wfac
    np.testing.assert_array_equal(w, want)


@pytest.mark.parametrize("i", range(len(REF["steps"])))
def test_product_weights_equal_script(i):
    want, wfac = _script_weights(i)
    w, fac = df.weights(float(REF["steps"][i]))
    assert fac == wfac
    np.testing.assert_array_equal(w, want)


def test_oracle_images_equal_script():
    dz = float(REF["dz"])
    got = odf.df_images(REF["fz"], dz)
    assert got.shape == REF["df"].shape == (int(REF["nshifts"]), 5, 5)
    np.testing.assert_array_equal(got, REF["df"])


@pytest.mark.gpu
def test_gpu_images_match_script():
    dz = float(REF["dz"])
    want = REF["df"]
    got = df.df_images(REF["fz"], dz)
    assert got.shape == want.shape
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-13 * np.abs(want).max())
