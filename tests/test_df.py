"""Frequency-shift images (mafm_df, mafm_df_adjoint) against the oracle's
numpy restatement of simple-vafm-image.py:77-89, 204.

Weights: bit-exact (host arithmetic in the same order).  Images: the GPU sums
the window in the same order in FP64; numpy's (FZ*W).sum uses pairwise
summation, so images agree to 1e-13 relative to the image's magnitude.
Adjoint: <df(x), y> = <x, df_adjoint(y)> to 1e-12 relative.
"""
import numpy as np
import pytest

from oracle import df as odf
from mechafm_gb300 import _abi, df

STEPS = [0.1, 0.05, 0.2, 0.25, 0.125, 0.3, 0.07, 0.5 / 3]


@pytest.mark.parametrize("dz", STEPS)
def test_weights_match_script(dz):
    w, fac = df.weights(dz)
    want, wfac = odf.weights(dz)
    assert fac == wfac
    assert len(w) == len(want)
    np.testing.assert_array_equal(w, want)


@pytest.mark.parametrize("amp,dz", [(0.3, 0.1), (1.0, 0.1), (0.45, 0.1), (2.0, 0.25), (0.8, 0.3)])
def test_weights_other_amplitudes(amp, dz):
    w, fac = df.weights(dz, df.params(amplitude=amp, k_cantilever=1000.0, f0=30e3))
    want, wfac = odf.weights(dz, amplitude=amp, k_cantilever=1000.0, f0=30e3)
    assert fac == wfac
    np.testing.assert_array_equal(w, want)


def test_weights_reject_bad_step():
    with pytest.raises(_abi.MafmError):
        df.weights(0.0)
    with pytest.raises(_abi.MafmError):
        df.weights(1e-5)      # window of more than 4096 heights


def _stack(seed, nx=7, ny=5, nz=40):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(nx, ny, nz)) * 0.3


@pytest.mark.gpu
@pytest.mark.parametrize("dz", [0.1, 0.05, 0.25])
def test_df_images_match_oracle(dz):
    fz = _stack(1)
    got = df.df_images(fz, dz)
    want = odf.df_images(fz, dz)
    assert got.shape == want.shape
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-13 * np.abs(want).max())


@pytest.mark.gpu
def test_df_images_from_points():
    fz = _stack(2, nz=30)
    pts = np.zeros(fz.size, dtype=_abi.POINT_DTYPE)
    pts["force"][:, 2] = fz.reshape(-1)
    pts["force"][:, 0] = 1e9          # must not be read
    got = df.df_images(pts, 0.1, shape=fz.shape)
    np.testing.assert_array_equal(got, df.df_images(fz, 0.1))


@pytest.mark.gpu
def test_df_too_few_heights_is_an_error():
    with pytest.raises(_abi.MafmError):
        df.df_images(_stack(3, nz=8), 0.1)     # 8-height window at dz = 0.1


@pytest.mark.gpu
def test_df_adjoint_is_transpose():
    dz, nz = 0.1, 33
    x = _stack(4, nz=nz)
    y = np.random.default_rng(5).normal(size=(nz - len(df.weights(dz)[0]), 7, 5))
    lhs = float((df.df_images(x, dz) * y).sum())
    rhs = float((x * df.df_adjoint(y, nz, dz)).sum())
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


@pytest.mark.gpu
def test_df_torch_device_and_grad():
    torch = pytest.importorskip("torch")
    dz = 0.1
    fz = torch.tensor(_stack(6, nz=25), device="cuda", requires_grad=True)
    img = df.df_image_torch(fz, dz)
    want = odf.df_images(fz.detach().cpu().numpy(), dz)
    np.testing.assert_allclose(img.detach().cpu().numpy(), want, rtol=0,
                               atol=1e-13 * np.abs(want).max())
    g = torch.randn_like(img)
    img.backward(g)
    np.testing.assert_allclose(fz.grad.cpu().numpy(),
                               df.df_adjoint(g.cpu().numpy(), 25, dz), rtol=0, atol=1e-15)


def test_oracle_df_adjoint_is_transpose():
    dz, nz = 0.1, 21
    x = _stack(7, nz=nz)
    y = np.random.default_rng(8).normal(size=(nz - len(odf.weights(dz)[0]), 7, 5))
    lhs = float((odf.df_images(x, dz) * y).sum())
    rhs = float((x * odf.df_adjoint(y, nz, dz)).sum())
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


@pytest.mark.gpu
def test_df_loss_backpropagates_through_the_relaxation(tmp_path):
    """fz_image -> df_image_torch -> loss: the atom-position gradient equals the
    oracle adjoint driven by the transposed df operator."""
    torch = pytest.importorskip("torch")
    import oracle
    from mechafm_gb300 import synth
    from mechafm_gb300.scan import Input
    from mechafm_gb300.torch_ops import fz_image
    spec = synth.cluster_60(area=0.3, step=0.1, zhigh=10.0, zlow=8.5, minterm="f",
                            ftol="1e-10", maxsteps="400000")
    desc = Input(spec.write(str(tmp_path))).desc()
    dz = desc.c.dz
    a = desc.atoms()
    pos = torch.tensor(a["pos"], requires_grad=True)
    fz = fz_image(desc, pos, torch.tensor(a["charge"]), torch.tensor(desc.pair_params()))
    img = df.df_image_torch(fz.cuda(), dz)
    g = torch.randn_like(img)
    (img * g).sum().backward()
    pts, _ = oracle.run(desc)
    w = odf.df_adjoint(g.cpu().numpy(), desc.c.nz, dz).reshape(-1)
    want = oracle.adjoint(desc, pts, w)["dpos"]
    np.testing.assert_allclose(pos.grad.numpy(), want, rtol=1e-6, atol=1e-9 * np.abs(want).max())
