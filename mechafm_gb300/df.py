"""Frequency-shift images from Fz stacks (libmafm's mafm_df / mafm_df_adjoint).

The reference's post-processing script (simple-vafm-image.py:77-89, 204)
converts the Fz of consecutive scan heights into frequency-shift images with
Giessibl's weights.  Here the same operator runs on the GPU through the C ABI:

* ``weights(dz, params)`` returns (W, fshiftfac) as the script builds them;
* ``df_images(fz, dz)`` takes Fz as (nx, ny, nz) in scan-level order (k = 0 at
  zhigh, the layout of a relaxed scan) or a mafm_point array, and returns
  df images (nshift, nx, ny), window s covering ascending heights s..s+nosc-1;
* ``df_image_torch(fz, dz)`` is the differentiable version (backward is
  mafm_df_adjoint), so a loss on df images back-propagates into fz_image.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import check, lib, ptr

AMPLITUDE = 0.50                 # Angstrom
K_CANTILEVER = 1800 * 1.438978   # 1800 N/m in kcal/mol/A^2
F0 = 25.000e3                    # Hz


def params(amplitude=AMPLITUDE, k_cantilever=K_CANTILEVER, f0=F0) -> _abi.DfParams:
    return _abi.DfParams(amplitude, k_cantilever, f0)


def weights(dz: float, prm: _abi.DfParams | None = None):
    n = C.c_int32()
    fac = C.c_double()
    pp = C.byref(prm) if prm is not None else None
    check(lib().mafm_df_weights(pp, dz, None, 0, C.byref(n), C.byref(fac)))
    w = np.zeros(n.value)
    check(lib().mafm_df_weights(pp, dz, ptr(w), n.value, C.byref(n), C.byref(fac)))
    return w, fac.value


def _fz_view(fz, shape):
    """(array, stride in doubles, nx, ny, nz) for an Fz stack or mafm_point array."""
    if isinstance(fz, np.ndarray) and fz.dtype == _abi.POINT_DTYPE:
        if shape is None:
            raise ValueError("a point array needs shape=(nx, ny, nz)")
        fz = np.ascontiguousarray(fz)
        base = fz.ctypes.data + _abi.POINT_DTYPE.fields["force"][1] + 16
        return fz, C.c_void_p(base), 8, shape
    fz = np.ascontiguousarray(fz, dtype=np.float64)
    if shape is None:
        shape = fz.shape
    return fz, ptr(fz), 1, tuple(shape)


def df_images(fz, dz: float, prm: _abi.DfParams | None = None, shape=None, stream=None):
    """df images (nshift, nx, ny) of an Fz stack on the host (copied through the GPU)."""
    keep, p, stride, (nx, ny, nz) = _fz_view(fz, shape)
    w, _ = weights(dz, prm)
    out = np.zeros((nz - len(w), nx, ny)) if nz > len(w) else np.zeros(0)
    pp = C.byref(prm) if prm is not None else None
    check(lib().mafm_df(p, stride, nx, ny, nz, dz, pp, ptr(out), stream))
    del keep
    return out


def df_adjoint(g_df, nz: int, dz: float, prm: _abi.DfParams | None = None, stream=None):
    """dL/dFz (nx, ny, nz) from dL/ddf (nshift, nx, ny)."""
    g_df = np.ascontiguousarray(g_df, dtype=np.float64)
    _, nx, ny = g_df.shape
    out = np.zeros((nx, ny, nz))
    pp = C.byref(prm) if prm is not None else None
    check(lib().mafm_df_adjoint(ptr(g_df), nx, ny, nz, dz, pp, ptr(out), stream))
    return out


def _torch_df(fz, dz, prm, adjoint):
    import torch
    x = fz.detach().contiguous().double()
    nx, ny = x.shape[-2:] if adjoint else x.shape[:2]
    pp = C.byref(prm) if prm is not None else None
    stream = C.c_void_p(torch.cuda.current_stream(x.device).cuda_stream) if x.is_cuda else None
    if adjoint:
        nz = adjoint
        out = torch.empty((nx, ny, nz), dtype=torch.float64, device=x.device)
        check(lib().mafm_df_adjoint(C.c_void_p(x.data_ptr()), nx, ny, nz, dz, pp,
                                    C.c_void_p(out.data_ptr()), stream))
    else:
        nz = x.shape[2]
        nw = len(weights(dz, prm)[0])
        out = torch.empty((max(nz - nw, 0), nx, ny), dtype=torch.float64, device=x.device)
        check(lib().mafm_df(C.c_void_p(x.data_ptr()), 1, nx, ny, nz, dz, pp,
                            C.c_void_p(out.data_ptr()), stream))
    return out


def df_image_torch(fz, dz: float, prm: _abi.DfParams | None = None):
    """Differentiable df images (nshift, nx, ny) of a (nx, ny, nz) Fz tensor."""
    import torch

    class _Df(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x):
            ctx.nz = x.shape[2]
            ctx.dtype = x.dtype
            return _torch_df(x, dz, prm, 0).to(x.dtype)

        @staticmethod
        def backward(ctx, g):
            return _torch_df(g, dz, prm, ctx.nz).to(ctx.dtype)

    return _Df.apply(fz)
