"""Differentiable Fz images for PyTorch (the optional Python binding).

`fz_image(desc, pos, charge, pair)` relaxes the scan on the GPU through the C
ABI and returns the tip–surface Fz of every point as a tensor (nx, ny, nz);
its backward calls mafm_adjoint_ex (implicit differentiation at the relaxed
points) in the forward's precision.  pos (n_atoms, 3) are the prepared surface positions, charge
(n_atoms,) the Coulomb charges, pair (n_types, 3) the tip pair parameters
(LJ es6, es12, 0; Morse De, a, re).  Give pair as a function of per-type
eps/sigma with `lj_pair_params` to get eps/sigma gradients by autograd.

Fz images are what simple-vafm-image.py turns into frequency-shift images;
`mechafm_gb300.df` holds that operator.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _abi
from .scan import Desc, Scan


class _FzImage(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, charge, pair, desc, precision, device):
        d = desc.with_terms(pos.detach().cpu().double().numpy(),
                            charge.detach().cpu().double().numpy(),
                            pair.detach().cpu().double().numpy())
        scan = Scan(d, device=device)
        # pinned host records: the kernel writes them directly, and the
        # backward's upload of them runs at the link's speed
        buf = torch.empty(d.n_points * _abi.POINT_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
        pts, _ = scan.run(precision, out=buf.numpy().view(_abi.POINT_DTYPE))
        ctx.buf = buf
        ctx.scan = scan
        ctx.pts = pts
        ctx.precision = precision
        ctx.shapes = (pos.shape, charge.shape, pair.shape)
        ctx.dtypes = (pos.dtype, charge.dtype, pair.dtype)
        ctx.devices = (pos.device, charge.device, pair.device)
        fz = torch.from_numpy(pts["force"][:, 2].copy()).reshape(d.shape)
        return fz.to(device=pos.device, dtype=pos.dtype)

    @staticmethod
    def backward(ctx, grad_fz):
        w = grad_fz.detach().double().cpu().numpy().reshape(-1)
        # a double-float forward differentiates with the FP32C adjoint (within
        # 1e-5 of the FP64 one); the others in their own precision
        prec = _abi.FP32C if ctx.precision == _abi.DF else ctx.precision
        g = ctx.scan.adjoint(ctx.pts, w, precision=prec)
        out = []
        for key, shape, dt, dev in zip(("dpos", "dcharge", "dpair"), ctx.shapes, ctx.dtypes,
                                       ctx.devices):
            out.append(torch.from_numpy(g[key]).reshape(shape).to(device=dev, dtype=dt))
        ctx.scan.close()
        return out[0], out[1], out[2], None, None, None


def fz_image(desc: Desc, pos, charge, pair, precision=_abi.FP64, device: int = 0):
    """Fz image (nx, ny, nz) of the scan with these terms; differentiable."""
    return _FzImage.apply(pos, charge, pair, desc, precision, device)


def lj_pair_params(eps, sigma, eps_tip: float, sigma_tip: float):
    """Tip–type LJ parameters by the reference's mixing (simulation.cpp:261-264):
    es6 = 4 sqrt(eps eps_tip) ((sigma + sigma_tip)/2)^6, es12 likewise with ^12."""
    e = torch.sqrt(eps * eps_tip)
    s = (sigma + sigma_tip) / 2
    return torch.stack([4 * e * s ** 6, 4 * e * s ** 12, torch.zeros_like(e)], dim=-1)
