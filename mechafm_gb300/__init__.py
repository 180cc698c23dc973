"""mechafm_gb300 — GB300 (sm_103a) implementation of the MechAFM scan hot path.

The compute path is libmafm.so (CUDA kernels + C++ host front-end, C ABI in
include/mafm.h).  This package holds the ctypes face of that ABI
(``scan.Input``, ``scan.Scan``, ``scan.run_batch``), the seeded synthetic
workload generator (``synth``) and the in-tree build (``build``).
"""
from ._abi import FP32C, FP64, MafmError  # noqa: F401
from .scan import Desc, Input, Scan, run_batch  # noqa: F401

__all__ = ["FP32C", "FP64", "MafmError", "Desc", "Input", "Scan", "run_batch"]
