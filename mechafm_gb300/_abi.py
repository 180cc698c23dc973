"""ctypes mirror of include/mafm.h (the libmafm C ABI).

Only plain pointers and sizes cross the boundary; numpy arrays are passed via
their data pointers.  The structure layouts must match the header exactly;
tests/test_abi.py checks the sizes against the compiled library.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmafm.so")

MAFM_OK = 0
MAFM_E_INVALID, MAFM_E_IO, MAFM_E_PARSE, MAFM_E_CUDA = 1, 2, 3, 4
MAFM_E_NOMEM, MAFM_E_RANGE, MAFM_E_DEVICE, MAFM_E_UNSUPPORTED = 5, 6, 7, 8

MIN_SD, MIN_FIRE = 0, 1
INT_EULER, INT_MIDPOINT, INT_RK4 = 0, 1, 2
TERM_E, TERM_F, TERM_EF = 0, 1, 2
PAIR_LJ, PAIR_MORSE = 0, 1
FP64, FP32C, DF = 0, 1, 2
PT_MAXSTEPS, PT_NONFINITE, PT_OUTSIDE, PT_NEAR_TIE, PT_FP64 = 1, 2, 4, 8, 16
NOALLOC_MAX_SCANS = 32


class Pair(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("p", C.c_double * 3)]


class ScanDesc(C.Structure):
    _fields_ = [
        ("n_atoms", C.c_int32), ("n_types", C.c_int32),
        ("pos", C.POINTER(C.c_double)), ("charge", C.POINTER(C.c_double)),
        ("type", C.POINTER(C.c_int32)), ("tip_pair", C.POINTER(Pair)),
        ("dummy_pair", Pair),
        ("tip_charge", C.c_double), ("dummy_charge", C.c_double), ("qbase", C.c_double),
        ("coulomb", C.c_int32), ("tip_dummy_coulomb", C.c_int32),
        ("harm_k", C.c_double), ("harm_r0", C.c_double), ("tip_dummy_d", C.c_double),
        ("vdw_pbc", C.c_int32), ("tip_pbc", C.c_int32),
        ("cell", C.c_double * 9), ("offset", C.c_double * 3),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("flexible", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("zhigh", C.c_double), ("zlow", C.c_double), ("area", C.c_double * 2),
        ("minimiser", C.c_int32), ("integrator", C.c_int32),
        ("minterm", C.c_int32), ("maxsteps", C.c_int32),
        ("etol", C.c_double), ("ftol", C.c_double), ("dt", C.c_double),
        ("rigidgrid", C.c_int32), ("use_external_potential", C.c_int32),
        ("epot", C.POINTER(C.c_double)), ("epot_n", C.c_int32 * 3), ("reserved1", C.c_int32),
        ("epot_basis", C.c_double * 9), ("epot_origin", C.c_double * 3),
    ]


class Point(C.Structure):
    _fields_ = [("tip", C.c_double * 3), ("force", C.c_double * 3), ("energy", C.c_double),
                ("steps", C.c_int32), ("status", C.c_int32)]


# numpy view of mafm_point (64 bytes)
POINT_DTYPE = np.dtype([("tip", "<f8", (3,)), ("force", "<f8", (3,)), ("energy", "<f8"),
                        ("steps", "<i4"), ("status", "<i4")])
assert POINT_DTYPE.itemsize == C.sizeof(Point) == 64


class RunOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("lanes_per_column", C.c_int32),
                ("block_threads", C.c_int32), ("columns_per_tile", C.c_int32),
                ("col_begin", C.c_int32), ("col_end", C.c_int32)]


class RunStats(C.Structure):
    _fields_ = [("total_steps", C.c_uint64), ("force_evals", C.c_uint64),
                ("pair_evals", C.c_uint64), ("error_word", C.c_uint32),
                ("fp64_columns", C.c_uint32), ("kernel_ms", C.c_double)]


class FlexDesc(C.Structure):
    _fields_ = [
        ("fixed", C.POINTER(C.c_int32)),
        ("n_bonds", C.c_int32), ("bond_atoms", C.POINTER(C.c_int32)),
        ("bond_param", C.POINTER(C.c_double)),
        ("n_angles", C.c_int32), ("angle_atoms", C.POINTER(C.c_int32)),
        ("angle_param", C.POINTER(C.c_double)),
        ("n_dihedrals", C.c_int32), ("dihedral_atoms", C.POINTER(C.c_int32)),
        ("dihedral_param", C.POINTER(C.c_double)),
        ("n_pairs", C.c_int32), ("pair_atoms", C.POINTER(C.c_int32)),
        ("pair_vdw", C.POINTER(Pair)), ("pair_qq", C.POINTER(C.c_double)),
        ("substrate", C.c_double * 5),
    ]


class DfParams(C.Structure):
    _fields_ = [("amplitude", C.c_double), ("k_cantilever", C.c_double), ("f0", C.c_double)]


class Grad(C.Structure):
    _fields_ = [("dpos", C.POINTER(C.c_double)), ("dcharge", C.POINTER(C.c_double)),
                ("dpair", C.POINTER(C.c_double))]


# Every symbol the header declares, with its ctypes signature.
_P = C.c_void_p
SIGNATURES = {
    "mafm_last_error": (C.c_char_p, []),
    "mafm_abi_version": (C.c_int, []),
    "mafm_input_load": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(_P)]),
    "mafm_input_desc": (C.c_int, [_P, C.POINTER(ScanDesc)]),
    "mafm_input_output_opts": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int32)]),
    "mafm_input_free": (C.c_int, [_P]),
    "mafm_scan_create": (C.c_int, [C.c_int, C.POINTER(ScanDesc), C.POINTER(_P)]),
    "mafm_scan_destroy": (C.c_int, [_P]),
    "mafm_scan_size": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "mafm_run": (C.c_int, [_P, C.POINTER(RunOpts), _P, C.POINTER(RunStats), _P]),
    "mafm_run_columns": (C.c_int, [_P, _P, C.c_int64, _P, C.POINTER(RunStats), _P]),
    "mafm_run_batch": (C.c_int, [C.POINTER(_P), C.c_int32, C.POINTER(RunOpts),
                                 C.POINTER(_P), C.POINTER(RunStats), _P]),
    "mafm_run_batch_noalloc": (C.c_int, [C.POINTER(_P), C.c_int32, C.POINTER(RunOpts),
                                         C.POINTER(_P), C.POINTER(RunStats), _P]),
    "mafm_plan_create": (C.c_int, [C.POINTER(_P), C.c_int32, C.POINTER(RunOpts), C.POINTER(_P),
                                   C.POINTER(_P)]),
    "mafm_plan_launch": (C.c_int, [_P, _P]),
    "mafm_plan_stats": (C.c_int, [_P, C.POINTER(RunStats), _P]),
    "mafm_plan_config": (C.c_int, [_P, C.POINTER(RunOpts)]),
    "mafm_plan_destroy": (C.c_int, [_P]),
    "mafm_autotune": (C.c_int, [C.POINTER(_P), C.c_int32, C.POINTER(RunOpts),
                                C.POINTER(C.c_double), _P]),
    "mafm_adjoint": (C.c_int, [_P, _P, _P, C.POINTER(Grad), _P]),
    "mafm_adjoint_ex": (C.c_int, [_P, C.c_int32, _P, _P, C.POINTER(Grad), _P]),
    "mafm_input_flex_desc": (C.c_int, [_P, C.POINTER(FlexDesc)]),
    "mafm_write_states": (C.c_int, [_P, _P, C.c_int32, C.c_char_p]),
    "mafm_flex_create": (C.c_int, [C.c_int, C.POINTER(ScanDesc), C.POINTER(FlexDesc),
                                   C.POINTER(C.c_void_p)]),
    "mafm_flex_destroy": (C.c_int, [_P]),
    "mafm_flex_run": (C.c_int, [_P, C.c_int32, C.c_int32, _P, C.POINTER(RunStats), C.c_int32,
                                _P, _P]),
    "mafm_df_weights": (C.c_int, [C.POINTER(DfParams), C.c_double, _P, C.c_int32,
                                  C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "mafm_df": (C.c_int, [_P, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                          C.POINTER(DfParams), _P, _P]),
    "mafm_df_adjoint": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                                  C.POINTER(DfParams), _P, _P]),
    "mafm_scan_sample": (C.c_int, [_P, C.c_int32, C.c_int32, _P, C.c_int64, _P]),
    "mafm_scan_grid_info": (C.c_int, [_P, C.c_int32, C.c_int32 * 3, C.c_double * 9,
                                      C.c_double * 3]),
    "mafm_scan_grid_copy": (C.c_int, [_P, C.c_int32, _P]),
    "mafm_scan_build_grid": (C.c_int, [_P, C.c_int32, _P]),
    "mafm_write_output": (C.c_int, [_P, _P, C.c_char_p, C.c_int32]),
    "mafm_writer_open": (C.c_int, [_P, C.c_char_p, C.c_int32, C.POINTER(_P)]),
    "mafm_writer_append": (C.c_int, [_P, _P, C.c_int32, C.c_int32]),
    "mafm_writer_close": (C.c_int, [_P]),
    "mafm_write_statistics": (C.c_int, [_P, C.c_char_p, C.c_uint64, C.c_double, C.c_double]),
}


class MafmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code
        self.msg = msg


_lib = None


def lib(path: str | None = None):
    """Load libmafm.so (built in-tree by mechafm_gb300.build) once."""
    global _lib
    if _lib is None:
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise OSError(f"{p} is missing: build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code: int) -> None:
    if code != MAFM_OK:
        raise MafmError(code, lib().mafm_last_error().decode(errors="replace"))


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)
