"""ORACLE — test infrastructure, not product.

ctypes access to liboracle_mafm.so (the plain-C FP64 restatement of the
reference's scan path, oracle/mafm_oracle.c) and to the reference's own
binaries in oracle/_ref/ when they were built (oracle/Makefile `ref`).
Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "liboracle_mafm.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_DUMP = os.path.join(REF_DIR, "ref_dump")
REF_CLI = os.path.join(REF_DIR, "mechafm-omp")

_port = None


def reference_dir(reference: str | None = None) -> str | None:
    """The reference checkout: the argument, else $MAFM_REFERENCE_DIR, else None."""
    return reference or os.environ.get("MAFM_REFERENCE_DIR") or None


def build(reference: str | None = None) -> None:
    """Build the port (gcc) and, when the reference sources are given (argument
    or $MAFM_REFERENCE_DIR) and exist, oracle/_ref."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    ref = reference_dir(reference)
    if ref and os.path.isdir(os.path.join(ref, "src")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref}", "-j8"], check=True)


def port():
    """The oracle port library (loaded once)."""
    global _port
    if _port is None:
        from mechafm_gb300 import _abi
        if not os.path.exists(PORT_LIB):
            build()
        L = C.CDLL(PORT_LIB)
        L.oracle_run.restype = C.c_int
        L.oracle_run.argtypes = [C.POINTER(_abi.ScanDesc), C.c_int, C.c_int, C.c_void_p,
                                 C.c_int, C.POINTER(C.c_uint64)]
        L.oracle_run_columns.restype = C.c_int
        L.oracle_run_columns.argtypes = [C.POINTER(_abi.ScanDesc), C.c_void_p, C.c_int64,
                                         C.c_void_p, C.c_int, C.POINTER(C.c_uint64)]
        L.oracle_run_split.restype = C.c_int
        L.oracle_run_split.argtypes = [C.POINTER(_abi.ScanDesc), C.c_int, C.c_int, C.c_void_p,
                                       C.c_int, C.POINTER(C.c_uint64), C.c_double * 2]
        L.oracle_flex_run.restype = C.c_int
        L.oracle_flex_run.argtypes = [C.POINTER(_abi.ScanDesc), C.POINTER(_abi.FlexDesc), C.c_int,
                                      C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_uint64),
                                      C.c_int, C.c_void_p]
        L.oracle_sample.restype = C.c_int
        L.oracle_sample.argtypes = [C.POINTER(_abi.ScanDesc), C.c_int, C.c_void_p,
                                    C.c_int64, C.c_void_p]
        L.oracle_grid.restype = C.c_int
        L.oracle_grid.argtypes = [C.POINTER(_abi.ScanDesc), C.c_int, C.c_int32 * 3,
                                  C.c_void_p, C.c_int64]
        L.oracle_adjoint.restype = C.c_int
        L.oracle_adjoint.argtypes = [C.POINTER(_abi.ScanDesc), C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p]
        L.oracle_last_error.restype = C.c_char_p
        _port = L
    return _port


def _check(code: int) -> None:
    if code:
        raise RuntimeError(f"oracle failed [{code}]: "
                           f"{port().oracle_last_error().decode(errors='replace')}")


def run(desc, col_begin: int = 0, col_end: int | None = None, threads: int = 0):
    """Relax columns [col_begin, col_end) with the FP64 port; returns (points, total_steps)."""
    from mechafm_gb300 import _abi
    d = desc.c
    if col_end is None:
        col_end = d.nx * d.ny
    out = np.zeros((col_end - col_begin) * d.nz, dtype=_abi.POINT_DTYPE)
    steps = C.c_uint64(0)
    _check(port().oracle_run(C.byref(d), col_begin, col_end, out.ctypes.data_as(C.c_void_p),
                             threads, C.byref(steps)))
    return out, int(steps.value)


def run_columns(desc, columns, threads: int = 0):
    """Relax the listed columns (i * ny + j) with the FP64 port; returns
    (points, total_steps) with column columns[i] at points[i*nz:(i+1)*nz]."""
    from mechafm_gb300 import _abi
    d = desc.c
    cols = np.ascontiguousarray(columns, dtype=np.int32)
    if len(cols) and (cols.min() < 0 or cols.max() >= d.nx * d.ny):
        raise ValueError("column outside the scan")
    out = np.zeros(len(cols) * d.nz, dtype=_abi.POINT_DTYPE)
    steps = C.c_uint64(0)
    _check(port().oracle_run_columns(C.byref(d), cols.ctypes.data_as(C.c_void_p), len(cols),
                                     out.ctypes.data_as(C.c_void_p), threads, C.byref(steps)))
    return out, int(steps.value)


def run_split(desc, col_begin: int = 0, col_end: int | None = None, threads: int = 0):
    """run() plus its wall time split: (points, total_steps, setup_s, relax_s)."""
    from mechafm_gb300 import _abi
    d = desc.c
    if col_end is None:
        col_end = d.nx * d.ny
    out = np.zeros((col_end - col_begin) * d.nz, dtype=_abi.POINT_DTYPE)
    steps = C.c_uint64(0)
    t = (C.c_double * 2)()
    _check(port().oracle_run_split(C.byref(d), col_begin, col_end, out.ctypes.data_as(C.c_void_p),
                                   threads, C.byref(steps), t))
    return out, int(steps.value), t[0], t[1]


def flex_run(desc, flex, col_begin: int = 0, col_end: int | None = None, threads: int = 0,
             state_column: int = -1):
    """Relax a flexible scan with the FP64 port: (points, total_steps, states)."""
    from mechafm_gb300 import _abi
    d = desc.c
    if col_end is None:
        col_end = d.nx * d.ny
    out = np.zeros((col_end - col_begin) * d.nz, dtype=_abi.POINT_DTYPE)
    steps = C.c_uint64(0)
    states = np.zeros((d.nz, d.n_atoms + 2, 3)) if state_column >= 0 else None
    _check(port().oracle_flex_run(C.byref(d), C.byref(flex.c), col_begin, col_end,
                                  out.ctypes.data_as(C.c_void_p), threads, C.byref(steps),
                                  state_column,
                                  states.ctypes.data_as(C.c_void_p) if states is not None else None))
    return out, int(steps.value), states


def sample(desc, pts: np.ndarray, what: int = 0) -> np.ndarray:
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((len(pts), 4))
    _check(port().oracle_sample(C.byref(desc.c), what, pts.ctypes.data_as(C.c_void_p),
                                len(pts), out.ctypes.data_as(C.c_void_p)))
    return out


def adjoint(desc, pts, w):
    """FP64 gradients of sum_p w_p Fz_p (see oracle_adjoint): dpos, dcharge, dpair."""
    d = desc.c
    dpos = np.zeros((d.n_atoms, 3))
    dq = np.zeros(d.n_atoms)
    dpair = np.zeros((d.n_types, 3))
    w = np.ascontiguousarray(w, dtype=np.float64)
    _check(port().oracle_adjoint(C.byref(d), pts.ctypes.data_as(C.c_void_p),
                                 w.ctypes.data_as(C.c_void_p), dpos.ctypes.data_as(C.c_void_p),
                                 dq.ctypes.data_as(C.c_void_p), dpair.ctypes.data_as(C.c_void_p)))
    return {"dpos": dpos, "dcharge": dq, "dpair": dpair}


def grid(desc, what: int = 0) -> np.ndarray:
    n = (C.c_int32 * 3)()
    _check(port().oracle_grid(C.byref(desc.c), what, n, None, 0))
    out = np.zeros(n[0] * n[1] * n[2] * 4)
    _check(port().oracle_grid(C.byref(desc.c), what, n, out.ctypes.data_as(C.c_void_p),
                              out.size))
    return out.reshape(n[0], n[1], n[2], 4)


# ---- the reference itself (oracle/_ref, built from the reference sources) ----

REF_FIELDS = ["i", "j", "k", "steps", "tip_x", "tip_y", "tip_z", "dum_x", "dum_y", "dum_z",
              "pos_x", "pos_y", "pos_z", "fx", "fy", "fz", "e", "rx", "ry", "rz", "r", "angle",
              "vx", "vy", "vz"]


def ref_available() -> bool:
    return os.path.exists(REF_DUMP)


def ref_time_columns(input_file: str, columns, tmp_prefix: str, threads: int = 0):
    """The reference's own relaxation of the listed columns, timed inside
    ref_dump (OpenMP over columns): returns (points, wall_s, total_steps)."""
    cols = np.ascontiguousarray(columns, dtype=np.int32)
    path = tmp_prefix + "_cols.bin"
    cols.tofile(path)
    env = dict(os.environ)
    if threads > 0:
        env["OMP_NUM_THREADS"] = str(threads)
    r = subprocess.run([REF_DUMP, "time_cols", os.path.abspath(input_file), path], check=True,
                       capture_output=True, text=True, env=env)
    last = [l for l in r.stdout.splitlines() if l.startswith("points ")][-1].split()
    return int(last[1]), float(last[3]), int(last[5])


def ref_scan(input_file: str, out_bin: str, i_range=None, j_range=None) -> np.ndarray:
    """Run the reference's own code (oracle/_ref/ref_dump) over a pixel block."""
    args = [REF_DUMP, "scan", os.path.abspath(input_file), os.path.abspath(out_bin)]
    if i_range is not None:
        args += [str(i_range[0]), str(i_range[1]), str(j_range[0]), str(j_range[1])]
    subprocess.run(args, check=True, cwd=os.path.dirname(os.path.abspath(input_file)),
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return np.fromfile(out_bin).reshape(-1, 25)


def ref_sample(input_file: str, pts: np.ndarray, mode: str, tmp_prefix: str) -> np.ndarray:
    pin, pout = tmp_prefix + ".pts", tmp_prefix + ".fe"
    np.ascontiguousarray(pts, dtype=np.float64).tofile(pin)
    subprocess.run([REF_DUMP, mode, os.path.abspath(input_file), pin, pout], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return np.fromfile(pout).reshape(-1, 4)


def ref_system(input_file: str, out_txt: str) -> dict:
    subprocess.run([REF_DUMP, "system", os.path.abspath(input_file), out_txt], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    info = {"atoms": []}
    with open(out_txt) as f:
        for line in f:
            t = line.split()
            if t[0] == "atom":
                info["atoms"].append((t[1], float(t[2]), float(t[3]), float(t[4]),
                                      float(t[5]), int(t[6])))
            elif t[0] in ("n_points", "offset"):
                info[t[0]] = [float(x) for x in t[1:]]
            else:
                info[t[0]] = float(t[1])
    return info
