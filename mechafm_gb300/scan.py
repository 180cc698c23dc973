"""Python face of the libmafm C ABI (include/mafm.h).

Mirrors the reference's process flow (src/mechafm.cpp:209-233): load the input
files (readInputFile / readXYZFile / readParameterFile), prepare the System,
relax every pixel column, write the scan files.  Every call goes through the
C ABI; there is no Python or CPU compute path, and a missing libmafm.so is an
error.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi
from ._abi import check, lib, ptr


class Input:
    """Parsed input files plus the prepared System (opaque mafm_input)."""

    def __init__(self, input_file: str, verbose: bool = False):
        h = C.c_void_p()
        check(lib().mafm_input_load(os.fsencode(input_file), int(verbose), C.byref(h)))
        self._h = h
        self.path = input_file

    def close(self):
        if getattr(self, "_h", None):
            lib().mafm_input_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def desc(self) -> "Desc":
        d = _abi.ScanDesc()
        check(lib().mafm_input_desc(self._h, C.byref(d)))
        return Desc(d, keep=self)

    def flex_desc(self) -> "FlexDesc":
        """The flexible topology of a `flexible on` input (mafm_input_flex_desc)."""
        f = _abi.FlexDesc()
        check(lib().mafm_input_flex_desc(self._h, C.byref(f)))
        return FlexDesc(f, keep=self)

    def output_opts(self):
        g, s, b = C.c_int32(), C.c_int32(), C.c_int32()
        check(lib().mafm_input_output_opts(self._h, C.byref(g), C.byref(s), C.byref(b)))
        return {"gzip": bool(g.value), "statistics": bool(s.value), "bufsize": b.value}

    def write_output(self, points: np.ndarray, folder: str, gzip: bool | None = None):
        if gzip is None:
            gzip = self.output_opts()["gzip"]
        if folder and not folder.endswith("/"):
            folder += "/"
        points = np.ascontiguousarray(points, dtype=_abi.POINT_DTYPE)
        check(lib().mafm_write_output(self._h, ptr(points), os.fsencode(folder), int(gzip)))


class Desc:
    """A mafm_scan_desc plus whatever owns the memory its pointers refer to."""

    def __init__(self, c: _abi.ScanDesc, keep=None):
        self.c = c
        self._keep = keep

    def with_terms(self, pos: np.ndarray, charge: np.ndarray, pair: np.ndarray) -> "Desc":
        """A copy of this descriptor with new atom positions (n, 3), charges (n,)
        and tip pair parameters (n_types, 3); the copy owns those arrays."""
        c = _abi.ScanDesc()
        C.pointer(c)[0] = self.c
        n, nt = self.c.n_atoms, self.c.n_types
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(n, 3)
        charge = np.ascontiguousarray(charge, dtype=np.float64).reshape(n)
        pair = np.ascontiguousarray(pair, dtype=np.float64).reshape(nt, 3)
        pairs = (_abi.Pair * max(nt, 1))()
        for t in range(nt):
            pairs[t].kind = self.c.tip_pair[t].kind
            for m in range(3):
                pairs[t].p[m] = pair[t, m]
        c.pos = pos.ctypes.data_as(C.POINTER(C.c_double))
        c.charge = charge.ctypes.data_as(C.POINTER(C.c_double))
        c.tip_pair = C.cast(pairs, C.POINTER(_abi.Pair))
        return Desc(c, keep=(self, pos, charge, pairs))

    def crop(self, i0: int, j0: int, ni: int, nj: int) -> "Desc":
        """The ni x nj pixel block starting at pixel (i0, j0) as a scan of its
        own: pixel (i, j) of the copy is pixel (i0 + i, j0 + j) of this scan.
        The surface, the cell offset and the external field's origin move by
        -(i0 dx, j0 dy), so every tip–surface distance is unchanged, and the
        rigid grid of the copy lies on the same lattice (its spacing, dx/2 and
        dy/2, divides the shift).  Used to time and check sub-areas of scans
        whose full grid is too large for the FP64 and CPU paths."""
        d = self.c
        if not (0 <= i0 and 0 <= j0 and ni >= 1 and nj >= 1 and i0 + ni <= d.nx and j0 + nj <= d.ny):
            raise ValueError("crop outside the pixel grid")
        c = _abi.ScanDesc()
        C.pointer(c)[0] = d
        sx, sy = i0 * d.dx, j0 * d.dy
        pos = self.atoms()["pos"]
        pos[:, 0] -= sx
        pos[:, 1] -= sy
        pos = np.ascontiguousarray(pos.reshape(-1))
        c.pos = pos.ctypes.data_as(C.POINTER(C.c_double))
        c.nx, c.ny = ni, nj
        c.area[0] = (ni - 1) * d.dx
        c.area[1] = (nj - 1) * d.dy
        c.offset[0] = d.offset[0] - sx
        c.offset[1] = d.offset[1] - sy
        c.epot_origin[0] = d.epot_origin[0] - sx
        c.epot_origin[1] = d.epot_origin[1] - sy
        return Desc(c, keep=(self, pos))

    def pair_params(self) -> np.ndarray:
        return np.array([[self.c.tip_pair[t].p[m] for m in range(3)]
                         for t in range(self.c.n_types)]).reshape(self.c.n_types, 3)

    def pair_kinds(self) -> np.ndarray:
        return np.array([self.c.tip_pair[t].kind for t in range(self.c.n_types)], dtype=np.int32)

    @property
    def n_columns(self) -> int:
        return self.c.nx * self.c.ny

    @property
    def n_points(self) -> int:
        return self.c.nx * self.c.ny * self.c.nz

    @property
    def shape(self):
        return (self.c.nx, self.c.ny, self.c.nz)

    def atoms(self) -> dict:
        n = self.c.n_atoms
        return {
            "pos": np.ctypeslib.as_array(self.c.pos, shape=(n * 3,)).reshape(n, 3).copy(),
            "charge": np.ctypeslib.as_array(self.c.charge, shape=(n,)).copy(),
            "type": np.ctypeslib.as_array(self.c.type, shape=(n,)).copy(),
        }


class FlexDesc:
    """A mafm_flex_desc plus whatever owns the memory its pointers refer to."""

    def __init__(self, c: _abi.FlexDesc, keep=None):
        self.c = c
        self._keep = keep


class FlexScan:
    """A device-resident flexible scan (mafm_flex): FP64, one warp per column."""

    def __init__(self, desc: Desc, flex: FlexDesc, device: int = -1):
        h = C.c_void_p()
        check(lib().mafm_flex_create(device, C.byref(desc.c), C.byref(flex.c), C.byref(h)))
        self._h = h
        self.desc = desc
        self.flex = flex

    def close(self):
        if getattr(self, "_h", None):
            lib().mafm_flex_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, col_begin=0, col_end=0, state_column=-1, stream=None):
        """Relax columns [col_begin, col_end); returns (points, stats, states)
        with states (nz, n_atoms + 2, 3) for state_column, or None."""
        d = self.desc.c
        n_cols = (col_end - col_begin) if col_end else d.nx * d.ny
        out = np.zeros(n_cols * d.nz, dtype=_abi.POINT_DTYPE)
        st = _abi.RunStats()
        states = np.zeros((d.nz, d.n_atoms + 2, 3)) if state_column >= 0 else None
        check(lib().mafm_flex_run(self._h, col_begin, col_end, ptr(out), C.byref(st), state_column,
                                  ptr(states) if states is not None else None, stream))
        return out, st, states


def run_opts(precision=_abi.FP64, lanes=0, block=0, tile=0, col_begin=0, col_end=0):
    return _abi.RunOpts(precision, lanes, block, tile, col_begin, col_end)


class Scan:
    """A device-resident scan (mafm_scan)."""

    def __init__(self, desc: Desc, device: int = -1):
        h = C.c_void_p()
        check(lib().mafm_scan_create(device, C.byref(desc.c), C.byref(h)))
        self._h = h
        self.desc = desc

    def close(self):
        if getattr(self, "_h", None):
            lib().mafm_scan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def run(self, precision=_abi.FP64, lanes=0, block=0, tile=0, col_begin=0, col_end=0,
            out: np.ndarray | None = None, stream=None):
        """Relax the scan; returns (points, stats) with points in host memory."""
        n_cols = (col_end - col_begin) if col_end else self.desc.n_columns
        if out is None:
            out = np.zeros(n_cols * self.desc.c.nz, dtype=_abi.POINT_DTYPE)
        stats = _abi.RunStats()
        o = run_opts(precision, lanes, block, tile, col_begin, col_end)
        check(lib().mafm_run(self._h, C.byref(o), ptr(out), C.byref(stats), stream))
        return out, stats

    def run_columns(self, columns, stream=None):
        """Plain FP64 relaxation of the listed columns (i * ny + j); returns
        (points, stats) with column columns[m] at points[m*nz:(m+1)*nz]."""
        cols = np.ascontiguousarray(columns, dtype=np.int32)
        out = np.zeros(len(cols) * self.desc.c.nz, dtype=_abi.POINT_DTYPE)
        stats = _abi.RunStats()
        check(lib().mafm_run_columns(self._h, ptr(cols), len(cols), ptr(out), C.byref(stats),
                                     stream))
        return out, stats

    def run_device(self, out_ptr: int, precision=_abi.FP32C, lanes=0, block=0, tile=0,
                   stream=None, stats: bool = False):
        """Relax into device memory at out_ptr (no copy back).  stats=True synchronises."""
        st = _abi.RunStats() if stats else None
        o = run_opts(precision, lanes, block, tile)
        check(lib().mafm_run(self._h, C.byref(o), C.c_void_p(out_ptr),
                             C.byref(st) if st is not None else None, stream))
        return st

    def adjoint(self, points: np.ndarray, dl_dfz: np.ndarray, stream=None,
                precision=_abi.FP64) -> dict:
        """Gradients of L through the relaxation, given the relaxed points of a
        run and dL/dFz per point (mafm_adjoint_ex): dpos (n_atoms, 3), dcharge
        (n_atoms,), dpair (n_types, 3) for tip_pair[t].p."""
        d = self.desc.c
        points = np.ascontiguousarray(points, dtype=_abi.POINT_DTYPE)
        w = np.ascontiguousarray(dl_dfz, dtype=np.float64).reshape(-1)
        if len(points) != self.desc.n_points or len(w) != self.desc.n_points:
            raise ValueError("adjoint needs every point of the scan")
        dpos = np.zeros((d.n_atoms, 3))
        dq = np.zeros(d.n_atoms)
        dpair = np.zeros((d.n_types, 3))
        g = _abi.Grad(dpos.ctypes.data_as(C.POINTER(C.c_double)),
                      dq.ctypes.data_as(C.POINTER(C.c_double)),
                      dpair.ctypes.data_as(C.POINTER(C.c_double)))
        check(lib().mafm_adjoint_ex(self._h, precision, ptr(points), ptr(w), C.byref(g), stream))
        return {"dpos": dpos, "dcharge": dq, "dpair": dpair}

    def sample(self, pts: np.ndarray, precision=_abi.FP64, what: int = 0) -> np.ndarray:
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((len(pts), 4))
        check(lib().mafm_scan_sample(self._h, precision, what, ptr(pts), len(pts), ptr(out)))
        return out

    def grid_info(self, what: int = 0):
        n = (C.c_int32 * 3)()
        b = (C.c_double * 9)()
        o = (C.c_double * 3)()
        check(lib().mafm_scan_grid_info(self._h, what, n, b, o))
        return tuple(n), np.array(b[:]).reshape(3, 3), np.array(o[:])

    def grid(self, what: int = 0) -> np.ndarray:
        n, _, _ = self.grid_info(what)
        out = np.zeros(n[0] * n[1] * n[2] * 4)
        check(lib().mafm_scan_grid_copy(self._h, what, ptr(out)))
        return out.reshape(n[0], n[1], n[2], 4)


def run_batch(scans: list, precision=_abi.FP32C, lanes=0, block=0, tile=0, stream=None):
    """Relax several scans in one persistent launch; returns (list of points, stats)."""
    n = len(scans)
    handles = (C.c_void_p * n)(*[s.handle for s in scans])
    outs = [np.zeros(s.desc.n_points, dtype=_abi.POINT_DTYPE) for s in scans]
    optrs = (C.c_void_p * n)(*[o.ctypes.data for o in outs])
    stats = _abi.RunStats()
    o = run_opts(precision, lanes, block, tile)
    check(lib().mafm_run_batch(handles, n, C.byref(o), optrs, C.byref(stats), stream))
    return outs, stats
