"""Bathymetry and current fields: owners of device (HBM) copies of the grids.

Python face of the field handles of the C ABI (mr_bathymetry / mr_current),
mirroring the reference's field types: CartesianNetcdf3
(src/bathymetry/cartesian_netcdf3.rs:35-256), ConstantDepth, ConstantSlope,
ArrayDepth, CartesianCurrent (src/current/cartesian_current.rs:18-213) and
ConstantCurrent.  The grids are staged to the GPU once, at construction.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _native as N


def _arr(a, dtype):
    return np.ascontiguousarray(np.asarray(a, dtype=dtype).ravel())


class Bathymetry:
    """A bathymetry field on the GPU."""

    def __init__(self, handle: int, kind: str, shape=None):
        self._h = ctypes.c_void_p(handle)
        self.kind = kind
        self.shape = shape  # (ny, nx) for grids

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    @classmethod
    def grid(cls, x, y, depth) -> "Bathymetry":
        """x[nx], y[ny] (stored f32, as the reference does), depth read with
        flat index nx*j + i (stored f64).  `depth` may be any array whose
        row-major flattening is that order, e.g. shape (ny, nx)."""
        L = N.load()
        x = _arr(x, np.float32)
        y = _arr(y, np.float32)
        d = _arr(depth, np.float64)
        out = ctypes.c_void_p()
        N.check(L.mr_bathymetry_grid(x.size, y.size, x.ctypes.data, y.ctypes.data, d.ctypes.data,
                                     d.size, ctypes.byref(out)))
        return cls(out.value, "grid", (y.size, x.size))

    @classmethod
    def open(cls, path, x_name="x", y_name="y", depth_name="depth") -> "Bathymetry":
        """CartesianNetcdf3::open: a NetCDF-3 classic / 64-bit-offset file."""
        L = N.load()
        out = ctypes.c_void_p()
        N.check(L.mr_bathymetry_open(os.fsencode(path), x_name.encode(), y_name.encode(),
                                     depth_name.encode(), ctypes.byref(out)))
        return cls(out.value, "grid")

    @classmethod
    def constant(cls, h: float = 1000.0) -> "Bathymetry":
        L = N.load()
        out = ctypes.c_void_p()
        N.check(L.mr_bathymetry_constant(h, ctypes.byref(out)))
        return cls(out.value, "constant")

    @classmethod
    def slope(cls, h0=50.0, x0=0.0, y0=0.0, dhdx=-5e-2, dhdy=0.0) -> "Bathymetry":
        """ConstantSlope with the reference builder's defaults
        (src/bathymetry/constant_slope.rs:28-44)."""
        L = N.load()
        out = ctypes.c_void_p()
        N.check(L.mr_bathymetry_slope(h0, x0, y0, dhdx, dhdy, ctypes.byref(out)))
        return cls(out.value, "slope")

    @classmethod
    def array(cls, arr) -> "Bathymetry":
        """ArrayDepth test field: square array, arr[i][j] with i the x index."""
        L = N.load()
        a = np.ascontiguousarray(arr, dtype=np.float32)
        if a.ndim != 2 or a.shape[0] != a.shape[1]:
            raise ValueError("ArrayDepth takes a square 2-D array")
        out = ctypes.c_void_p()
        N.check(L.mr_bathymetry_array(a.shape[0], a.ctypes.data, ctypes.byref(out)))
        return cls(out.value, "array")

    def close(self) -> None:
        if self._h and self._h.value:
            N.load().mr_bathymetry_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001  (interpreter shutdown)
            pass


class Current:
    """A current field on the GPU."""

    def __init__(self, handle: int, kind: str, shape=None):
        self._h = ctypes.c_void_p(handle)
        self.kind = kind
        self.shape = shape

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    @classmethod
    def grid(cls, x, y, u, v) -> "Current":
        L = N.load()
        x = _arr(x, np.float64)
        y = _arr(y, np.float64)
        u = _arr(u, np.float64)
        v = _arr(v, np.float64)
        out = ctypes.c_void_p()
        N.check(L.mr_current_grid(x.size, y.size, x.ctypes.data, y.ctypes.data, u.ctypes.data,
                                  u.size, v.ctypes.data, v.size, ctypes.byref(out)))
        return cls(out.value, "grid", (y.size, x.size))

    @classmethod
    def open(cls, path, x_name="x", y_name="y", u_name="u", v_name="v") -> "Current":
        """CartesianCurrent::open on a NetCDF-3 file."""
        L = N.load()
        out = ctypes.c_void_p()
        N.check(L.mr_current_open(os.fsencode(path), x_name.encode(), y_name.encode(),
                                  u_name.encode(), v_name.encode(), ctypes.byref(out)))
        return cls(out.value, "grid")

    @classmethod
    def constant(cls, u: float = 0.0, v: float = 0.0) -> "Current":
        L = N.load()
        out = ctypes.c_void_p()
        N.check(L.mr_current_constant(u, v, ctypes.byref(out)))
        return cls(out.value, "constant")

    def close(self) -> None:
        if self._h and self._h.value:
            N.load().mr_current_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def read_netcdf3_variable(path, name) -> np.ndarray:
    """Reads one NetCDF-3 variable as float64 with the library's own reader."""
    L = N.load()
    n = ctypes.c_size_t()
    t = ctypes.c_int()
    N.check(L.mr_netcdf3_read_f64(os.fsencode(path), name.encode(), None, 0, ctypes.byref(n),
                                  ctypes.byref(t)))
    out = np.empty(n.value, np.float64)
    N.check(L.mr_netcdf3_read_f64(os.fsencode(path), name.encode(), out.ctypes.data, out.size,
                                  ctypes.byref(n), ctypes.byref(t)))
    return out
