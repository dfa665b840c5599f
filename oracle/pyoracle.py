"""ctypes binding of the CPU oracle (oracle/mantaray_oracle.cpp).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, as the checker.  The product package
(mantaray_gb300) never imports this module.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libmantaray_oracle.so")

OK = 0
ARGUMENT_OUT_OF_BOUNDS = 1
INVALID_ARGUMENT = 2
INDEX_OUT_OF_BOUNDS = 3

STOP_STAGE1 = 0
STOP_FRESH = 1

RAY_COMPLETE = 0
RAY_STOPPED = 1

_lib = None


def build() -> str:
    """Compile the oracle with its Makefile (g++, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
        os.path.join(_HERE, "mantaray_oracle.cpp")
    ):
        build()
    L = ctypes.CDLL(LIB_PATH)
    vp, sz, f32, f64, i32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_float, ctypes.c_double, ctypes.c_int
    P = ctypes.POINTER
    L.or_bathy_grid.restype = vp
    L.or_bathy_grid.argtypes = [sz, sz, P(f32), P(f32), P(f64), sz]
    L.or_bathy_constant.restype = vp
    L.or_bathy_constant.argtypes = [f32]
    L.or_bathy_slope.restype = vp
    L.or_bathy_slope.argtypes = [f32] * 5
    L.or_bathy_array.restype = vp
    L.or_bathy_array.argtypes = [sz, P(f32)]
    L.or_bathy_free.argtypes = [vp]
    L.or_current_grid.restype = vp
    L.or_current_grid.argtypes = [sz, sz, P(f64), P(f64), P(f64), sz, P(f64), sz]
    L.or_current_constant.restype = vp
    L.or_current_constant.argtypes = [f64, f64]
    L.or_current_free.argtypes = [vp]
    L.or_bilinear.restype = i32
    L.or_bilinear.argtypes = [P(f32), f32, f32, P(f32)]
    L.or_nearest_f32.restype = i32
    L.or_nearest_f32.argtypes = [f32, P(f32), sz, P(f32)]
    L.or_nearest_f64.restype = i32
    L.or_nearest_f64.argtypes = [f64, P(f64), sz, P(f64)]
    L.or_bathy_four_corners.restype = i32
    L.or_bathy_four_corners.argtypes = [vp, f32, f32, P(ctypes.c_uint64)]
    L.or_current_four_corners.restype = i32
    L.or_current_four_corners.argtypes = [vp, f64, f64, P(ctypes.c_uint64)]
    L.or_depth_and_gradient.restype = i32
    L.or_depth_and_gradient.argtypes = [vp, f32, f32, P(f32)]
    L.or_current_and_gradient.restype = i32
    L.or_current_and_gradient.argtypes = [vp, f64, f64, P(f64)]
    L.or_group_velocity.restype = i32
    L.or_group_velocity.argtypes = [f64, f64, P(f64)]
    L.or_dkdt_bathy.restype = None
    L.or_dkdt_bathy.argtypes = [f64, f64, f64, f64, P(f64)]
    L.or_odes.restype = i32
    L.or_odes.argtypes = [vp, vp, f64, f64, f64, f64, P(f64)]
    L.or_num_steps.restype = ctypes.c_uint64
    L.or_num_steps.argtypes = [f64, f64, f64]
    L.or_trace.restype = i32
    L.or_trace.argtypes = [vp, vp, sz, P(f64), P(f64), P(f64), P(f64), f64, f64, f64,
                           i32, sz, P(f64), P(ctypes.c_int32), P(ctypes.c_uint8), i32]
    L.or_trace_final.restype = i32
    L.or_trace_final.argtypes = [vp, vp, sz, P(f64), P(f64), P(f64), P(f64), f64, f64, f64,
                                 i32, P(f64), P(ctypes.c_int32), P(ctypes.c_uint8), i32]
    L.or_diff_end_states.restype = i32
    L.or_diff_end_states.argtypes = [P(f64), sz, sz, f64, f64, f64, f64, P(f64), P(f64), sz, sz,
                                     f64, f64, f64, f64, sz, P(f64), P(f64), P(f64), P(f64), f64,
                                     ctypes.c_uint64, P(f64), P(ctypes.c_uint8), i32]
    _lib = L
    return L


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


class Bathymetry:
    """A bathymetry field held by the oracle (grid or analytic)."""

    def __init__(self, handle, keep=()):
        if not handle:
            raise MemoryError("oracle bathymetry allocation failed")
        self.handle = handle
        self._keep = keep

    @classmethod
    def grid(cls, x, y, depth):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        d = np.ascontiguousarray(np.asarray(depth, dtype=np.float64).ravel())
        h = lib().or_bathy_grid(x.size, y.size, _ptr(x, ctypes.c_float), _ptr(y, ctypes.c_float),
                                _ptr(d, ctypes.c_double), d.size)
        return cls(h)

    @classmethod
    def constant(cls, h):
        return cls(lib().or_bathy_constant(h))

    @classmethod
    def slope(cls, h0=50.0, x0=0.0, y0=0.0, dhdx=-5e-2, dhdy=0.0):
        return cls(lib().or_bathy_slope(h0, x0, y0, dhdx, dhdy))

    @classmethod
    def array(cls, arr):
        a = np.ascontiguousarray(arr, dtype=np.float32)
        assert a.ndim == 2 and a.shape[0] == a.shape[1]
        return cls(lib().or_bathy_array(a.shape[0], _ptr(a, ctypes.c_float)))

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.or_bathy_free(self.handle)
            self.handle = None

    def depth_and_gradient(self, x, y):
        out = np.zeros(3, np.float32)
        e = lib().or_depth_and_gradient(self.handle, x, y, _ptr(out, ctypes.c_float))
        return e, out

    def four_corners(self, x, y):
        out = np.zeros(8, np.uint64)
        e = lib().or_bathy_four_corners(self.handle, x, y, _ptr(out, ctypes.c_uint64))
        return e, [(int(out[2 * i]), int(out[2 * i + 1])) for i in range(4)]


class Current:
    """A current field held by the oracle (grid or constant)."""

    def __init__(self, handle):
        if not handle:
            raise MemoryError("oracle current allocation failed")
        self.handle = handle

    @classmethod
    def grid(cls, x, y, u, v):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        u = np.ascontiguousarray(np.asarray(u, dtype=np.float64).ravel())
        v = np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel())
        h = lib().or_current_grid(x.size, y.size, _ptr(x, ctypes.c_double), _ptr(y, ctypes.c_double),
                                  _ptr(u, ctypes.c_double), u.size, _ptr(v, ctypes.c_double), v.size)
        return cls(h)

    @classmethod
    def constant(cls, u=0.0, v=0.0):
        return cls(lib().or_current_constant(u, v))

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.or_current_free(self.handle)
            self.handle = None

    def current_and_gradient(self, x, y):
        out = np.zeros(6, np.float64)
        e = lib().or_current_and_gradient(self.handle, x, y, _ptr(out, ctypes.c_double))
        return e, out

    def four_corners(self, x, y):
        out = np.zeros(8, np.uint64)
        e = lib().or_current_four_corners(self.handle, x, y, _ptr(out, ctypes.c_uint64))
        return e, [(int(out[2 * i]), int(out[2 * i + 1])) for i in range(4)]


def bilinear(points, target):
    p = np.ascontiguousarray(points, dtype=np.float32).reshape(12)
    out = np.zeros(1, np.float32)
    e = lib().or_bilinear(_ptr(p, ctypes.c_float), target[0], target[1], _ptr(out, ctypes.c_float))
    return e, out[0]


def nearest_f32(target, arr):
    a = np.ascontiguousarray(arr, dtype=np.float32)
    out = np.zeros(1, np.float32)
    e = lib().or_nearest_f32(target, _ptr(a, ctypes.c_float), a.size, _ptr(out, ctypes.c_float))
    return e, out[0]


def nearest_f64(target, arr):
    a = np.ascontiguousarray(arr, dtype=np.float64)
    out = np.zeros(1, np.float64)
    e = lib().or_nearest_f64(target, _ptr(a, ctypes.c_double), a.size, _ptr(out, ctypes.c_double))
    return e, out[0]


def group_velocity(k, h):
    out = np.zeros(1, np.float64)
    e = lib().or_group_velocity(k, h, _ptr(out, ctypes.c_double))
    return e, out[0]


def dkdt_bathy(k, h, dhdx, dhdy):
    out = np.zeros(2, np.float64)
    lib().or_dkdt_bathy(k, h, dhdx, dhdy, _ptr(out, ctypes.c_double))
    return out


def odes(bathy, current, x, y, kx, ky):
    out = np.zeros(4, np.float64)
    e = lib().or_odes(bathy.handle, current.handle, x, y, kx, ky, _ptr(out, ctypes.c_double))
    return e, out


def num_steps(t0, t_end, dt):
    return int(lib().or_num_steps(t0, t_end, dt))


def trace(bathy, current, x0, y0, kx0, ky0, t0, t_end, dt, stop_rule=STOP_STAGE1,
          rows_cap=None, threads=0):
    """Trace rays; returns (traj[5][rows][n], n_rows[n], status[n])."""
    x0, y0, kx0, ky0 = (np.ascontiguousarray(np.atleast_1d(a), dtype=np.float64)
                        for a in (x0, y0, kx0, ky0))
    n = x0.size
    if rows_cap is None:
        rows_cap = num_steps(t0, t_end, dt) + 1
    traj = np.empty((5, rows_cap, n), np.float64)
    n_rows = np.zeros(n, np.int32)
    status = np.zeros(n, np.uint8)
    rc = lib().or_trace(bathy.handle, current.handle, n, _ptr(x0, ctypes.c_double),
                        _ptr(y0, ctypes.c_double), _ptr(kx0, ctypes.c_double),
                        _ptr(ky0, ctypes.c_double), t0, t_end, dt, stop_rule, rows_cap,
                        _ptr(traj, ctypes.c_double), _ptr(n_rows, ctypes.c_int32),
                        _ptr(status, ctypes.c_uint8), threads)
    if rc != 0:
        raise ValueError("rows_cap too small")
    return traj, n_rows, status


def trace_final(bathy, current, x0, y0, kx0, ky0, t0, t_end, dt, stop_rule=STOP_STAGE1,
                threads=0):
    """Trace rays keeping only each ray's last row: (final[5][n], n_rows, status)."""
    x0, y0, kx0, ky0 = (np.ascontiguousarray(np.atleast_1d(a), dtype=np.float64)
                        for a in (x0, y0, kx0, ky0))
    n = x0.size
    final = np.empty((5, n), np.float64)
    n_rows = np.zeros(n, np.int32)
    status = np.zeros(n, np.uint8)
    lib().or_trace_final(bathy.handle, current.handle, n, _ptr(x0, ctypes.c_double),
                         _ptr(y0, ctypes.c_double), _ptr(kx0, ctypes.c_double),
                         _ptr(ky0, ctypes.c_double), t0, t_end, dt, stop_rule,
                         _ptr(final, ctypes.c_double), _ptr(n_rows, ctypes.c_int32),
                         _ptr(status, ctypes.c_uint8), threads)
    return final, n_rows, status


def diff_end_states(depth, bgeom, u, v, cgeom, x0, y0, kx0, ky0, dt, steps, threads=0):
    """End states [4][n] of the differentiation model (f64 lookups).
    bgeom/cgeom = (x0, y0, dx, dy); depth, u, v shaped [ny][nx]."""
    depth = np.ascontiguousarray(depth, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    x0, y0, kx0, ky0 = (np.ascontiguousarray(np.atleast_1d(a), dtype=np.float64)
                        for a in (x0, y0, kx0, ky0))
    n = x0.size
    end = np.empty((4, n), np.float64)
    status = np.zeros(n, np.uint8)
    d = ctypes.c_double
    rc = lib().or_diff_end_states(
        _ptr(depth, d), depth.shape[1], depth.shape[0], *bgeom, _ptr(u, d), _ptr(v, d), u.shape[1],
        u.shape[0], *cgeom, n, _ptr(x0, d), _ptr(y0, d), _ptr(kx0, d), _ptr(ky0, d), dt, steps,
        _ptr(end, d), _ptr(status, ctypes.c_uint8), threads)
    if rc != 0:
        raise ValueError("grids need at least 2 x 2 points")
    return end, status
