"""ctypes binding of libmantaray_gpu.so (C ABI: include/mantaray_gpu.h).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when the shared library has not been built.
"""

from __future__ import annotations

import ctypes
import os

from . import build as _build

OK = 0
ERR_INVALID_ARGUMENT = -1
ERR_CUDA = -2
ERR_IO = -3
ERR_READ = -4
ERR_CAPACITY = -5
ERR_OUT_OF_MEMORY = -6

RAY_COMPLETE = 0
RAY_STOPPED = 1

STOP_STAGE1 = 0x0
STOP_FRESH = 0x1
MATH_IDENTITY = 0x0
MATH_LIBM = 0x10

# Exported symbols (checked by the CPU test that loads the library).
SYMBOLS = (
    "mr_bathymetry_grid", "mr_bathymetry_open", "mr_bathymetry_constant", "mr_bathymetry_slope",
    "mr_bathymetry_array", "mr_bathymetry_destroy", "mr_current_grid", "mr_current_open",
    "mr_current_constant", "mr_current_destroy", "mr_num_steps", "mr_trace", "mr_trace_device",
    "mr_single_ray", "mr_single_ray_files", "mr_ray_tracing_files", "mr_netcdf3_read_f64",
    "mr_last_error", "mr_version", "mr_measure_fma_peak",
    "mr_batch_default_config", "mr_batch_create", "mr_batch_destroy", "mr_batch_trace_device",
    "mr_batch_graph_create", "mr_batch_graph_launch", "mr_batch_graph_destroy",
    "mr_batch_trace_device_static", "mr_diff_forward", "mr_diff_backward", "mr_diff_tangent",
    "mr_seed_point_sources", "mr_seed_line",
)

SEED_EVEN_DIRECTIONS = 0x1

STAGING_NONE = 0
STAGING_TILE = 1
STAGING_AHEAD = 2

BATCH_STATIC_MAX_SCENARIOS = 64

BATCH_COMPLETE = 0
BATCH_OUT_OF_DOMAIN = 1
BATCH_DRY = 2
BATCH_BAD_WAVENUMBER = 3


class DiffGrid(ctypes.Structure):
    """mr_diff_grid: a regular grid (points, origin, spacing)."""

    _fields_ = [("nx", ctypes.c_size_t), ("ny", ctypes.c_size_t), ("x0", ctypes.c_double),
                ("y0", ctypes.c_double), ("dx", ctypes.c_double), ("dy", ctypes.c_double)]


class BatchConfig(ctypes.Structure):
    """mr_batch_config: launch shape of the persistent batched kernel."""

    _fields_ = [("block", ctypes.c_int), ("blocks_per_sm", ctypes.c_int),
                ("rays_per_lane", ctypes.c_int), ("rebase_interval", ctypes.c_int),
                ("order", ctypes.c_int), ("staging", ctypes.c_int),
                ("sweep_steps", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class MantarayError(RuntimeError):
    """A C-ABI call returned a negative code."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class MantarayIOError(MantarayError, OSError):
    pass


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads the library (building it first if it is absent or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        _build.build()
    if not os.path.exists(path):
        raise ImportError(f"libmantaray_gpu.so is not built ({path}); run mantaray_gb300.build.build()")
    L = ctypes.CDLL(path)
    vp, sz, f32, f64, i32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_float, ctypes.c_double, ctypes.c_int
    P = ctypes.POINTER
    pp = P(ctypes.c_void_p)
    cs = ctypes.c_char_p
    sig = {
        "mr_bathymetry_grid": (i32, [sz, sz, vp, vp, vp, sz, pp]),
        "mr_bathymetry_open": (i32, [cs, cs, cs, cs, pp]),
        "mr_bathymetry_constant": (i32, [f32, pp]),
        "mr_bathymetry_slope": (i32, [f32, f32, f32, f32, f32, pp]),
        "mr_bathymetry_array": (i32, [sz, vp, pp]),
        "mr_bathymetry_destroy": (None, [vp]),
        "mr_current_grid": (i32, [sz, sz, vp, vp, vp, sz, vp, sz, pp]),
        "mr_current_open": (i32, [cs, cs, cs, cs, cs, pp]),
        "mr_current_constant": (i32, [f64, f64, pp]),
        "mr_current_destroy": (None, [vp]),
        "mr_num_steps": (ctypes.c_uint64, [f64, f64, f64]),
        "mr_trace": (i32, [vp, vp, sz, vp, vp, vp, vp, f64, f64, f64, i32, sz, vp, vp, vp]),
        "mr_trace_device": (i32, [vp, vp, sz, vp, vp, vp, vp, f64, f64, f64, i32, sz, vp, vp, vp, vp]),
        "mr_single_ray": (i32, [vp, vp, f64, f64, f64, f64, f64, f64, sz, vp, vp]),
        "mr_single_ray_files": (i32, [cs, cs, f64, f64, f64, f64, f64, f64, sz, vp, vp]),
        "mr_ray_tracing_files": (i32, [cs, cs, sz, vp, vp, vp, vp, f64, f64, sz, vp, vp, vp]),
        "mr_netcdf3_read_f64": (i32, [cs, cs, vp, sz, P(sz), P(i32)]),
        "mr_last_error": (cs, []),
        "mr_version": (i32, []),
        "mr_measure_fma_peak": (i32, [i32, P(f64)]),
        "mr_batch_default_config": (i32, [P(BatchConfig)]),
        "mr_batch_create": (i32, [sz, P(vp), P(vp), pp]),
        "mr_batch_destroy": (None, [vp]),
        "mr_batch_trace_device": (i32, [vp, sz, vp, vp, vp, vp, vp, f64, f64, ctypes.c_int64,
                                        ctypes.c_int64, sz, vp, vp, vp, vp, vp, P(BatchConfig), vp]),
        "mr_batch_graph_create": (i32, [vp, sz, vp, vp, vp, vp, vp, f64, f64, ctypes.c_int64,
                                        ctypes.c_int64, sz, vp, vp, vp, vp, vp, P(BatchConfig),
                                        pp]),
        "mr_batch_graph_launch": (i32, [vp, sz, vp]),
        "mr_diff_forward": (i32, [i32, P(DiffGrid), vp, P(DiffGrid), vp, vp, sz, vp, vp, vp, vp,
                                  f64, ctypes.c_int64, ctypes.c_int64, vp, vp, vp, vp]),
        "mr_diff_backward": (i32, [i32, P(DiffGrid), vp, P(DiffGrid), vp, vp, sz, vp, vp, vp, vp,
                                   f64, ctypes.c_int64, ctypes.c_int64, vp, vp, vp, vp, vp, vp,
                                   vp, vp, vp]),
        "mr_diff_tangent": (i32, [i32, P(DiffGrid), vp, P(DiffGrid), vp, vp, sz, vp, vp, vp, vp,
                                  vp, vp, vp, vp, f64, ctypes.c_int64, vp, vp, vp, vp]),
        "mr_batch_trace_device_static": (i32, [vp, sz, vp, vp, vp, vp, vp, f64, f64,
                                               ctypes.c_int64, ctypes.c_int64, sz, vp, vp, vp,
                                               vp, vp, P(BatchConfig), vp]),
        "mr_batch_graph_destroy": (None, [vp]),
        "mr_seed_point_sources": (i32, [vp, sz, vp, vp, sz, f64, f64, f64, f64, ctypes.c_uint64,
                                        i32, vp, vp, vp, vp, vp]),
        "mr_seed_line": (i32, [vp, f64, f64, f64, f64, sz, f64, f64, f64, f64, ctypes.c_uint64,
                               i32, vp, vp, vp, vp, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc: int) -> None:
    """Raises MantarayError for a negative return code."""
    if rc == OK:
        return
    msg = (load().mr_last_error() or b"").decode(errors="replace")
    if rc == ERR_IO:
        raise MantarayIOError(rc, msg)
    raise MantarayError(rc, msg)
