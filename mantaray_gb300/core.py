"""Ray tracing entry points.

`single_ray` and `ray_tracing` keep the signatures and results of the
reference's Python API (python/mantaray/core.py:9-132), which calls the Rust
extension `_mantaray` (src/ffi.rs:25-85); here the work runs in the CUDA
library through its C ABI.  `trace` and `trace_device` are the array forms
(ManyRays::trace_many, src/ray.rs:98-127) over field objects that stay
resident on the GPU between calls.
"""

from __future__ import annotations

import datetime
import os
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .dataset import make_dataset
from .fields import Bathymetry, Current

VARNAMES = ("time", "x", "y", "kx", "ky")

_STOP_RULES = {"stage1": N.STOP_STAGE1, "fresh": N.STOP_FRESH}
_MATH = {"libm": N.MATH_LIBM, "identity": N.MATH_IDENTITY}


def _options(stop_rule, math) -> int:
    """Option bits of a trace call.  Named choices map to their bits; integers
    go to the library as they are (it rejects unknown bits)."""
    bits = 0
    for value, table, what in ((stop_rule, _STOP_RULES, "stop rule"), (math, _MATH, "math")):
        if isinstance(value, str):
            if value not in table:
                raise ValueError(f"unknown {what} {value!r} (one of {sorted(table)})")
            bits |= table[value]
        else:
            bits |= int(value)
    return bits


def num_steps(t0: float, t_end: float, dt: float) -> int:
    """ceil((t_end - t0) / dt) as the stepper counts its steps."""
    return int(N.load().mr_num_steps(float(t0), float(t_end), float(dt)))


@dataclass
class TraceResult:
    """Trajectories of n rays: traj[5][rows][n] (t, x, y, kx, ky)."""

    traj: np.ndarray
    n_rows: np.ndarray
    status: np.ndarray

    @property
    def rows(self) -> int:
        """Rows up to the longest ray (the reference's padded length)."""
        return int(self.n_rows.max()) if self.n_rows.size else 0

    def ray(self, i: int) -> np.ndarray:
        """Ray i as the reference's list of (t, x, y, kx, ky) rows."""
        return np.ascontiguousarray(self.traj[:, : self.n_rows[i], i].T)

    def ray_result(self, i: int) -> dict:
        """Ray i as the reference's RayResult (src/ray_result.rs:123-150)."""
        from . import results

        return results.ray_result(self.ray(i))

    def as_json(self, i: int) -> str:
        """Ray i serialised as RayResult::as_json (src/ray_result.rs:74-76)."""
        from . import results

        return results.as_json(self.ray_result(i))

    def append_tsv(self, path, i: int) -> None:
        """Ray i appended to a TSV file as src/ray.rs:219-243 writes it."""
        from . import results

        results.append_tsv(path, self.ray(i))


def _f64(a):
    return np.ascontiguousarray(np.atleast_1d(np.asarray(a, dtype=np.float64)))


def trace(bathymetry: Bathymetry, current: Current, x0, y0, kx0, ky0, duration: float,
          step_size: float, t0: float = 0.0, stop_rule="stage1", math="identity",
          out: np.ndarray | None = None, rows_cap: int | None = None) -> TraceResult:
    """Traces rays from t0 to t0 + duration with step `step_size` (plain FP64
    kernel).  stop_rule: "stage1" or "fresh"; math: "identity" (default: the
    reference's quantities with fewer FP64 instructions) or "libm" (the
    reference's transcendental calls in its order); both within 1e-9 of the
    reference at every step.  `out` may be a preallocated (page-locked for speed)
    float64 array of shape (5, rows_cap, n)."""
    L = N.load()
    x0, y0, kx0, ky0 = (_f64(a) for a in (x0, y0, kx0, ky0))
    n = x0.size
    if not (y0.size == kx0.size == ky0.size == n):
        raise ValueError("x0, y0, kx0 and ky0 must have the same length")
    t_end = t0 + duration
    if rows_cap is None:
        rows_cap = num_steps(t0, t_end, step_size) + 1 if out is None else out.shape[1]
    if out is None:
        out = np.empty((5, rows_cap, n), np.float64)
    elif out.shape != (5, rows_cap, n) or out.dtype != np.float64 or not out.flags.c_contiguous:
        raise ValueError("out must be a C-contiguous float64 array of shape (5, rows_cap, n)")
    n_rows = np.zeros(n, np.int32)
    status = np.zeros(n, np.uint8)
    N.check(L.mr_trace(bathymetry.handle, current.handle, n, x0.ctypes.data, y0.ctypes.data,
                       kx0.ctypes.data, ky0.ctypes.data, float(t0), float(t_end),
                       float(step_size), _options(stop_rule, math), rows_cap, out.ctypes.data,
                       n_rows.ctypes.data, status.ctypes.data))
    return TraceResult(out, n_rows, status)


def trace_device(bathymetry: Bathymetry, current: Current, x0, y0, kx0, ky0, t0: float,
                 t_end: float, step_size: float, traj, n_rows, status, stop_rule="stage1",
                 math="identity", stream=None) -> None:
    """Device-buffer form: every array argument is a CUDA tensor (torch) or any
    object with `data_ptr()`; traj has shape (5, rows_cap, n).  Asynchronous on
    `stream` (a torch.cuda.Stream, a raw handle, or None for the current
    torch stream)."""
    L = N.load()
    n = int(x0.numel())
    rows_cap = int(traj.shape[1])
    if stream is None:
        import torch

        stream = torch.cuda.current_stream()
    handle = getattr(stream, "cuda_stream", stream)
    N.check(L.mr_trace_device(bathymetry.handle, current.handle, n, x0.data_ptr(), y0.data_ptr(),
                              kx0.data_ptr(), ky0.data_ptr(), float(t0), float(t_end),
                              float(step_size), _options(stop_rule, math), rows_cap,
                              traj.data_ptr(), n_rows.data_ptr(), status.data_ptr(),
                              handle))


def _open_fields(bathymetry, current):
    b = bathymetry if isinstance(bathymetry, Bathymetry) else Bathymetry.open(os.fspath(bathymetry))
    c = current if isinstance(current, Current) else Current.open(os.fspath(current))
    return b, c


def single_ray(x0: float, y0: float, kx0: float, ky0: float, duration: float, step_size: float,
               bathymetry, current, math: str = "identity"):
    """Propagates one ray (reference: python/mantaray/core.py:9-65).

    `bathymetry` / `current` are NetCDF-3 paths (variables x, y, depth and
    x, y, u, v, as src/ffi.rs:36-38 requires) or field objects.  Returns a
    dataset over `time_step` with variables time, x, y, kx, ky.  `math`
    (not in the reference): "identity" (default) evaluates the reference's
    quantities with fewer FP64 instructions, "libm" its expressions with its
    transcendental calls (about 3x slower; it also reproduces the reference's
    single-step known answers to f64::EPSILON).  Both stay within 1e-9 of the
    reference at every step."""
    b, c = _open_fields(bathymetry, current)
    res = trace(b, c, x0, y0, kx0, ky0, duration, step_size, math=math)
    rows = int(res.n_rows[0])
    tmp = res.traj[:, :rows, 0]
    return make_dataset(
        {v: (("time_step",), tmp[i]) for i, v in enumerate(VARNAMES)},
        coords=("time", "x", "y"),
        attrs={"date_created": str(datetime.datetime.now())},
    )


def ray_tracing(x0, y0, kx0, ky0, duration: float, step_size: float, bathymetry, current,
                math: str = "identity"):
    """Traces many rays (reference: python/mantaray/core.py:68-132).

    Returns a dataset over (`time_step`, `ray`), rays shorter than the longest
    one padded with NaN.  `math` as in single_ray."""
    b, c = _open_fields(bathymetry, current)
    res = trace(b, c, x0, y0, kx0, ky0, duration, step_size, math=math)
    if res.n_rows.size == 0:
        raise ValueError("ray_tracing needs at least one ray")
    rows = res.rows
    data = res.traj[:, :rows, :]
    return make_dataset(
        {v: (("time_step", "ray"), data[i]) for i, v in enumerate(VARNAMES)},
        coords=("time", "x", "y"),
        attrs={"date_created": str(datetime.datetime.now())},
        index_coords={"time_step": np.arange(rows), "ray": np.arange(data.shape[2])},
    )
