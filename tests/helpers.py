"""Shared test helpers: NetCDF-3 fixture writers and trajectory predicates.

The writers restate the reference's test-file generators
(src/io/utility.rs:29-90 for bathymetry, :108-181 for current): f32 x and y
axes built as `i as f32 * step`, f64 fields laid out [y][x] (row-major, x
fastest), written as NetCDF-3 classic with scipy.
"""

from __future__ import annotations

import math

import numpy as np
from scipy.io import netcdf_file


def axes(x_num, y_num, x_step, y_step):
    x = np.arange(x_num, dtype=np.float32) * np.float32(x_step)
    y = np.arange(y_num, dtype=np.float32) * np.float32(y_step)
    return x, y


def bathymetry_arrays(x_num, y_num, x_step, y_step, depth_fn):
    """Arrays of create_netcdf3_bathymetry (src/io/utility.rs:29-45)."""
    x, y = axes(x_num, y_num, x_step, y_step)
    depth = np.array([[depth_fn(xx, yy) for xx in x] for yy in y], dtype=np.float64)
    return x, y, depth


def current_arrays(x_num, y_num, x_step, y_step, current_fn):
    """Arrays of create_netcdf3_current (src/io/utility.rs:108-128)."""
    x, y = axes(x_num, y_num, x_step, y_step)
    uv = [[current_fn(xx, yy) for xx in x] for yy in y]
    u = np.array([[p[0] for p in row] for row in uv], dtype=np.float64)
    v = np.array([[p[1] for p in row] for row in uv], dtype=np.float64)
    return x, y, u, v


def write_nc(path, variables, dims, version=1):
    """variables: name -> (dim names, array); dims: name -> length."""
    with netcdf_file(str(path), "w", version=version) as f:
        for name, n in dims.items():
            f.createDimension(name, n)
        for name, (dn, arr) in variables.items():
            arr = np.asarray(arr)
            var = f.createVariable(name, arr.dtype, dn)
            var[...] = arr
    return path


def write_bathymetry_nc(path, x_num, y_num, x_step, y_step, depth_fn):
    x, y, depth = bathymetry_arrays(x_num, y_num, x_step, y_step, depth_fn)
    write_nc(path, {"y": (("y",), y), "x": (("x",), x), "depth": (("y", "x"), depth)},
             {"y": y_num, "x": x_num})
    return x, y, depth


def write_current_nc(path, x_num, y_num, x_step, y_step, current_fn):
    x, y, u, v = current_arrays(x_num, y_num, x_step, y_step, current_fn)
    write_nc(path, {"y": (("y",), y), "x": (("x",), x), "u": (("y", "x"), u),
                    "v": (("y", "x"), v)}, {"y": y_num, "x": x_num})
    return x, y, u, v


# Predicates of src/tests/helper/mod.rs:12-66 over rows (x, y, kx, ky):
# rows whose x is NaN are skipped, the first row is the reference value.
def _rows(data):
    first = data[0]
    rest = [r for r in data[1:] if not math.isnan(r[0])]
    return first, rest


def increase(data, index):
    last, rest = _rows(data)
    last = last[index]
    for r in rest:
        if not r[index] > last:
            return False
        last = r[index]
    return True


def decrease(data, index):
    last, rest = _rows(data)
    last = last[index]
    for r in rest:
        if not r[index] < last:
            return False
        last = r[index]
    return True


def same(data, index):
    last, rest = _rows(data)
    last = last[index]
    for r in rest:
        if not r[index] == last:
            return False
        last = r[index]
    return True


XI, YI, KXI, KYI = 0, 1, 2, 3


def ray_rows(traj, n_rows, i):
    """Ray i of a [5][rows][n] trajectory as rows of (x, y, kx, ky)."""
    return traj[1:, : int(n_rows[i]), i].T


def assert_parity(gpu_traj, gpu_rows, cpu_traj, cpu_rows, rtol=1e-9, floors=(1.0, 1.0, 1e-6, 1e-6)):
    """Per-step agreement of the plain FP64 form with the oracle:
    |a - b| <= rtol * max(|b|, floor) for x, y (floor 1 m) and kx, ky
    (floor 1e-6 rad/m) over all rows before a ray's first non-finite row; t
    must match exactly there; row counts must match.  Returns the largest
    scaled error seen."""
    assert gpu_traj.shape == cpu_traj.shape
    np.testing.assert_array_equal(gpu_rows, cpu_rows)
    rows = gpu_traj.shape[1]
    n = gpu_traj.shape[2]
    cpu = cpu_traj[1:]
    gpu = gpu_traj[1:]
    finite = np.all(np.isfinite(cpu), axis=0)  # [rows][n]
    # rows before the first non-finite row of each ray
    first_bad = np.where(finite.all(axis=0), rows, np.argmin(finite, axis=0))
    valid = np.arange(rows)[:, None] < first_bad[None, :]
    np.testing.assert_array_equal(np.where(valid, gpu_traj[0], 0.0), np.where(valid, cpu_traj[0], 0.0))
    worst = 0.0
    for v in range(4):
        b = cpu[v]
        a = gpu[v]
        scale = rtol * np.maximum(np.abs(b), floors[v])
        err = np.where(valid, np.abs(a - b) / scale, 0.0)
        m = float(np.nanmax(err)) if err.size else 0.0
        if not m <= 1.0:
            idx = np.unravel_index(np.nanargmax(err), err.shape)
            raise AssertionError(
                f"variable {('x', 'y', 'kx', 'ky')[v]} row {idx[0]} ray {idx[1]}: gpu {a[idx]!r} "
                f"oracle {b[idx]!r} (scaled error {m:.3g} > 1)")
        worst = max(worst, m)
    # NaN appears in the same places (termination rows, NaN padding)
    np.testing.assert_array_equal(np.isnan(gpu), np.isnan(cpu))
    # beyond each ray's length both are NaN padding
    pad = np.arange(rows)[:, None] >= cpu_rows[None, :]
    assert np.all(np.isnan(gpu_traj[:, pad])) and np.all(np.isnan(cpu_traj[:, pad]))
    _ = n
    return worst
