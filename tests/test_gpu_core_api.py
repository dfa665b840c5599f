"""The reference-facing API on the GPU: single_ray / ray_tracing over NetCDF-3
files (the port of python/tests/test_core.py), the file-path C entry points,
host-buffer forms (pageable and page-locked), the device form, and error
behaviour."""

import ctypes
import math

import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mr():
    import mantaray_gb300 as m

    m._native.load()
    return m


def deep_water_constant_depth(path):
    # python/tests/test_core.py:9-21 (depth declared on dims ("x", "y"), a
    # square constant array, written NETCDF3_CLASSIC)
    H.write_nc(path, {"depth": (("x", "y"), 10_000 * np.ones((3, 3))),
                      "x": (("x",), np.array([-1e4, 0, 1e4])),
                      "y": (("y",), np.array([-1e4, 0, 1e4]))}, {"x": 3, "y": 3})
    return path


def zero_current_field(path):
    # python/tests/test_core.py:24-37
    H.write_nc(path, {"u": (("x", "y"), 0.01 * np.ones((3, 3))),
                      "v": (("x", "y"), 0.01 * np.ones((3, 3))),
                      "x": (("x",), np.array([-1e8, 0, 1e8])),
                      "y": (("y",), np.array([-1e8, 0, 1e8]))}, {"x": 3, "y": 3})
    return path


@pytest.fixture
def files(tmp_path):
    return (deep_water_constant_depth(tmp_path / "island.nc"),
            zero_current_field(tmp_path / "current.nc"))


def test_single_ray(mr, files):
    # python/tests/test_core.py:40-53
    ds = mr.single_ray(-1000, 0, 0.01, 0, 10, 2, files[0], files[1])
    assert ds.sizes["time_step"] == 6
    assert (ds.kx == 0.01).all()
    assert (ds.ky == 0.0).all()
    assert set(ds.coords) == {"time", "x", "y"}


def test_multiple_rays(mr, files):
    # python/tests/test_core.py:56-78
    ds = mr.ray_tracing(3 * [-1000], 3 * [0], 3 * [0.01], 3 * [0], 10, 2, str(files[0]),
                        str(files[1]))
    assert ds.sizes["time_step"] == 6
    assert ds.sizes["ray"] == 3
    assert (ds.kx == 0.01).all()
    assert (ds.ky == 0.0).all()


def test_libm_math_through_the_drop_in(mr, oracle, files):
    # the reference's own transcendental calls through the reference-shaped
    # call: same rows, values within the parity bar of the default call
    x0, y0 = [-1000.0, 200.0, 3000.0], [0.0, -500.0, 250.0]
    kx0, ky0 = [0.01, 0.02, 0.005], [0.0, 0.01, -0.01]
    a = mr.ray_tracing(x0, y0, kx0, ky0, 200, 1, str(files[0]), str(files[1]), math="libm")
    b = mr.ray_tracing(x0, y0, kx0, ky0, 200, 1, str(files[0]), str(files[1]))
    assert a.sizes == b.sizes
    for v, floor in (("x", 1.0), ("y", 1.0), ("kx", 1e-6), ("ky", 1e-6)):
        va, vb = np.asarray(a[v]), np.asarray(b[v])
        np.testing.assert_array_equal(np.isnan(va), np.isnan(vb))
        ok = np.isfinite(va)
        assert np.all(np.abs(va[ok] - vb[ok]) <= 1e-9 * np.maximum(np.abs(va[ok]), floor))


def test_rays_variable_length(mr, oracle, files):
    # python/tests/test_core.py:81-101 (no assertion there): one ray reaches
    # the grid edge first; the shorter ray is NaN padded to the longer one.
    ds = mr.ray_tracing(2 * [-1e3], 2 * [0], [-0.01, 0.01], 2 * [0], 1e6, 20, str(files[0]),
                        str(files[1]))
    x = np.asarray(ds["x"])
    lengths = np.sum(~np.isnan(np.asarray(ds["time"])), axis=0)
    assert lengths[0] != lengths[1]
    assert ds.sizes["time_step"] == lengths.max()
    short = int(np.argmin(lengths))
    assert np.all(np.isnan(x[lengths[short]:, short]))
    # agreement with the oracle on the same file contents
    b = oracle.Bathymetry.grid(np.array([-1e4, 0, 1e4], np.float32), np.array([-1e4, 0, 1e4], np.float32),
                               10_000 * np.ones(9))
    c = oracle.Current.grid(np.array([-1e8, 0, 1e8]), np.array([-1e8, 0, 1e8]), 0.01 * np.ones(9),
                            0.01 * np.ones(9))
    o = oracle.trace(b, c, [-1e3, -1e3], [0.0, 0.0], [-0.01, 0.01], [0.0, 0.0], 0.0, 1e6, 20.0)
    np.testing.assert_array_equal(lengths, o[1])
    rows = int(lengths.max())
    g = np.stack([np.asarray(ds[v]) for v in ("time", "x", "y", "kx", "ky")])
    H.assert_parity(g, lengths.astype(np.int32), o[0][:, :rows], o[1])


def test_file_entry_points_match_array_form(mr, files):
    L = mr._native.load()
    rows_cap = 6
    buf = np.empty((rows_cap, 5))
    n_rows = ctypes.c_int32()
    mr._native.check(L.mr_single_ray_files(str(files[0]).encode(), str(files[1]).encode(),
                                           -1000.0, 0.0, 0.01, 0.0, 10.0, 2.0, rows_cap,
                                           buf.ctypes.data, ctypes.byref(n_rows)))
    assert n_rows.value == 6
    ds = mr.single_ray(-1000, 0, 0.01, 0, 10, 2, files[0], files[1])
    np.testing.assert_array_equal(buf[:, 0], np.asarray(ds["time"]))
    np.testing.assert_array_equal(buf[:, 1], np.asarray(ds["x"]))
    traj = np.empty((5, rows_cap, 2))
    nr = np.zeros(2, np.int32)
    st = np.zeros(2, np.uint8)
    x0 = np.array([-1000.0, -500.0])
    z = np.zeros(2)
    k = np.full(2, 0.01)
    mr._native.check(L.mr_ray_tracing_files(str(files[0]).encode(), str(files[1]).encode(), 2,
                                            x0.ctypes.data, z.ctypes.data, k.ctypes.data,
                                            z.ctypes.data, 10.0, 2.0, rows_cap, traj.ctypes.data,
                                            nr.ctypes.data, st.ctypes.data))
    np.testing.assert_array_equal(traj[:, :, 0].T, buf)


def test_missing_file_raises(mr, tmp_path, files):
    with pytest.raises(mr.MantarayIOError):
        mr.single_ray(0, 0, 0.01, 0, 10, 2, tmp_path / "nope.nc", files[1])
    with pytest.raises(mr.MantarayError):
        mr.Bathymetry.open(files[1])  # no "depth" variable


def _case(mr):
    x, y, depth = H.bathymetry_arrays(200, 150, 25.0, 25.0, lambda a, b: 30.0 + 0.02 * float(a) + 0.01 * float(b))
    b = mr.Bathymetry.grid(x, y, depth)
    cx, cy, u, v = H.current_arrays(200, 150, 25.0, 25.0, lambda a, b: (0.2 * math.sin(float(b) / 500.0), 0.1))
    c = mr.Current.grid(cx.astype(np.float64), cy.astype(np.float64), u, v)
    rng = np.random.default_rng(2)
    n = 1000
    th = rng.uniform(-1, 1, n)
    k = rng.uniform(0.01, 0.1, n)
    return b, c, (rng.uniform(100, 4000, n), rng.uniform(100, 3500, n), k * np.cos(th), k * np.sin(th))


def test_pinned_and_pageable_outputs_agree(mr):
    import torch

    b, c, rays = _case(mr)
    rows = mr.num_steps(0.0, 300.0, 0.5) + 1
    pageable = mr.trace(b, c, *rays, 300.0, 0.5)
    pinned = torch.empty((5, rows, rays[0].size), dtype=torch.float64, pin_memory=True)
    out = pinned.numpy()
    res = mr.trace(b, c, *rays, 300.0, 0.5, out=out)
    np.testing.assert_array_equal(np.nan_to_num(res.traj, nan=-9.0), np.nan_to_num(pageable.traj, nan=-9.0))
    np.testing.assert_array_equal(res.n_rows, pageable.n_rows)
    np.testing.assert_array_equal(res.status, pageable.status)


def test_device_form_matches_host_form(mr):
    import torch

    b, c, rays = _case(mr)
    host = mr.trace(b, c, *rays, 300.0, 0.5, rows_cap=700)  # extra rows: NaN padding
    assert np.all(np.isnan(host.traj[:, 601:, :]))
    dev = torch.device("cuda")
    ins = [torch.from_numpy(a).to(dev) for a in rays]
    traj = torch.empty((5, 700, rays[0].size), dtype=torch.float64, device=dev)
    n_rows = torch.empty(rays[0].size, dtype=torch.int32, device=dev)
    status = torch.empty(rays[0].size, dtype=torch.uint8, device=dev)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        mr.trace_device(b, c, *ins, 0.0, 300.0, 0.5, traj, n_rows, status, stream=s)
    s.synchronize()
    np.testing.assert_array_equal(np.nan_to_num(traj.cpu().numpy(), nan=-9.0),
                                  np.nan_to_num(host.traj, nan=-9.0))
    np.testing.assert_array_equal(n_rows.cpu().numpy(), host.n_rows)


def test_argument_errors(mr):
    b, c, rays = _case(mr)
    with pytest.raises(mr.MantarayError) as ei:
        mr.trace(b, c, *rays, 300.0, 0.5, rows_cap=10)
    assert ei.value.code == mr._native.ERR_CAPACITY
    with pytest.raises(ValueError):
        mr.trace(b, c, rays[0], rays[1][:5], rays[2], rays[3], 10.0, 1.0)
    with pytest.raises(mr.MantarayError) as ei:
        mr.trace(b, c, *rays, 10.0, 1.0, stop_rule=7)
    assert ei.value.code == mr._native.ERR_INVALID_ARGUMENT
    # a one-point axis opens (as in the reference) but cannot be traced
    one = mr.Current.grid([0.0], [0.0], [1.0], [1.0])
    with pytest.raises(mr.MantarayError) as ei:
        mr.trace(b, one, *rays, 10.0, 1.0)
    assert ei.value.code == mr._native.ERR_INVALID_ARGUMENT
    # zero rays is a no-op
    res = mr.trace(b, c, [], [], [], [], 10.0, 1.0)
    assert res.traj.shape == (5, 11, 0)


def test_many_calls_reuse_fields(mr):
    b, c, rays = _case(mr)
    first = mr.trace(b, c, *rays, 100.0, 1.0)
    for _ in range(5):
        again = mr.trace(b, c, *rays, 100.0, 1.0)
    np.testing.assert_array_equal(np.nan_to_num(first.traj, nan=0.0), np.nan_to_num(again.traj, nan=0.0))
