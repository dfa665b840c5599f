"""The CPU oracle against the reference's own known answers (runs on CPU).

Each test ports a unit or integration test of mines-oceanography/mantaray
(cited path:line) onto the oracle, which pins the restatement before it is
trusted as the checker of the CUDA kernels.
"""

import math

import numpy as np
import pytest

from tests import helpers as H

F64_EPS = np.finfo(np.float64).eps
F32_EPS = float(np.finfo(np.float32).eps)


# ---------------------------------------------------------------- RHS pins --

@pytest.mark.parametrize("k,ans", [(1.0, 1.565247584249853), (3.0, 0.9036961141150639),
                                   (5.0, 0.7), (10.0, 0.4949747468305833)])
def test_group_velocity(oracle, k, ans):
    # src/wave_ray_path.rs:294-315 (Wolfram values, tolerance 1e-4)
    e, v = oracle.group_velocity(k, 1000.0)
    assert e == oracle.OK and abs(v - ans) < 1e-4


def test_negative_k(oracle):
    # src/wave_ray_path.rs:317-326
    assert oracle.group_velocity(-1.0, 1000.0)[0] == oracle.ARGUMENT_OUT_OF_BOUNDS
    assert oracle.group_velocity(-12.0, 1000.0)[0] == oracle.ARGUMENT_OUT_OF_BOUNDS


@pytest.mark.parametrize("kx,ky,dx,dy", [(1.0, 0.0, 1.565247584249853, 0.0),
                                         (0.0, 1.0, 0.0, 1.565247584249853),
                                         (-1.0, 0.0, -1.565247584249853, 0.0),
                                         (0.0, -1.0, 0.0, -1.565247584249853)])
def test_odes(oracle, kx, ky, dx, dy):
    # src/wave_ray_path.rs:328-358 and the builder test :643-695
    b = oracle.Bathymetry.constant(1000.0)
    c = oracle.Current.constant(0.0, 0.0)
    e, d = oracle.odes(b, c, 0.0, 0.0, kx, ky)
    assert e == oracle.OK
    assert abs(d[0] - dx) < 1e-4 and abs(d[1] - dy) < 1e-4


def _last(oracle, bathy, x0, y0, kx, ky, tf, dt, current=None):
    c = current or oracle.Current.constant(0.0, 0.0)
    traj, n_rows, status = oracle.trace(bathy, c, x0, y0, kx, ky, 0.0, tf, dt)
    return traj[1:, n_rows[0] - 1, 0], traj, n_rows, status


def test_zero_k(oracle):
    # src/wave_ray_path.rs:360-380
    last, *_ = _last(oracle, oracle.Bathymetry.constant(1000.0), 0.0, 0.0, 0.0, 0.0, 10.0, 1.0)
    assert np.all(np.isnan(last))


def test_zero_h(oracle):
    # src/wave_ray_path.rs:382-401
    last, *_ = _last(oracle, oracle.Bathymetry.constant(0.0), 0.0, 0.0, 1.0, 1.0, 10.0, 1.0)
    assert np.all(np.isnan(last))


AXIS = [(0.0, 1.0, 0.0, math.sqrt(9.8) / 2.0), (1.0, 0.0, math.sqrt(9.8) / 2.0, 0.0),
        (0.0, -1.0, 0.0, -math.sqrt(9.8) / 2.0), (-1.0, 0.0, -math.sqrt(9.8) / 2.0, 0.0)]


@pytest.mark.parametrize("kx,ky,xf,yf", AXIS)
def test_axis(oracle, kx, ky, xf, yf):
    # src/wave_ray_path.rs:403-416: one RK4 step lands within f64::EPSILON
    last, *_ = _last(oracle, oracle.Bathymetry.constant(1000.0), 0.0, 0.0, kx, ky, 1.0, 1.0)
    assert abs(last[0] - xf) < F64_EPS and abs(last[1] - yf) < F64_EPS


@pytest.mark.parametrize("kx,ky,xf,yf", AXIS)
def test_array_as_parameter(oracle, kx, ky, xf, yf):
    # src/wave_ray_path.rs:418-435
    b = oracle.Bathymetry.array(np.full((3, 3), 1000.0))
    last, *_ = _last(oracle, b, 0.0, 0.0, kx, ky, 1.0, 1.0)
    assert abs(last[0] - xf) < F64_EPS and abs(last[1] - yf) < F64_EPS


@pytest.mark.parametrize("state,check", [((math.nan, 0.0, 1.0, 0.0), (0,)),
                                         ((0.0, math.nan, 1.0, 0.0), (1,)),
                                         ((0.0, 0.0, math.nan, 0.0), (0, 1)),
                                         ((0.0, 0.0, 0.0, math.nan), (0, 1))])
def test_nan_inputs(oracle, state, check):
    # src/wave_ray_path.rs:437-517
    last, *_ = _last(oracle, oracle.Bathymetry.constant(1000.0), *state, 1.0, 1.0)
    for i in check:
        assert math.isnan(last[i])


SHALLOW = [(0.0, 1.0, 0.00000000000000006031543168844801, 0.9850257515953494),
           (1.0, 0.0, 0.9850257515953494, 0.0),
           (0.0, -1.0, 0.00000000000000006031543168844801, -0.9850257515953494),
           (-1.0, 0.0, -0.9850257515953494, 0.00000000000000012063086337689602)]


@pytest.mark.parametrize("kx,ky,xf,yf", SHALLOW)
def test_shallow(oracle, kx, ky, xf, yf):
    # src/wave_ray_path.rs:519-548; the tiny cross terms come from cos/sin of
    # atan2 at +-pi/2 and pi and pin the RK4 update order to the bit.
    last, *_ = _last(oracle, oracle.Bathymetry.constant(0.1), 0.0, 0.0, kx, ky, 1.0, 1.0)
    assert abs(last[0] - xf) < F64_EPS and abs(last[1] - yf) < F64_EPS
    assert last[0] == xf and last[1] == yf  # bit-identical in fact


def test_out_of_range_gives_nan(oracle):
    # src/wave_ray_path.rs:550-570
    b = oracle.Bathymetry.array(np.full((2, 2), 1000.0))
    last, *_ = _last(oracle, b, 0.0, 0.0, 0.0, 1.0, 10.0, 1.0)
    assert math.isnan(last[0]) and math.isnan(last[1])


def test_dk_deep(oracle):
    # src/wave_ray_path.rs:572-597
    d = oracle.dkdt_bathy(1000.0, 1000.0, 0.2, 0.2)
    assert abs(d[0]) < F64_EPS and abs(d[1]) < F64_EPS


@pytest.mark.parametrize("stop_rule", [0, 1])
def test_solout(oracle, stop_rule):
    # src/wave_ray_path.rs:599-626: 3 rows, the last one all NaN (both rules)
    b = oracle.Bathymetry.array(np.full((2, 2), 1000.0))
    c = oracle.Current.constant(0.0, 0.0)
    traj, n_rows, status = oracle.trace(b, c, 0.0, 0.0, 0.0, 1.0, 0.0, 10.0, 1.0,
                                        stop_rule=stop_rule)
    assert n_rows[0] == 3 and status[0] == oracle.RAY_STOPPED
    assert np.all(np.isnan(traj[1:, 2, 0]))
    assert np.all(np.isnan(traj[:, 3:, 0]))


@pytest.mark.parametrize("u,v,dx,dy", [(1.0, 0.0, 1.565247584249853 + 1.0, 0.0),
                                       (-1.0, 0.0, 1.565247584249853 - 1.0, 0.0),
                                       (0.0, 1.0, 1.565247584249853, 1.0),
                                       (0.0, -1.0, 1.565247584249853, -1.0),
                                       (1.0, 1.0, 1.565247584249853 + 1.0, 1.0),
                                       (-1.0, -1.0, 1.565247584249853 - 1.0, -1.0)])
def test_constant_depth_current(oracle, u, v, dx, dy):
    # src/wave_ray_path.rs:697-768 (f64::EPSILON)
    b = oracle.Bathymetry.constant(1000.0)
    e, d = oracle.odes(b, oracle.Current.constant(u, v), 0.0, 0.0, 1.0, 0.0)
    assert e == oracle.OK
    assert abs(d[0] - dx) < F64_EPS and abs(d[1] - dy) < F64_EPS


def stop_rule_case(rng_seed=5, n=4000):
    """Random 6x6 depth grid and rays, seeded: a case where some rays leave
    the grid with every RK4 stage inside it (the two stop rules then differ)."""
    rng = np.random.default_rng(rng_seed)
    depth = rng.uniform(1, 200, size=(6, 6))
    x = np.arange(6, dtype=np.float32) * np.float32(20.0)
    x0 = rng.uniform(0, 100, n)
    y0 = rng.uniform(0, 100, n)
    th = rng.uniform(0, 2 * np.pi, n)
    return (x, x, depth), (x0, y0, 0.05 * np.cos(th), 0.05 * np.sin(th))


def test_stop_rules_differ_only_by_the_final_nan_row(oracle):
    # Where the new state is finite but outside the grid, FRESH stops on its
    # NaN derivative; STAGE1 records one more, all-NaN, row.  Elsewhere the
    # two rules give identical trajectories.
    grid, rays = stop_rule_case()
    b = oracle.Bathymetry.grid(*grid)
    c = oracle.Current.constant(0.0, 0.0)
    tr0, n0, _ = oracle.trace(b, c, *rays, 0.0, 30.0, 1.0, stop_rule=0)
    tr1, n1, _ = oracle.trace(b, c, *rays, 0.0, 30.0, 1.0, stop_rule=1)
    diff = np.nonzero(n0 != n1)[0]
    assert 0 < diff.size < rays[0].size // 50
    assert np.all(n0[diff] == n1[diff] + 1)
    same = np.nonzero(n0 == n1)[0]
    np.testing.assert_array_equal(tr0[:, :, same], tr1[:, :, same])
    for i in diff:
        np.testing.assert_array_equal(tr0[:, : n1[i], i], tr1[:, : n1[i], i])
        assert np.all(np.isnan(tr0[1:, n0[i] - 1, i]))
        assert np.all(np.isfinite(tr1[:, n1[i] - 1, i]))


# ------------------------------------------------------------ interpolation --

def test_interp(oracle):
    # src/interpolator.rs:86-123
    x, y, x1, y1, x2, y2, q11, q21, q12, q22, t, val = (
        20.0, 23.0, -77.0, -19.0, 123.0, 145.0, 10.0, 20.0, 30.0, 40.0, 1230.0, 19.971951219512192)
    pts = [(x1 + t, y1 + t, q11), (x1 + t, y2 + t, q12), (x2 + t, y2 + t, q22), (x2 + t, y1 + t, q21)]
    e, ans = oracle.bilinear(pts, (x + t, y + t))
    # the reference compares in f32 (`val` is an f32 literal there)
    assert e == oracle.OK and abs(np.float32(ans) - np.float32(val)) < np.float32(F32_EPS)


@pytest.mark.parametrize("x,y,val", [(0.0, 0.0, 0.0), (10.0, 0.0, 5.0), (0.0, 10.0, 10.0),
                                     (10.0, 10.0, 15.0)])
def test_edges(oracle, x, y, val):
    # src/interpolator.rs:125-161
    x1, y1, x2, y2, q11, q21, q12, q22 = 0.0, 0.0, 10.0, 10.0, 0.0, 5.0, 10.0, 15.0
    pts = [(x1, y1, q11), (x1, y2, q12), (x2, y2, q22), (x2, y1, q21)]
    e, ans = oracle.bilinear(pts, (x, y))
    assert e == oracle.OK and abs(float(ans) - val) < F32_EPS


def test_bilinear_degenerate(oracle):
    # src/interpolator.rs:64-67: zero determinant -> InvalidArgument
    pts = [(0.0, 0.0, 1.0)] * 4
    assert oracle.bilinear(pts, (1.0, 1.0))[0] == oracle.INVALID_ARGUMENT


# ------------------------------------------------------- gridded bathymetry --

def four_depth_fn(x, y):
    # src/bathymetry/cartesian_netcdf3.rs:487-501
    if x < 25000.0:
        return 20.0 if y < 12500.0 else 10.0
    return 5.0 if y < 12500.0 else 15.0


@pytest.fixture(scope="module")
def four_depth(oracle):
    x, y, depth = H.bathymetry_arrays(101, 51, 500.0, 500.0, four_depth_fn)
    return oracle.Bathymetry.grid(x, y, depth), x, y


def test_vars(four_depth):
    # cartesian_netcdf3.rs:503-514
    _, x, _ = four_depth
    assert abs(x[10] - 5000.0) < F32_EPS


def test_nearest(oracle, four_depth):
    # cartesian_netcdf3.rs:516-537
    _, x, y = four_depth
    e, i = oracle.nearest_f32(5499.0, x)
    assert e == 0 and round(float(i)) == 11.0
    assert oracle.nearest_f32(-1.0, y)[0] == oracle.INDEX_OUT_OF_BOUNDS
    assert oracle.nearest_f32(25501.0, y)[0] == oracle.INDEX_OUT_OF_BOUNDS
    assert abs(oracle.nearest_f32(5500.0, x)[1] - 11.0) <= F32_EPS


CORNERS = [
    ((0.0, 25000.0), [(0, 49), (0, 50), (1, 50), (1, 49)]),
    ((0.0, 5500.0), [(0, 11), (0, 12), (1, 12), (1, 11)]),
    ((0.0, 0.0), [(0, 0), (0, 1), (1, 1), (1, 0)]),
    ((5500.0, 25000.0), [(11, 49), (11, 50), (12, 50), (12, 49)]),
    ((5500.0, 0.0), [(11, 0), (11, 1), (12, 1), (12, 0)]),
    ((50000.0, 25000.0), [(99, 49), (99, 50), (100, 50), (100, 49)]),
    ((50000.0, 5500.0), [(99, 11), (99, 12), (100, 12), (100, 11)]),
    ((50000.0, 0.0), [(99, 0), (99, 1), (100, 1), (100, 0)]),
    ((5500.0, 5500.0), [(11, 11), (11, 12), (12, 12), (12, 11)]),
    ((5500.0, 5750.0), [(11, 11), (11, 12), (12, 12), (12, 11)]),
    ((5750.0, 5500.0), [(11, 11), (11, 12), (12, 12), (12, 11)]),
    ((5750.0, 5750.0), [(11, 11), (11, 12), (12, 12), (12, 11)]),
]
CORNERS_OOB = [(50001.0, 0.0), (50000.0, 25001.0), (-1.0, 0.0), (50000.0, -1.0)]


@pytest.mark.parametrize("pt,expected", CORNERS)
def test_get_corners(oracle, four_depth, pt, expected):
    # cartesian_netcdf3.rs:562-659
    e, c = four_depth[0].four_corners(*pt)
    assert e == 0 and c == expected


@pytest.mark.parametrize("pt", CORNERS_OOB)
def test_get_corners_out_of_bounds(oracle, four_depth, pt):
    assert four_depth[0].four_corners(*pt)[0] == oracle.INDEX_OUT_OF_BOUNDS


@pytest.mark.parametrize("x,y,h", [(10099.0, 5099.0, 20.0), (30099.0, 5099.0, 5.0),
                                   (10099.0, 15099.0, 10.0), (30099.0, 15099.0, 15.0)])
def test_depth(oracle, four_depth, x, y, h):
    # cartesian_netcdf3.rs:661-689
    e, out = four_depth[0].depth_and_gradient(x, y)
    assert e == 0 and abs(out[0] - h) < F32_EPS


@pytest.mark.parametrize("pt", [(-500.1, 500.1), (500.1, -500.1)])
def test_depth_out_of_bounds(oracle, four_depth, pt):
    # cartesian_netcdf3.rs:691-725
    assert four_depth[0].depth_and_gradient(*pt)[0] == oracle.INDEX_OUT_OF_BOUNDS


@pytest.mark.parametrize("pt", [(math.nan, math.nan), (10000.0, math.nan), (math.nan, 10000.0)])
def test_depth_nan(oracle, four_depth, pt):
    # cartesian_netcdf3.rs:727-742
    e, out = four_depth[0].depth_and_gradient(*pt)
    assert e == 0 and np.isnan(out[0])


@pytest.mark.parametrize("axis", ["x", "y"])
def test_depth_and_gradient_ramp(oracle, axis):
    # cartesian_netcdf3.rs:744-834: a 100x100 linear ramp, exact at every node
    def depth_fn(x, y):
        return float(x if axis == "x" else y) * 0.05

    x, y, depth = H.bathymetry_arrays(100, 100, 1.0, 1.0, depth_fn)
    b = oracle.Bathymetry.grid(x, y, depth)
    gx, gy = (0.05, 0.0) if axis == "x" else (0.0, 0.05)
    for i in range(100):
        for j in range(100):
            e, out = b.depth_and_gradient(float(i), float(j))
            assert e == 0
            assert abs(out[1] - gx) < F32_EPS and abs(out[2] - gy) < F32_EPS
            assert abs(out[0] - np.float32(depth_fn(np.float32(i), np.float32(j)))) < F32_EPS


def test_constant_slope_depth(oracle):
    # src/ray.rs:562-563 (ConstantSlope builder defaults)
    b = oracle.Bathymetry.slope()
    assert b.depth_and_gradient(10.0, 1000.0)[1][0] == np.float32(49.5)
    assert b.depth_and_gradient(300.0, 1000.0)[1][0] == np.float32(35.0)


# ----------------------------------------------------------- gridded current --

def _current(oracle, nx, ny, step, fn):
    x, y, u, v = H.current_arrays(nx, ny, step, step, fn)
    return oracle.Current.grid(x.astype(np.float64), y.astype(np.float64), u, v), x, y, u, v


def test_current_nearest_and_corners(oracle):
    # src/current/cartesian_current.rs:639-776
    c, x, y, *_ = _current(oracle, 101, 51, 500.0, lambda a, b: (5.0, 0.0))
    e, i = oracle.nearest_f64(5499.0, x.astype(np.float64))
    assert e == 0 and round(i) == 11.0
    assert oracle.nearest_f64(-1.0, y.astype(np.float64))[0] == oracle.INDEX_OUT_OF_BOUNDS
    assert oracle.nearest_f64(25501.0, y.astype(np.float64))[0] == oracle.INDEX_OUT_OF_BOUNDS
    for pt, expected in CORNERS:
        e, got = c.four_corners(*pt)
        assert e == 0 and got == expected
    for pt in CORNERS_OOB:
        assert c.four_corners(*pt)[0] == oracle.INDEX_OUT_OF_BOUNDS


def test_current_zero_gradient(oracle):
    # cartesian_current.rs:842-875
    c, *_ = _current(oracle, 100, 50, 1.0, lambda a, b: (5.0, 0.0))
    for i in range(100):
        for j in range(50):
            e, out = c.current_and_gradient(float(i), float(j))
            assert e == 0
            assert list(out) == [5.0, 0.0, 0.0, 0.0, 0.0, 0.0]
    assert c.current_and_gradient(50001.0, 1000.0)[0] == oracle.INDEX_OUT_OF_BOUNDS
    assert c.current_and_gradient(-50001.0, -1000.0)[0] == oracle.INDEX_OUT_OF_BOUNDS


@pytest.mark.parametrize("axis", ["x", "y"])
def test_current_gradient_ramp(oracle, axis):
    # cartesian_current.rs:877-992 (assert_eq!: exact)
    def fn(x, y):
        v = float(x if axis == "x" else y)
        return (v, v)

    c, *_ = _current(oracle, 100, 100, 1.0, fn)
    g = [1.0, 0.0] if axis == "x" else [0.0, 1.0]
    for i in range(100):
        for j in range(100):
            e, out = c.current_and_gradient(float(i), float(j))
            v = float(i if axis == "x" else j)
            assert e == 0 and list(out) == [v, v, g[0], g[1], g[0], g[1]]


def test_current_nan_point_is_an_error(oracle):
    # NaN position: nearest passes NaN through, floor/ceil saturate to 0, all
    # four corners coincide and bilinear reports a zero determinant.
    c, *_ = _current(oracle, 10, 10, 1.0, lambda a, b: (1.0, 1.0))
    assert c.current_and_gradient(math.nan, 1.0)[0] == oracle.INVALID_ARGUMENT


# ------------------------------------------------- trajectory integrations --

def test_constant_wave_properties(oracle):
    # src/ray.rs:268-397
    b = oracle.Bathymetry.constant(10.0)
    c = oracle.Current.constant(0.0, 0.0)
    for (x0, y0, kx, ky, tf) in [(10.0, 50.0, 0.01, 0.0, 8.0), (10.0, 50.0, 1.0, 0.0, 18.0)]:
        traj, n_rows, _ = oracle.trace(b, c, x0, y0, kx, ky, 0.0, tf, 1.0)
        d = H.ray_rows(traj, n_rows, 0)
        assert np.all(d[:, 1] == 50.0) and np.all(d[:, 2] == kx) and np.all(d[:, 3] == 0.0)
        assert H.increase(d, H.XI)
    for (kx, ky, tf) in [(0.007, 0.007, 8.0), (0.7, 0.7, 18.0)]:
        traj, n_rows, _ = oracle.trace(b, c, 10.0, 10.0, kx, ky, 0.0, tf, 1.0)
        d = H.ray_rows(traj, n_rows, 0)
        assert np.all(d[:, 2] == kx) and np.all(d[:, 3] == ky)
        assert np.all(np.diff(d[:, 0]) >= 0) and np.all(np.diff(d[:, 1]) >= 0)


def two_depth_fn(x, y):
    # src/ray.rs:259-266
    return 20.0 if x >= 50.0 else 50.0


def test_two_depth_waves(oracle):
    # src/ray.rs:399-548
    x, y, depth = H.bathymetry_arrays(100, 100, 1.0, 1.0, two_depth_fn)
    b = oracle.Bathymetry.grid(x, y, depth)
    c = oracle.Current.constant(0.0, 0.0)
    traj, n, _ = oracle.trace(b, c, 10.0, 50.0, 0.01, 0.0, 0.0, 5.0, 1.0)
    d = H.ray_rows(traj, n, 0)
    assert np.all(d[:, 1] == 50.0) and np.all(d[:, 3] == 0.0)
    assert np.all(np.diff(d[:, 0]) >= 0) and np.all(np.diff(d[:, 2]) >= 0) and d[-1, 2] > d[0, 2]
    traj, n, _ = oracle.trace(b, c, 10.0, 10.0, 0.007, 0.007, 0.0, 6.8, 0.1)
    d = H.ray_rows(traj, n, 0)
    assert np.all(d[:, 3] == 0.007)
    assert np.all(np.diff(d[:, 0]) >= 0) and np.all(np.diff(d[:, 1]) >= 0)
    assert np.all(np.diff(d[:, 2]) >= 0) and np.all(d[:, 0] >= d[:, 1]) and d[-1, 2] > d[0, 2]
    traj, n, _ = oracle.trace(b, c, 10.0, 50.0, 1.0, 0.0, 0.0, 30.0, 1.0)
    d = H.ray_rows(traj, n, 0)
    assert np.all(d[:, 3] == 0.0) and np.all(d[:, 1] == 50.0) and np.all(d[:, 2] == 1.0)
    assert np.all(np.diff(d[:, 0]) >= 0)
    traj, n, _ = oracle.trace(b, c, 10.0, 10.0, 0.7, 0.7, 0.0, 40.0, 1.0)
    d = H.ray_rows(traj, n, 0)
    assert np.all(d[:, 2] == 0.7) and np.all(d[:, 3] == 0.7) and np.all(np.diff(d[:, 0]) >= 0)


def test_slope_depth_wave(oracle):
    # src/ray.rs:550-584
    b = oracle.Bathymetry.slope()
    c = oracle.Current.constant(0.0, 0.0)
    traj, n, _ = oracle.trace(b, c, 10.0, 1000.0, 0.1, 0.0, 0.0, 100.0, 1.0)
    d = H.ray_rows(traj, n, 0)
    d = d[~np.isnan(d[:, 0])]
    assert np.all(np.diff(d[:, 0]) >= 0) and d[-1, 2] > d[0, 2]


@pytest.mark.parametrize("u,v,kx,ky,sx,sy", [
    (0.5, 0.0, 0.1, 0.0, 1, 0),   # ray.rs:615-643 (h = 10)
    (0.0, 0.5, 0.1, 0.0, 1, 1),   # :645-679
    (0.0, -0.5, 0.1, 0.0, 1, -1),  # :681-717
    (0.5, 0.0, 0.0, 0.1, 1, 1),   # :719-755
    (-0.5, 0.0, 0.0, 0.1, -1, 1),  # :757-792
    (0.5, 0.5, 0.1, 0.0, 1, 1),   # :794-830
    (-0.5, -0.5, -0.1, 0.0, -1, -1),  # :832-867
])
def test_constant_current_rays(oracle, u, v, kx, ky, sx, sy):
    depth = 10.0 if (u, v) == (0.5, 0.0) and ky == 0.0 else 1000.0
    b = oracle.Bathymetry.constant(depth)
    traj, n, _ = oracle.trace(b, oracle.Current.constant(u, v), 0.0, 0.0, kx, ky, 1.0, 10.0, 1.0)
    d = H.ray_rows(traj, n, 0)
    assert np.all(d[:, 2] == kx) and np.all(d[:, 3] == ky)
    for col, s in ((0, sx), (1, sy)):
        diffs = np.diff(d[:, col])
        if s > 0:
            assert np.all(diffs >= 0) and d[-1, col] > d[0, col]
        elif s < 0:
            assert np.all(diffs <= 0) and d[-1, col] < d[0, col]
        else:
            assert np.all(d[:, col] == 0.0)


def test_many_waves_ok(oracle):
    # src/ray.rs:1331-1361: nine rays on the default slope to t = 1e5 s
    b = oracle.Bathymetry.slope()
    c = oracle.Current.constant(0.0, 0.0)
    ys = np.arange(10.0, 100.0, 10.0)
    steps = oracle.num_steps(0.0, 100000.0, 1.0)
    final, n_rows, status = oracle.trace_final(b, c, np.full(9, 10.0), ys, np.ones(9),
                                               np.zeros(9), 0.0, 100000.0, 1.0)
    assert len(n_rows) == 9 and np.all(n_rows >= 1) and np.all(n_rows <= steps + 1)


BEACHES = {
    # name: (slope h0, dhdx, dhdy), rays (x, y, kx, ky), expectations per ray
    "right": ((100.0, -0.05, 0.0),
              [(0.0, 0.0, math.cos(math.pi / 6), math.sin(math.pi / 6)),
               (0.0, 0.0, math.cos(-math.pi / 6), math.sin(-math.pi / 6)),
               (0.0, 0.0, 1.0, 0.0)],
              [("inc", "inc", "inc", "same"), ("inc", "dec", "inc", "same"),
               ("inc", "same", "inc", "same")]),
    "left": ((0.0, 0.05, 0.0),
             [(2000.0, 0.0, -math.cos(math.pi / 6), math.sin(math.pi / 6)),
              (2000.0, 0.0, -math.cos(-math.pi / 6), math.sin(-math.pi / 6)),
              (2000.0, 100.0, -1.0, 0.0)],
             [("dec", "inc", "dec", "same"), ("dec", "dec", "dec", "same"),
              ("dec", "same", "dec", "same")]),
    "top": ((100.0, 0.0, -0.05),
            [(0.0, 0.0, math.cos(4 * math.pi / 6), math.sin(4 * math.pi / 6)),
             (0.0, 0.0, math.cos(2 * math.pi / 6), math.sin(2 * math.pi / 6)),
             (100.0, 0.0, 0.0, 1.0)],
            [("dec", "inc", "same", "inc"), ("inc", "inc", "same", "inc"),
             ("same", "inc", "same", "inc")]),
    "bottom": ((0.0, 0.0, 0.05),
               [(0.0, 2000.0, math.cos(4 * math.pi / 6), -math.sin(4 * math.pi / 6)),
                (0.0, 2000.0, math.cos(2 * math.pi / 6), -math.sin(2 * math.pi / 6)),
                (100.0, 2000.0, 0.0, -1.0)],
               [("dec", "dec", "same", "dec"), ("inc", "dec", "same", "dec"),
                ("same", "dec", "same", "dec")]),
}


def beach_rays(name):
    (h0, dhdx, dhdy), rays, expect = BEACHES[name]
    k = 0.05
    x0 = np.array([r[0] for r in rays])
    y0 = np.array([r[1] for r in rays])
    kx0 = np.array([k * r[2] for r in rays])
    ky0 = np.array([k * r[3] for r in rays])
    return (h0, dhdx, dhdy), (x0, y0, kx0, ky0), expect


def check_beach(traj, n_rows, expect):
    preds = {"inc": H.increase, "dec": H.decrease, "same": H.same}
    for i, e in enumerate(expect):
        d = H.ray_rows(traj, n_rows, i)
        for col, p in enumerate(e):
            assert preds[p](d, col), (i, col, p)


@pytest.mark.parametrize("name", list(BEACHES))
def test_linear_beach(oracle, name):
    # src/tests/linear_beach.rs:14-416 (ManyRays over 1000 s)
    (h0, dhdx, dhdy), rays, expect = beach_rays(name)
    b = oracle.Bathymetry.slope(h0=h0, x0=0.0, y0=0.0, dhdx=dhdx, dhdy=dhdy)
    traj, n_rows, _ = oracle.trace(b, oracle.Current.constant(0.0, 0.0), *rays, 0.0, 1000.0, 1.0)
    check_beach(traj, n_rows, expect)


def circle_rays():
    i = np.arange(12)
    return (np.full(12, 50000.0), np.full(12, 25000.0), 0.05 * np.cos(np.pi * i / 6.0),
            0.05 * np.sin(np.pi * i / 6.0))


def check_circle(traj, n_rows, kx0, ky0):
    for i in range(12):
        d = H.ray_rows(traj, n_rows, i)
        for col, k in ((0, kx0[i]), (1, ky0[i])):
            if abs(k) < F64_EPS:
                assert H.same(d, col)
            elif k > 0:
                assert H.increase(d, col)
            else:
                assert H.decrease(d, col)
        assert H.same(d, 2) and H.same(d, 3)


@pytest.mark.parametrize("depth", [2000.0, 10.0])
def test_constant_depth_circle(oracle, depth):
    # src/tests/test_constant_depth.rs:38-160 (12 rays, 5000 s)
    b = oracle.Bathymetry.constant(depth)
    rays = circle_rays()
    traj, n_rows, _ = oracle.trace(b, oracle.Current.constant(0.0, 0.0), *rays, 0.0, 5000.0, 1.0)
    check_circle(traj, n_rows, rays[2], rays[3])


def test_python_core_row_count(oracle):
    # python/tests/test_core.py:40-78: duration 10, step 2 -> 6 rows, k unchanged
    x = np.array([-1e4, 0.0, 1e4], np.float32)
    b = oracle.Bathymetry.grid(x, x, np.full(9, 10000.0))
    cx = np.array([-1e8, 0.0, 1e8])
    c = oracle.Current.grid(cx, cx, np.full(9, 0.01), np.full(9, 0.01))
    traj, n_rows, _ = oracle.trace(b, c, [-1000.0] * 3, [0.0] * 3, [0.01] * 3, [0.0] * 3,
                                   0.0, 10.0, 2.0)
    assert traj.shape[1] == 6 and np.all(n_rows == 6)
    assert np.all(traj[3] == 0.01) and np.all(traj[4] == 0.0)


@pytest.mark.parametrize("t0,t_end,dt,steps", [(0.0, 10.0, 2.0, 5), (0.0, 10.0, 3.0, 4),
                                               (1.0, 10.0, 1.0, 9), (0.0, -1.0, 1.0, 0),
                                               (0.0, 1.0, 0.0, 2 ** 64 - 1),
                                               (0.0, math.nan, 1.0, 0), (0.0, 6.8, 0.1, 68)])
def test_num_steps(oracle, t0, t_end, dt, steps):
    # ceil((t_end - t0)/h) with Rust's saturating usize cast
    assert oracle.num_steps(t0, t_end, dt) == steps
