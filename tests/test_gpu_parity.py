"""Parity of the plain FP64 CUDA kernel with the CPU oracle (GPU tests).

The bar (the plain form's contract): every x, y, kx, ky of every row before a
ray's first non-finite row agrees with the oracle to 1e-9 relative
(|a - b| <= 1e-9 * max(|b|, floor), floors 1 m and 1e-6 rad/m), t and row
counts agree exactly, and NaN appears in the same places.  The reference's own
known answers are checked on the GPU results directly as well.
"""

import math

import numpy as np
import pytest

from tests import helpers as H
from tests.test_oracle_golden import (AXIS, BEACHES, SHALLOW, beach_rays, check_beach,
                                      check_circle, circle_rays, four_depth_fn, stop_rule_case,
                                      two_depth_fn)

pytestmark = pytest.mark.gpu

RTOL = 1e-9
F64_EPS = np.finfo(np.float64).eps
MATH = "libm"


@pytest.fixture(autouse=True, params=["libm", "identity"])
def math_mode(request):
    """Every parity test runs for both right-hand-side arithmetic options."""
    global MATH
    MATH = request.param
    yield request.param


@pytest.fixture(scope="module")
def mr():
    import mantaray_gb300 as m

    m._native.load()
    return m


def both(mr, oracle, bathy, current, x0, y0, kx0, ky0, t0, t_end, dt, stop_rule=0):
    """(gpu traj, gpu rows, gpu status, oracle traj, oracle rows, oracle status)
    for the same field description.  bathy/current: ("constant", h) etc."""
    gb, ob = make_bathy(mr, oracle, bathy)
    gc, oc = make_current(mr, oracle, current)
    g = mr.trace(gb, gc, x0, y0, kx0, ky0, t_end - t0, dt, t0=t0, stop_rule=stop_rule, math=MATH)
    o = oracle.trace(ob, oc, x0, y0, kx0, ky0, t0, t_end, dt, stop_rule=stop_rule)
    return g.traj, g.n_rows, g.status, o[0], o[1], o[2]


def make_bathy(mr, oracle, spec):
    kind, args = spec[0], spec[1:]
    if kind == "grid":
        return mr.Bathymetry.grid(*args), oracle.Bathymetry.grid(*args)
    if kind == "constant":
        return mr.Bathymetry.constant(*args), oracle.Bathymetry.constant(*args)
    if kind == "slope":
        return mr.Bathymetry.slope(*args), oracle.Bathymetry.slope(*args)
    if kind == "array":
        return mr.Bathymetry.array(*args), oracle.Bathymetry.array(*args)
    raise ValueError(kind)


def make_current(mr, oracle, spec):
    kind, args = spec[0], spec[1:]
    if kind == "grid":
        return mr.Current.grid(*args), oracle.Current.grid(*args)
    return mr.Current.constant(*args), oracle.Current.constant(*args)


def eps_pin():
    """Tolerance of the reference's single-step known answers (f64::EPSILON,
    src/wave_ray_path.rs:280).  The libm arithmetic meets it; the identity
    arithmetic computes the same quantities a few ulps apart, so it is held to
    4 ulps there (and to the 1e-9 parity bar everywhere)."""
    return F64_EPS if MATH == "libm" else 4 * F64_EPS


def check(g, gr, gs, o, orr, os_):
    worst = H.assert_parity(g, gr, o, orr, rtol=RTOL)
    np.testing.assert_array_equal(gs, os_)
    return worst


ZERO = ("constant", 0.0, 0.0)


# ------------------------------------------- the reference's known answers --

@pytest.mark.parametrize("kx,ky,xf,yf", AXIS)
def test_axis(mr, oracle, kx, ky, xf, yf):
    # src/wave_ray_path.rs:403-416
    r = both(mr, oracle, ("constant", 1000.0), ZERO, 0.0, 0.0, kx, ky, 0.0, 1.0, 1.0)
    check(*r)
    assert abs(r[0][1, 1, 0] - xf) < eps_pin() and abs(r[0][2, 1, 0] - yf) < eps_pin()


@pytest.mark.parametrize("kx,ky,xf,yf", SHALLOW)
def test_shallow(mr, oracle, kx, ky, xf, yf):
    # src/wave_ray_path.rs:519-548 (f64::EPSILON)
    r = both(mr, oracle, ("constant", 0.1), ZERO, 0.0, 0.0, kx, ky, 0.0, 1.0, 1.0)
    check(*r)
    assert abs(r[0][1, 1, 0] - xf) < eps_pin() and abs(r[0][2, 1, 0] - yf) < eps_pin()


@pytest.mark.parametrize("kx,ky,xf,yf", AXIS)
def test_array_as_parameter(mr, oracle, kx, ky, xf, yf):
    # src/wave_ray_path.rs:418-435
    r = both(mr, oracle, ("array", np.full((3, 3), 1000.0)), ZERO, 0.0, 0.0, kx, ky, 0.0, 1.0, 1.0)
    check(*r)
    assert abs(r[0][1, 1, 0] - xf) < eps_pin() and abs(r[0][2, 1, 0] - yf) < eps_pin()


@pytest.mark.parametrize("bathy,state,tf", [
    (("constant", 1000.0), (0.0, 0.0, 0.0, 0.0), 10.0),       # zero k, :360-380
    (("constant", 0.0), (0.0, 0.0, 1.0, 1.0), 10.0),          # zero h, :382-401
    (("constant", 1000.0), (math.nan, 0.0, 1.0, 0.0), 1.0),   # :437-455
    (("constant", 1000.0), (0.0, math.nan, 1.0, 0.0), 1.0),   # :457-475
    (("constant", 1000.0), (0.0, 0.0, math.nan, 0.0), 1.0),   # :477-496
    (("constant", 1000.0), (0.0, 0.0, 0.0, math.nan), 1.0),   # :498-517
    (("array", np.full((2, 2), 1000.0)), (0.0, 0.0, 0.0, 1.0), 10.0),  # :550-626
    (("constant", -5.0), (0.0, 0.0, 1.0, 0.0), 5.0),          # negative depth
])
@pytest.mark.parametrize("stop_rule", [0, 1])
def test_nan_and_termination(mr, oracle, bathy, state, tf, stop_rule):
    r = both(mr, oracle, bathy, ZERO, *state, 0.0, tf, 1.0, stop_rule=stop_rule)
    check(*r)


def test_solout_three_rows(mr, oracle):
    # src/wave_ray_path.rs:599-626
    r = both(mr, oracle, ("array", np.full((2, 2), 1000.0)), ZERO, 0.0, 0.0, 0.0, 1.0, 0.0, 10.0, 1.0)
    assert r[1][0] == 3 and r[2][0] == 1
    assert np.all(np.isnan(r[0][1:, 2, 0]))


@pytest.mark.parametrize("u,v", [(1.0, 0.0), (-1.0, 0.0), (0.0, 1.0), (0.0, -1.0), (1.0, 1.0),
                                 (-1.0, -1.0)])
def test_constant_current(mr, oracle, u, v):
    # src/wave_ray_path.rs:697-768 through a one-step trajectory
    r = both(mr, oracle, ("constant", 1000.0), ("constant", u, v), 0.0, 0.0, 1.0, 0.0, 0.0, 5.0, 1.0)
    check(*r)


# ------------------------------------------------------------------- grids --

def test_four_depth_grid(mr, oracle):
    # cartesian_netcdf3.rs:487-501 quadrants, rays crossing the depth steps
    x, y, depth = H.bathymetry_arrays(101, 51, 500.0, 500.0, four_depth_fn)
    rng = np.random.default_rng(7)
    n = 300
    th = rng.uniform(0, 2 * np.pi, n)
    k = rng.uniform(0.005, 0.2, n)
    r = both(mr, oracle, ("grid", x, y, depth), ZERO, rng.uniform(0, 50000, n),
             rng.uniform(0, 25000, n), k * np.cos(th), k * np.sin(th), 0.0, 600.0, 2.0)
    check(*r)


def test_two_depth_grid(mr, oracle):
    # src/ray.rs:399-548
    x, y, depth = H.bathymetry_arrays(100, 100, 1.0, 1.0, two_depth_fn)
    for (x0, y0, kx, ky, tf, dt) in [(10.0, 50.0, 0.01, 0.0, 5.0, 1.0),
                                     (10.0, 10.0, 0.007, 0.007, 6.8, 0.1),
                                     (10.0, 50.0, 1.0, 0.0, 30.0, 1.0),
                                     (10.0, 10.0, 0.7, 0.7, 40.0, 1.0)]:
        r = both(mr, oracle, ("grid", x, y, depth), ZERO, x0, y0, kx, ky, 0.0, tf, dt)
        check(*r)


@pytest.mark.parametrize("fn", [
    lambda a, b: (float(a) / 100.0, 0.0),            # src/ray.rs:879-960 (du/dx)
    lambda a, b: (float(b) / 100.0, 0.0),            # :962-1060 (du/dy)
    lambda a, b: (0.0, float(b) / 100.0),            # :1062-1160 (dv/dy)
    lambda a, b: (0.0, float(a) / 100.0),            # :1162-1254 (dv/dx)
    lambda a, b: (float(a) / 100.0, float(b) / 100.0),  # :1254-1320 (all)
])
def test_current_gradient_grids(mr, oracle, fn):
    x, y, u, v = H.current_arrays(100, 100, 1.0, 1.0, fn)
    cur = ("grid", x.astype(np.float64), y.astype(np.float64), u, v)
    x0 = np.array([1.0, 1.0, 50.0, 1.0])
    y0 = np.array([1.0, 1.0, 1.0, 50.0])
    kx0 = np.array([0.1, 0.0, 0.0, 0.1])
    ky0 = np.array([0.0, 0.1, 0.1, 0.0])
    r = both(mr, oracle, ("constant", 1000.0), cur, x0, y0, kx0, ky0, 1.0, 10.0, 1.0)
    check(*r)


def _around(v, k=3):
    """v and its k nearest doubles on each side."""
    out = [v]
    lo = hi = v
    for _ in range(k):
        lo = np.nextafter(lo, -np.inf)
        hi = np.nextafter(hi, np.inf)
        out += [lo, hi]
    return out


def test_current_cells_at_grid_lines(mr, oracle):
    # The current's cell index at and next to every grid line, on axes whose
    # spacing is not a binary fraction, over a random current: a wrong cell
    # changes the cell-constant gradients (cartesian_current.rs:515-536) and
    # with them the first stage of the step.
    rng = np.random.default_rng(31)
    nx, ny = 48, 40
    xs = 3.3 + 0.7 * np.arange(nx)
    ys = -1.1 + 0.3 * np.arange(ny)
    u = rng.normal(0.0, 0.3, (ny, nx))
    v = rng.normal(0.0, 0.3, (ny, nx))
    cur = ("grid", xs, ys, u, v)
    px = np.array([t for a in xs for t in _around(float(a))] + [xs[0] - 0.01, xs[-1] + 0.01])
    py = np.array([t for a in ys for t in _around(float(a))] + [ys[0] - 0.01, ys[-1] + 0.01])
    x0 = np.concatenate([px, rng.uniform(xs[1], xs[-2], py.size)])
    y0 = np.concatenate([rng.uniform(ys[1], ys[-2], px.size), py])
    th = rng.uniform(0, 2 * np.pi, x0.size)
    r = both(mr, oracle, ("constant", 50.0), cur, x0, y0, 0.05 * np.cos(th), 0.05 * np.sin(th),
             0.0, 2.0, 0.5)
    check(*r)
    assert np.any(r[2] == 1) and np.any(r[1] > 2)


def test_depth_len_shorter_than_grid(mr, oracle):
    # depth_at_indexes checks the flat index against the array length
    # (cartesian_netcdf3.rs:465-471): lookups past the end are errors (NaN).
    x, y, depth = H.bathymetry_arrays(20, 20, 10.0, 10.0, lambda a, b: 50.0 + float(a))
    short = depth.ravel()[: 20 * 12]
    n = 64
    th = np.linspace(0, 2 * np.pi, n, endpoint=False)
    r = both(mr, oracle, ("grid", x, y, short), ZERO, np.full(n, 95.0), np.full(n, 95.0),
             0.05 * np.cos(th), 0.05 * np.sin(th), 0.0, 60.0, 0.5)
    check(*r)
    assert np.any(r[2] == 1)


@pytest.mark.parametrize("stop_rule", [0, 1])
def test_random_grid_stop_rules(mr, oracle, stop_rule):
    grid, rays = stop_rule_case()
    r = both(mr, oracle, ("grid",) + grid, ZERO, *rays, 0.0, 30.0, 1.0, stop_rule=stop_rule)
    check(*r)


# ------------------------------------------------------ integration tests --

@pytest.mark.parametrize("name", list(BEACHES))
def test_linear_beach(mr, oracle, name):
    # src/tests/linear_beach.rs
    (h0, dhdx, dhdy), rays, expect = beach_rays(name)
    r = both(mr, oracle, ("slope", h0, 0.0, 0.0, dhdx, dhdy), ZERO, *rays, 0.0, 1000.0, 1.0)
    check(*r)
    check_beach(r[0], r[1], expect)


@pytest.mark.parametrize("depth", [2000.0, 10.0])
def test_constant_depth_circle(mr, oracle, depth):
    # src/tests/test_constant_depth.rs
    rays = circle_rays()
    r = both(mr, oracle, ("constant", depth), ZERO, *rays, 0.0, 5000.0, 1.0)
    check(*r)
    check_circle(r[0], r[1], rays[2], rays[3])


@pytest.mark.parametrize("t0,t_end,dt", [
    (0.0, 0.0, 1.0),      # zero duration: the initial row only
    (0.0, 10.25, 1.0),    # fractional: ceil(10.25 / 1) = 11 steps, the last past t_end
    (0.0, 0.5, 2.0),      # one step longer than the whole duration
    (37.5, 87.5, 0.5),    # a start time other than 0 (t accumulates from t0)
])
def test_durations_and_start_times(mr, oracle, t0, t_end, dt):
    # the stepper's step count and time rows (ceil((t_end - t0) / dt) steps,
    # t += dt) on a grid with a current, rays of several directions
    from mantaray_gb300.workloads import seamount

    w = seamount(n_rays=64, steps=10)
    bathy = ("grid", w.bx, w.by, w.depth)
    current = ("grid", w.cx, w.cy, w.u, w.v)
    r = both(mr, oracle, bathy, current, w.x0 + 500.0, w.y0, w.kx0, w.ky0, t0, t_end, dt)
    check(*r)
    steps = math.ceil((t_end - t0) / dt)
    assert r[0].shape[1] == steps + 1
    assert np.all(r[1] == steps + 1)
    t = t0
    for row in range(steps + 1):
        assert np.all(r[0][0, row] == t)
        t = t + dt


def test_slope_and_many_waves(mr, oracle):
    # src/ray.rs:550-584 and :1331-1361
    r = both(mr, oracle, ("slope",), ZERO, 10.0, 1000.0, 0.1, 0.0, 0.0, 100.0, 1.0)
    check(*r)
    ys = np.arange(10.0, 100.0, 10.0)
    r = both(mr, oracle, ("slope",), ZERO, np.full(9, 10.0), ys, np.ones(9), np.zeros(9),
             0.0, 3000.0, 1.0)
    check(*r)


# --------------------------------------------------------- benchmark cases --

def _workload_both(mr, oracle, w, stop_rule=0):
    bathy = ("grid", w.bx, w.by, w.depth)
    cur = ("grid", w.cx, w.cy, w.u, w.v)
    return both(mr, oracle, bathy, cur, w.x0, w.y0, w.kx0, w.ky0, w.t0, w.t_end, w.dt, stop_rule)


def test_planar_beach_full(mr, oracle):
    # The CPU reference case at full size: 1,024 rays x 2,000 steps.
    from mantaray_gb300.workloads import planar_beach

    r = _workload_both(mr, oracle, planar_beach())
    worst = check(*r)
    assert worst <= 1.0


def test_seamount_subset(mr, oracle):
    # The GPU drop-in case's fields and step count with a seeded subset of
    # 768 of its 65,536 rays (all 4,000 steps).
    from mantaray_gb300.workloads import seamount

    w = seamount()
    idx = np.random.default_rng(11).choice(w.n, 768, replace=False)
    r = _workload_both(mr, oracle, w.subset(np.sort(idx)))
    check(*r)


def test_seamount_full_size_properties(mr, oracle):
    # All 65,536 rays x 4,000 steps on the GPU (10.5 GB of trajectories kept on
    # the device); size-independent checks: determinism, t exact, rows, and a
    # seeded sample of rays compared with the oracle.
    import torch

    from mantaray_gb300.workloads import seamount

    w = seamount()
    b = mr.Bathymetry.grid(w.bx, w.by, w.depth)
    c = mr.Current.grid(w.cx, w.cy, w.u, w.v)
    rows = mr.num_steps(w.t0, w.t_end, w.dt) + 1
    dev = torch.device("cuda")
    ins = [torch.from_numpy(a).to(dev) for a in (w.x0, w.y0, w.kx0, w.ky0)]
    traj = torch.empty((5, rows, w.n), dtype=torch.float64, device=dev)
    n_rows = torch.empty(w.n, dtype=torch.int32, device=dev)
    status = torch.empty(w.n, dtype=torch.uint8, device=dev)
    mr.trace_device(b, c, *ins, w.t0, w.t_end, w.dt, traj, n_rows, status, math=MATH)
    torch.cuda.synchronize()
    checksum1 = torch.nansum(traj[1:], dim=(1, 2)).cpu().numpy()
    rows1 = n_rows.cpu().numpy()
    # determinism: a second run is bitwise identical
    traj2 = torch.empty_like(traj)
    mr.trace_device(b, c, *ins, w.t0, w.t_end, w.dt, traj2, n_rows, status, math=MATH)
    torch.cuda.synchronize()
    assert torch.equal(torch.nan_to_num(traj, nan=-1e300), torch.nan_to_num(traj2, nan=-1e300))
    del traj2
    # every ray that completed has t exactly as the stepper accumulates it
    t_last = traj[0, rows - 1].cpu().numpy()
    done = rows1 == rows
    t = 0.0
    for _ in range(rows - 1):
        t = t + w.dt
    assert np.all(t_last[done] == t)
    assert np.all(np.isfinite(checksum1))
    # seeded sample against the oracle
    idx = np.sort(np.random.default_rng(3).choice(w.n, 96, replace=False))
    sub = traj[:, :, torch.from_numpy(idx).to(dev)].cpu().numpy()
    ob = oracle.Bathymetry.grid(w.bx, w.by, w.depth)
    oc = oracle.Current.grid(w.cx, w.cy, w.u, w.v)
    o = oracle.trace(ob, oc, w.x0[idx], w.y0[idx], w.kx0[idx], w.ky0[idx], w.t0, w.t_end, w.dt)
    H.assert_parity(np.ascontiguousarray(sub), rows1[idx], o[0], o[1], rtol=RTOL)
    # The same rays traced alone (a small call) give the same bits; and
    # repeated into a call of 78,720 rays, more blocks than one wave of the
    # build that keeps each lane's last cells holds, so that call runs the
    # build without that cache.
    del traj
    small = mr.trace(b, c, w.x0[idx], w.y0[idx], w.kx0[idx], w.ky0[idx], w.t_end - w.t0, w.dt,
                     t0=w.t0, math=MATH)
    assert np.array_equal(small.n_rows, rows1[idx])
    assert np.array_equal(np.nan_to_num(small.traj, nan=-1e300), np.nan_to_num(sub, nan=-1e300))
    reps = 820
    big_in = [torch.from_numpy(np.tile(a[idx], reps)).to(dev) for a in (w.x0, w.y0, w.kx0, w.ky0)]
    nb = len(idx) * reps
    big = torch.empty((5, rows, nb), dtype=torch.float64, device=dev)
    nr_big = torch.empty(nb, dtype=torch.int32, device=dev)
    st_big = torch.empty(nb, dtype=torch.uint8, device=dev)
    mr.trace_device(b, c, *big_in, w.t0, w.t_end, w.dt, big, nr_big, st_big, math=MATH)
    torch.cuda.synchronize()
    for k in (0, reps - 1):
        part = big[:, :, k * len(idx):(k + 1) * len(idx)].cpu().numpy()
        assert np.array_equal(nr_big[k * len(idx):(k + 1) * len(idx)].cpu().numpy(), rows1[idx])
        assert np.array_equal(np.nan_to_num(part, nan=-1e300), np.nan_to_num(sub, nan=-1e300))


def test_vortex_field_and_shelf_bump(mr, oracle):
    # Smooth fields where every lookup matters: the multi-source case's
    # generator (Gaussian shoals, 16 Gaussian vortices) at 512^2, and the
    # differentiation case's shelf with its shoal and jet, 256 rays each,
    # 2,000 steps, every row against the oracle.
    from mantaray_gb300.workloads import multi_source, shelf_bump

    scen, rays = multi_source(n_sources=8, rays_per_source=32, n_scenarios=1, n=512,
                              steps=2000)
    bx, by, depth, cx, cy, u, v = scen[0]
    r = both(mr, oracle, ("grid", bx, by, depth), ("grid", cx, cy, u, v), rays["x0"],
             rays["y0"], rays["kx0"], rays["ky0"], 0.0, 2000 * rays["dt"], rays["dt"])
    check(*r)
    w = shelf_bump(n_rays=256, steps=2000)
    check(*_workload_both(mr, oracle, w))


@pytest.mark.parametrize("size", ["fine_corner", "whole_domain"])
def test_shelf_slope_fields_every_row(mr, oracle, size):
    # The large single-scenario case's generator (shelf-slope profile, k^-3
    # roughness at 50 m rms, meandering jet and 64 eddies; |k0| at the launch
    # depth), every row of every ray against the oracle: at its own 50 m
    # spacing on a 2,048^2 corner of the domain (the roughness at full
    # resolution; 2,048 rays x 2,000 steps), and over its whole 409.6 km
    # domain on a 1,024^2 grid at 400 m, where the rays cross the slope onto
    # the 60 m shelf (512 rays x 20,000 steps; about half end at the shore
    # or a side edge).
    from mantaray_gb300.workloads import shelf_slope

    kw = (dict(n=2048, n_rays=2048, steps=2000) if size == "fine_corner"
          else dict(n=1024, spacing=400.0, n_rays=512, steps=20000))
    f, r = shelf_slope(**kw)
    res = both(mr, oracle, ("grid",) + tuple(f[:3]), ("grid",) + tuple(f[3:]), r["x0"], r["y0"],
               r["kx0"], r["ky0"], r["t0"], r["t0"] + r["steps"] * r["dt"], r["dt"])
    check(*res)
    assert np.any(res[2] != 0) or size == "fine_corner"
