"""Refraction against Snell's law, the analytic check of the reference's
notebooks/theoretical_comparison (snells_law_verification.ipynb, forcing
from data_generation.ipynb: a 300 x 150 grid at 50 m; ten shelves stepping
from 100 m to 10 m along x; or 10,000 m deep water with a v = 2 m/s current
on the right half).  With fields that vary in x only, k_y is conserved
exactly by the ray equations and the absolute frequency
omega = sqrt(g k tanh(k h)) + k . U by the flow, so on each shelf the
direction follows from the full dispersion relation:
k solves (omega - k_y V)^2 = g k tanh(k h), sin(phi) = k_y / k.
The oracle (CPU) and the plain FP64 kernel through the drop-in single_ray
(GPU, NetCDF files) are checked mid-shelf to 1% of the angle (the discrete
model conserves omega only approximately where the depth or current jumps
within one cell: measured 0.2% for the shelves, 0.5% for the shear), and
k_y bit for bit."""

import math

import numpy as np
import pytest

from tests import helpers as H

G = 9.8
NX, NY, DL = 300, 150, 50.0


def _step_depth(x, _y):
    # data_generation.ipynb: depth_max - floor(linspace(0, 10, NX, endpoint=False)) * 10
    i = int(round(x / DL))
    return 100.0 - math.floor(i * 10 / NX) * 10.0


def _shear(x, _y):
    return (0.0, 2.0 if int(round(x / DL)) >= NX // 2 else 0.0)


def _k_for(omega, ky, h, v):
    """|k| with (omega - ky v)^2 = g k tanh(k h) (Newton)."""
    s2 = (omega - ky * v) ** 2
    k = max(s2 / G, math.sqrt(s2 / (G * h)))
    for _ in range(100):
        th = math.tanh(k * h)
        f = G * k * th - s2
        k -= f / (G * th + G * k * h * (1 - th * th))
    return k


def _check(traj, rows, depth_of, v_of, k0, phi0, mids):
    x, y, kx, ky = (traj[q, :rows, 0] for q in range(1, 5))
    ok = np.isfinite(x)
    x, y, kx, ky = x[ok], y[ok], kx[ok], ky[ok]
    ky0 = k0 * math.sin(phi0)
    assert np.all(ky == ky[0]) and ky[0] == ky0  # k_y conserved exactly
    omega = math.sqrt(G * k0 * math.tanh(k0 * depth_of(50.0))) + ky0 * v_of(50.0)
    checked = 0
    for xm in mids:
        if xm > x.max():
            continue
        j = int(np.argmin(np.abs(x - xm)))
        phi = math.atan2(ky[j], kx[j])
        k_th = _k_for(omega, ky0, depth_of(x[j]), v_of(x[j]))
        phi_th = math.asin(ky0 / k_th)
        assert abs(phi - phi_th) <= 1e-2 * abs(phi_th), (xm, phi, phi_th)
        checked += 1
    assert checked >= min(3, len(mids))


def _shelf_mids():
    edges = [i * DL for i in range(NX) if i == 0 or _step_depth(i * DL, 0) != _step_depth((i - 1) * DL, 0)]
    return [e + 15 * DL for e in edges]


CASES = {
    # notebook parameters: lambda = 10 km, phi0 = pi/8, start (50, 500), 1000 s at dt 0.5
    "step_bathymetry": (_step_depth, lambda x, y: (0.0, 0.0), 2 * math.pi / 10000, math.pi / 8,
                        1000.0, 0.5),
    # deep water, shear current: a 400 m wave at 30 degrees
    "shear_current": (lambda x, y: 10000.0, _shear, 2 * math.pi / 400, math.pi / 6, 1000.0, 0.5),
}


def _mids(name):
    return _shelf_mids() if name == "step_bathymetry" else [NX // 4 * DL, 9000.0, 10000.0]


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_follows_snells_law(oracle, name):
    depth_fn, cur_fn, k0, phi0, dur, dt = CASES[name]
    x, y, depth = H.bathymetry_arrays(NX, NY, DL, DL, depth_fn)
    cx, cy, u, v = H.current_arrays(NX, NY, DL, DL, cur_fn)
    ob = oracle.Bathymetry.grid(x, y, depth)
    oc = oracle.Current.grid(cx.astype(np.float64), cy.astype(np.float64), u, v)
    traj, rows, _ = oracle.trace(ob, oc, [50.0], [500.0], [k0 * math.cos(phi0)],
                                 [k0 * math.sin(phi0)], 0.0, dur, dt)
    _check(traj, int(rows[0]), lambda xx: depth_fn(xx, 0), lambda xx: cur_fn(xx, 0)[1], k0, phi0,
           _mids(name))


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_gpu_single_ray_follows_snells_law(tmp_path, name):
    import mantaray_gb300 as mr

    depth_fn, cur_fn, k0, phi0, dur, dt = CASES[name]
    bp, cp = tmp_path / "b.nc", tmp_path / "c.nc"
    H.write_bathymetry_nc(bp, NX, NY, DL, DL, depth_fn)
    H.write_current_nc(cp, NX, NY, DL, DL, cur_fn)
    ds = mr.single_ray(50.0, 500.0, k0 * math.cos(phi0), k0 * math.sin(phi0), dur, dt, str(bp),
                       str(cp))
    traj = np.stack([np.asarray(ds[v]) for v in ("time", "x", "y", "kx", "ky")])[:, :, None]
    _check(traj, traj.shape[1], lambda xx: depth_fn(xx, 0), lambda xx: cur_fn(xx, 0)[1], k0,
           phi0, _mids(name))
