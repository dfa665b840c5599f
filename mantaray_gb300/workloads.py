"""Synthetic workloads with the shapes, sizes and value distributions of the
benchmark configurations (no public dataset is involved).

Every generator is deterministic: numpy PCG64 seeded with 1000 + the
configuration index.  Fields are built on the host in float64; initial
|k0| solves the dispersion relation at the launch depth (initial.wavenumber).
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .initial import wavenumber_vector


@dataclass
class Workload:
    name: str
    # bathymetry grid (f32 axes, f64 depth [ny][nx]) and current grid (f64)
    bx: np.ndarray
    by: np.ndarray
    depth: np.ndarray
    cx: np.ndarray
    cy: np.ndarray
    u: np.ndarray
    v: np.ndarray
    # rays
    x0: np.ndarray
    y0: np.ndarray
    kx0: np.ndarray
    ky0: np.ndarray
    t0: float
    t_end: float
    dt: float
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.x0.size)

    def subset(self, idx) -> "Workload":
        """The same fields with a subset of the rays."""
        return Workload(self.name, self.bx, self.by, self.depth, self.cx, self.cy, self.u, self.v,
                        self.x0[idx], self.y0[idx], self.kx0[idx], self.ky0[idx], self.t0,
                        self.t_end, self.dt, dict(self.meta))


def planar_beach(n_rays: int = 1024) -> Workload:
    """Plain method, CPU reference case: 1,024 rays at x = 0, y evenly spaced
    0-9,990 m, 30 degrees from +x, T = 10 s; 1,000 x 1,000 grid at 10 m,
    h(x) = max(2, 100 - 0.009 x); zero current; dt = 0.5 s for 2,000 steps."""
    x = np.arange(1000, dtype=np.float64) * 10.0
    depth1d = np.maximum(2.0, 100.0 - 0.009 * x)
    depth = np.broadcast_to(depth1d[None, :], (1000, 1000)).copy()
    y0 = np.linspace(0.0, 9990.0, n_rays)
    x0 = np.zeros(n_rays)
    h0 = np.maximum(2.0, 100.0 - 0.009 * x0)
    kx0, ky0 = wavenumber_vector(np.full(n_rays, 10.0), h0, np.full(n_rays, np.deg2rad(30.0)))
    zeros = np.zeros((1000, 1000))
    return Workload("planar_beach_1024rays_1000x1000_dt0.5_2000steps", x.astype(np.float32),
                    x.astype(np.float32), depth, x, x, zeros, zeros.copy(), x0, y0, kx0, ky0,
                    0.0, 1000.0, 0.5, {"grid": (1000, 1000), "spacing": 10.0})


def seamount(n_rays: int = 65536, steps: int = 4000, seed: int = 1001) -> Workload:
    """Plain FP64 GPU drop-in case: 65,536 rays at x = 0, y ~ U[0, 100 km),
    directions ~ U(+-20 deg), T ~ U[8, 16] s; 2,001 x 2,001 grid at 50 m with a
    Gaussian seamount h = 4000 - 3800 exp(-r^2 / (2 (15 km)^2)) centred in the
    domain, floored at 5 m; uniform current (0.5, 0) m/s on the same grid;
    dt = 1 s for 4,000 steps."""
    rng = np.random.default_rng(seed)
    n = 2001
    x = np.arange(n, dtype=np.float64) * 50.0
    xc = yc = 50000.0
    r2 = (x[None, :] - xc) ** 2 + (x[:, None] - yc) ** 2
    depth = np.maximum(5.0, 4000.0 - 3800.0 * np.exp(-r2 / (2.0 * 15000.0 ** 2)))
    y0 = rng.uniform(0.0, 100000.0, n_rays)
    theta = rng.uniform(-np.deg2rad(20.0), np.deg2rad(20.0), n_rays)
    period = rng.uniform(8.0, 16.0, n_rays)
    x0 = np.zeros(n_rays)
    h0 = np.maximum(5.0, 4000.0 - 3800.0 * np.exp(-((x0 - xc) ** 2 + (y0 - yc) ** 2) / (2.0 * 15000.0 ** 2)))
    kx0, ky0 = wavenumber_vector(period, h0, theta)
    u = np.full((n, n), 0.5)
    v = np.zeros((n, n))
    return Workload(f"seamount_{n_rays}rays_2001x2001_dt1_{steps}steps", x.astype(np.float32),
                    x.astype(np.float32), depth, x, x, u, v, x0, y0, kx0, ky0, 0.0, float(steps),
                    1.0, {"grid": (n, n), "spacing": 50.0})
