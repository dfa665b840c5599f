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


def shelf_bump(n_rays: int = 262144, steps: int = 3000, bump_scale: float = 1.0,
               seed: int = 1002) -> Workload:
    """Differentiation case: 262,144 rays on a 512 x 512 grid at 200 m.
    Bathymetry: a linear shelf from 3,000 m (x = 0) to 20 m (far edge) with a
    1,500 m Gaussian shoal (sigma 8 km) at the centre of the domain, where the
    shelf is 1,510 m deep (so its top is at 10 m), floored at 5 m;
    `bump_scale` multiplies the shoal (1.1 gives the loss targets).  Current:
    a Gaussian jet u(y) = 1.0 exp(-(y - 51.2 km)^2 / (2 (5 km)^2)), v = 0.
    Rays start at x = 25 km, y ~ U[25, 77] km, directions ~ U(+-30 deg),
    T ~ U[8, 14] s, so that in 3,000 s they cross the shoal; dt = 1 s."""
    rng = np.random.default_rng(seed)
    n = 512
    x = np.arange(n, dtype=np.float64) * 200.0
    L = x[-1]
    shelf = 3000.0 - 2980.0 * (x / L)
    r2 = (x[None, :] - 51200.0) ** 2 + (x[:, None] - 51200.0) ** 2
    depth = np.maximum(5.0, shelf[None, :] - bump_scale * 1500.0 * np.exp(-r2 / (2.0 * 8000.0 ** 2)))
    u = np.broadcast_to(np.exp(-((x[:, None] - 51200.0) ** 2) / (2.0 * 5000.0 ** 2)), (n, n)).copy()
    v = np.zeros((n, n))
    y0 = rng.uniform(25000.0, 77000.0, n_rays)
    theta = rng.uniform(-np.deg2rad(30.0), np.deg2rad(30.0), n_rays)
    period = rng.uniform(8.0, 14.0, n_rays)
    x0 = np.full(n_rays, 25000.0)
    h0 = 3000.0 - 2980.0 * (x0 / L)
    kx0, ky0 = wavenumber_vector(period, h0, theta)
    return Workload(f"shelf_bump_{n_rays}rays_512x512_dt1_{steps}steps", x.astype(np.float32),
                    x.astype(np.float32), depth, x, x, u, v, x0, y0, kx0, ky0, 0.0, float(steps),
                    1.0, {"grid": (n, n), "spacing": 200.0, "bump_scale": bump_scale})


def _gaussian_vortices(rng, x, y, count, speed_lo, speed_hi, sigma_lo, sigma_hi):
    """u = d(psi)/dy, v = -d(psi)/dx of a streamfunction made of `count`
    Gaussian vortices psi_j = A_j exp(-r^2 / (2 s_j^2)); each vortex's peak
    speed (at r = s_j) is drawn from [speed_lo, speed_hi] with a random sign.
    Each vortex is evaluated within 6 sigma of its centre (beyond that its
    velocity is below 1e-7 of its peak)."""
    u = np.zeros((y.size, x.size))
    v = np.zeros((y.size, x.size))
    dxg, dyg = x[1] - x[0], y[1] - y[0]
    for _ in range(count):
        cx, cy = rng.uniform(x[0], x[-1]), rng.uniform(y[0], y[-1])
        s = rng.uniform(sigma_lo, sigma_hi)
        a = rng.choice([-1.0, 1.0]) * rng.uniform(speed_lo, speed_hi) * s * np.exp(0.5)
        i0 = max(0, int((cx - 6 * s - x[0]) / dxg)); i1 = min(x.size, int((cx + 6 * s - x[0]) / dxg) + 2)
        j0 = max(0, int((cy - 6 * s - y[0]) / dyg)); j1 = min(y.size, int((cy + 6 * s - y[0]) / dyg) + 2)
        dx = x[None, i0:i1] - cx
        dy = y[j0:j1, None] - cy
        g = a * np.exp(-(dx * dx + dy * dy) / (2.0 * s * s)) / (s * s)
        u[j0:j1, i0:i1] += -dy * g
        v[j0:j1, i0:i1] += dx * g
    return u, v


def multi_source(n_sources: int = 1024, rays_per_source: int = 4096, n_scenarios: int = 8,
                 n: int = 2048, steps: int = 20000, seed: int = 1003):
    """Batching + precision case: 8 scenarios of 2,048 x 2,048 grids at 100 m.
    Each scenario's bathymetry is 4,000 m minus 32 seeded Gaussian shoals
    (amplitude 500-4,500 m, sigma 5-40 km) clipped to 20-4,000 m; its current
    comes from a streamfunction of 16 Gaussian vortices with peak speeds
    0.2-1.5 m/s (sigma 5-25 km).  1,024 point sources (128 per scenario, away
    from the edges) emit 4,096 rays each, directions ~ U[0, 2 pi), periods
    ~ U[6, 18] s.  dt = 2 s, up to 20,000 steps.  Returns (scenarios, rays):
    scenarios = [(bx, by, depth, cx, cy, u, v)], rays = dict of arrays with a
    `scenario` column; rays are grouped by scenario."""
    rng = np.random.default_rng(seed)
    x = np.arange(n, dtype=np.float64) * 100.0
    scenarios = []
    depth_fns = []
    for _ in range(n_scenarios):
        bumps = [(rng.uniform(x[0], x[-1]), rng.uniform(x[0], x[-1]), rng.uniform(500, 4500),
                  rng.uniform(5000, 40000)) for _ in range(32)]
        X, Y = x[None, :], x[:, None]
        h = np.full((n, n), 4000.0)
        for cx, cy, a, s in bumps:
            h -= a * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2.0 * s * s))
        h = np.clip(h, 20.0, 4000.0)
        u, v = _gaussian_vortices(rng, x, x, 16, 0.2, 1.5, 5000.0, 25000.0)
        scenarios.append((x.astype(np.float32), x.astype(np.float32), h, x, x, u, v))

        def depth_at(px, py, bumps=bumps):
            hh = np.full(px.shape, 4000.0)
            for cx, cy, a, s in bumps:
                hh -= a * np.exp(-((px - cx) ** 2 + (py - cy) ** 2) / (2.0 * s * s))
            return np.clip(hh, 20.0, 4000.0)

        depth_fns.append(depth_at)
    per_scen = n_sources // n_scenarios
    xs, ys, kxs, kys, sid = [], [], [], [], []
    margin = 10000.0
    for s in range(n_scenarios):
        sx = rng.uniform(margin, x[-1] - margin, per_scen)
        sy = rng.uniform(margin, x[-1] - margin, per_scen)
        px = np.repeat(sx, rays_per_source)
        py = np.repeat(sy, rays_per_source)
        theta = rng.uniform(0.0, 2.0 * np.pi, px.size)
        period = rng.uniform(6.0, 18.0, px.size)
        kx, ky = wavenumber_vector(period, depth_fns[s](px, py), theta)
        xs.append(px); ys.append(py); kxs.append(kx); kys.append(ky)
        sid.append(np.full(px.size, s, np.uint8))
    rays = {"x0": np.concatenate(xs), "y0": np.concatenate(ys), "kx0": np.concatenate(kxs),
            "ky0": np.concatenate(kys), "scenario": np.concatenate(sid), "t0": 0.0, "dt": 2.0,
            "steps": steps}
    return scenarios, rays


def shelf_slope(n: int = 8192, n_rays: int = 16777216, steps: int = 50000, seed: int = 1004,
                spacing: float = 50.0):
    """Large single-scenario case: 8,192 x 8,192 grid at 50 m.  Bathymetry: a
    continental shelf-slope profile along x (4,000 m deep at the entry edge,
    a tanh slope centred at 300 km, 15 km wide, up to a 60 m shelf) plus
    seeded 2-D random-phase roughness with a k^-3 spectrum scaled to 50 m rms,
    floored at 5 m.  Current: a meandering jet along x (1 m/s, 20 km wide,
    meander amplitude 30 km, wavelength 150 km) plus 64 seeded Gaussian eddies
    (0.2-1.0 m/s, sigma 5-20 km).  Swell enters at x = 0 with y ~ U over the
    edge, directions ~ U(+-15 deg), periods ~ U[10, 16] s; dt = 2 s, up to
    50,000 steps.  Returns (fields, rays) like multi_source (one scenario).
    A smaller n at the same spacing is a corner of that domain; n = 1,024 at
    a `spacing` of 400 m keeps the whole domain (slope, shelf, jet, eddies)
    on a coarser grid."""
    rng = np.random.default_rng(seed)
    x = np.arange(n, dtype=np.float64) * spacing
    profile = 60.0 + (4000.0 - 60.0) * 0.5 * (1.0 - np.tanh((x - 300000.0) / 15000.0))
    # random-phase k^-3 roughness (FFT synthesis on the grid)
    kx = np.fft.fftfreq(n, d=spacing)
    ky = np.fft.rfftfreq(n, d=spacing)
    kk = np.hypot(kx[:, None], ky[None, :])
    amp = np.zeros_like(kk)
    nz = kk > 0
    amp[nz] = kk[nz] ** -1.5  # |F|^2 ~ k^-3
    phase = np.exp(2j * np.pi * rng.random(kk.shape))
    rough = np.fft.irfft2(amp * phase, s=(n, n))
    rough *= 50.0 / np.sqrt(np.mean(rough * rough))
    depth = np.maximum(5.0, profile[None, :] + rough)
    del rough, amp, phase, kk
    Y = x[:, None]
    yc = x[-1] / 2 + 30000.0 * np.sin(2.0 * np.pi * x[None, :] / 150000.0)
    u = 1.0 * np.exp(-((Y - yc) ** 2) / (2.0 * 20000.0 ** 2))
    v = np.zeros_like(u)
    eu, ev = _gaussian_vortices(rng, x, x, 64, 0.2, 1.0, 5000.0, 20000.0)
    u += eu
    v += ev
    del eu, ev
    y0 = rng.uniform(0.0, x[-1], n_rays)
    theta = rng.uniform(-np.deg2rad(15.0), np.deg2rad(15.0), n_rays)
    period = rng.uniform(10.0, 16.0, n_rays)
    x0 = np.zeros(n_rays)
    # |k0| at the launch depth h(0, y0): the grid's x = 0 column interpolated
    # linearly in y (the bilinear at a zero x fraction), roughness included
    kx0, ky0 = wavenumber_vector(period, np.interp(y0, x, depth[:, 0]), theta)
    fields = (x.astype(np.float32), x.astype(np.float32), depth, x, x, u, v)
    rays = {"x0": x0, "y0": y0, "kx0": kx0, "ky0": ky0, "scenario": None, "t0": 0.0, "dt": 2.0,
            "steps": steps}
    return fields, rays
