"""Initial conditions for rays: wavenumber from wave period and depth.

The reference's notebooks set |k0| from the linear dispersion relation
(notebooks/canonical_examples/utils.py:11-26).  Here the intrinsic relation
(2*pi/T)^2 = g k tanh(k h) is solved for k by Newton iteration in float64,
vectorised over rays.
"""

from __future__ import annotations

import numpy as np

G = 9.8  # src/wave_ray_path.rs:23


def wavenumber(period, depth, iterations: int = 60) -> np.ndarray:
    """|k| solving (2*pi/T)^2 = g k tanh(k h) for every (T, h)."""
    T = np.asarray(period, dtype=np.float64)
    h = np.asarray(depth, dtype=np.float64)
    omega2 = (2.0 * np.pi / T) ** 2
    # deep-water guess, raised to the shallow-water value where that is larger
    k = np.maximum(omega2 / G, np.sqrt(omega2 / (G * h)))
    for _ in range(iterations):
        th = np.tanh(k * h)
        f = G * k * th - omega2
        df = G * th + G * k * h * (1.0 - th * th)
        step = f / df
        k = k - step
        if np.all(np.abs(step) <= 1e-15 * np.abs(k)):
            break
    return k


def wavenumber_vector(period, depth, direction):
    """(kx, ky) for rays with periods T, launch depths h and directions (rad from +x)."""
    k = wavenumber(period, depth)
    d = np.asarray(direction, dtype=np.float64)
    return k * np.cos(d), k * np.sin(d)


def cfl_step(grid_spacing: float, period, depth) -> float:
    """Time step in which the fastest ray crosses one grid cell: the CFL step
    of notebooks/canonical_examples/utils.py:47-67, with the finite-depth group
    velocity in place of the deep-water one used there."""
    k = wavenumber(period, depth)
    kh = k * np.asarray(depth, dtype=np.float64)
    cg = 0.5 * np.sqrt(G / k * np.tanh(kh)) * (1.0 + 2.0 * kh / np.sinh(2.0 * kh))
    return float(grid_spacing / np.max(cg))


# ---- the reference notebooks' helpers (notebooks/canonical_examples/utils.py,
# notebooks/agulhas/notebook/src.py); those notebooks use g = 9.81 ----------

G_NOTEBOOK = 9.81  # notebooks/canonical_examples/utils.py:8


def period_to_wavenumber_deep(period, g: float = G_NOTEBOOK):
    """Deep-water wavenumber (2 pi)^2 / (g T^2) (utils.py:11-26)."""
    T = np.asarray(period, dtype=np.float64)
    return (2.0 * np.pi) ** 2 / (g * T * T)


def deep_water_group_velocity(k, g: float = G_NOTEBOOK):
    """Deep-water group velocity sqrt(g / k) / 2 (utils.py:29-44)."""
    return np.sqrt(g / np.asarray(k, dtype=np.float64)) / 2.0


def cfl_time_step(x, y, k0, g: float = G_NOTEBOOK) -> float:
    """Smallest mean grid spacing over the deep-water group velocity of k0
    (utils.py:47-67)."""
    dd = min(float(np.diff(np.asarray(x, dtype=np.float64)).mean()),
             float(np.diff(np.asarray(y, dtype=np.float64)).mean()))
    return dd / float(deep_water_group_velocity(k0, g))


def duration_to_cross(x, k0, g: float = G_NOTEBOOK) -> int:
    """max(x) over the deep-water group velocity, rounded (utils.py:71-87)."""
    return int(round(float(np.max(x)) / float(deep_water_group_velocity(k0, g))))


def start_line_points(x_line, y_line, x_grid, y_grid, num_points):
    """num_points evenly spaced on the segment (x_line[0], y_line[0]) ->
    (x_line[1], y_line[1]), each moved to the nearest grid node, as
    start_line_ray_tracing does (notebooks/agulhas/notebook/src.py:60-82).
    The nearest node of a regular grid is found per axis (the squared
    distance separates), first index on ties as numpy.argmin."""
    xg = np.asarray(x_grid, dtype=np.float64)
    yg = np.asarray(y_grid, dtype=np.float64)
    px = np.linspace(x_line[0], x_line[1], num_points)
    py = np.linspace(y_line[0], y_line[1], num_points)
    ix = np.argmin(np.abs(xg[None, :] - px[:, None]), axis=1)
    iy = np.argmin(np.abs(yg[None, :] - py[:, None]), axis=1)
    return xg[ix], yg[iy]


# ---- device seeding (include/mantaray_gpu.h, mr_seed_*) ---------------------

def _seed_outputs(n, device):
    import torch

    return [torch.empty(n, dtype=torch.float64, device=device) for _ in range(4)]


def seed_point_sources(bathymetry, sx, sy, rays_per_source, direction_range=(0.0, 2 * np.pi),
                       period_range=(10.0, 10.0), seed=0, even_directions=False, stream=None):
    """Initial states (x0, y0, kx0, ky0) as CUDA float64 tensors for
    rays_per_source rays from each point (sx[s], sy[s]) (CUDA float64
    tensors), directions and periods uniform over the ranges (directions
    evenly spaced with even_directions), |k| from the dispersion relation at
    the launch depth.  Computed on the device."""
    import torch

    from . import _native as N

    sx = sx.contiguous()
    sy = sy.contiguous()
    out = _seed_outputs(sx.numel() * int(rays_per_source), sx.device)
    st = stream if stream is not None else torch.cuda.current_stream(sx.device).cuda_stream
    N.check(N.load().mr_seed_point_sources(
        bathymetry.handle, sx.numel(), sx.data_ptr(), sy.data_ptr(), int(rays_per_source),
        float(direction_range[0]), float(direction_range[1]), float(period_range[0]),
        float(period_range[1]), int(seed) & (2 ** 64 - 1),
        N.SEED_EVEN_DIRECTIONS if even_directions else 0, *[t.data_ptr() for t in out], st))
    return tuple(out)


def seed_line(bathymetry, start, end, n, direction_range=(0.0, 0.0), period_range=(10.0, 10.0),
              seed=0, even_directions=False, device="cuda", stream=None):
    """Initial states for n rays at numpy.linspace points from `start` to
    `end` (x, y), as seed_point_sources.  Computed on the device."""
    import torch

    from . import _native as N

    out = _seed_outputs(int(n), torch.device(device))
    st = stream if stream is not None else torch.cuda.current_stream(out[0].device).cuda_stream
    N.check(N.load().mr_seed_line(
        bathymetry.handle, float(start[0]), float(start[1]), float(end[0]), float(end[1]), int(n),
        float(direction_range[0]), float(direction_range[1]), float(period_range[0]),
        float(period_range[1]), int(seed) & (2 ** 64 - 1),
        N.SEED_EVEN_DIRECTIONS if even_directions else 0, *[t.data_ptr() for t in out], st))
    return tuple(out)


def splitmix_uniform(seed, index):
    """The device seeding's uniforms: SplitMix64 (Steele, Lea and Flood 2014)
    of seed + (index + 1) * 0x9E3779B97F4A7C15, top 53 bits over 2^53."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (np.asarray(index, dtype=np.uint64) + np.uint64(1)) * \
            np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
