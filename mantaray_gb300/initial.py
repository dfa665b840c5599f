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
