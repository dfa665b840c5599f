"""Device seeding of initial states (mr_seed_point_sources / mr_seed_line)
against the host: positions exactly, directions and periods from the same
SplitMix64 uniforms, |k| against the host dispersion solve (1e-12)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host_k(periods, h):
    from mantaray_gb300.initial import wavenumber

    return wavenumber(periods, h)


def test_point_sources_constant_depth():
    import torch

    import mantaray_gb300 as mr
    from mantaray_gb300.initial import seed_point_sources, splitmix_uniform

    b = mr.Bathymetry.constant(50.0)
    sx = torch.tensor([100.0, 2500.5, -7.25], dtype=torch.float64, device="cuda")
    sy = torch.tensor([0.0, 333.0, 1e4], dtype=torch.float64, device="cuda")
    m, seed = 1000, 987654321
    x0, y0, kx0, ky0 = (t.cpu().numpy() for t in seed_point_sources(
        b, sx, sy, m, (-0.5, 2.0), (6.0, 18.0), seed=seed))
    r = np.arange(3 * m)
    th = -0.5 + (2.0 - -0.5) * splitmix_uniform(seed, 2 * r)
    T = 6.0 + (18.0 - 6.0) * splitmix_uniform(seed, 2 * r + 1)
    k = _host_k(T, np.full(r.size, 50.0))
    np.testing.assert_array_equal(x0, np.repeat(sx.cpu().numpy(), m))
    np.testing.assert_array_equal(y0, np.repeat(sy.cpu().numpy(), m))
    np.testing.assert_allclose(np.hypot(kx0, ky0), k, rtol=1e-12)
    np.testing.assert_allclose(np.arctan2(ky0, kx0), np.angle(np.exp(1j * th)), rtol=0, atol=1e-12)


def test_line_on_a_slope_with_even_directions():
    import torch  # noqa: F401

    import mantaray_gb300 as mr
    from mantaray_gb300.initial import seed_line, splitmix_uniform

    b = mr.Bathymetry.slope(h0=80.0, x0=0.0, y0=0.0, dhdx=-0.01, dhdy=0.002)
    n = 777
    x0, y0, kx0, ky0 = (t.cpu().numpy() for t in seed_line(
        b, (10.0, 20.0), (3010.0, 520.0), n, (-0.3, 0.3), (8.0, 12.0), seed=5,
        even_directions=True))
    np.testing.assert_array_equal(x0, np.linspace(10.0, 3010.0, n))
    np.testing.assert_array_equal(y0, np.linspace(20.0, 520.0, n))
    # ConstantSlope's depth in f32 (src/bathymetry/constant_slope.rs)
    xf, yf = x0.astype(np.float32), y0.astype(np.float32)
    h = (np.float32(80.0) + np.float32(-0.01) * (xf - np.float32(0.0)) +
         np.float32(0.002) * (yf - np.float32(0.0))).astype(np.float64)
    r = np.arange(n)
    T = 8.0 + (12.0 - 8.0) * splitmix_uniform(5, 2 * r + 1)
    th = -0.3 + (0.3 - -0.3) * ((r + 0.5) / n)
    np.testing.assert_allclose(np.hypot(kx0, ky0), _host_k(T, h), rtol=1e-12)
    np.testing.assert_allclose(np.arctan2(ky0, kx0), th, rtol=0, atol=1e-12)


def test_sources_off_the_grid_get_nan():
    import torch

    import mantaray_gb300 as mr
    from mantaray_gb300.initial import seed_point_sources
    from tests import helpers as H

    x, y, depth = H.bathymetry_arrays(50, 40, 10.0, 10.0, lambda a, b: 30.0)
    b = mr.Bathymetry.grid(x, y, depth)
    sx = torch.tensor([100.0, -50.0, 100.0], dtype=torch.float64, device="cuda")
    sy = torch.tensor([100.0, 100.0, 1e6], dtype=torch.float64, device="cuda")
    _, _, kx0, ky0 = (t.cpu().numpy() for t in seed_point_sources(b, sx, sy, 4))
    assert np.all(np.isfinite(kx0[:4])) and np.all(np.isnan(kx0[4:]))
    np.testing.assert_allclose(np.hypot(kx0[:4], ky0[:4]), _host_k(np.full(4, 10.0),
                                                                   np.full(4, 30.0)), rtol=1e-12)


def test_seeded_rays_trace_in_the_batched_form():
    # seeding and tracing both on the device: every seeded ray is traced
    import torch

    import mantaray_gb300 as mr
    from mantaray_gb300.batch import BatchTracer
    from mantaray_gb300.initial import seed_point_sources
    from tests import helpers as H

    x, y, depth = H.bathymetry_arrays(200, 200, 50.0, 50.0, lambda a, b: 20.0 + 0.2 * float(a))
    cx, cy, u, v = H.current_arrays(200, 200, 50.0, 50.0, lambda a, b: (0.1, 0.0))
    b = mr.Bathymetry.grid(x, y, depth)
    c = mr.Current.grid(cx.astype(np.float64), cy.astype(np.float64), u, v)
    sx = torch.tensor([5000.0, 3000.0], dtype=torch.float64, device="cuda")
    sy = torch.tensor([5000.0, 7000.0], dtype=torch.float64, device="cuda")
    rays = seed_point_sources(b, sx, sy, 2048, period_range=(6.0, 14.0), seed=1)
    res = BatchTracer([(b, c)]).trace(*rays, 1.0, 400)
    torch.cuda.synchronize()
    steps = res.n_steps.cpu().numpy()
    assert steps.size == 4096 and np.all(steps >= 1)
