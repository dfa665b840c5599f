"""The allocation-free batched entry point, mr_batch_trace_device_static.

Some callers cannot call cudaMalloc when they trace: their device memory
belongs to another runtime's pool (a framework that reserved the GPU's memory
up front, an engine with a fixed budget), or their loop must not allocate
because an allocation can synchronise the device.  This entry point keeps the
kernel's scratch (the work-queue head and the scenario table) in a static
device array instead of allocated memory.  Its results must be exactly those
of the allocating entry point, mr_batch_trace_device, bit for bit and call
after call: the array keeps the previous call's contents, so every case runs
two static calls in a row, and the second shows that the scratch is reset.

Cases: the scenario-table builds (two scenarios, and a scenario index past
the table), and the single-scenario builds (current on the bathymetry's
grid, on its own offset grid, constant), which read their scenario from the
kernel's parameters.  This file is collected last on purpose.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _static_call(L, tracer, ins, dt, steps, decimation, out, cfg, stream, scenario=None):
    n = int(ins[0].numel())
    return L.mr_batch_trace_device_static(
        tracer._h, n, scenario.data_ptr() if scenario is not None else None,
        *[t.data_ptr() for t in ins], 0.0, float(dt), int(steps), int(decimation),
        int(out.saved.shape[1]), out.saved.data_ptr() if out.saved.numel() else None,
        out.end_state.data_ptr(), out.n_steps.data_ptr(), out.n_saved.data_ptr(),
        out.status.data_ptr(), ctypes.byref(cfg), stream.cuda_stream)


def _bits(out):
    """The outputs as integer bit patterns (NaN payloads included)."""
    return [out.saved.cpu().numpy().view(np.uint32), out.end_state.cpu().numpy().view(np.uint64),
            out.n_steps.cpu().numpy(), out.n_saved.cpu().numpy(), out.status.cpu().numpy()]


def _check_static_equals_allocating(tracer, ins, dt, steps, dec, scenario=None):
    import torch

    from mantaray_gb300 import _native as N
    from mantaray_gb300.batch import BatchTracer, default_config

    L = N.load()
    n = int(ins[0].numel())
    cfg = default_config()
    stream = torch.cuda.current_stream()
    ref = tracer.trace(*ins, dt, steps, decimation=dec, scenario=scenario, config=cfg)
    torch.cuda.synchronize()
    expected = _bits(ref)
    assert np.any(expected[4] != 0) and np.any(expected[4] == 0)  # uneven lifetimes
    for _ in range(2):  # two calls in a row through the same static scratch
        out = BatchTracer.alloc(n, steps, dec)
        N.check(_static_call(L, tracer, ins, dt, steps, dec, out, cfg, stream, scenario))
        torch.cuda.synchronize()
        for got, exp in zip(_bits(out), expected):
            np.testing.assert_array_equal(got, exp)


def _small_fields(n=192, spacing=100.0, seed=5):
    """A 192^2 grid at 100 m: 3,000 m deep with a seeded shoal that dries at
    its top, and a vortex current."""
    rng = np.random.default_rng(seed)
    x = np.arange(n, dtype=np.float64) * spacing
    X, Y = x[None, :], x[:, None]
    cx, cy = rng.uniform(0.3, 0.7, 2) * x[-1]
    depth = 3000.0 - 3100.0 * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2.0 * 3000.0 ** 2))
    r2 = (X - x[-1] / 2) ** 2 + (Y - x[-1] / 2) ** 2
    g = 0.8 * np.exp(-r2 / (2.0 * 4000.0 ** 2))
    u = -(Y - x[-1] / 2) / 4000.0 * g
    v = (X - x[-1] / 2) / 4000.0 * g
    return x, depth, u, v


def _small_rays(x, n_rays, seed=6):
    import torch

    from mantaray_gb300.initial import wavenumber_vector

    rng = np.random.default_rng(seed)
    x0 = rng.uniform(0.05, 0.95, n_rays) * x[-1]
    y0 = rng.uniform(0.05, 0.95, n_rays) * x[-1]
    kx0, ky0 = wavenumber_vector(rng.uniform(8.0, 14.0, n_rays), np.full(n_rays, 3000.0),
                                 rng.uniform(0.0, 2.0 * np.pi, n_rays))
    return [torch.from_numpy(a).cuda() for a in (x0, y0, kx0, ky0)]


def test_static_entry_point_matches_the_allocating_one():
    import torch

    import mantaray_gb300 as mr
    from mantaray_gb300.batch import BatchTracer
    from mantaray_gb300.workloads import multi_source

    scenarios, rays = multi_source(n_sources=16, rays_per_source=256, n_scenarios=2, n=256,
                                   steps=400)
    fields = [(mr.Bathymetry.grid(s[0], s[1], s[2]), mr.Current.grid(s[3], s[4], s[5], s[6]))
              for s in scenarios]
    tracer = BatchTracer(fields)
    ins = [torch.from_numpy(rays[k]).cuda() for k in ("x0", "y0", "kx0", "ky0")]
    sid = torch.from_numpy(rays["scenario"]).cuda()
    _check_static_equals_allocating(tracer, ins, rays["dt"], 400, 40, sid)


def test_static_entry_point_scenario_index_past_the_table():
    # scenario indices >= the number of scenarios trace scenario 0, in both calls
    import torch

    import mantaray_gb300 as mr
    from mantaray_gb300.batch import BatchTracer

    x, depth, u, v = _small_fields()
    x2, depth2, u2, v2 = _small_fields(seed=9)
    xf = x.astype(np.float32)
    tracer = BatchTracer([(mr.Bathymetry.grid(xf, xf, depth), mr.Current.grid(x, x, u, v)),
                          (mr.Bathymetry.grid(xf, xf, depth2), mr.Current.grid(x, x, u2, v2))])
    ins = _small_rays(x, 2048)
    sid = torch.from_numpy(np.arange(2048, dtype=np.uint8) % 4).cuda()  # 2 and 3: past the table
    _check_static_equals_allocating(tracer, ins, 2.0, 600, 50, sid)


@pytest.mark.parametrize("current", ["same_grid", "own_grid", "constant"])
def test_static_entry_point_single_scenario_builds(current):
    import mantaray_gb300 as mr
    from mantaray_gb300.batch import BatchTracer

    x, depth, u, v = _small_fields()
    xf = x.astype(np.float32)
    b = mr.Bathymetry.grid(xf, xf, depth)
    if current == "same_grid":
        c = mr.Current.grid(x, x, u, v)
    elif current == "own_grid":
        xc = np.arange(160, dtype=np.float64) * 130.0 - 500.0  # offset, coarser, smaller grid
        Xc, Yc = xc[None, :], xc[:, None]
        c = mr.Current.grid(xc, xc, 0.3 * np.sin(Yc / 5000.0) + 0.0 * Xc,
                            0.2 * np.cos(Xc / 7000.0) + 0.0 * Yc)
    else:
        c = mr.Current.constant(0.4, -0.2)
    tracer = BatchTracer([(b, c)])
    _check_static_equals_allocating(tracer, _small_rays(x, 2048), 2.0, 600, 50)


def test_static_entry_point_refuses_pageable_outputs():
    # the kernel cannot write pageable host memory: refused before any work
    import torch

    import mantaray_gb300 as mr
    from mantaray_gb300 import _native as N
    from mantaray_gb300.batch import BatchResult, BatchTracer, default_config

    L = N.load()
    x, depth, u, v = _small_fields()
    xf = x.astype(np.float32)
    tracer = BatchTracer([(mr.Bathymetry.grid(xf, xf, depth), mr.Current.grid(x, x, u, v))])
    ins = _small_rays(x, 64)
    dev = BatchTracer.alloc(64, 10, 0)
    host = BatchResult(dev.saved, torch.empty((5, 64), dtype=torch.float64), dev.n_steps,
                       dev.n_saved, dev.status)
    rc = _static_call(L, tracer, ins, 2.0, 10, 0, host, default_config(),
                      torch.cuda.current_stream())
    assert rc == N.ERR_INVALID_ARGUMENT
    assert b"page-locked" in L.mr_last_error()


def test_static_entry_point_rejects_too_many_scenarios():
    import torch

    import mantaray_gb300 as mr
    from mantaray_gb300 import _native as N
    from mantaray_gb300.batch import BatchTracer, default_config

    L = N.load()
    x = np.arange(4, dtype=np.float32) * 10.0
    b = mr.Bathymetry.grid(x, x, np.full(16, 100.0))
    c = mr.Current.constant(0.0, 0.0)
    tracer = BatchTracer([(b, c)] * (N.BATCH_STATIC_MAX_SCENARIOS + 1))
    ins = [torch.full((8,), v, dtype=torch.float64, device="cuda") for v in (5.0, 5.0, 0.05, 0.0)]
    out = BatchTracer.alloc(8, 10, 0)
    rc = _static_call(L, tracer, ins, 1.0, 10, 0, out, default_config(),
                      torch.cuda.current_stream())
    assert rc == N.ERR_CAPACITY
    assert b"at most 64 scenarios" in L.mr_last_error()


def test_static_entry_point_rejects_ray_ordering():
    # ordering needs scratch memory: the static entry point refuses it
    import torch

    import mantaray_gb300 as mr
    from mantaray_gb300 import _native as N
    from mantaray_gb300.batch import BatchTracer, make_config

    L = N.load()
    x = np.arange(4, dtype=np.float32) * 10.0
    tracer = BatchTracer([(mr.Bathymetry.grid(x, x, np.full(16, 100.0)),
                           mr.Current.constant(0.0, 0.0))])
    ins = [torch.full((8,), v, dtype=torch.float64, device="cuda") for v in (5.0, 5.0, 0.05, 0.0)]
    out = BatchTracer.alloc(8, 10, 0)
    rc = _static_call(L, tracer, ins, 1.0, 10, 0, out, make_config(128, 4, 1, 32, 1),
                      torch.cuda.current_stream())
    assert rc == N.ERR_INVALID_ARGUMENT
    assert b"ordering" in L.mr_last_error()
