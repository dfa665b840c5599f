"""The allocation-free batched entry point, mr_batch_trace_device_static.

It serves callers that cannot call cudaMalloc when they trace -- their
device memory is owned by another runtime's pool, or their loop must not
allocate -- by keeping the kernel's scratch (work-queue head, scenario table)
in a static device array instead of allocated memory.  Its results must be
exactly those of the allocating entry point, mr_batch_trace_device, call
after call (the array keeps the previous call's contents, so the second call
checks that it is reset).  This file is collected last on purpose.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _nan_equal(a, b):
    np.testing.assert_array_equal(np.nan_to_num(a, nan=-7.0), np.nan_to_num(b, nan=-7.0))


def _static_call(L, N, tracer, ins, dt, steps, decimation, out, cfg, stream, scenario=None):
    n = int(ins[0].numel())
    return L.mr_batch_trace_device_static(
        tracer._h, n, scenario.data_ptr() if scenario is not None else None,
        *[t.data_ptr() for t in ins], 0.0, float(dt), int(steps), int(decimation),
        int(out.saved.shape[1]), out.saved.data_ptr() if out.saved.numel() else None,
        out.end_state.data_ptr(), out.n_steps.data_ptr(), out.n_saved.data_ptr(),
        out.status.data_ptr(), ctypes.byref(cfg), stream.cuda_stream)


def test_static_entry_point_matches_the_allocating_one():
    import torch

    import mantaray_gb300 as mr
    from mantaray_gb300 import _native as N
    from mantaray_gb300.batch import BatchTracer, default_config
    from mantaray_gb300.workloads import multi_source

    L = N.load()
    scenarios, rays = multi_source(n_sources=16, rays_per_source=256, n_scenarios=2, n=256,
                                   steps=400)
    fields = [(mr.Bathymetry.grid(s[0], s[1], s[2]), mr.Current.grid(s[3], s[4], s[5], s[6]))
              for s in scenarios]
    tracer = BatchTracer(fields)
    ins = [torch.from_numpy(rays[k]).cuda() for k in ("x0", "y0", "kx0", "ky0")]
    sid = torch.from_numpy(rays["scenario"]).cuda()
    n = int(ins[0].numel())
    steps, dec, dt = 400, 40, rays["dt"]
    cfg = default_config()
    stream = torch.cuda.current_stream()
    ref = tracer.trace(*ins, dt, steps, decimation=dec, scenario=sid, config=cfg)
    torch.cuda.synchronize()
    expected = [t.cpu().numpy() for t in (ref.saved, ref.end_state, ref.n_steps, ref.n_saved,
                                          ref.status)]
    assert np.any(expected[4] != 0) and np.any(expected[4] == 0)  # uneven lifetimes
    for _ in range(2):  # two calls in a row through the same static scratch
        out = BatchTracer.alloc(n, steps, dec)
        N.check(_static_call(L, N, tracer, ins, dt, steps, dec, out, cfg, stream, sid))
        torch.cuda.synchronize()
        got = [t.cpu().numpy() for t in (out.saved, out.end_state, out.n_steps, out.n_saved,
                                         out.status)]
        for a, b in zip(got, expected):
            _nan_equal(a, b)


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
    rc = _static_call(L, N, tracer, ins, 1.0, 10, 0, out, default_config(),
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
    rc = _static_call(L, N, tracer, ins, 1.0, 10, 0, out, make_config(128, 4, 1, 32, 1),
                      torch.cuda.current_stream())
    assert rc == N.ERR_INVALID_ARGUMENT
    assert b"ordering" in L.mr_last_error()
