"""Batched FP32 form: millions of rays over several scenarios in one
persistent kernel, with CUDA-graph replay and a launch-shape autotuner.

Python face of the mr_batch_* entry points of include/mantaray_gpu.h.  Device
memory is torch CUDA tensors (plumbing only: the integration runs in the
library's own kernels).
"""

from __future__ import annotations

import ctypes
import itertools
import json
import os
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .fields import Bathymetry, Current


def _torch():
    import torch

    return torch


def default_config() -> N.BatchConfig:
    cfg = N.BatchConfig()
    N.check(N.load().mr_batch_default_config(ctypes.byref(cfg)))
    return cfg


def make_config(block=128, blocks_per_sm=4, rays_per_lane=1, rebase_interval=32,
                order=0, staging=0, sweep_steps=0) -> N.BatchConfig:
    return N.BatchConfig(block, blocks_per_sm, rays_per_lane, rebase_interval, order, staging,
                         sweep_steps)


@dataclass
class BatchResult:
    """Outputs of one batched call: torch CUDA tensors, or page-locked CPU
    tensors (`pin_memory()`), which the kernel writes in place."""

    saved: object       # [5][save_cap][n] f32 (t, x, y, kx, ky), NaN past each ray's rows
    end_state: object   # [5][n] f64 last valid state
    n_steps: object     # [n] int32
    n_saved: object     # [n] int32
    status: object      # [n] uint8 (MR_BATCH_*)


class BatchTracer:
    """Rays over a list of (bathymetry, current) scenarios in FP32."""

    def __init__(self, scenarios):
        L = N.load()
        self._fields = list(scenarios)  # keep the field handles alive
        n = len(self._fields)
        bs = (ctypes.c_void_p * n)(*[b.handle.value for b, _ in self._fields])
        cs = (ctypes.c_void_p * n)(*[c.handle.value for _, c in self._fields])
        out = ctypes.c_void_p()
        N.check(L.mr_batch_create(n, bs, cs, ctypes.byref(out)))
        self._h = out
        self.n_scenarios = n
        self._staging = {}

    def supports(self, staging: int) -> bool:
        """Whether mr_batch_config.staging = `staging` is accepted for this
        batch (tried once per value with a call of no rays, which checks the
        configuration and traces nothing): tiles need one scenario with its
        current gridded on the bathymetry's grid, staging ahead every
        scenario's current on its bathymetry's grid."""
        if staging not in self._staging:
            torch = _torch()
            z = torch.empty(0, dtype=torch.float64, device="cuda")
            out = self.alloc(0, 1, 0, device="cuda")
            rc = N.load().mr_batch_trace_device(
                self._h, 0, None, z.data_ptr(), z.data_ptr(), z.data_ptr(), z.data_ptr(), 0.0,
                1.0, 1, 0, 0, None, out.end_state.data_ptr(), out.n_steps.data_ptr(),
                out.n_saved.data_ptr(), out.status.data_ptr(),
                ctypes.byref(make_config(128, 4, 1, 32, 0, staging)), None)
            self._staging[staging] = rc == N.OK
        return self._staging[staging]

    @property
    def tiles_supported(self) -> bool:
        return self.supports(N.STAGING_TILE)

    def close(self):
        if self._h and self._h.value:
            N.load().mr_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    @staticmethod
    def alloc(n, max_steps, decimation, device="cuda"):
        torch = _torch()
        save_cap = (max_steps // decimation + 1) if decimation > 0 else 0
        return BatchResult(
            saved=torch.empty((5, save_cap, n), dtype=torch.float32, device=device)
            if save_cap else torch.empty((5, 0, n), dtype=torch.float32, device=device),
            end_state=torch.empty((5, n), dtype=torch.float64, device=device),
            n_steps=torch.empty(n, dtype=torch.int32, device=device),
            n_saved=torch.empty(n, dtype=torch.int32, device=device),
            status=torch.empty(n, dtype=torch.uint8, device=device))

    def trace(self, x0, y0, kx0, ky0, dt, max_steps, t0=0.0, decimation=0, scenario=None,
              config=None, out: BatchResult | None = None, stream=None) -> BatchResult:
        """Traces the rays (float64 CUDA tensors) asynchronously on `stream`."""
        torch = _torch()
        n = int(x0.numel())
        cfg = config or default_config()
        if out is None:
            out = self.alloc(n, max_steps, decimation, device=x0.device)
        if stream is None:
            stream = torch.cuda.current_stream(x0.device)
        sp = scenario.data_ptr() if scenario is not None else None
        N.check(N.load().mr_batch_trace_device(
            self._h, n, sp, x0.data_ptr(), y0.data_ptr(), kx0.data_ptr(), ky0.data_ptr(),
            float(t0), float(dt), int(max_steps), int(decimation), int(out.saved.shape[1]),
            out.saved.data_ptr() if out.saved.numel() else None, out.end_state.data_ptr(),
            out.n_steps.data_ptr(), out.n_saved.data_ptr(), out.status.data_ptr(),
            ctypes.byref(cfg), getattr(stream, "cuda_stream", stream)))
        return out

    def graph(self, x0, y0, kx0, ky0, dt, max_steps, t0=0.0, decimation=0, scenario=None,
              config=None) -> "BatchGraph":
        """Captures the call in a CUDA graph over buffers for x0.numel() rays."""
        return BatchGraph(self, x0, y0, kx0, ky0, dt, max_steps, t0, decimation, scenario,
                          config or default_config())

    def autotune(self, x0, y0, kx0, ky0, dt, probe_steps, t0=0.0, scenario=None,
                 candidates=None, repeats=2, cache_key=None, long_steps=None,
                 long_rays=None, finalists=4, sweeps=(96, 128),
                 probe_rays=None, final_rays=None, final_steps=None,
                 final_count=3) -> N.BatchConfig:
        """Times every candidate launch shape on a probe run (the first
        `probe_rays` of the given rays, default all, for `probe_steps` steps,
        endpoints only) and returns the fastest.
        With `long_steps`, the `finalists` fastest are timed again on the
        first `long_rays` rays for `long_steps` steps, once each, and the
        fastest of that run wins: a short probe keeps the rays near their
        starts, where the fields they read may fit in L2, while a long trace
        spreads them over the whole field.  There the four fastest ordered
        one-ray finalists (or the fastest such candidate, if no finalist is
        one) are also timed in sweeps of each length in `sweeps`, a form that
        only pays once the rays have spread.  With `final_steps`, the
        `final_count` fastest of that stage are timed once more on the first
        `final_rays` rays for `final_steps` steps (the workload itself), and
        the fastest there wins.  Results are cached in memory and in
        $MANTARAY_TUNE_CACHE (a JSON file) when that is set."""
        torch = _torch()
        key = cache_key
        cache_path = os.environ.get("MANTARAY_TUNE_CACHE")
        if key and key in _TUNE_CACHE:
            return make_config(**_TUNE_CACHE[key])
        if key and cache_path and os.path.exists(cache_path):
            stored = json.load(open(cache_path))
            if key in stored:
                _TUNE_CACHE[key] = stored[key]
                return make_config(**stored[key])
        if candidates is None:
            candidates = [make_config(b, bps, rpl, 32, order)
                          for b, bps, rpl, order in itertools.product((64, 128, 256),
                                                                      (2, 4, 6, 8, 12),
                                                                      (1, 2), (0, 1))
                          if b * bps <= 2048]
            # staged cell records (one ray per lane): shared-memory tiles
            # (ordered rays), records loaded ahead
            for staging, orders in ((N.STAGING_TILE, (1,)), (N.STAGING_AHEAD, (0, 1))):
                if self.supports(staging):
                    candidates += [make_config(b, bps, 1, 32, order, staging)
                                   for b, bps, order in itertools.product(
                                       (64, 128, 256), (2, 4, 6, 8, 12), orders)
                                   if b * bps <= 2048]
        stream = torch.cuda.current_stream(x0.device)

        def timed(cfg, rays, steps, reps, out):
            self.trace(*rays, dt, steps, t0, 0, sc(rays), cfg, out, stream)
            ts = []
            for _ in range(reps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                self.trace(*rays, dt, steps, t0, 0, sc(rays), cfg, out, stream)
                e1.record(stream)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            return min(ts)

        def sc(rays):
            return None if scenario is None else scenario[: rays[0].numel()]

        p = int(min(x0.numel(), probe_rays or x0.numel()))
        rays = tuple(t[:p] for t in (x0, y0, kx0, ky0))
        out = self.alloc(p, probe_steps, 0, device=x0.device)
        ranked = sorted((timed(cfg, rays, probe_steps, repeats, out), i)
                        for i, cfg in enumerate(candidates))
        best = candidates[ranked[0][1]]
        if long_steps:
            m = int(min(x0.numel(), long_rays or x0.numel()))
            rays = tuple(t[:m] for t in (x0, y0, kx0, ky0))
            out = self.alloc(m, long_steps, 0, device=x0.device)
            finals = [candidates[i] for _, i in ranked[:finalists]]

            def sweepable(c):
                return c.order == 1 and c.rays_per_lane == 1 and c.staging == 0 and \
                    c.sweep_steps == 0

            bases = [c for c in finals if sweepable(c)][:4]
            if not bases:
                bases = [candidates[i] for _, i in ranked if sweepable(candidates[i])][:1]
            finals += [make_config(**dict(c.as_dict(), sweep_steps=sw))
                       for c in bases for sw in sweeps if 0 < sw < long_steps]
            ranked_long = sorted(((timed(cfg, rays, long_steps, 1, out), i)
                                  for i, cfg in enumerate(finals)), key=lambda t: t[0])
            best = finals[ranked_long[0][1]]
            if final_steps:
                f = int(min(x0.numel(), final_rays or x0.numel()))
                rays = tuple(t[:f] for t in (x0, y0, kx0, ky0))
                del out
                out = self.alloc(f, final_steps, 0, device=x0.device)
                last = [finals[i] for _, i in ranked_long[:final_count]]
                best = min(last, key=lambda cfg: timed(cfg, rays, final_steps, 1, out))
        if key:
            _TUNE_CACHE[key] = best.as_dict()
            if cache_path:
                stored = json.load(open(cache_path)) if os.path.exists(cache_path) else {}
                stored[key] = best.as_dict()
                json.dump(stored, open(cache_path, "w"), indent=1)
        return best


    def tune_decimation(self, x0, y0, kx0, ky0, dt, max_steps, choices, max_saved_bytes,
                        probe_steps=None, t0=0.0, scenario=None, config=None, slowdown=1.05,
                        repeats=2):
        """Output decimation: the finest of `choices` (steps between stored
        rows) whose stored rows for these rays over max_steps fit in
        max_saved_bytes and whose probe run (`probe_steps`, default
        min(max_steps, 1,000)) takes at most `slowdown` times the coarsest
        fitting choice's.  Returns (decimation, {decimation: probe ms}); raises
        ValueError when no choice fits."""
        torch = _torch()
        n = int(x0.numel())
        fits = sorted(d for d in choices
                      if d > 0 and 5 * 4 * n * (max_steps // d + 1) <= max_saved_bytes)
        if not fits:
            raise ValueError("no decimation in `choices` fits max_saved_bytes")
        probe = min(max_steps, 1000) if probe_steps is None else probe_steps
        cfg = config or default_config()
        stream = torch.cuda.current_stream(x0.device)
        times = {}
        for d in fits:
            out = self.alloc(n, probe, d, device=x0.device)
            self.trace(x0, y0, kx0, ky0, dt, probe, t0, d, scenario, cfg, out, stream)
            ts = []
            for _ in range(repeats):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                self.trace(x0, y0, kx0, ky0, dt, probe, t0, d, scenario, cfg, out, stream)
                e1.record(stream)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            times[d] = min(ts)
            del out
        limit = slowdown * times[fits[-1]]
        return next(d for d in fits if times[d] <= limit), times


_TUNE_CACHE: dict = {}


class BatchGraph:
    """A batched call captured once and replayed for any n <= capacity."""

    def __init__(self, tracer, x0, y0, kx0, ky0, dt, max_steps, t0, decimation, scenario, cfg):
        self.tracer = tracer
        self.n_max = int(x0.numel())
        self.inputs = (x0, y0, kx0, ky0, scenario)  # kept alive: the graph reads them
        self.out = tracer.alloc(self.n_max, max_steps, decimation, device=x0.device)
        self.cfg = cfg
        g = ctypes.c_void_p()
        o = self.out
        N.check(N.load().mr_batch_graph_create(
            tracer._h, self.n_max, scenario.data_ptr() if scenario is not None else None,
            x0.data_ptr(), y0.data_ptr(), kx0.data_ptr(), ky0.data_ptr(), float(t0), float(dt),
            int(max_steps), int(decimation), int(o.saved.shape[1]),
            o.saved.data_ptr() if o.saved.numel() else None, o.end_state.data_ptr(),
            o.n_steps.data_ptr(), o.n_saved.data_ptr(), o.status.data_ptr(), ctypes.byref(cfg),
            ctypes.byref(g)))
        self._g = g

    def launch(self, n=None, stream=None):
        torch = _torch()
        n = self.n_max if n is None else int(n)
        if stream is None:
            stream = torch.cuda.current_stream(self.inputs[0].device)
        N.check(N.load().mr_batch_graph_launch(self._g, n, getattr(stream, "cuda_stream", stream)))

    def close(self):
        if self._g and self._g.value:
            N.load().mr_batch_graph_destroy(self._g)
            self._g = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def endpoint_errors(end_state, n_steps, oracle_traj, oracle_rows, per_ray=False):
    """Endpoint error of batched results against full-precision trajectories
    (traj[5][rows][n], e.g. the plain FP64 form's) at the batched form's last
    valid step: relative position error |dx| / path length (path length along
    the full-precision trajectory up to that step) and direction error
    |d theta| (rad).  Rays that the batched form carried past the
    full-precision trajectory's last finite row are counted, not compared.
    per_ray: the error arrays hold every ray, NaN where not compared."""
    end = np.asarray(end_state)
    steps = np.asarray(n_steps).astype(np.int64)
    n = end.shape[1]
    rows = np.asarray(oracle_rows).astype(np.int64)
    traj = np.asarray(oracle_traj)
    idx = np.arange(n)
    last_ok = np.all(np.isfinite(traj[1:, rows - 1, idx]), axis=0)
    last_finite = np.where(last_ok, rows - 1, rows - 2)
    cmp = steps <= last_finite
    row = np.where(cmp, steps, 0)
    ox, oy = traj[1, row, idx], traj[2, row, idx]
    okx, oky = traj[3, row, idx], traj[4, row, idx]
    dxy = np.hypot(end[1] - ox, end[2] - oy)
    seg = np.hypot(np.diff(traj[1], axis=0), np.diff(traj[2], axis=0))
    seg = np.where(np.arange(seg.shape[0])[:, None] < row[None, :], seg, 0.0)
    path = np.nansum(seg, axis=0)
    rel = np.where(path > 0, dxy / np.maximum(path, 1e-300), 0.0)
    dth = np.abs(np.angle(np.exp(1j * (np.arctan2(end[4], end[3]) - np.arctan2(oky, okx)))))
    if per_ray:
        rel, dth = np.where(cmp, rel, np.nan), np.where(cmp, dth, np.nan)
    else:
        rel, dth = rel[cmp], dth[cmp]
    return {"rel_position": rel, "direction": dth, "compared": int(np.sum(cmp)),
            "past_end": int(np.sum(~cmp)), "early_stop": int(np.sum(steps < last_finite)),
            "n": n}
