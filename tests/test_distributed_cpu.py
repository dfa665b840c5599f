"""The multi-GPU host logic on CPU: two gloo ranks each trace their shard of
the rays with the oracle and gather; the result must equal one trace of all
rays, and the timing reductions must be the max / sum over ranks."""

import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist

    from mantaray_gb300 import distributed as D
    from mantaray_gb300.workloads import planar_beach
    from oracle import pyoracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = planar_beach(n_rays=37)
        a, b = D.shard_range(w.n, rank, world)
        ob = pyoracle.Bathymetry.grid(w.bx, w.by, w.depth)
        oc = pyoracle.Current.grid(w.cx, w.cy, w.u, w.v)
        traj, rows, _ = pyoracle.trace(ob, oc, w.x0[a:b], w.y0[a:b], w.kx0[a:b], w.ky0[a:b],
                                       w.t0, w.t0 + 50.0, w.dt, threads=1)
        full = D.gather_rays(traj, w.n)
        full_rows = D.gather_rays(rows.astype(np.float64)[None, :], w.n)
        t_max = D.reduce_scalar(float(rank + 1), "max")
        total = D.reduce_scalar(float(b - a), "sum")
        # node gradients of each rank's shard summed over ranks (in place)
        import torch

        g = torch.full((3, 4), float(rank + 1), dtype=torch.float64)
        D.allreduce_node_gradients(g)
        assert bool((g == 3.0).all())
        if rank == 0:
            np.savez(out_path, traj=full, rows=full_rows, t_max=t_max, total=total)
        else:
            assert full is None
    finally:
        dist.destroy_process_group()


def test_shard_range_partitions():
    from mantaray_gb300.distributed import shard_range

    for n in (0, 1, 7, 64, 1001):
        for world in (1, 2, 3, 8):
            spans = [shard_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def test_two_gloo_ranks_gather_the_full_trace(tmp_path, oracle):
    import torch.multiprocessing as mp

    from mantaray_gb300.workloads import planar_beach

    out = str(tmp_path / "gathered.npz")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(out)
    w = planar_beach(n_rays=37)
    ob = oracle.Bathymetry.grid(w.bx, w.by, w.depth)
    oc = oracle.Current.grid(w.cx, w.cy, w.u, w.v)
    traj, rows, _ = oracle.trace(ob, oc, w.x0, w.y0, w.kx0, w.ky0, w.t0, w.t0 + 50.0, w.dt)
    np.testing.assert_array_equal(np.nan_to_num(got["traj"], nan=-9.0),
                                  np.nan_to_num(traj, nan=-9.0))
    np.testing.assert_array_equal(got["rows"][0], rows)
    assert float(got["t_max"]) == 2.0 and float(got["total"]) == 37.0
