"""The N > 1 path on CPU: two gloo ranks (127.0.0.1) agree on the slowest
rank's timing, render independent replica views (the CPU oracle stands in
for the GPU kernels here), and report the whole job's rate."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import oracle_lib as OL

R = __import__("importlib").import_module("exposure-render_gb300.replicas")


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, lr = R.rank_info()
        assert (r, w, lr) == (rank, world, rank)
        # each rank renders its own view: the tiny scene with the rank's seed
        sc = OL.PKG.scenes.scene_tiny(res=16, film=(12, 10), seed=3)
        sc.tracer.settings.seed = R.view_seed(1, rank)
        h = OL.SceneHandle(OL.load_oracle(), sc)
        img = h.render_sum(2, view=rank, nthreads=1)
        h.close()
        local_ms = 10.0 * (rank + 1)                 # a stand-in timing, slower on rank 1
        R.barrier(dist)
        ms = R.max_over_ranks(local_ms, dist, device="cpu")
        rate = R.whole_job_rate(12 * 10 * 2, ms / 1e3, world)
        sums = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
        dist.all_gather(sums, torch.tensor([float(img.astype(np.float64).sum())], dtype=torch.float64))
        out[rank] = (ms, rate, [float(t.item()) for t in sums])
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(worker, args=(world, free_port(), out), nprocs=world, start_method="spawn", join=True)
    (ms0, rate0, sums0), (ms1, rate1, sums1) = out[0], out[1]
    assert ms0 == ms1 == 20.0                          # both ranks report the slowest
    assert rate0 == rate1 == pytest.approx(2 * 240 / 0.020)
    assert sums0 == sums1 and sums0[0] != sums0[1]    # independent replica views


def test_single_process_identities():
    assert R.max_over_ranks(3.5, None) == 3.5
    assert R.whole_job_rate(100.0, 2.0, 1) == 50.0
    assert R.view_seed(1, 0) == 1 and R.view_seed(1, 3) == 4
