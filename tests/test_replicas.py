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


def split_worker(rank, world, port, out):
    """one view's samples split across ranks, sums all-reduced; the adjoint's
    gradients of each rank's share all-reduced"""
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        S = OL.PKG.scenes
        sc = S.scene_tiny(res=16, film=(12, 10), seed=3)
        first, count = R.split_samples(6, rank, world)
        h = OL.SceneHandle(OL.load_oracle(), sc)
        part = torch.from_numpy(h.render_sum(count, view=0, first=first, nthreads=1).astype(np.float64))
        h.close()
        R.sum_over_ranks(part, dist)
        # differentiable medium: each rank's samples, gradients summed
        res, n = (12, 12, 12), 12
        rho = S.blob_density(res, n_blobs=3, seed=5)
        tf = S.ramp_opacity(n)
        maj = S.spline_majorant(rho, tf, 30.0, brick=4)
        msc = S.medium_scene(res=res, film=(10, 8))
        mh = OL.MediumHandle(OL.load_oracle(), msc, rho, tf, 30.0, np.array([0.8, 0.8, 0.8]), 0.5, maj, 4)
        img, smp = mh.render(count, first=first, keep_samples=True, nthreads=1)
        dimg = np.ones_like(img) * 1e-2
        g_rho, g_tf = mh.adjoint(count, dimg, smp, first=first, nthreads=1)
        mh.close()
        g = torch.from_numpy(np.concatenate([g_rho.ravel(), g_tf]).astype(np.float64))
        R.sum_over_ranks(g, dist)
        out[rank] = (part.numpy(), g.numpy())
    finally:
        dist.destroy_process_group()


def test_split_samples_and_reduce():
    """the exchange step of a split view: rank shares of the sample stream
    sum to the one-process render (up to float re-association), and the
    shares' adjoint gradients sum to the whole adjoint"""
    assert [R.split_samples(7, r, 3) for r in range(3)] == [(0, 3), (3, 2), (5, 2)]
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(split_worker, args=(world, free_port(), out), nprocs=world, start_method="spawn", join=True)
    (img0, g0), (img1, g1) = out[0], out[1]
    assert np.array_equal(img0, img1) and np.array_equal(g0, g1)
    S = OL.PKG.scenes
    sc = S.scene_tiny(res=16, film=(12, 10), seed=3)
    h = OL.SceneHandle(OL.load_oracle(), sc)
    whole = h.render_sum(6, view=0, first=0, nthreads=1).astype(np.float64)
    h.close()
    assert np.allclose(img0, whole, rtol=1e-5, atol=1e-6)
    res, n = (12, 12, 12), 12
    rho = S.blob_density(res, n_blobs=3, seed=5)
    tf = S.ramp_opacity(n)
    maj = S.spline_majorant(rho, tf, 30.0, brick=4)
    mh = OL.MediumHandle(OL.load_oracle(), S.medium_scene(res=res, film=(10, 8)), rho, tf, 30.0, np.array([0.8, 0.8, 0.8]), 0.5,
                         maj, 4)
    img, smp = mh.render(6, keep_samples=True, nthreads=1)
    g_rho, g_tf = mh.adjoint(6, np.ones_like(img) * 1e-2, smp, nthreads=1)
    mh.close()
    g = np.concatenate([g_rho.ravel(), g_tf]).astype(np.float64)
    assert np.allclose(g0, g, rtol=1e-4, atol=1e-6 * np.abs(g).max())


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
