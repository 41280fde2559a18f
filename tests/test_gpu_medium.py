"""Differentiable medium on the GPU (er_medium_*, medium.py): forward samples
bit-exact with the CPU oracle, the path-replay adjoint against the oracle's
adjoint and against central finite differences (h = 1e-3) of the binary64
evaluation of the same samples, at the differentiable workload's size (128^3
density, 64 opacity values, 256^2 x 32 spp)."""
import importlib

import numpy as np
import pytest

import oracle_lib as OL

pytestmark = pytest.mark.gpu

C = OL.C
S = OL.PKG.scenes
ALB = (0.8, 0.7, 0.6)


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def torch():
    import torch as T
    assert T.cuda.is_available(), "GPU tests need CUDA"
    return T


@pytest.fixture(scope="module")
def lib(torch):
    L = C.load_library()
    C.check(L.er_set_device(0))
    yield L
    L.er_reset()


@pytest.fixture(scope="module")
def pkg():
    return importlib.import_module("exposure-render_gb300.runtime"), importlib.import_module("exposure-render_gb300.medium")


def make(torch, lib, pkg, res, n, film, scale, brick, seed=3, blobs=4):
    runtime, medium = pkg
    sc = S.medium_scene(res=res, film=film)
    r = runtime.Renderer(sc, lib)
    rho = torch.from_numpy(S.blob_density(res, n_blobs=blobs, seed=seed)).cuda()
    tf = torch.from_numpy(S.ramp_opacity(n)).cuda()
    m = medium.Medium(r, rho, tf, scale, albedo=ALB, nee_probability=0.5, brick=brick)
    return sc, r, m, rho, tf


def test_forward_bit_exact_and_adjoint_matches_oracle(torch, lib, pkg, oracle):
    sc, r, m, rho, tf = make(torch, lib, pkg, (16, 16, 16), 16, (24, 20), 30.0, 4)
    try:
        spp = 4
        smp, s = m.render_samples(rho, tf, spp)
        torch.cuda.synchronize()
        maj = m.majorant.cpu().numpy()
        h = OL.MediumHandle(oracle, sc, rho.cpu().numpy(), tf.cpu().numpy(), 30.0, np.array(ALB), 0.5, maj, 4)
        ref_sum, ref_smp = h.render(spp, keep_samples=True, nthreads=4)
        assert np.array_equal(bits(smp.cpu().numpy()), bits(ref_smp))
        assert np.array_equal(bits(s.cpu().numpy()), bits(ref_sum))
        rng = np.random.default_rng(2)
        dimg = rng.normal(size=ref_sum.shape).astype(np.float32)
        g_rho, g_tf = m.adjoint(rho, tf, spp, torch.from_numpy(dimg).cuda(), smp)
        o_rho, o_tf = h.adjoint(spp, dimg, ref_smp, nthreads=4)
        h.close()
        # same terms, summed in another order (atomics vs per-thread buffers)
        assert np.allclose(g_tf.cpu().numpy(), o_tf, rtol=1e-4, atol=1e-5 * np.abs(o_tf).max())
        assert np.allclose(g_rho.cpu().numpy(), o_rho, rtol=1e-4, atol=1e-5 * np.abs(o_rho).max())
        # recomputing each sample instead of reading it gives the same gradients
        r_rho, r_tf = m.adjoint(rho, tf, spp, torch.from_numpy(dimg).cuda(), None)
        assert torch.allclose(r_tf, g_tf, rtol=1e-5, atol=1e-6 * float(g_tf.abs().max()))
        assert torch.allclose(r_rho, g_rho, rtol=1e-5, atol=1e-6 * float(g_rho.abs().max()))
    finally:
        r.close()


def test_autograd_function(torch, lib, pkg):
    sc, r, m, rho, tf = make(torch, lib, pkg, (16, 16, 16), 16, (24, 20), 30.0, 4)
    try:
        spp = 4
        target = torch.full((r.height, r.width, 3), 0.02, device="cuda")
        rho_p = rho.clone().requires_grad_(True)
        tf_p = tf.clone().requires_grad_(True)
        img = m(rho_p, tf_p, spp)
        loss = ((img - target) ** 2).sum()
        loss.backward()
        smp, s = m.render_samples(rho, tf, spp)
        dsum = 2.0 * (s / spp - target) / spp
        g_rho, g_tf = m.adjoint(rho, tf, spp, dsum, smp)
        # two walks of the same samples: the gradients agree up to the order
        # of the atomic sums (a density entry that sums terms of both signs
        # keeps ~1e-7 of the largest gradient from that order)
        assert torch.allclose(tf_p.grad, g_tf, rtol=1e-5, atol=1e-6 * float(g_tf.abs().max()))
        assert torch.allclose(rho_p.grad, g_rho, rtol=1e-5, atol=1e-6 * float(g_rho.abs().max()))
    finally:
        r.close()


def test_binary64_evaluation_tracks_float(torch, lib, pkg):
    sc, r, m, rho, tf = make(torch, lib, pkg, (16, 16, 16), 16, (24, 20), 30.0, 4)
    try:
        s64 = m.render_sums64(rho, tf, 4)
        _, s32 = m.render_samples(rho, tf, 4)
        assert torch.allclose(s64.float(), s32, rtol=1e-4, atol=1e-6)
    finally:
        r.close()


def test_c4_adjoint_matches_finite_differences(torch, lib, pkg):
    """128^3 density, 64 opacity values, 256^2 x 32 spp; target rendered at
    1024 spp from parameters perturbed by N(0, 0.05); 32 random parameters
    (up to 16 opacity values the image depends on, the rest voxels)"""
    res, n, scale, spp = (128, 128, 128), 64, 40.0, 32
    sc, r, m, rho, tf = make(torch, lib, pkg, res, n, (256, 256), scale, 8, seed=40, blobs=10)
    try:
        gen = torch.Generator(device="cuda").manual_seed(7)
        rho_t = rho + 0.05 * torch.randn(rho.shape, device="cuda", generator=gen)
        tf_t = tf + 0.05 * torch.randn(tf.shape, device="cuda", generator=gen)
        # one majorant that bounds both parameter sets
        maj0 = m.majorant.clone()
        m.rebuild_majorant(rho_t.contiguous(), tf_t.contiguous())
        m.majorant = torch.maximum(maj0, m.majorant).contiguous()
        _, ts = m.render_samples(rho_t.contiguous(), tf_t.contiguous(), 1024, view=1)
        target = (ts / 1024).double()

        def loss64(rh, t):
            s = m.render_sums64(rh, t, spp)
            return float(((s / spp - target) ** 2).mean())

        smp, s = m.render_samples(rho, tf, spp)
        dsum = 2.0 * (s.double() / spp - target) / spp / target.numel()
        g_rho, g_tf = m.adjoint(rho, tf, spp, dsum.float(), smp)
        C.check(lib.er_synchronize())
        # 32 parameters drawn uniformly among those the loss depends on (a
        # non-zero gradient, however small): up to 16 opacity values, the rest
        # voxels.  The error is relative to the finite difference, with a floor
        # of 1e-4 of the largest gradient of the parameter's kind (float
        # atomics sum many samples' contributions, which cancel in the
        # smallest gradients)
        rng = np.random.default_rng(11)
        gt = g_tf.cpu().numpy()
        live_tf = np.flatnonzero(gt != 0.0)
        tf_idx = rng.choice(live_tf, min(16, len(live_tf)), replace=False)
        gr = g_rho.cpu().numpy().ravel()
        rho_idx = rng.choice(np.flatnonzero(gr != 0.0), 32 - len(tf_idx), replace=False)
        floor = {"tf": 1e-4 * float(np.abs(gt).max()), "rho": 1e-4 * float(np.abs(gr).max())}
        h = 1e-3
        worst = 0.0
        for kind, idx in [("tf", i) for i in tf_idx] + [("rho", i) for i in rho_idx]:
            base = tf if kind == "tf" else rho
            p, q = base.clone(), base.clone()
            p.view(-1)[idx] += h
            q.view(-1)[idx] -= h
            if kind == "tf":
                fd = (loss64(rho, p) - loss64(rho, q)) / (2 * h)
                adj = float(gt[idx])
            else:
                fd = (loss64(p, tf) - loss64(q, tf)) / (2 * h)
                adj = float(gr[idx])
            rel = abs(adj - fd) / max(abs(fd), floor[kind])
            worst = max(worst, rel)
            assert rel <= 1e-3, (kind, int(idx), adj, fd, rel)
        print(f"worst relative error over 32 parameters: {worst:.2e}")
    finally:
        r.close()
