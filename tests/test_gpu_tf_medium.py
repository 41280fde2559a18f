"""The differentiable tracer model (er_medium_* with ER_MEDIUM_TRACER) on
the GPU: the bound tracer's opacity PLF (node values as parameters), its
diffuse / specular / glossiness / emission transfer functions over a float
intensity grid, and its BRDF / phase / hybrid shading.  Forward samples
bit-exact with the CPU oracle; the path-replay adjoint against the oracle's
adjoint, against central differences of the GPU's binary64 evaluation at the
differentiable workload's size (128^3 grid, 64-node opacity, 256^2 x 32
spp), and through torch.autograd; and the estimator's converged image
against the product's own (delta tracking, stochastic hybrid choice, full
MIS) on the same scene."""
import importlib

import numpy as np
import pytest

import oracle_lib as OL

pytestmark = pytest.mark.gpu

C = OL.C
S = OL.PKG.scenes


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


def make(torch, lib, pkg, res, n, film, scale, brick, shading=C.SHADING_HYBRID, seed=3, blobs=4, emission=0.8, q=0.5):
    runtime, medium = pkg
    sc = S.tf_medium_scene(res=res, film=film, n_nodes=n, shading=shading, emission=emission)
    r = runtime.Renderer(sc, lib)
    rho_np = S.blob_density(res, n_blobs=blobs, seed=seed)
    rho = torch.from_numpy(rho_np).cuda()
    vals = torch.from_numpy(S.plf_node_values(sc.tracer.opacity)).cuda()
    m = medium.Medium(r, rho, vals, scale, nee_probability=q, brick=brick, model="tracer",
                      gradient_magnitude_inv=S.gradient_magnitude_range(rho_np))
    return sc, r, m, rho, vals


@pytest.mark.parametrize("shading", [C.SHADING_BRDF_ONLY, C.SHADING_PHASE_ONLY, C.SHADING_HYBRID])
def test_forward_bit_exact_and_adjoint_matches_oracle(torch, lib, pkg, oracle, shading):
    sc, r, m, rho, vals = make(torch, lib, pkg, (16, 16, 16), 12, (24, 20), 30.0, 4, shading=shading)
    try:
        spp = 4
        smp, s = m.render_samples(rho, vals, spp)
        torch.cuda.synchronize()
        maj = m.majorant.cpu().numpy()
        # the same bound up to float rounding (the GPU sums in float, numpy in double)
        assert np.allclose(maj, S.plf_majorant(rho.cpu().numpy(), sc.tracer.opacity, vals.cpu().numpy(), 30.0, brick=4), rtol=1e-6)
        h = OL.MediumHandle(oracle, sc, rho.cpu().numpy(), vals.cpu().numpy(), 30.0, np.array([0.8, 0.8, 0.8]), 0.5, maj, 4,
                            model=1, gm_inv=m.gm_inv)
        ref_sum, ref_smp = h.render(spp, keep_samples=True, nthreads=4)
        assert np.array_equal(bits(smp.cpu().numpy()), bits(ref_smp))
        assert np.array_equal(bits(s.cpu().numpy()), bits(ref_sum))
        assert np.abs(ref_sum).max() > 0.0
        rng = np.random.default_rng(2)
        dimg = rng.normal(size=ref_sum.shape).astype(np.float32)
        g_rho, g_tf = m.adjoint(rho, vals, spp, torch.from_numpy(dimg).cuda(), smp)
        o_rho, o_tf = h.adjoint(spp, dimg, ref_smp, nthreads=4)
        h.close()
        # the same terms, summed in another order (atomics vs per-thread buffers)
        assert np.allclose(g_tf.cpu().numpy(), o_tf, rtol=1e-4, atol=1e-5 * np.abs(o_tf).max())
        assert np.allclose(g_rho.cpu().numpy(), o_rho, rtol=1e-4, atol=1e-5 * np.abs(o_rho).max())
        r_rho, r_tf = m.adjoint(rho, vals, spp, torch.from_numpy(dimg).cuda(), None)
        assert torch.allclose(r_tf, g_tf, rtol=1e-5, atol=1e-6 * float(g_tf.abs().max()))
        assert torch.allclose(r_rho, g_rho, rtol=1e-5, atol=1e-6 * float(g_rho.abs().max()))
    finally:
        r.close()


def test_adjoint_on_kept_jobs_matches_a_fresh_walk(torch, lib, pkg):
    """An adjoint right after its forward replays against the job list the
    forward kept; after another walk (here view 3) the same adjoint call
    runs the count, jobs and shadow stages again.  Both give the same
    gradients up to the order of the atomic sums."""
    sc, r, m, rho, vals = make(torch, lib, pkg, (16, 16, 16), 12, (24, 20), 30.0, 4)
    try:
        spp = 4
        smp, s = m.render_samples(rho, vals, spp)
        dimg = torch.from_numpy(np.random.default_rng(5).normal(size=tuple(s.shape)).astype(np.float32)).cuda()
        k_rho, k_tf = m.adjoint(rho, vals, spp, dimg, smp)
        m.render_samples(rho, vals, spp, view=3)
        f_rho, f_tf = m.adjoint(rho, vals, spp, dimg, smp)
        k2_rho, k2_tf = m.adjoint(rho, vals, spp, dimg, smp)      # kept again after the fresh walk
        torch.cuda.synchronize()
        assert float(f_tf.abs().max()) > 0 and float(f_rho.abs().max()) > 0
        for a, b in ((k_tf, f_tf), (k_rho, f_rho), (k2_tf, f_tf), (k2_rho, f_rho)):
            assert torch.allclose(a, b, rtol=1e-5, atol=1e-6 * float(b.abs().max()))
    finally:
        r.close()


def test_binary64_tracks_float_and_the_oracle(torch, lib, pkg):
    """The GPU's binary64 evaluation (every medium-dependent quantity in
    double; the camera and light geometry stays float) against its float
    forward and against the oracle's binary64 build (which has the geometry
    in double too)"""
    sc, r, m, rho, vals = make(torch, lib, pkg, (16, 16, 16), 12, (24, 20), 30.0, 4)
    try:
        s64 = m.render_sums64(rho, vals, 4).cpu().numpy()
        _, s32 = m.render_samples(rho, vals, 4)
        s32 = s32.cpu().numpy()
        # a collision or roulette decision whose threshold falls between the
        # float and the double value takes another path: such pixels differ
        # by a whole sample; every other pixel agrees to float rounding of
        # its path (products of transmittances: ~1e-4 of the image's peak)
        close = np.isclose(s32, s64, rtol=1e-4, atol=2e-4 * np.abs(s64).max()).all(-1)
        flips = int((~close).sum())
        assert flips <= max(2, close.size // 100), (flips, float(np.abs(s32 - s64).max()))
        assert abs(float(s32.sum()) - float(s64.sum())) <= 2e-2 * float(np.abs(s64).sum()), (s32.sum(), s64.sum())
        f64 = OL.load_fp64()
        h = OL.MediumHandle(f64, sc, rho.cpu().numpy(), vals.cpu().numpy(), 30.0, np.array([0.8, 0.8, 0.8]), 0.5,
                            m.majorant.cpu().numpy(), 4, model=1, gm_inv=m.gm_inv)
        ref = h.render(4, nthreads=4)
        h.close()
        # the geometry (float on the GPU, double in the oracle) moves the
        # collision points by float rounding: pixels agree to 1e-3 of the
        # image's largest value but for the rare decision flips
        near = (np.abs(s64 - ref) <= 1e-3 * np.abs(ref).max()).all(-1)
        assert int((~near).sum()) <= max(2, near.size // 100), (int((~near).sum()), float(np.abs(s64 - ref).max()))
    finally:
        r.close()


def test_c4_tracer_adjoint_matches_finite_differences(torch, lib, pkg):
    """128^3 float intensity grid, the 64-node opacity PLF, hybrid shader
    with emission, 256^2 x 32 spp; the target is rendered at 1024 spp from
    the parameters perturbed by N(0, 0.05).  32 parameters drawn uniformly
    among those the loss depends on: 16 opacity node values (central
    differences at h = 1e-3 of the binary64 evaluation of the same samples;
    sigma is linear in the node values) and 16 voxels (h = 1e-5: the PLF is
    piecewise linear in the intensity, and a 1e-3 step of a voxel moves some
    lookups across a node position).  Pass: |adjoint - difference| <= 1e-3
    |difference| + 1e-5 of the largest gradient of the parameter's kind."""
    res, n, scale, spp = (128, 128, 128), 64, 40.0, 32
    sc, r, m, rho, vals = make(torch, lib, pkg, res, n, (256, 256), scale, 8, seed=40, blobs=10)
    try:
        gen = torch.Generator(device="cuda").manual_seed(7)
        rho_t = (rho + 0.05 * torch.randn(rho.shape, device="cuda", generator=gen)).contiguous()
        vals_t = (vals + 0.05 * torch.randn(vals.shape, device="cuda", generator=gen)).contiguous()
        maj0 = m.majorant.clone()
        m.rebuild_majorant(rho_t, vals_t)
        m.majorant = torch.maximum(maj0, m.majorant).contiguous()
        _, ts = m.render_samples(rho_t, vals_t, 1024, view=1)
        target = (ts / 1024).double()

        def loss64(rh, v):
            s = m.render_sums64(rh, v, spp)
            return float(((s / spp - target) ** 2).mean())

        smp, s = m.render_samples(rho, vals, spp)
        dsum = 2.0 * (s.double() / spp - target) / spp / target.numel()
        g_rho, g_tf = m.adjoint(rho, vals, spp, dsum.float(), smp)
        C.check(lib.er_synchronize())
        rng = np.random.default_rng(11)
        gt = g_tf.cpu().numpy()
        gr = g_rho.cpu().numpy().ravel()
        tf_idx = rng.choice(np.flatnonzero(gt != 0.0), 16, replace=False)
        rho_idx = rng.choice(np.flatnonzero(gr != 0.0), 16, replace=False)
        floor = {"tf": 1e-5 * float(np.abs(gt).max()), "rho": 1e-5 * float(np.abs(gr).max())}
        worst = 0.0
        for kind, idx in [("tf", i) for i in tf_idx] + [("rho", i) for i in rho_idx]:
            base = vals if kind == "tf" else rho
            h = 1e-3 if kind == "tf" else 1e-5
            p, q = base.clone(), base.clone()
            p.view(-1)[idx] += h
            q.view(-1)[idx] -= h
            # the float32 parameters' actual step
            step = float(p.view(-1)[idx].double() - q.view(-1)[idx].double())
            if kind == "tf":
                fd = (loss64(rho, p) - loss64(rho, q)) / step
                adj = float(gt[idx])
            else:
                fd = (loss64(p, vals) - loss64(q, vals)) / step
                adj = float(gr[idx])
            # |adj - fd| <= 1e-3 |fd| + floor
            rel = abs(adj - fd) / (abs(fd) + floor[kind] / 1e-3)
            worst = max(worst, rel)
            assert rel <= 1e-3, (kind, int(idx), adj, fd, rel)
        print(f"worst relative error over 32 parameters: {worst:.2e}")
    finally:
        r.close()


def test_autograd_function(torch, lib, pkg):
    sc, r, m, rho, vals = make(torch, lib, pkg, (16, 16, 16), 12, (24, 20), 30.0, 4)
    try:
        spp = 4
        target = torch.full((r.height, r.width, 3), 0.02, device="cuda")
        rho_p = rho.clone().requires_grad_(True)
        v_p = vals.clone().requires_grad_(True)
        img = m(rho_p, v_p, spp)
        loss = ((img - target) ** 2).sum()
        loss.backward()
        smp, s = m.render_samples(rho, vals, spp)
        dsum = 2.0 * (s / spp - target) / spp
        g_rho, g_tf = m.adjoint(rho, vals, spp, dsum, smp)
        # two walks of the same samples: equal up to the order of the atomic sums
        assert torch.allclose(v_p.grad, g_tf, rtol=1e-5, atol=1e-6 * float(g_tf.abs().max()))
        assert torch.allclose(rho_p.grad, g_rho, rtol=1e-5, atol=1e-6 * float(g_rho.abs().max()))
    finally:
        r.close()


def test_tracer_model_converges_to_the_product_image(torch, lib, pkg):
    """The tiny blob scene with the hybrid shader: the product's estimator
    (delta tracking, stochastic shader choice, full MIS) on the uint16
    volume and the differentiable tracer model on the same volume as a float
    grid, each at 4096 spp from two independent halves: the images agree to
    within their noise.  The product's lookups truncate each lerp stage to an
    integer (Source/buffer3d.h:234-241), the float grid's do not; the
    intensities and transfer-function positions are scaled by 16 so that
    this truncation (under 2 units of 64000) stays below the noise."""
    runtime, medium = pkg
    sc = S.scene_tiny(res=32, film=(48, 40), seed=3)
    sc.volume = np.clip(sc.volume.astype(np.int64) * 16, 0, 65535).astype(np.uint16)

    def scaled(plf):
        # off the integers, so that no truncated lookup lands on a node
        return C.make_plf([(16.0 * plf.position[i] + 0.25, plf.value[i]) for i in range(plf.count)])
    t = sc.tracer
    t.opacity, t.glossiness = scaled(t.opacity), scaled(t.glossiness)
    for tf in (t.diffuse, t.specular, t.emission):
        for c in range(3):
            tf.plf[c] = scaled(tf.plf[c])
    s = sc.tracer.settings
    s.free_flight, s.mis, s.stratify, s.apply_shading_type, s.shading_type = 1, 1, 0, 1, C.SHADING_HYBRID
    s.majorant_brick = 4
    r = runtime.Renderer(sc, lib)
    try:
        spp = 2048
        W, H = sc.width, sc.height

        def product(first):
            d = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
            r.trace_sum_device(d.data_ptr(), spp, 5, first, 0, None)
            return d[..., :3].double() / spp

        a1, a2 = product(0), product(spp)
        grid = torch.from_numpy(sc.volume.astype(np.float32)).cuda()
        vals = torch.from_numpy(S.plf_node_values(sc.tracer.opacity)).cuda()
        ds = float(np.float32(s.density_scale) * np.float32(s.density_scale))
        m = medium.Medium(r, grid, vals, ds, nee_probability=1.0, brick=4, model="tracer",
                          gradient_magnitude_inv=1.0 / r.gradient_magnitude())

        def tracer_model(first):
            acc = torch.zeros((H, W, 3), dtype=torch.float64, device="cuda")
            for k in range(0, spp, 256):
                _, sm = m.render_samples(grid, vals, 256, view=6, first=first + k)
                acc += sm.double()
            return acc / spp

        b1, b2 = tracer_model(0), tracer_model(spp)
        A, B = 0.5 * (a1 + a2), 0.5 * (b1 + b2)
        var_a = float(((a1 - a2) ** 2).mean()) / 4.0
        var_b = float(((b1 - b2) ** 2).mean()) / 4.0
        d2 = float(((A - B) ** 2).mean())
        assert float(A.abs().max()) > 0.0
        assert d2 <= 1.5 * (var_a + var_b), (d2, var_a, var_b)
    finally:
        r.close()
