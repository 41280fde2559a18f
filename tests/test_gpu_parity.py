"""GPU kernels against the CPU oracle, through the C ABI of
libexposurerender.so.  The parity kernels evaluate the reference's
floating-point operations in the reference's order, so every comparison on
the transport path is bit-exact (a float XYZA per pixel compared as uint32)."""
import ctypes
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
def runtime():
    return importlib.import_module("exposure-render_gb300.runtime")


def dev_sum(torch, r, spp, view=0, first=0):
    d = torch.zeros((r.height, r.width, 4), dtype=torch.float32, device="cuda")
    r.trace_sum_device(d.data_ptr(), spp, view, first, 0, None)
    torch.cuda.synchronize()
    return d.cpu().numpy()


@pytest.mark.parametrize("fn", range(8))
def test_math_device_bits_equal_host(torch, lib, oracle, fn):
    rng = np.random.default_rng(100 + fn)
    if fn == 0:
        x = np.exp(rng.uniform(-60, 60, 65536))
    elif fn == 6:
        x = rng.uniform(-1, 1, 65536)
    elif fn == 5:
        x = rng.uniform(0, 1.2, 65536)
    else:
        x = rng.uniform(-20, 20, 65536)
    x = x.astype(np.float32)
    y = (np.exp(rng.uniform(-3, 14, 65536)) if fn == 5 else rng.normal(size=65536)).astype(np.float32)
    host = np.zeros_like(x)
    oracle.math_eval(fn, len(x), OL.ptr(x), OL.ptr(y), OL.ptr(host))
    dx, dy = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    do = torch.zeros_like(dx)
    C.check(lib.er_math_eval_device(fn, len(x), dx.data_ptr(), dy.data_ptr(), do.data_ptr(), None))
    torch.cuda.synchronize()
    assert np.array_equal(bits(do.cpu().numpy()), bits(host))


@pytest.fixture(scope="module")
def tiny(lib, runtime, oracle):
    sc = S.scene_tiny()
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    yield sc, r, h
    r.close()
    h.close()


def test_frames_stateful_lanes(torch, tiny):
    sc, r, h = tiny
    lanes = OL.initial_lanes(int(sc.tracer.settings.seed), sc.width, sc.height)
    d_lanes = torch.from_numpy(lanes.view(np.int32).copy()).cuda()
    d_frame = torch.zeros((sc.height, sc.width, 4), dtype=torch.float32, device="cuda")
    for f in range(3):
        cpu = h.render_frame(lanes, nthreads=4)
        r.trace_frame_device(d_lanes.data_ptr(), d_frame.data_ptr(), None)
        torch.cuda.synchronize()
        assert np.array_equal(bits(d_frame.cpu().numpy()), bits(cpu)), f"frame {f}"
        assert np.array_equal(d_lanes.cpu().numpy().view(np.uint32), lanes), f"lanes {f}"


@pytest.mark.parametrize("spp,view,first", [(1, 0, 0), (4, 0, 0), (3, 7, 11)])
def test_counter_seeded_sums(torch, tiny, spp, view, first):
    sc, r, h = tiny
    assert np.array_equal(bits(dev_sum(torch, r, spp, view, first)), bits(h.render_sum(spp, view, first, nthreads=4)))


@pytest.mark.parametrize("shape", ["plane", "disk", "ring", "box", "sphere"])
@pytest.mark.parametrize("gradient_mode", [0, 1, 2])
def test_light_shapes_and_gradient_modes(torch, lib, runtime, oracle, shape, gradient_mode):
    sc = S.scene_tiny(res=20, film=(24, 20), seed=5)
    L = sc.lights[0]
    L.shape.type = {"plane": 0, "disk": 1, "ring": 2, "box": 3, "sphere": 4}[shape]
    L.shape.inner_radius, L.shape.outer_radius = 0.1, 0.3
    L.shape.size[0], L.shape.size[1], L.shape.size[2] = 0.4, 0.3, 0.2
    L.shape.one_sided = 1 if shape in ("plane", "disk") else 0
    L.unit = C.UNIT_LUX if shape in ("disk", "box") else C.UNIT_POWER
    sc.tracer.settings.gradient_computation = gradient_mode
    sc.tracer.camera.aperture_size = 0.03 if shape == "ring" else 0.0
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        assert np.array_equal(bits(dev_sum(torch, r, 3)), bits(h.render_sum(3, nthreads=4)))
    finally:
        r.close()
        h.close()


def test_environment_sphere_two_lights(torch, lib, runtime, oracle):
    sc = S.scene_tiny(res=20, film=(24, 20), seed=6)
    tm = np.eye(4).tolist()
    env = C.er_light_desc()
    env.visible = 1
    env.shape = S.make_shape(C.SHAPE_SPHERE, (tm, tm), outer=4.0)
    env.texture_id = 1
    env.multiplier = 0.7
    sc.lights.append(env)
    sc.textures.append(S.gradient_texture([(0.0, (0.2, 0.2, 0.3)), (0.5, (0.5, 0.5, 0.6)), (1.0, (1.0, 1.0, 1.0))]))
    sc.tracer.light_count = 2
    sc.tracer.light_ids[1] = 1
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        assert np.array_equal(bits(dev_sum(torch, r, 4)), bits(h.render_sum(4, nthreads=4)))
    finally:
        r.close()
        h.close()


def test_c1_crop_bit_exact(torch, lib, runtime, oracle):
    """The 128^3 / 256^2 plain-forward workload: GPU over the whole film, the
    oracle over a 40x40 crop through the volume centre."""
    sc = S.scene_c1()
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        g = dev_sum(torch, r, 6)
        c = h.render_sum(6, rect=(108, 108, 40, 40), nthreads=8)
        assert np.array_equal(bits(g[108:148, 108:148]), bits(c))
        assert (c[..., 3] > 0).mean() > 0.5
    finally:
        r.close()
        h.close()


def test_c1_full_size_properties(torch, lib, runtime):
    """Full 256^2 x 64 spp: deterministic across launches, and one 64-spp
    launch equals two 32-spp launches of the same counter stream up to float
    re-association."""
    sc = S.scene_c1()
    r = runtime.Renderer(sc, lib)
    try:
        a = dev_sum(torch, r, 64)
        b = dev_sum(torch, r, 64)
        assert np.array_equal(bits(a), bits(b))
        d = torch.zeros((r.height, r.width, 4), dtype=torch.float32, device="cuda")
        r.trace_sum_device(d.data_ptr(), 32, 0, 0, 0, None)
        r.trace_sum_device(d.data_ptr(), 32, 0, 32, 1, None)
        torch.cuda.synchronize()
        s = d.cpu().numpy()
        assert np.allclose(s, a, rtol=1e-5, atol=1e-6)
        alpha = a[..., 3] / 64.0
        assert 0.2 < alpha.mean() < 0.6 and alpha.max() == 1.0 and alpha.min() == 0.0
    finally:
        r.close()


def test_render_estimate_api_matches_reference_pipeline(torch, lib, runtime, oracle):
    """RenderEstimate x3 through the C ABI (transport, 3x3 Gaussian, running
    average, tone map) against the oracle's restatement of the same pipeline."""
    sc = S.scene_tiny(res=24, film=(30, 22), seed=12)
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        W, H = sc.width, sc.height
        lanes = OL.initial_lanes(int(sc.tracer.settings.seed), W, H)
        assert np.array_equal(r.get_seeds(), lanes)
        running = np.zeros((H, W, 4), np.float32)
        for n in range(3):
            frame = h.render_frame(lanes, nthreads=4)
            raw = frame.copy()
            rgba = np.zeros((H, W, 4), np.uint8)
            oracle.post_frame(OL.ptr(frame), OL.ptr(running), OL.ptr(rgba), W, H, n, float(sc.tracer.camera.exposure))
            r.render_estimate()
            assert np.array_equal(bits(r.get_frame_estimate()), bits(raw)), n
            assert np.array_equal(bits(r.get_running_estimate()), bits(running)), n
            assert np.array_equal(r.get_estimate(), rgba), n
        assert r.no_iterations() == 3
        assert np.array_equal(r.get_seeds(), lanes)
    finally:
        r.close()
        h.close()


def test_post_frame_device(torch, lib, oracle):
    rng = np.random.default_rng(21)
    W, H = 37, 23
    run_c = np.zeros((H, W, 4), np.float32)
    d_run = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    d_rgba = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    for n in range(4):
        f = rng.uniform(0, 3, (H, W, 4)).astype(np.float32)
        f[..., 3] = (rng.uniform(0, 1, (H, W)) > 0.3).astype(np.float32)
        d_f = torch.from_numpy(f.copy()).cuda()
        rgba = np.zeros((H, W, 4), np.uint8)
        oracle.post_frame(OL.ptr(f), OL.ptr(run_c), OL.ptr(rgba), W, H, n, 0.7)
        C.check(lib.er_post_frame_device(d_f.data_ptr(), d_run.data_ptr(), d_rgba.data_ptr(), W, H, n, 0.7, 1, None))
        torch.cuda.synchronize()
        assert np.array_equal(bits(d_run.cpu().numpy()), bits(run_c))
        assert np.array_equal(d_rgba.cpu().numpy(), rgba)


@pytest.mark.parametrize("radius,sd,sr", [(0, 1.0, 10.0), (2, 1.5, 20.0), (5, 3.0, 8.0)])
def test_bilateral_device(torch, lib, oracle, radius, sd, sr):
    rng = np.random.default_rng(radius)
    W, H = 41, 29
    img = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
    tmp = np.zeros_like(img)
    out = np.zeros_like(img)
    oracle.bilateral(OL.ptr(img), OL.ptr(tmp), OL.ptr(out), W, H, radius, sd, sr)
    d_in = torch.from_numpy(img).cuda()
    d_tmp = torch.zeros_like(d_in)
    d_out = torch.zeros_like(d_in)
    C.check(lib.er_bilateral_device(d_in.data_ptr(), d_tmp.data_ptr(), d_out.data_ptr(), W, H, radius, sd, sr, None))
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy(), out)
    assert (out[..., 3] == 255).all()


def test_gradient_magnitude_volume(torch, lib, runtime, oracle):
    sc = S.scene_tiny(res=28, film=(8, 8), seed=4)
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        gm = np.zeros(sc.volume.shape, np.uint16)
        mx = oracle.gradient_magnitude_volume(h.h, OL.ptr(gm))
        d_gm = torch.zeros(sc.volume.shape, dtype=torch.int16, device="cuda")
        m = r.gradient_magnitude(d_gm.data_ptr())
        assert np.array_equal(d_gm.cpu().numpy().view(np.uint16), gm)
        assert np.float32(m) == np.float32(mx) and mx > 0
    finally:
        r.close()
        h.close()


def test_render_spp_mean(torch, lib, runtime, oracle):
    sc = S.scene_tiny(res=24, film=(30, 22), seed=13)
    sc.tracer.settings.frame_filter = -1
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        r.render_spp(3)
        r.render_spp(2)
        s = h.render_sum(3, nthreads=4) + h.render_sum(2, first=3, nthreads=4)
        assert np.allclose(r.get_running_estimate(), s / 5.0, rtol=1e-6, atol=1e-7)
        assert r.no_iterations() == 5
    finally:
        r.close()
        h.close()


def test_bind_list_semantics_and_errors(torch, lib):
    lib.er_reset()
    ids = []
    t = S.uniform_texture()
    for k in range(31):
        i = ctypes.c_int32(-1)
        C.check(lib.er_bind_texture(ctypes.byref(t), ctypes.byref(i)))
        ids.append(i.value)
    assert ids == list(range(31))
    i = ctypes.c_int32(-1)
    assert lib.er_bind_texture(ctypes.byref(t), ctypes.byref(i)) == 3          # list full
    # the capacity check comes before update-or-insert (Source/list.cuh:63-83)
    i = ctypes.c_int32(5)
    assert lib.er_bind_texture(ctypes.byref(t), ctypes.byref(i)) == 3
    C.check(lib.er_unbind_texture(5))
    assert lib.er_unbind_texture(5) == 1                                        # invalid id
    i = ctypes.c_int32(-1)
    C.check(lib.er_bind_texture(ctypes.byref(t), ctypes.byref(i)))
    assert i.value == 31                                                        # IDs are not reused
    C.check(lib.er_unbind_texture(31))                                          # back to 30 items
    i2 = ctypes.c_int32(7)
    C.check(lib.er_bind_texture(ctypes.byref(t), ctypes.byref(i2)))
    assert i2.value == 7                                                        # update in place
    assert lib.er_render_estimate(12345) == 1
    assert b"does not exist" in lib.er_last_error_message()
    lib.er_reset()
    sc = S.scene_tiny()
    sc.tracer.object_count = 1
    rt = importlib.import_module("exposure-render_gb300.runtime")
    r = rt.Renderer(sc, lib)
    # ObjectIDs.Count above the bound objects: only bound objects are walked
    assert lib.er_render_estimate(r.tracer_id) == 0
    r.close()
    lib.er_reset()


@pytest.mark.parametrize("uv", [(24, 20), (0, 0), (47, 39), (10, 30)])
def test_autofocus_bits_equal_oracle(torch, lib, runtime, oracle, uv):
    """er_get_auto_focus_distance against the oracle's restatement of
    KrnlComputeAutoFocusDistance, with the same seed lanes (a scene of its
    own: the resource tests before it reset the library)"""
    sc = S.scene_tiny()
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    u, v = uv
    d = ctypes.c_float(0.0)
    C.check(lib.er_get_auto_focus_distance(r.tracer_id, u, v, ctypes.byref(d)))
    l0, l1 = OL.seed_lanes(sc.tracer.settings.seed, 0x41F0C05E, v * sc.width + u, 0)
    ref = h.orc.autofocus(h.h, u, v, l0, l1)
    assert np.float32(d.value).view(np.uint32) == np.float32(ref).view(np.uint32)
    assert lib.er_get_auto_focus_distance(r.tracer_id, sc.width, 0, ctypes.byref(d)) == C.ER_ERR_INVALID_ARGUMENT
    r.close()
    h.close()
