"""Clipping objects and the zero-size volume box on the GPU against the CPU
oracle, through the C ABI.  Clipping objects (ErClippingObject,
Source/erclippingobject.h:27-58) remove the volume inside their shape (outside
with Invert) from free flight and shadow rays; a volume bound without
NormalizeSize has no extent (Source/volume.h:106-117), so renders show only
the lights and objects.  Float XYZA sums compared as uint32."""
import ctypes
import importlib

import numpy as np
import pytest

import oracle_lib as OL
from test_clipping import with_environment

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


def fast_settings(s, engine):
    s.free_flight = C.FREE_FLIGHT_DELTA
    s.mis = C.MIS_FULL
    s.apply_shading_type = 1
    s.shading_type = C.SHADING_HYBRID
    s.majorant_brick = 4
    s.engine = engine


@pytest.mark.parametrize("mode", ["march", "delta-wavefront", "delta-one-kernel", "delta-persistent"])
def test_clipped_scene_bit_exact(torch, lib, runtime, oracle, mode):
    sc = with_environment(S.scene_clipped())
    s = sc.tracer.settings
    if mode != "march":
        fast_settings(s, 1 if mode == "delta-one-kernel" else 2)
        if mode == "delta-persistent":
            s.tune_stages = C.PERSISTENT_BOTH
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        g = dev_sum(torch, r, 3, view=2, first=5)
        c = h.render_sum(3, view=2, first=5, nthreads=8)
        assert np.array_equal(bits(g), bits(c))
        assert 0.0 < c[..., 3].sum()
    finally:
        r.close()
        h.close()


def test_clipped_reference_frames(torch, lib, runtime, oracle):
    """The reference-order frame path (RenderEstimate's kernel, stateful
    per-pixel lanes) with clipping objects"""
    sc = S.scene_clipped()
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        lanes = OL.initial_lanes(int(sc.tracer.settings.seed), sc.width, sc.height)
        d_lanes = torch.from_numpy(lanes.view(np.int32).copy()).cuda()
        d_frame = torch.zeros((sc.height, sc.width, 4), dtype=torch.float32, device="cuda")
        for f in range(2):
            cpu = h.render_frame(lanes, nthreads=4)
            r.trace_frame_device(d_lanes.data_ptr(), d_frame.data_ptr(), None)
            torch.cuda.synchronize()
            assert np.array_equal(bits(d_frame.cpu().numpy()), bits(cpu)), f"frame {f}"
    finally:
        r.close()
        h.close()


def test_clipping_rebind_updates_renders(torch, lib, runtime, oracle):
    """Rebinding a clipping object with a new shape (same ID) changes the
    next render; unbinding it leaves the tracer's ID dangling, which is
    skipped (the unclipped render)"""
    sc = S.scene_clipped()
    fast_settings(sc.tracer.settings, 2)
    r = runtime.Renderer(sc, lib)
    try:
        before = dev_sum(torch, r, 2)
        k = S.make_clipping_object(S.make_shape(C.SHAPE_SPHERE, S.look_at_tm((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), (0.0, 1.0, 0.0)),
                                                outer=0.2))
        cid = ctypes.c_int32(r.clipping_ids[1])
        C.check(lib.er_bind_clipping_object(ctypes.byref(k), ctypes.byref(cid)))
        after = dev_sum(torch, r, 2)
        sc2 = S.scene_clipped()
        fast_settings(sc2.tracer.settings, 2)
        sc2.clipping_objects[1] = k
        h = OL.SceneHandle(oracle, sc2)
        try:
            assert np.array_equal(bits(after), bits(h.render_sum(2, nthreads=8)))
        finally:
            h.close()
        assert not np.array_equal(bits(before), bits(after))
        for i in r.clipping_ids:
            C.check(lib.er_unbind_clipping_object(i))
        r.clipping_ids = []
        plain = dev_sum(torch, r, 2)
        sc3 = S.scene_tiny()
        fast_settings(sc3.tracer.settings, 2)
        h = OL.SceneHandle(oracle, sc3)
        try:
            assert np.array_equal(bits(plain), bits(h.render_sum(2, nthreads=8)))
        finally:
            h.close()
    finally:
        r.close()


def test_clipped_views_in_a_batch(torch, lib, runtime, oracle):
    """A batch mixing a clipped tracer's views with an unclipped tracer's:
    every view bit-exact with the oracle"""
    a = with_environment(S.scene_clipped())
    fast_settings(a.tracer.settings, 2)
    b = S.scene_tiny(res=40, film=(40, 32), seed=4)
    fast_settings(b.tracer.settings, 2)
    ra, rb = runtime.Renderer(a, lib), runtime.Renderer(b, lib)
    rng = np.random.default_rng(9)
    cam = S.orbit_camera(rng, (36, 28), radius=2.1)
    sums = [torch.zeros((a.height, a.width, 4), dtype=torch.float32, device="cuda"),
            torch.zeros((b.height, b.width, 4), dtype=torch.float32, device="cuda"),
            torch.zeros((28, 36, 4), dtype=torch.float32, device="cuda")]
    batch = runtime.Batch([(ra.tracer_id, 3, sums[0].data_ptr(), None), (rb.tracer_id, 2, sums[1].data_ptr(), None),
                           (ra.tracer_id, 2, sums[2].data_ptr(), cam)], flags=C.ER_BATCH_GRAPH, window_items=1500, lib=lib)
    try:
        batch.launch(None)
        torch.cuda.synchronize()
        for i, (sc, spp, camera) in enumerate(((a, 3, None), (b, 2, None), (a, 2, cam))):
            if camera is not None:
                sc = S.Scene(sc.name, sc.volume, tracer=C.er_tracer_desc.from_buffer_copy(sc.tracer), lights=sc.lights,
                             textures=sc.textures, clipping_objects=sc.clipping_objects)
                sc.tracer.camera = camera
            h = OL.SceneHandle(oracle, sc)
            try:
                assert np.array_equal(bits(sums[i].cpu().numpy()), bits(h.render_sum(spp, view=i, nthreads=8))), f"view {i}"
            finally:
                h.close()
    finally:
        batch.close()
        ra.close()
        rb.close()


@pytest.mark.parametrize("free_flight", [0, 1])
def test_volume_without_normalize_size(torch, lib, runtime, oracle, free_flight):
    """normalize_size = 0 binds, as in the reference, and renders only the
    lights: bit-exact with the oracle (which keeps the reference's zero-size
    box), and every pixel sees the environment light"""
    sc = with_environment(S.scene_tiny(res=20, film=(24, 20), seed=5))
    sc.normalize_size = 0
    if free_flight:
        fast_settings(sc.tracer.settings, 2)
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        g = dev_sum(torch, r, 3)
        c = h.render_sum(3, nthreads=8)
        assert np.array_equal(bits(g), bits(c))
        assert c[..., :3].all(-1).all()
        # the RenderEstimate / GetEstimate pipeline runs and reads back
        r.render_estimate()
        r.render_estimate()
        img = r.get_estimate()
        assert img.shape == (sc.height, sc.width, 4)
    finally:
        r.close()
        h.close()
