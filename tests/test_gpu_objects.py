"""Surface objects (SampleRay's third event type, Source/objects.h:26-80,
Source/transport.h:141-149) on the GPU against the oracle, through the C ABI:
the one-kernel path, the wavefront stages, the stateful frame kernel and a
batch, each bit-exact per pixel."""
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
def env():
    import torch
    assert torch.cuda.is_available()
    lib = C.load_library()
    C.check(lib.er_set_device(0))
    rt = importlib.import_module("exposure-render_gb300.runtime")
    yield torch, lib, rt
    lib.er_reset()


def gpu_sum(torch, r, spp, view=0, first=0):
    d = torch.zeros((r.height, r.width, 4), dtype=torch.float32, device="cuda")
    r.trace_sum_device(d.data_ptr(), spp, view, first, 0, None)
    torch.cuda.synchronize()
    return d.cpu().numpy()


MODES = [
    dict(),                                                                   # the reference's live estimator
    dict(free_flight=1, mis=1, apply_shading_type=1, shading_type=2),          # delta tracking, full MIS, hybrid
    dict(free_flight=0, mis=1),
]


@pytest.mark.parametrize("engine", [1, 2], ids=["one-kernel", "wavefront"])
@pytest.mark.parametrize("mode", MODES, ids=["reference", "delta-mis-hybrid", "march-mis"])
def test_objects_sum_bit_exact(env, oracle, engine, mode):
    torch, lib, rt = env
    sc = S.scene_objects()
    sc.tracer.settings.engine = engine
    for k, v in mode.items():
        setattr(sc.tracer.settings, k, v)
    r = rt.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        g = gpu_sum(torch, r, 4, view=2, first=3)
        cpu = h.render_sum(4, view=2, first=3, nthreads=4)
        assert np.array_equal(bits(g), bits(cpu))
        assert cpu[..., 3].mean() > 0.5                      # the floor fills the frame
    finally:
        r.close()
        h.close()


def test_objects_change_the_image(env, oracle):
    """the same scene without its objects renders differently (the objects are
    intersected, shade and shadow), and the one with them matches the oracle"""
    torch, lib, rt = env
    sc = S.scene_objects()
    r = rt.Renderer(sc, lib)
    with_objects = gpu_sum(torch, r, 2)
    r.close()
    sc.tracer.object_count = 0
    r = rt.Renderer(sc, lib)
    without = gpu_sum(torch, r, 2)
    r.close()
    assert (np.abs(with_objects - without).max(-1) > 0).mean() > 0.3


def test_objects_frames_stateful_lanes(env, oracle):
    torch, lib, rt = env
    sc = S.scene_objects(film=(40, 36))
    r = rt.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        lanes = OL.initial_lanes(21, sc.width, sc.height)
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


@pytest.mark.parametrize("shape", ["disk", "ring", "box"])
def test_object_shapes(env, oracle, shape):
    torch, lib, rt = env
    sc = S.scene_objects(res=20, film=(28, 24), seed=8)
    sh = sc.objects[1].shape
    sh.type = {"disk": C.SHAPE_DISK, "ring": C.SHAPE_RING, "box": C.SHAPE_BOX}[shape]
    sh.inner_radius, sh.outer_radius = 0.1, 0.3
    sh.size[0], sh.size[1], sh.size[2] = 0.4, 0.3, 0.2
    sc.objects[0].glossiness_texture_id = 2                     # luminance of a checker
    for engine in (1, 2):
        sc.tracer.settings.engine = engine
        r = rt.Renderer(sc, lib)
        h = OL.SceneHandle(oracle, sc)
        try:
            assert np.array_equal(bits(gpu_sum(torch, r, 3)), bits(h.render_sum(3, nthreads=4))), engine
        finally:
            r.close()
            h.close()


def test_objects_in_a_batch(env, oracle):
    """a batch mixing a view with objects and one without equals the views
    rendered alone, which equal the oracle"""
    torch, lib, rt = env
    a = S.scene_objects()
    b = S.scene_tiny(seed=3)
    b.tracer.settings.free_flight = C.FREE_FLIGHT_DELTA
    ra, rb = rt.Renderer(a, lib), rt.Renderer(b, lib)
    try:
        outs, recs = [], (C.er_batch_view * 2)()
        for i, (r, spp) in enumerate([(ra, 5), (rb, 3)]):
            d = torch.zeros((r.height, r.width, 4), dtype=torch.float32, device="cuda")
            outs.append(d)
            recs[i].tracer_id = r.tracer_id
            recs[i].spp = spp
            recs[i].view = i
            recs[i].first_sample = 0
            recs[i].d_sum_xyza = d.data_ptr()
            recs[i].accumulate = 0
            recs[i].display = 0
        bid = ctypes.c_int32(-1)
        C.check(lib.er_batch_create(recs, 2, C.ER_BATCH_GRAPH, 0, ctypes.byref(bid)))
        C.check(lib.er_batch_launch(bid.value, None))
        torch.cuda.synchronize()
        h = OL.SceneHandle(oracle, a)
        assert np.array_equal(bits(outs[0].cpu().numpy()), bits(h.render_sum(5, view=0, nthreads=4)))
        h.close()
        assert np.array_equal(bits(outs[1].cpu().numpy()), bits(gpu_sum(torch, rb, 3, view=1)))
        C.check(lib.er_batch_destroy(bid.value))
    finally:
        ra.close()
        rb.close()


@pytest.mark.parametrize("engine", [1, 2], ids=["one-kernel", "wavefront"])
def test_bitmap_textures(env, oracle, engine):
    """bitmap textures on the light and on both objects (Source/textures.h:101-107)"""
    torch, lib, rt = env
    sc = S.scene_bitmaps()
    sc.tracer.settings.engine = engine
    r = rt.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        cpu = h.render_sum(4, nthreads=4)
        assert np.array_equal(bits(gpu_sum(torch, r, 4)), bits(cpu))
        assert cpu[..., :3].max() > 0
    finally:
        r.close()
        h.close()
