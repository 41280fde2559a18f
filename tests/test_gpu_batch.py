"""Batched multi-view transport (er_batch_*) against one-view renders
(er_trace_sum_device, er_render_spp), through the C ABI.  A batch cuts the
samples of all its views into windows that mix views; every view's sums must
still be bit-identical to rendering that view alone."""
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


@pytest.fixture(scope="module")
def pair(lib, runtime):
    """Two bound tiny scenes: A marches with light-only MIS (the reference
    estimator), B delta-tracks with full MIS and the hybrid shader."""
    a = S.scene_tiny(seed=3)
    b = S.scene_tiny(res=40, film=(40, 32), seed=4)
    b.tracer.settings.free_flight = C.FREE_FLIGHT_DELTA
    b.tracer.settings.mis = C.MIS_FULL
    b.tracer.settings.apply_shading_type = 1
    b.tracer.settings.shading_type = C.SHADING_HYBRID
    ra, rb = runtime.Renderer(a, lib), runtime.Renderer(b, lib)
    yield ra, rb
    ra.close()
    rb.close()


def bind_with_camera(lib, r, cam):
    t = C.er_tracer_desc.from_buffer_copy(r.tracer_desc)
    t.camera = cam
    tid = ctypes.c_int32(-1)
    C.check(lib.er_bind_tracer(ctypes.byref(t), ctypes.byref(tid)))
    return tid.value


def single(torch, lib, tracer, w, h, spp, view, first, accumulate=0, init=None):
    d = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") if init is None else init.clone()
    C.check(lib.er_trace_sum_device(tracer, spp, view, first, d.data_ptr(), accumulate, None))
    torch.cuda.synchronize()
    return d.cpu().numpy()


def view_table(ra, rb):
    """(renderer, camera or None, spp, view, first) of six views of uneven size"""
    rng = np.random.default_rng(5)
    cam1 = S.orbit_camera(rng, (24, 20), radius=2.2)
    cam2 = S.orbit_camera(rng, (64, 16), radius=2.0)
    cam3 = S.orbit_camera(rng, (8, 8), radius=2.4)
    return [(ra, None, 5, 0, 0), (rb, None, 3, 1, 0), (ra, cam1, 7, 2, 0), (rb, cam2, 2, 3, 0), (ra, None, 4, 5, 11),
            (rb, cam3, 1, 6, 0)]


def make_batch(torch, lib, table, flags, window, accumulate=0):
    recs = (C.er_batch_view * len(table))()
    outs = []
    for i, (r, cam, spp, view, first) in enumerate(table):
        w, h = (cam.film_size[0], cam.film_size[1]) if cam is not None else (r.width, r.height)
        d = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
        outs.append(d)
        recs[i].tracer_id = r.tracer_id
        recs[i].spp = spp
        recs[i].view = view
        recs[i].first_sample = first
        recs[i].d_sum_xyza = d.data_ptr()
        recs[i].accumulate = accumulate
        recs[i].display = 0
        if cam is not None:
            recs[i].camera = ctypes.pointer(cam)
    bid = ctypes.c_int32(-1)
    C.check(lib.er_batch_create(recs, len(table), flags, window, ctypes.byref(bid)))
    return bid.value, outs


def expected(torch, lib, table):
    out = []
    for r, cam, spp, view, first in table:
        if cam is None:
            out.append(single(torch, lib, r.tracer_id, r.width, r.height, spp, view, first))
        else:
            tid = bind_with_camera(lib, r, cam)
            out.append(single(torch, lib, tid, cam.film_size[0], cam.film_size[1], spp, view, first))
            C.check(lib.er_unbind_tracer(tid))
    return out


@pytest.mark.parametrize("flags,window", [(0, 0), (C.ER_BATCH_GRAPH, 0), (0, 3000), (C.ER_BATCH_GRAPH, 3000), (C.ER_BATCH_GRAPH, 517)])
def test_batch_equals_single_views(torch, lib, pair, flags, window):
    ra, rb = pair
    table = view_table(ra, rb)
    ref = expected(torch, lib, table)
    bid, outs = make_batch(torch, lib, table, flags, window)
    nw, ns, qb = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int64(0)
    C.check(lib.er_batch_info(bid, ctypes.byref(nw), ctypes.byref(ns), ctypes.byref(qb)))
    if window:
        assert nw.value > 1 and ns.value > len(table)     # views cut across windows
    else:
        assert nw.value == 1 and ns.value == len(table)
    for _ in range(2):                                     # a replay gives the same sums
        C.check(lib.er_batch_launch(bid, None))
        torch.cuda.synchronize()
        for k, d in enumerate(outs):
            assert np.array_equal(bits(d.cpu().numpy()), bits(ref[k])), f"view {k}"
    C.check(lib.er_synchronize())
    C.check(lib.er_batch_destroy(bid))


def test_batch_tuning_variants_equal(torch, lib, pair):
    ra, rb = pair
    table = view_table(ra, rb)
    ref = expected(torch, lib, table)
    bid, outs = make_batch(torch, lib, table, C.ER_BATCH_GRAPH, 2000)
    for p, s in [(2, 8), (3, 6), (6, 3), (8, 2), (4, 4)]:
        C.check(lib.er_batch_set_tuning(bid, p, s))
        for d in outs:
            d.zero_()
        C.check(lib.er_batch_launch(bid, None))
        torch.cuda.synchronize()
        for k, d in enumerate(outs):
            assert np.array_equal(bits(d.cpu().numpy()), bits(ref[k])), f"tuning {p}/{s} view {k}"
    C.check(lib.er_batch_destroy(bid))


def test_batch_progressive_accumulation(torch, lib, pair):
    """launch, advance by spp, launch == two accumulating one-view calls"""
    ra, rb = pair
    table = [t for t in view_table(ra, rb) if t[4] == 0]
    bid, outs = make_batch(torch, lib, table, C.ER_BATCH_GRAPH, 1500, accumulate=1)
    C.check(lib.er_batch_launch(bid, None))
    spp0 = table[0][2]
    # every view advances by the same count; views with another spp skip or overlap samples, as documented
    C.check(lib.er_batch_advance(bid, spp0, None))
    C.check(lib.er_batch_launch(bid, None))
    torch.cuda.synchronize()
    for k, (r, cam, spp, view, first) in enumerate(table):
        tid = r.tracer_id if cam is None else bind_with_camera(lib, r, cam)
        w, h = (r.width, r.height) if cam is None else (cam.film_size[0], cam.film_size[1])
        d = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
        C.check(lib.er_trace_sum_device(tid, spp, view, 0, d.data_ptr(), 1, None))
        C.check(lib.er_trace_sum_device(tid, spp, view, spp0, d.data_ptr(), 1, None))
        torch.cuda.synchronize()
        if cam is not None:
            C.check(lib.er_unbind_tracer(tid))
        assert np.array_equal(bits(outs[k].cpu().numpy()), bits(d.cpu().numpy())), f"view {k}"
    C.check(lib.er_batch_destroy(bid))


def test_batch_display_equals_render_spp(torch, lib, runtime):
    """display pass: mean -> 3x3 Gaussian -> tone map -> bilateral, into the
    tracer's own buffers, equal to er_render_spp from a reset tracer"""
    sc = S.scene_tiny(seed=6)
    sc.tracer.settings.bilateral = 1
    r = runtime.Renderer(sc, lib)
    sc2 = S.scene_tiny(res=24, film=(32, 24), seed=7)
    r2 = runtime.Renderer(sc2, lib)
    try:
        spp = 6
        ref = []
        for rr in (r, r2):
            C.check(lib.er_reset_accumulation(rr.tracer_id))
            rr.render_spp(spp)
            ref.append((rr.get_estimate(), rr.get_running_estimate()))
            C.check(lib.er_reset_accumulation(rr.tracer_id))
        recs = (C.er_batch_view * 2)()
        for k, rr in enumerate((r, r2)):
            recs[k].tracer_id = rr.tracer_id
            recs[k].spp = spp
            recs[k].view = 0          # er_render_spp renders view 0 of each tracer's stream
            recs[k].first_sample = 0
            recs[k].d_sum_xyza = None  # the tracer's own sum buffer
            recs[k].accumulate = 0
            recs[k].display = 1
        bid = ctypes.c_int32(-1)
        C.check(lib.er_batch_create(recs, 2, C.ER_BATCH_GRAPH, 700, ctypes.byref(bid)))
        C.check(lib.er_batch_launch(bid, None))
        C.check(lib.er_synchronize())
        for rr, (e, run) in zip((r, r2), ref):
            assert np.array_equal(rr.get_estimate(), e)
            assert np.array_equal(bits(rr.get_running_estimate()), bits(run))
        C.check(lib.er_batch_destroy(bid))
    finally:
        r.close()
        r2.close()


def test_batch_replans_after_bind(torch, lib, pair):
    ra, rb = pair
    table = view_table(ra, rb)[:3]
    bid, outs = make_batch(torch, lib, table, C.ER_BATCH_GRAPH, 0)
    C.check(lib.er_batch_launch(bid, None))
    saved = C.er_tracer_desc.from_buffer_copy(ra.tracer_desc)
    try:
        ra.tracer_desc.settings.density_scale = 37.0
        ra.rebind_tracer()
        ref = expected(torch, lib, table)
        for d in outs:
            d.zero_()
        C.check(lib.er_batch_launch(bid, None))
        torch.cuda.synchronize()
        for k, d in enumerate(outs):
            assert np.array_equal(bits(d.cpu().numpy()), bits(ref[k])), f"view {k}"
    finally:
        ctypes.memmove(ctypes.byref(ra.tracer_desc), ctypes.byref(saved), ctypes.sizeof(saved))
        ra.rebind_tracer()
        C.check(lib.er_batch_destroy(bid))


def test_batch_argument_errors(torch, lib, pair):
    ra, rb = pair
    d = torch.zeros((ra.height, ra.width, 4), dtype=torch.float32, device="cuda")
    bid = ctypes.c_int32(-1)

    def create(recs, n=None):
        return lib.er_batch_create(recs, len(recs) if n is None else n, 0, 0, ctypes.byref(bid))

    recs = (C.er_batch_view * 2)()
    for i in range(2):
        recs[i].tracer_id = ra.tracer_id
        recs[i].spp = 2
        recs[i].d_sum_xyza = d.data_ptr()
    assert create(recs) == C.ER_ERR_INVALID_ARGUMENT          # two views share one sum buffer
    one = (C.er_batch_view * 1)()
    one[0].tracer_id = ra.tracer_id
    one[0].spp = 0
    one[0].d_sum_xyza = d.data_ptr()
    assert create(one) == C.ER_ERR_INVALID_ARGUMENT            # spp must be positive
    one[0].spp = 1
    one[0].tracer_id = 9999
    assert create(one) == C.ER_ERR_INVALID_ID
    one[0].tracer_id = ra.tracer_id
    cam = S.orbit_camera(np.random.default_rng(1), (16, 16))
    one[0].camera = ctypes.pointer(cam)
    one[0].d_sum_xyza = None
    assert create(one) == C.ER_ERR_INVALID_ARGUMENT            # a camera override needs its own buffer
    one[0].d_sum_xyza = d.data_ptr()
    one[0].display = 1
    assert create(one) == C.ER_ERR_INVALID_ARGUMENT            # and cannot use the tracer's display
    assert create(one, 0) == C.ER_ERR_INVALID_ARGUMENT
    assert lib.er_batch_launch(12345, None) == C.ER_ERR_INVALID_ID
    one[0].display = 0
    assert create(one) == C.ER_OK
    assert lib.er_batch_set_tuning(bid.value, 5, 0) == C.ER_ERR_INVALID_ARGUMENT
    C.check(lib.er_batch_destroy(bid.value))
    assert lib.er_batch_destroy(bid.value) == C.ER_ERR_INVALID_ID


def test_stage_profiler(torch, lib, pair):
    """er_profile_*: per-stage launch counts of a one-view render (one window)
    and of a batch launched without its graph; graph replays record nothing"""
    ra, rb = pair
    ms = np.zeros(4, dtype=np.float64)
    n = np.zeros(4, dtype=np.int64)
    C.check(lib.er_profile_read(ms.ctypes.data, n.ctypes.data))          # clear
    C.check(lib.er_profile_enable(1))
    d = torch.zeros((ra.height, ra.width, 4), dtype=torch.float32, device="cuda")
    C.check(lib.er_trace_sum_device(ra.tracer_id, 3, 0, 0, d.data_ptr(), 0, None))
    C.check(lib.er_profile_read(ms.ctypes.data, n.ctypes.data))
    assert list(n) == [1, 1, 1, 1] and (ms > 0).all()
    table = view_table(ra, rb)
    for flags in (0, C.ER_BATCH_GRAPH):
        bid, outs = make_batch(torch, lib, table, flags, 3000)
        nw = ctypes.c_int32(0)
        C.check(lib.er_batch_info(bid, ctypes.byref(nw), None, None))
        C.check(lib.er_profile_read(ms.ctypes.data, n.ctypes.data))      # the plan's capture records nothing either
        C.check(lib.er_batch_launch(bid, None))
        C.check(lib.er_profile_read(ms.ctypes.data, n.ctypes.data))
        assert list(n) == ([nw.value] * 4 if flags == 0 else [0, 0, 0, 0])
        C.check(lib.er_batch_destroy(bid))
    C.check(lib.er_profile_enable(0))
    C.check(lib.er_trace_sum_device(ra.tracer_id, 1, 0, 0, d.data_ptr(), 0, None))
    C.check(lib.er_profile_read(ms.ctypes.data, n.ctypes.data))
    assert list(n) == [0, 0, 0, 0]


def test_batch_stages_and_autotune(torch, lib, pair):
    """a batch's tune_stages (set or autotuned on whole launches) changes which
    kernels run, not the sums"""
    ra, rb = pair
    table = [(rb, None, 3, 1, 0), (rb, S.orbit_camera(np.random.default_rng(2), (40, 24), radius=2.1), 2, 2, 0)]
    ref = expected(torch, lib, table)
    bid, outs = make_batch(torch, lib, table, C.ER_BATCH_GRAPH, 0)
    for stages in (1, 1 | C.TUNE_NO_SKIP, 2, 3 | C.TUNE_NO_SKIP_SHADOW):
        C.check(lib.er_batch_set_stages(bid, stages))
        C.check(lib.er_batch_launch(bid, None))
        torch.cuda.synchronize()
        for k, d in enumerate(outs):
            assert np.array_equal(bits(d.cpu().numpy()), bits(ref[k])), (stages, k)
    st, m = ctypes.c_int32(-1), ctypes.c_float(0.0)
    C.check(lib.er_batch_autotune(bid, None, ctypes.byref(st), ctypes.byref(m)))
    assert 0 <= st.value <= 15 and m.value > 0
    # the tuner may have changed the tracer's majorant brick (which random
    # numbers a sample draws): the batch still equals the views rendered alone
    s = C.er_render_settings()
    C.check(lib.er_get_render_settings(rb.tracer_id, s))
    assert s.majorant_brick in (1, 2, 4, 8)
    orig = C.er_render_settings.from_buffer_copy(rb.tracer_desc.settings)
    rb.tracer_desc.settings = s                 # the camera-override view copies the descriptor
    ref2 = expected(torch, lib, table)
    C.check(lib.er_batch_launch(bid, None))
    torch.cuda.synchronize()
    for k, d in enumerate(outs):
        assert np.array_equal(bits(d.cpu().numpy()), bits(ref2[k]))
    assert lib.er_batch_set_stages(bid, 16) == C.ER_ERR_INVALID_ARGUMENT
    C.check(lib.er_batch_destroy(bid))
    rb.tracer_desc.settings = orig
    rb.rebind_tracer()          # the fixture's settings for the tests that follow
