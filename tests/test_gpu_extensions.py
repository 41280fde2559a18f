"""GPU extension estimators (delta/ratio tracking, hybrid shader switch,
full MIS) against the oracle's restatement: bit-exact per path."""
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


def two_light_scene(seed, film=(24, 20)):
    sc = S.scene_tiny(res=20, film=film, seed=seed)
    tm = np.eye(4).tolist()
    envl = C.er_light_desc()
    envl.visible = 1
    envl.shape = S.make_shape(C.SHAPE_SPHERE, (tm, tm), outer=3.0)
    envl.texture_id = 1
    envl.multiplier = 0.5
    sc.lights.append(envl)
    sc.textures.append(S.gradient_texture([(0.0, (0.2, 0.2, 0.3)), (1.0, (1.0, 1.0, 1.0))]))
    sc.tracer.light_count = 2
    sc.tracer.light_ids[1] = 1
    return sc


MODES = [
    dict(free_flight=1),
    dict(free_flight=1, majorant_brick=4),
    dict(free_flight=1, majorant_brick=16),
    dict(free_flight=0, mis=1),
    dict(free_flight=1, mis=1),
    dict(free_flight=0, apply_shading_type=1, shading_type=1),
    dict(free_flight=1, mis=1, apply_shading_type=1, shading_type=1),
    dict(free_flight=1, mis=1, apply_shading_type=1, shading_type=2),
    dict(free_flight=0, mis=0, apply_shading_type=1, shading_type=2, opacity_modulated=0),
    dict(free_flight=1, mis=1, apply_shading_type=1, shading_type=3),
    dict(free_flight=1, mis=0, apply_shading_type=1, shading_type=4),
]


@pytest.mark.parametrize("mode", MODES, ids=[",".join(f"{k}={v}" for k, v in m.items()) for m in MODES])
def test_extension_mode_bit_exact(env, oracle, mode):
    torch, lib, rt = env
    sc = two_light_scene(9)
    for k, v in mode.items():
        setattr(sc.tracer.settings, k, v)
    r = rt.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        d = torch.zeros((sc.height, sc.width, 4), dtype=torch.float32, device="cuda")
        r.trace_sum_device(d.data_ptr(), 4, 3, 5, 0, None)
        torch.cuda.synchronize()
        cpu = h.render_sum(4, view=3, first=5, nthreads=4)
        g = d.cpu().numpy()
        assert np.array_equal(bits(g), bits(cpu))
        assert cpu[..., 3].sum() > 0
    finally:
        r.close()
        h.close()


def test_delta_c1_crop_bit_exact(env, oracle):
    torch, lib, rt = env
    sc = S.scene_c1()
    sc.tracer.settings.free_flight = 1
    sc.tracer.settings.mis = 1
    r = rt.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        d = torch.zeros((sc.height, sc.width, 4), dtype=torch.float32, device="cuda")
        r.trace_sum_device(d.data_ptr(), 8, 0, 0, 0, None)
        torch.cuda.synchronize()
        cpu = h.render_sum(8, rect=(100, 96, 48, 40), nthreads=8)
        assert np.array_equal(bits(d.cpu().numpy()[96:136, 100:148]), bits(cpu))
    finally:
        r.close()
        h.close()


def sigma_table(oracle, plf, n, ds):
    xs = np.arange(n, dtype=np.float32)
    op = np.zeros(n, np.float32)
    oracle.plf_evaluate(OL.ctypes.byref(plf), n, OL.ptr(xs), OL.ptr(op))
    return (np.float32(ds) * op).astype(np.float32)


@pytest.mark.parametrize("shape,brick", [((20, 24, 28), 8), ((33, 17, 40), 4), ((16, 16, 16), 16), ((9, 10, 11), 1), ((40, 40, 40), 64)])
def test_majorant_grid_device_bit_exact(env, oracle, shape, brick):
    torch, lib, rt = env
    vol = S.blob_volume(shape, n_blobs=5, seed=brick)
    plf = C.make_plf([(0.0, 0.0), (300.0, 0.0), (1200.0, 0.7), (3000.5, 1.0)])
    n = int(vol.max()) + 1
    ds = 100.0
    sig = sigma_table(oracle, plf, n, ds)
    res = np.array([shape[2], shape[1], shape[0]], np.int32)
    nb = [(int(r) + brick - 1) // brick for r in res]
    want = np.zeros(nb[0] * nb[1] * nb[2], np.float32)
    oracle.majorant_grid(OL.ptr(vol), OL.ptr(res), brick, OL.ptr(sig), n, ds, OL.ptr(want))
    d_vol = torch.from_numpy(vol.view(np.int16).copy()).cuda()
    d_sig = torch.from_numpy(sig).cuda()
    d_out = torch.full((want.size,), -1.0, dtype=torch.float32, device="cuda")
    C.check(lib.er_build_majorant_device(d_vol.data_ptr(), res.ctypes.data_as(OL.ctypes.POINTER(OL.ctypes.c_int32)), brick,
                                         d_sig.data_ptr(), n, ds, d_out.data_ptr(), None))
    torch.cuda.synchronize()
    assert np.array_equal(bits(d_out.cpu().numpy()), bits(want))
    assert want.max() > 0


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 0 | 12, 1 | 12, 1 | 8, 2 | 4], ids=["shadow", "both", "none", "primary", "shadow-noskip",
                                                                        "both-noskip", "both-skip-primary", "none-skip-shadow"])
def test_persistent_stage_modes_bit_exact(env, oracle, mode):
    """every persistent-lane mode of the delta-tracking stages (tune_stages;
    the ER_TUNE_NO_SKIP_* bits are accepted and ignored) gives the oracle's
    sums with the hybrid shader and full MIS"""
    torch, lib, rt = env
    sc = two_light_scene(13)
    sc.tracer.settings.free_flight = 1
    sc.tracer.settings.mis = 1
    sc.tracer.settings.apply_shading_type = 1
    sc.tracer.settings.shading_type = 2
    sc.tracer.settings.tune_stages = mode
    r = rt.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        for tp, ts in ((4, 4), (2, 3), (8, 8)):
            r.tracer_desc.settings.tune_primary, r.tracer_desc.settings.tune_shadow = tp, ts
            r.rebind_tracer()
            d = torch.zeros((sc.height, sc.width, 4), dtype=torch.float32, device="cuda")
            r.trace_sum_device(d.data_ptr(), 5, 1, 2, 0, None)
            torch.cuda.synchronize()
            assert np.array_equal(bits(d.cpu().numpy()), bits(h.render_sum(5, view=1, first=2, nthreads=4))), (tp, ts)
    finally:
        r.close()
        h.close()


@pytest.mark.parametrize("stages", [0, 1, 2], ids=["persistent-shadow", "persistent-both", "per-thread"])
def test_stratified_light_samples_bit_exact(env, oracle, stages):
    """settings.stratify on the GPU (wavefront stages in each mode, the
    one-kernel path) gives the oracle's sums"""
    torch, lib, rt = env
    sc = two_light_scene(17)
    sc.tracer.settings.free_flight = 1
    sc.tracer.settings.mis = 1
    sc.tracer.settings.stratify = 1
    sc.tracer.settings.tune_stages = stages
    h = OL.SceneHandle(oracle, sc)
    cpu = h.render_sum(6, view=2, first=7, nthreads=4)
    h.close()
    for engine in (2, 1):
        sc.tracer.settings.engine = engine
        r = rt.Renderer(sc, lib)
        try:
            d = torch.zeros((sc.height, sc.width, 4), dtype=torch.float32, device="cuda")
            r.trace_sum_device(d.data_ptr(), 6, 2, 7, 0, None)
            torch.cuda.synchronize()
            assert np.array_equal(bits(d.cpu().numpy()), bits(cpu)), engine
        finally:
            r.close()
    sc.tracer.settings.stratify = 0
    h = OL.SceneHandle(oracle, sc)
    assert not np.array_equal(h.render_sum(6, view=2, first=7, nthreads=4), cpu)
    h.close()


def sparse_scene(film=(40, 32)):
    """80^3 voxels, empty but for two small dense boxes: empty-space
    distances run up to the 32-brick cap at 1^3 and 2^3 bricks"""
    vol = np.zeros((80, 80, 80), dtype=np.uint16)
    vol[10:30, 8:28, 12:34] = 3000
    vol[50:66, 54:72, 44:60] = 2200
    lights, textures = S.c1_lights()
    return S.Scene("sparse", vol, tracer=S.c1_tracer(film), lights=lights, textures=textures)


@pytest.mark.parametrize("brick,stages,engine", [(1, 0, 0), (1, 1, 0), (1, 2, 0), (2, 0, 0), (2, 1, 0), (2, 3, 0), (1, 0, 1), (2, 0, 1)],
                         ids=["b1-persistent-shadow", "b1-persistent-both", "b1-per-thread", "b2-persistent-shadow",
                              "b2-persistent-both", "b2-persistent-primary", "b1-one-kernel", "b2-one-kernel"])
def test_empty_space_jump_bit_exact(env, oracle, brick, stages, engine):
    """delta and ratio tracking that jump across cubes of empty bricks (the
    wavefront stages in each persistent-lane mode and the one-kernel path)
    give the oracle's sums bit for bit"""
    torch, lib, rt = env
    sc = sparse_scene()
    s = sc.tracer.settings
    s.free_flight, s.mis, s.majorant_brick, s.tune_stages, s.engine = 1, 1, brick, stages, engine
    r = rt.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        d = torch.zeros((sc.height, sc.width, 4), dtype=torch.float32, device="cuda")
        r.trace_sum_device(d.data_ptr(), 4, 2, 1, 0, None)
        torch.cuda.synchronize()
        cpu = h.render_sum(4, view=2, first=1, nthreads=4)
        assert np.array_equal(bits(d.cpu().numpy()), bits(cpu))
        assert cpu[..., 3].sum() > 0
    finally:
        r.close()
        h.close()


@pytest.mark.parametrize("shading", [2, 3, 4], ids=["hybrid", "modulation", "threshold"])
@pytest.mark.parametrize("tune_shade", [2, 3, 4, 6])
def test_sorted_shade_stage_bit_exact(env, oracle, shading, tune_shade):
    """a shader switch that mixes BRDF and phase events runs the shade stage
    as classification + shading sorted by shader (k_wf_classify,
    k_wf_shade_sorted) in every occupancy variant: the oracle's sums"""
    torch, lib, rt = env
    sc = two_light_scene(17)
    s = sc.tracer.settings
    s.free_flight, s.mis, s.apply_shading_type, s.shading_type, s.tune_shade = 1, 1, 1, shading, tune_shade
    r = rt.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        d = torch.zeros((sc.height, sc.width, 4), dtype=torch.float32, device="cuda")
        r.trace_sum_device(d.data_ptr(), 6, 4, 3, 0, None)
        torch.cuda.synchronize()
        cpu = h.render_sum(6, view=4, first=3, nthreads=4)
        assert np.array_equal(bits(d.cpu().numpy()), bits(cpu))
        assert cpu[..., 3].sum() > 0
    finally:
        r.close()
        h.close()
