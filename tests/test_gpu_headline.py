"""The measured workloads themselves against the CPU oracle, bit for bit,
through the C ABI: crops of the 512^3 CT-like c2 scene on the reference's
live path (fixed-step march, BRDF, light sampling) and on the fast path the
benchmark times (delta tracking, hybrid shader, full MIS, stratified
samples); one view of each c3 volume inside a batch of all 64 c3 views; and
a crop of a volume with more than 2^30 voxels (64-bit voxel, corner-quad and
brick indices), whose majorant grid at 1^3 bricks (more than 2^30 bricks) is
checked against numpy.  The GPU renders whole films; the oracle renders
crops of them.  Float XYZA sums compared as uint32."""
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


def compare_crops(gpu, h, spp, crops, view=0, first=0):
    for (x0, y0, w, hh) in crops:
        cpu = h.render_sum(spp, view=view, first=first, rect=(x0, y0, w, hh), nthreads=16)
        g = gpu[y0:y0 + hh, x0:x0 + w]
        assert np.array_equal(bits(g), bits(cpu)), "crop %s: %d of %d pixels differ" % ((x0, y0, w, hh), int((g != cpu).any(-1).sum()),
                                                                                     w * hh)
        assert cpu[..., 3].sum() > 0.0, "crop %s sees no volume" % ((x0, y0, w, hh),)


# crops of the 1024^2 c2 film: the volume centre (inner shells), the
# ellipsoid's edge and a region between the shells
C2_CROPS = [(496, 496, 32, 32), (300, 620, 24, 24), (640, 380, 24, 24)]


@pytest.fixture(scope="module")
def c2():
    return S.scene_c2(res=512, film=(1024, 1024))


def test_c2_reference_order_crops(torch, lib, runtime, oracle, c2):
    """The reference's live estimator on the c2 workload (bench.py's
    reference_order figure): fixed-step march, BRDF at every volume event,
    light sampling only"""
    sc = S.Scene(c2.name, c2.volume, tracer=C.er_tracer_desc.from_buffer_copy(c2.tracer), lights=c2.lights, textures=c2.textures)
    s = sc.tracer.settings
    s.free_flight, s.mis, s.apply_shading_type, s.stratify = 0, 0, 0, 0
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        compare_crops(dev_sum(torch, r, 2, view=3, first=1), h, 2, C2_CROPS, view=3, first=1)
    finally:
        r.close()
        h.close()


@pytest.mark.parametrize("stages", [0, C.PERSISTENT_BOTH, C.PERSISTENT_PRIMARY | C.TUNE_NO_SKIP_SHADOW])
def test_c2_fast_path_crops(torch, lib, runtime, oracle, c2, stages):
    """The benchmark's estimator on the c2 workload: delta tracking over 8^3
    majorant bricks, ratio-tracked shadows, hybrid shader, full MIS,
    stratified samples (the per-thread and persistent-lane stages; the
    ER_TUNE_NO_SKIP_* bits are accepted and ignored)"""
    sc = S.Scene(c2.name, c2.volume, tracer=C.er_tracer_desc.from_buffer_copy(c2.tracer), lights=c2.lights, textures=c2.textures)
    s = sc.tracer.settings
    s.free_flight, s.mis, s.stratify, s.majorant_brick, s.tune_stages = 1, 1, 1, 8, stages
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        compare_crops(dev_sum(torch, r, 4, view=0, first=8), h, 4, C2_CROPS, view=0, first=8)
    finally:
        r.close()
        h.close()


def test_c3_views_inside_the_batch(torch, lib, runtime, oracle):
    """All 64 c3 views in one CUDA-graph batch, each at its full spp, with
    the benchmark's per-volume bricks (1, 4, 4) and persistent-lane stages;
    the first view of each of the three volumes (96^3, 256^3, 384x384x256)
    is compared with the oracle on a crop through its centre"""
    scenes = S.c3_scenes()
    views = S.c3_views()
    for sc, b in zip(scenes, (1, 4, 4)):
        sc.tracer.settings.majorant_brick = b
        sc.tracer.settings.tune_stages = C.PERSISTENT_BOTH | C.TUNE_NO_SKIP_SHADOW
    rs = [runtime.Renderer(sc, lib) for sc in scenes]
    sums = [torch.zeros((cam.film_size[1], cam.film_size[0], 4), dtype=torch.float32, device="cuda") for _, cam, _ in views]
    batch = runtime.Batch([(rs[k].tracer_id, spp, d.data_ptr(), cam) for (k, cam, spp), d in zip(views, sums)],
                          flags=C.ER_BATCH_GRAPH, lib=lib)
    try:
        batch.launch(None)
        torch.cuda.synchronize()
        done = set()
        for i, (k, cam, spp) in enumerate(views):
            if k in done:
                continue
            done.add(k)
            sc = S.Scene(scenes[k].name, scenes[k].volume, tracer=C.er_tracer_desc.from_buffer_copy(scenes[k].tracer),
                         lights=scenes[k].lights, textures=scenes[k].textures)
            sc.tracer.camera = cam
            W, H = cam.film_size[0], cam.film_size[1]
            h = OL.SceneHandle(oracle, sc)
            try:
                compare_crops(sums[i].cpu().numpy(), h, spp, [(W // 2 - 8, H // 2 - 8, 16, 16)], view=i)
            finally:
                h.close()
        assert done == {0, 1, 2}
    finally:
        batch.close()
        for r in rs:
            r.close()


# more than 2^30 voxels: 1024 x 1024 x 1088 (x, y, z); the voxels' byte
# offsets pass 2^31 and the corner quads' 2^33
BIG = (1088, 1024, 1024)


@pytest.fixture(scope="module")
def big_volume():
    return S.lattice_volume(BIG)


@pytest.mark.parametrize("free_flight", [1, 0])
def test_large_volume_crop(torch, lib, runtime, oracle, big_volume, free_flight):
    """Crops through a volume of 1.14e9 voxels filled in every slice, seen
    from above so that the collisions fall in the highest slices (voxel
    indices above 2^30): delta tracking over 8^3 bricks with full MIS and
    stratified samples, and the fixed-step march; the c2 lights and
    transfer functions, BRDF shading"""
    assert big_volume.size > (1 << 30)
    lights, textures = S.c2_lights()
    t = S.c2_tracer((96, 96))
    s = t.settings
    s.free_flight, s.mis, s.stratify, s.majorant_brick, s.bilateral, s.apply_shading_type = free_flight, 1, free_flight, 8, 0, 0
    t.camera = S.make_camera((96, 96), (0.15, -0.35, 1.2), (0.0, 0.0, 0.1), (0.0, 1.0, 0.0), fov=40.0)
    sc = S.Scene("big", big_volume, tracer=t, lights=lights, textures=textures)
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        if free_flight:
            compare_crops(dev_sum(torch, r, 3, view=1), h, 3, [(40, 40, 16, 16), (0, 0, 12, 12), (80, 10, 16, 16)], view=1)
        else:
            compare_crops(dev_sum(torch, r, 1, view=1), h, 1, [(44, 44, 8, 8), (4, 80, 8, 8)], view=1)
        assert OL.render_stats(oracle)["lookups"] > 10.0
    finally:
        r.close()
        h.close()


def test_majorant_grid_beyond_2e30_bricks(torch, lib, big_volume):
    """er_build_majorant_device at 1^3 bricks of the 1.14e9-voxel volume
    (more than 2^30 bricks, each the max of sigma over the 2^3 voxels of its
    footprint): slabs at both ends of the grid equal numpy's"""
    Z, Y, X = big_volume.shape
    vol = torch.from_numpy(big_volume.view(np.int16)).cuda()
    vmax = int(big_volume.max())
    # an opacity ramp with flat steps, as the workloads' transfer functions
    sigma = np.clip((np.arange(vmax + 1, dtype=np.float32) - 900.0) / 1600.0, 0.0, 1.0).astype(np.float32) * np.float32(100.0)
    d_sigma = torch.from_numpy(sigma).cuda()
    maj = torch.empty((Z, Y, X), dtype=torch.float32, device="cuda")
    res = (ctypes.c_int32 * 3)(X, Y, Z)
    C.check(lib.er_build_majorant_device(ctypes.c_void_p(vol.data_ptr()), res, 1, ctypes.c_void_p(d_sigma.data_ptr()), vmax + 1,
                                         ctypes.c_float(100.0), ctypes.c_void_p(maj.data_ptr()), None))
    torch.cuda.synchronize()
    del vol
    for z in (0, 1, Z // 2, Z - 2, Z - 1):
        # a 1^3 brick b covers the voxels [b, b + 1] a lookup clamped to it
        # blends, clamped to the volume
        lo, hi = z, min(z + 2, Z)
        slab = big_volume[lo:hi].astype(np.int32)
        mx = slab.max(axis=0)
        mn = slab.min(axis=0)
        pad_mx = np.pad(mx, ((0, 1), (0, 1)), mode="edge")
        pad_mn = np.pad(mn, ((0, 1), (0, 1)), mode="edge")
        offs = (0, 1)
        bmx = np.max([pad_mx[dy:dy + Y, dx:dx + X] for dy in offs for dx in offs], axis=0)
        bmn = np.min([pad_mn[dy:dy + Y, dx:dx + X] for dy in offs for dx in offs], axis=0)
        # max of sigma over [bmn - 1, bmx]: sigma is non-decreasing here, so sigma[bmx]
        expect = np.float32(100.0) * sigma[bmx]
        assert (bmn <= bmx).all()
        got = maj[z].cpu().numpy()
        nonempty = expect > 0.0
        assert np.array_equal(got[nonempty], expect[nonempty]), f"slab {z}"
        assert (got[~nonempty] <= 0.0).all(), f"slab {z}"


def test_c2_bricked_quad_layout(torch, lib, runtime, oracle, c2, monkeypatch):
    """The corner quads in 8^3 bricks (ER_QUAD_LAYOUT=bricked at bind time)
    read the same intensities: the c2 fast path's crops stay bit-exact, and
    the whole film equals the x-fastest layout's"""
    sc = S.Scene(c2.name, c2.volume, tracer=C.er_tracer_desc.from_buffer_copy(c2.tracer), lights=c2.lights, textures=c2.textures)
    s = sc.tracer.settings
    s.free_flight, s.mis, s.stratify, s.majorant_brick = 1, 1, 1, 8
    r = runtime.Renderer(sc, lib)
    try:
        flat = dev_sum(torch, r, 2, view=4)
    finally:
        r.close()
    monkeypatch.setenv("ER_QUAD_LAYOUT", "bricked")
    r = runtime.Renderer(sc, lib)
    h = OL.SceneHandle(oracle, sc)
    try:
        bricked = dev_sum(torch, r, 2, view=4)
        assert np.array_equal(bits(bricked), bits(flat))
        compare_crops(bricked, h, 2, C2_CROPS[:2], view=4)
    finally:
        r.close()
        h.close()
