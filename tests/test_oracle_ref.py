"""The C restatement against the reference's own code built on this host
(oracle/_ref/liberref.so), on fresh inputs.  Skipped where the reference
sources were not available at build time."""
import ctypes

import numpy as np
import pytest

import oracle_lib as OL

C = OL.C
S = OL.PKG.scenes


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def scenes(oracle, ref):
    sc = S.scene_tiny(res=24, film=(36, 28), seed=11)
    sc.tracer.camera.aperture_size = 0.05          # thin-lens path (Source/singlescattering.h:41-49)
    yield sc, OL.SceneHandle(oracle, sc), OL.SceneHandle(ref, sc)


def test_frames_bit_exact(scenes):
    sc, a, b = scenes
    la = OL.initial_lanes(9, sc.width, sc.height)
    lb = la.copy()
    for _ in range(2):
        assert np.array_equal(bits(a.render_frame(la, 4)), bits(b.render_frame(lb, 4)))
        assert np.array_equal(la, lb)


@pytest.mark.parametrize("gradient_mode", [0, 1, 2])
@pytest.mark.parametrize("shape", ["plane", "disk", "ring", "box", "sphere"])
def test_light_shapes_and_gradients(oracle, ref, shape, gradient_mode):
    sc = S.scene_tiny(res=20, film=(24, 20), seed=5)
    L = sc.lights[0]
    st = {"plane": C.SHAPE_PLANE, "disk": C.SHAPE_DISK, "ring": C.SHAPE_RING, "box": C.SHAPE_BOX, "sphere": C.SHAPE_SPHERE}[shape]
    L.shape.type = st
    L.shape.inner_radius, L.shape.outer_radius = 0.1, 0.3
    L.shape.size[0], L.shape.size[1], L.shape.size[2] = 0.4, 0.3, 0.2
    L.shape.one_sided = 1 if shape in ("plane", "disk") else 0
    L.unit = C.UNIT_LUX if shape in ("disk", "box") else C.UNIT_POWER
    sc.tracer.settings.gradient_computation = gradient_mode
    a, b = OL.SceneHandle(oracle, sc), OL.SceneHandle(ref, sc)
    assert np.array_equal(bits(a.render_sum(3, nthreads=4)), bits(b.render_sum(3, nthreads=4)))


def test_environment_sphere_and_gradient_texture(oracle, ref):
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
    a, b = OL.SceneHandle(oracle, sc), OL.SceneHandle(ref, sc)
    assert np.array_equal(bits(a.render_sum(4, nthreads=4)), bits(b.render_sum(4, nthreads=4)))


def test_kats_against_reference(oracle, ref, scenes):
    sc, a, b = scenes
    rng = np.random.default_rng(3)
    pts = rng.uniform(-0.6, 0.6, size=(500, 3)).astype(np.float32)
    for name, width in (("get_intensity", 1), ("normalized_gradient", 3), ("gradient_magnitude", 1)):
        oa = np.zeros((500, width), np.float32)
        ob = np.zeros((500, width), np.float32)
        getattr(oracle, name)(a.h, 500, OL.ptr(pts), OL.ptr(oa))
        getattr(ref, name)(b.h, 500, OL.ptr(pts), OL.ptr(ob))
        assert np.array_equal(bits(oa), bits(ob)), name
    rays = np.concatenate([rng.uniform(-2, 2, (500, 3)), rng.normal(size=(500, 3)), np.zeros((500, 1)), np.full((500, 1), 10.0)], 1).astype(np.float32)
    ia = np.zeros((500, 3), np.float32)
    ib = np.zeros((500, 3), np.float32)
    oracle.intersect_volume_box(a.h, 500, OL.ptr(rays), OL.ptr(ia))
    ref.intersect_volume_box(b.h, 500, OL.ptr(rays), OL.ptr(ib))
    assert np.array_equal(bits(ia), bits(ib))
    u = rng.uniform(0, 1, (500, 2)).astype(np.float32)
    u[0] = 0.5
    da = np.zeros((500, 2), np.float32)
    db = np.zeros((500, 2), np.float32)
    oracle.concentric_sample_disk(500, OL.ptr(u), OL.ptr(da))
    ref.concentric_sample_disk(500, OL.ptr(u), OL.ptr(db))
    assert np.array_equal(bits(da), bits(db))
    for x, y in ((0, 0), (17, 5), (35, 27)):
        uv = rng.uniform(0, 1, 4).astype(np.float32)
        ra = np.zeros(6, np.float32)
        rb = np.zeros(6, np.float32)
        oracle.camera_ray(a.h, x, y, OL.ptr(uv), OL.ptr(ra))
        ref.camera_ray(b.h, x, y, OL.ptr(uv), OL.ptr(rb))
        assert np.array_equal(bits(ra), bits(rb))


def test_post_pipeline(oracle, ref):
    rng = np.random.default_rng(4)
    W, H = 19, 13
    ra = np.zeros((H, W, 4), np.float32)
    rb = ra.copy()
    for n in range(4):
        f = rng.uniform(0, 2, (H, W, 4)).astype(np.float32)
        f[..., 3] = (rng.uniform(0, 1, (H, W)) > 0.4).astype(np.float32)
        fa, fb = f.copy(), f.copy()
        ga = np.zeros((H, W, 4), np.uint8)
        gb = ga.copy()
        oracle.post_frame(OL.ptr(fa), OL.ptr(ra), OL.ptr(ga), W, H, n, 1.3)
        ref.post_frame(OL.ptr(fb), OL.ptr(rb), OL.ptr(gb), W, H, n, 1.3)
        assert np.array_equal(bits(fa), bits(fb))
        assert np.array_equal(bits(ra), bits(rb))
        assert np.array_equal(ga, gb)


def test_plf_random_unsorted(oracle, ref):
    rng = np.random.default_rng(8)
    for trial in range(20):
        n = int(rng.integers(0, 130))
        plf = C.make_plf([(float(p), float(v)) for p, v in zip(rng.uniform(-100, 5000, n), rng.uniform(0, 1, n))])
        xs = np.concatenate([rng.uniform(-200, 5200, 200), np.array([plf.position[i] for i in range(plf.count)])]).astype(np.float32)
        ya = np.zeros_like(xs)
        yb = np.zeros_like(xs)
        oracle.plf_evaluate(ctypes.byref(plf), len(xs), OL.ptr(xs), OL.ptr(ya))
        ref.plf_evaluate(ctypes.byref(plf), len(xs), OL.ptr(xs), OL.ptr(yb))
        assert np.array_equal(bits(ya), bits(yb))
        assert plf.count <= 127


def test_surface_objects_sum_and_frames(oracle, ref):
    """objects (SampleRay's third event type, Source/objects.h) against the
    reference: textured floor and sphere, shadowed by and shadowing the volume"""
    sc = S.scene_objects()
    a, b = OL.SceneHandle(oracle, sc), OL.SceneHandle(ref, sc)
    sa = a.render_sum(4, nthreads=4)
    assert np.array_equal(bits(sa), bits(b.render_sum(4, nthreads=4)))
    la = OL.initial_lanes(21, sc.width, sc.height)
    lb = la.copy()
    for _ in range(2):
        assert np.array_equal(bits(a.render_frame(la, 4)), bits(b.render_frame(lb, 4)))
    sc.tracer.object_count = 0
    c = OL.SceneHandle(oracle, sc)
    assert not np.array_equal(sa, c.render_sum(4, nthreads=4))       # the objects show


@pytest.mark.parametrize("shape", ["disk", "ring", "box"])
def test_surface_object_shapes(oracle, ref, shape):
    sc = S.scene_objects(res=20, film=(28, 24), seed=8)
    st = {"disk": C.SHAPE_DISK, "ring": C.SHAPE_RING, "box": C.SHAPE_BOX}[shape]
    sh = sc.objects[1].shape
    sh.type = st
    sh.inner_radius, sh.outer_radius = 0.1, 0.3
    sh.size[0], sh.size[1], sh.size[2] = 0.4, 0.3, 0.2
    sc.objects[0].glossiness_texture_id = 2                     # luminance of a checker
    a, b = OL.SceneHandle(oracle, sc), OL.SceneHandle(ref, sc)
    assert np.array_equal(bits(a.render_sum(3, nthreads=4)), bits(b.render_sum(3, nthreads=4)))


def test_bitmap_textures(oracle, ref):
    """bitmap textures on a light and on objects (Source/textures.h:101-107,
    Source/buffer2d.h:227-254) against the reference"""
    sc = S.scene_bitmaps()
    a, b = OL.SceneHandle(oracle, sc), OL.SceneHandle(ref, sc)
    sa = a.render_sum(4, nthreads=4)
    assert np.array_equal(bits(sa), bits(b.render_sum(4, nthreads=4)))
    assert sa[..., :3].max() > 0
    sc.tracer.settings.free_flight = 1
    sc.tracer.settings.mis = 1
    c = OL.SceneHandle(oracle, sc)
    assert c.render_sum(2, nthreads=4)[..., :3].max() > 0


def random_scene(seed):
    """A scene on the reference's live path with every parameter drawn from a
    seeded generator: a non-cubic blob volume with anisotropic spacing, random
    unsorted transfer-function nodes, step factors, shadow settings and
    gradient mode, an orbit camera (thin lens on odd seeds), and one to three
    lights of random shape, orientation, size, sidedness, unit and texture
    (uniform, checker or gradient with random offset, repeat and flips).
    The volume's size is normalised: without NormalizeSize the reference
    scales the spacing by 0 (Source/volume.h:106-114), an empty box, which
    test_volume_without_normalize_size_is_empty covers."""
    rng = np.random.default_rng(1000 + seed)
    shape_zyx = tuple(int(v) for v in rng.integers(10, 26, size=3))
    sc = S.scene_tiny(res=16, film=(22, 18), seed=3)
    sc.volume = S.blob_volume(shape_zyx, n_blobs=5, seed=seed + 20)
    sc.spacing = tuple(float(v) for v in rng.uniform(0.6, 1.8, size=3))
    sc.normalize_size = 1
    t = sc.tracer

    def nodes(n, lo, hi):
        return [(float(rng.uniform(0.0, 4500.0)), float(rng.uniform(lo, hi))) for _ in range(n)]

    t.opacity = C.make_plf(nodes(int(rng.integers(2, 8)), 0.0, 1.0))
    t.diffuse = C.make_color_tf([(p, tuple(float(x) for x in rng.uniform(0.1, 1.0, 3)))
                                 for p, _ in nodes(int(rng.integers(1, 5)), 0, 1)])
    t.specular = C.make_color_tf([(p, tuple(float(x) for x in rng.uniform(0.0, 0.5, 3)))
                                  for p, _ in nodes(int(rng.integers(1, 4)), 0, 1)])
    t.glossiness = C.make_plf(nodes(int(rng.integers(1, 4)), 0.05, 0.95))
    t.emission = C.make_color_tf([(p, tuple(float(x) for x in rng.uniform(0.0, 0.3, 3)))
                                  for p, _ in nodes(int(rng.integers(1, 3)), 0, 1)])
    s = t.settings
    s.density_scale = float(rng.uniform(20.0, 200.0))
    s.step_factor_primary = float(rng.uniform(0.5, 2.0))
    s.step_factor_shadow = float(rng.uniform(0.5, 3.0))
    s.shadows = int(rng.integers(0, 2))
    s.max_shadow_distance = float(rng.uniform(0.3, 1.5))
    s.gradient_computation = int(rng.integers(0, 3))
    s.seed = int(rng.integers(1, 1 << 30))
    cam = S.orbit_camera(rng, (22, 18), radius=float(rng.uniform(1.6, 2.6)), fov=float(rng.uniform(25.0, 55.0)),
                         exposure=float(rng.uniform(0.5, 2.0)))
    if seed % 2:
        cam.aperture_size = float(rng.uniform(0.01, 0.08))
        cam.focal_distance = float(rng.uniform(1.0, 2.5))
    t.camera = cam
    sc.textures = []
    for k in range(3):
        kind = int(rng.integers(0, 3))
        if kind == 0:
            tex = S.uniform_texture(tuple(float(x) for x in rng.uniform(0.3, 1.0, 3)), level=float(rng.uniform(0.5, 2.0)))
        elif kind == 1:
            tex = S.checker_texture(tuple(float(x) for x in rng.uniform(0.0, 1.0, 3)),
                                    tuple(float(x) for x in rng.uniform(0.0, 1.0, 3)),
                                    level=float(rng.uniform(0.5, 2.0)), repeat=tuple(float(x) for x in rng.uniform(0.5, 4.0, 2)))
        else:
            tex = S.gradient_texture([(0.0, tuple(float(x) for x in rng.uniform(0, 1, 3))),
                                      (float(rng.uniform(0.2, 0.8)), tuple(float(x) for x in rng.uniform(0, 1, 3))),
                                      (1.0, tuple(float(x) for x in rng.uniform(0, 1, 3)))],
                                     level=float(rng.uniform(0.5, 2.0)))
        tex.offset[0], tex.offset[1] = (float(x) for x in rng.uniform(-0.5, 0.5, 2))
        tex.flip[0], tex.flip[1] = (int(x) for x in rng.integers(0, 2, 2))
        sc.textures.append(tex)
    shapes = [C.SHAPE_PLANE, C.SHAPE_DISK, C.SHAPE_RING, C.SHAPE_BOX, C.SHAPE_SPHERE]
    sc.lights = []
    n_lights = int(rng.integers(1, 4))
    for i in range(n_lights):
        L = C.er_light_desc()
        L.visible = int(rng.integers(0, 2))
        d = rng.normal(size=3)
        pos = tuple(float(x) for x in d / np.linalg.norm(d) * rng.uniform(0.9, 1.6))
        up = tuple(float(x) for x in rng.normal(size=3))
        st = shapes[int(rng.integers(0, len(shapes)))]
        inner = float(rng.uniform(0.05, 0.15))
        L.shape = S.make_shape(st, S.look_at_tm(pos, (0.0, 0.0, 0.0), up),
                               size=tuple(float(x) for x in rng.uniform(0.2, 0.6, 3)),
                               inner=inner, outer=inner + float(rng.uniform(0.1, 0.3)),
                               one_sided=int(rng.integers(0, 2)) if st in (C.SHAPE_PLANE, C.SHAPE_DISK, C.SHAPE_RING) else 0)
        L.texture_id = int(rng.integers(0, len(sc.textures)))
        L.multiplier = float(rng.uniform(2.0, 30.0))
        L.unit = int(rng.integers(0, 2))
        sc.lights.append(L)
        t.light_ids[i] = i
    t.light_count = n_lights
    return sc


@pytest.mark.parametrize("seed", range(16))
def test_random_scenes_bit_exact(oracle, ref, seed):
    """seeded random scenes on the live path: sample sums and two stateful
    frames equal the reference build bit for bit"""
    sc = random_scene(seed)
    a, b = OL.SceneHandle(oracle, sc), OL.SceneHandle(ref, sc)
    try:
        sa, sb = a.render_sum(3, nthreads=4), b.render_sum(3, nthreads=4)
        assert np.array_equal(bits(sa), bits(sb))
        assert np.isfinite(sa).all() and sa[..., 3].max() > 0
        la = OL.initial_lanes(seed + 1, sc.width, sc.height)
        lb = la.copy()
        for _ in range(2):
            assert np.array_equal(bits(a.render_frame(la, 4)), bits(b.render_frame(lb, 4)))
            assert np.array_equal(la, lb)
    finally:
        a.close()
        b.close()


def test_volume_without_normalize_size_is_empty(oracle, ref):
    """ErVolume without NormalizeSize: Volume's copy leaves Scale at 0 and
    multiplies the spacing by it (Source/volume.h:106-114), so the box has
    size 0 and no camera ray meets the volume; both builds render an empty,
    finite image, bit for bit"""
    sc = random_scene(0)
    sc.normalize_size = 0
    for L in sc.lights:
        L.visible = 0
    a, b = OL.SceneHandle(oracle, sc), OL.SceneHandle(ref, sc)
    try:
        sa, sb = a.render_sum(2, nthreads=4), b.render_sum(2, nthreads=4)
        assert np.array_equal(bits(sa), bits(sb))
        assert np.isfinite(sa).all() and not sa.any()
    finally:
        a.close()
        b.close()
