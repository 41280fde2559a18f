"""The oracle's delta and ratio trackers jump across cubes of empty
majorant bricks (one DDA step per cube, oracle/er_oracle.c dda_jump): on a
volume that is empty but for two small boxes, the majorant reads per
sample stay far below the bricks a ray crosses, and the image matches the
binary64 build (which jumps the same way) within noise."""
import numpy as np
import pytest

import oracle_lib as OL

C = OL.C
S = OL.PKG.scenes


def sparse_scene(film=(40, 32)):
    vol = np.zeros((80, 80, 80), dtype=np.uint16)
    vol[10:30, 8:28, 12:34] = 3000
    vol[50:66, 54:72, 44:60] = 2200
    lights, textures = S.c1_lights()
    sc = S.Scene("sparse", vol, tracer=S.c1_tracer(film), lights=lights, textures=textures)
    s = sc.tracer.settings
    s.free_flight, s.mis, s.majorant_brick = 1, 1, 1
    return sc


def test_jump_reads_few_majorants(oracle):
    sc = sparse_scene()
    h = OL.SceneHandle(oracle, sc)
    try:
        h.render_sum(8, nthreads=4)
        st = OL.render_stats(oracle)
    finally:
        h.close()
    # an 80-brick ray through the box takes ~80 to ~240 face crossings brick by
    # brick; with the jump a few per cube of empty bricks
    assert 0 < st["majorant_reads"] < 20, st
    assert st["shadow_majorant_reads"] < 20 * max(st["shadow_rays"], 1.0), st


def test_jump_float_and_binary64_agree():
    f32, f64 = OL.load_oracle(), OL.load_fp64()
    sc = sparse_scene()
    a = OL.SceneHandle(f32, sc)
    b = OL.SceneHandle(f64, sc)
    try:
        n = 256
        ma, ma2 = a.render_moments(n, view=1, nthreads=4)
        mb, mb2 = b.render_moments(n, view=2, nthreads=4)
    finally:
        a.close()
        b.close()
    ma, mb = (ma / n)[..., :3].astype(np.float64), (mb / n)[..., :3]
    va = np.maximum((ma2 / n)[..., :3] - ma ** 2, 0.0)
    vb = np.maximum((mb2 / n)[..., :3] - mb ** 2, 0.0)
    v = va + vb
    noisy = v > 1e-9 * (1.0 + ma ** 2)
    assert noisy.sum() > 50
    z = (ma - mb)[noisy] / np.sqrt(v[noisy] / n)
    assert np.mean(z * z) < 1.5


def test_majorant_brick_size_does_not_change_the_image():
    """Delta and ratio tracking are unbiased for any majorant that bounds the
    extinction of every lookup they make; the majorant of a brick covers only
    the voxels a lookup clamped to that brick blends.  If a brick's bound
    missed a lookup, the tight 1^3 bricks (a 2^3-voxel footprint each) would
    render another image than 8^3 bricks: the c3 96^3 blob volume, 48^2
    film, independent streams, per-pixel and whole-image z-tests."""
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location("bench_for_test", os.path.join(OL.ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    scenes, views, _ = bench.batched_workload("c3", 0)
    cam = [c for (k, c, _) in views if k == 0][0]
    f32 = OL.load_oracle()
    n = 512
    out = []
    for brick, view in ((1, 1), (8, 2)):
        sc = scenes[0]
        t = C.er_tracer_desc.from_buffer_copy(sc.tracer)
        t.camera = cam
        t.camera.film_size[0] = t.camera.film_size[1] = 48
        t.settings.free_flight, t.settings.mis, t.settings.majorant_brick, t.settings.stratify = 1, 1, brick, 0
        sc.tracer = t
        h = OL.SceneHandle(f32, sc)
        try:
            out.append(h.render_moments(n, view=view, nthreads=os.cpu_count() or 4))
        finally:
            h.close()
    (a, a2), (b, b2) = out
    ma, mb = (a / n)[..., :3].astype(np.float64), (b / n)[..., :3].astype(np.float64)
    va = np.maximum((a2 / n)[..., :3] - ma ** 2, 0.0)
    vb = np.maximum((b2 / n)[..., :3] - mb ** 2, 0.0)
    noisy = (va + vb) > 1e-9 * (1.0 + ma ** 2)
    assert noisy.sum() > 500
    z = (ma - mb)[noisy] / np.sqrt((va + vb)[noisy] / n)
    assert np.mean(z * z) < 1.5
    for c in range(3):
        d = ma[..., c].sum() - mb[..., c].sum()
        assert abs(d) < 4.0 * np.sqrt((va[..., c].sum() + vb[..., c].sum()) / n)


@pytest.mark.parametrize("brick", [1, 2, 4])
def test_jump_crosses_the_same_non_empty_bricks(oracle, brick):
    """Along 3000 random rays through the box, the walk with the empty-space
    jump meets the same non-empty bricks, in the same order and over the
    same ray segments (to float rounding of the face times), as the walk
    brick by brick, in fewer DDA iterations: the jump never steps over a
    brick whose majorant is positive."""
    sc = sparse_scene()
    sc.tracer.settings.majorant_brick = brick
    h = OL.SceneHandle(oracle, sc)
    try:
        vf = np.zeros(13, dtype=np.float32)
        oracle.volume_frame(h.h, OL.ptr(vf))
        lo, size = vf[0:3].astype(np.float64), vf[10:13].astype(np.float64)
        rng = np.random.default_rng(21 + brick)
        n, cap = 3000, 256
        target = lo + rng.uniform(0.0, 1.0, size=(n, 3)) * size
        d = rng.normal(size=(n, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        origin = target - 2.0 * float(size.max()) * d
        rays = np.zeros((n, 8), dtype=np.float32)
        rays[:, 0:3], rays[:, 3:6], rays[:, 6], rays[:, 7] = origin, d, 0.0, 1e6
        walks = []
        for jump in (0, 1):
            out = np.zeros((n, cap, 5), dtype=np.float32)
            counts = np.zeros((n, 2), dtype=np.int32)
            oracle.dda_walk(h.h, n, OL.ptr(rays), jump, cap, OL.ptr(out), OL.ptr(counts))
            walks.append((out, counts))
    finally:
        h.close()
    (a, ca), (b, cb) = walks
    assert (ca[:, 0] < cap).all() and ca[:, 0].sum() > 1000          # the rays meet the boxes
    assert cb[:, 1].sum() < 0.5 * ca[:, 1].sum()                      # far fewer iterations
    scale = float(size.max()) * 4.0
    for i in range(n):
        sa = [r for r in a[i, :ca[i, 0]] if r[1] - r[0] > 1e-5 * scale]
        sb = [r for r in b[i, :cb[i, 0]] if r[1] - r[0] > 1e-5 * scale]
        assert len(sa) == len(sb), i
        for ra, rb in zip(sa, sb):
            assert np.array_equal(ra[2:], rb[2:]), i
            assert np.allclose(ra[:2], rb[:2], rtol=1e-5, atol=1e-5 * scale), i


@pytest.mark.parametrize("brick", [1, 2, 3, 8])
def test_majorant_bounds_every_tracker_lookup(oracle, brick):
    """The extinction a tracker looks up at any point of a brick (local
    coordinates clamped to the brick, here also points a little outside it,
    as float rounding can place them) never exceeds the brick's majorant, and
    is zero in empty bricks: a rough random volume, a transfer function that
    rises and falls steeply, and a constant block where a blend rounding one
    intensity below the corners' minimum reads a higher extinction."""
    rng = np.random.default_rng(brick)
    vol = rng.integers(0, 3000, size=(23, 19, 21)).astype(np.uint16)
    vol[-12:, -12:, -12:] = 0                             # an empty corner (a whole 8^3 brick's footprint)
    # a constant block just above a falling edge of the transfer function, at
    # the origin: with a full-precision weight t (local coordinates below 1),
    # a blend (1 - t) a + t a rounds below a for about 4% of t, and the
    # truncation then reads the intensity one below, where the opacity is higher
    vol[:7, :7, :7] = 501
    lights, textures = S.c1_lights()
    t = S.c1_tracer((16, 16))
    t.opacity = C.make_plf([(0.0, 0.0), (499.0, 0.0), (500.0, 0.9), (501.0, 0.05), (1200.0, 0.5), (1201.0, 0.0),
                            (2000.0, 0.0), (2999.5, 1.0)])
    sc = S.Scene("rough", vol, tracer=t, lights=lights, textures=textures)
    s = sc.tracer.settings
    s.free_flight, s.majorant_brick = 1, brick
    h = OL.SceneHandle(oracle, sc)
    try:
        vf = np.zeros(13, dtype=np.float32)
        oracle.volume_frame(h.h, OL.ptr(vf))
        res = np.array([21, 19, 23], dtype=np.float64)     # x, y, z
        nb = np.ceil(res / brick).astype(np.int64)
        n = 200000
        b = np.stack([rng.integers(0, nb[a], size=n) for a in range(3)], axis=1)
        # points up to 0.3 brick outside their brick: the clamp must keep every blend in the footprint
        L = (b + rng.uniform(-0.3, 1.3, size=(n, 3))) * brick
        L = np.minimum(L, res)
        p = (vf[0:3].astype(np.float64) + L / (vf[3:6].astype(np.float64) * res)).astype(np.float32)
        out = np.zeros((n, 2), dtype=np.float32)
        oracle.brick_bound(h.h, n, OL.ptr(np.ascontiguousarray(p)), OL.ptr(np.ascontiguousarray(b.astype(np.int32))), OL.ptr(out))
    finally:
        h.close()
    sig, mu = out[:, 0], out[:, 1]
    full = mu > 0.0
    assert full.sum() > 1000 and (~full).sum() > 100
    assert (sig[full] <= mu[full]).all(), float((sig[full] - mu[full]).max())
    assert (sig[~full] == 0.0).all()
