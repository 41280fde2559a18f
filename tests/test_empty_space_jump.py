"""The oracle's delta and ratio trackers jump across cubes of empty
majorant bricks (one DDA step per cube, oracle/er_oracle.c dda_jump): on a
volume that is empty but for two small boxes, the majorant reads per
sample stay far below the bricks a ray crosses, and the image matches the
binary64 build (which jumps the same way) within noise."""
import numpy as np

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
