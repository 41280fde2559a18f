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
