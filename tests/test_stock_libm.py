"""The reference's own transport code built with the C library's elementary
functions (oracle/Makefile ref-stock: no routing of logf/expf/powf/... to
include/er_math.h) against the oracle, which the GPU path equals bit for
bit.  This is the unmodified reference's numerics: the comparison measures
how far the GPU path is from them, per pixel, on the reference's live
estimator (fixed-step march, BRDF, light sampling) over the c1 film (256^2,
two frames) and the c2 scene's whole field of view at 256^2 (one frame).

A threshold flip is a sample whose path took another branch (a Sum < S
crossing, a light pick) because an elementary function differed in its
last bits: it shows as a different number of random draws, i.e. different
RNG lane states after the frame (each draw advances both MWC lanes one
step, Source/rng.h:35-51).  Pixels without a flip must agree to 1e-4
relative (the FP32 tolerance of this path's parity); flips are counted and each is
traced to the draw counts of both builds."""
import os

import numpy as np
import pytest

import oracle_lib as OL

S = OL.PKG.scenes
STOCK_SO = os.path.join(OL.ROOT, "oracle", "_ref", "liberref_stock.so")


@pytest.fixture(scope="module")
def stock():
    if not os.path.exists(STOCK_SO):
        pytest.skip("stock-libm reference build (oracle/_ref/liberref_stock.so) not present on this machine")
    return OL.Oracle(STOCK_SO, "ref_")


def draws(lane0_before, lane0_after, cap=1 << 20):
    """MWC steps of lane 0 (Source/rng.h:37) from one state to another"""
    s, k = int(lane0_before), 0
    while s != int(lane0_after) and k < cap:
        s = (36969 * (s & 65535) + (s >> 16)) & 0xFFFFFFFF
        k += 1
    return k


def frames(lib, sc, n):
    h = OL.SceneHandle(lib, sc)
    lanes = OL.initial_lanes(int(sc.tracer.settings.seed), sc.width, sc.height)
    out = []
    try:
        for _ in range(n):
            before = lanes.copy()
            out.append((before, h.render_frame(lanes, nthreads=os.cpu_count() or 8), lanes.copy()))
    finally:
        h.close()
    return out


def live_path(sc):
    s = sc.tracer.settings
    s.free_flight, s.mis, s.apply_shading_type, s.stratify = 0, 0, 0, 0
    return sc


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_gpu_path_against_stock_libm_reference(oracle, stock, name):
    sc = live_path(S.scene_c1() if name == "c1" else S.scene_c2(res=512, film=(256, 256)))
    n_frames = 2 if name == "c1" else 1
    a, b = frames(oracle, sc, n_frames), frames(stock, sc, n_frames)
    npix = sc.width * sc.height
    total = flips = identical = 0
    worst = 0.0
    traced = []
    for (la0, fa, la1), (lb0, fb, lb1) in zip(a, b):
        assert np.array_equal(la0, lb0)
        flip = ((la1[:npix] != lb1[:npix]) | (la1[npix:] != lb1[npix:])).reshape(sc.height, sc.width)
        den = np.maximum(np.abs(fa), np.abs(fb))
        rel = np.where(den > 0, np.abs(fa - fb) / np.where(den > 0, den, 1.0), 0.0).max(-1)
        total += npix
        flips += int(flip.sum())
        identical += int((fa.view(np.uint32) == fb.view(np.uint32)).all(-1).sum())
        if (~flip).any():
            worst = max(worst, float(rel[~flip].max()))
        for p in np.flatnonzero(flip.ravel())[:8]:
            traced.append((int(p), draws(la0[p], la1[p]), draws(lb0[p], lb1[p])))
    print(f"{name}: {total} pixel samples, {identical / total:.4f} bit-identical, {flips} threshold flips "
          f"(draws oracle/stock: {traced}), worst relative error without a flip {worst:.2e}")
    assert worst <= 1e-4
    assert flips <= 1e-3 * total
    assert identical > 0.9 * total
