"""Generates the golden fixtures of tests/golden/ from the reference's own
transport and post-processing code (oracle/_ref/liberref.so, built by
oracle/Makefile from the reference sources).  Each fixture stores its inputs
(volume, descriptors as raw bytes) next to the reference outputs, so the
golden tests do not depend on regenerating the inputs bit-for-bit.

    python tests/golden/make_golden.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import oracle_lib as OL  # noqa: E402

C = OL.C
S = OL.PKG.scenes


def scene_bytes(sc):
    return {
        "volume": sc.volume,
        "spacing": np.array(sc.spacing, np.float32),
        "tracer": np.frombuffer(bytes(sc.tracer), np.uint8),
        "lights": np.frombuffer(b"".join(bytes(l) for l in sc.lights), np.uint8),
        "textures": np.frombuffer(b"".join(bytes(t) for t in sc.textures), np.uint8),
    }


def main():
    ref = OL.load_ref()
    if ref is None:
        raise SystemExit("build oracle/_ref/liberref.so first (make -C oracle ref)")
    out = {}
    # RNG sequences and the Get2/Get3 component order
    lanes = [(1, 2), (12345, 67890), (0xDEADBEEF, 0x12345678), (0x9068FFFE, 0x464FFFFE)]
    draws = np.zeros((len(lanes), 64), np.float32)
    g23 = np.zeros((len(lanes), 5), np.float32)
    for i, (a, b) in enumerate(lanes):
        ref.rng_draws(a, b, 64, OL.ptr(draws[i]))
        ref.rng_get2_get3(a, b, OL.ptr(g23[i]))
    out["rng_lanes"] = np.array(lanes, np.uint32)
    out["rng_draws"] = draws
    out["rng_get23"] = g23
    # PLF including the node edges (value at the last node is 0)
    plf = C.make_plf([(0.0, 0.0), (400.0, 0.1), (1500.0, 0.6), (4000.0, 1.0)])
    xs = np.array([-1.0, 0.0, 0.5, 399.0, 400.0, 401.0, 1499.5, 1500.0, 2000.0, 3999.0, 4000.0, 4000.5, 65535.0], np.float32)
    ys = np.zeros_like(xs)
    ref.plf_evaluate(ctypes.byref(plf), len(xs), OL.ptr(xs), OL.ptr(ys))
    out["plf_bytes"] = np.frombuffer(bytes(plf), np.uint8)
    out["plf_x"] = xs
    out["plf_y"] = ys
    # tone map
    rng = np.random.default_rng(5)
    xyza = rng.uniform(0.0, 3.0, size=(256, 4)).astype(np.float32)
    xyza[:, 3] = rng.uniform(0.0, 1.0, size=256).astype(np.float32)
    rgba = np.zeros((256, 4), np.uint8)
    ref.tonemap(256, OL.ptr(xyza), 0.8, OL.ptr(rgba))
    out["tonemap_in"] = xyza
    out["tonemap_out"] = rgba
    # tiny scene: three stateful frames, then counter-seeded sums
    sc = S.scene_tiny()
    for k, v in scene_bytes(sc).items():
        out["tiny_" + k] = v
    h = OL.SceneHandle(ref, sc)
    W, H = sc.width, sc.height
    lanes0 = OL.initial_lanes(int(sc.tracer.settings.seed), W, H)
    out["tiny_lanes0"] = lanes0.copy()
    la = lanes0.copy()
    frames = []
    for f in range(3):
        frames.append(h.render_frame(la, nthreads=8))
    out["tiny_frames"] = np.stack(frames)
    out["tiny_lanes3"] = la
    out["tiny_sum4"] = h.render_sum(4, view=0, first=0, nthreads=8)
    out["tiny_sum3_view7_first11"] = h.render_sum(3, view=7, first=11, nthreads=8)
    # reference post pipeline over the three frames
    running = np.zeros((H, W, 4), np.float32)
    disp = []
    for f in range(3):
        fr = frames[f].copy()
        rgba = np.zeros((H, W, 4), np.uint8)
        ref.post_frame(OL.ptr(fr), OL.ptr(running), OL.ptr(rgba), W, H, f, float(sc.tracer.camera.exposure))
        disp.append(rgba)
    out["tiny_running3"] = running
    out["tiny_display"] = np.stack(disp)
    # camera and volume derivations
    cf = np.zeros(15, np.float32)
    ref.camera_frame(h.h, OL.ptr(cf))
    vf = np.zeros(13, np.float32)
    ref.volume_frame(h.h, OL.ptr(vf))
    out["tiny_camera_frame"] = cf
    out["tiny_volume_frame"] = vf
    h.close()
    np.savez_compressed(os.path.join(HERE, "reference_kats.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_kats.npz"))


if __name__ == "__main__":
    main()
