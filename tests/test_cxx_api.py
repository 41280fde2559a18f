"""The C++ API of include/exposurerender.h, used the way a reference
application uses Source/exposurerender.h: compiled against the header,
linked against libexposurerender.so."""
import os
import subprocess

import numpy as np
import pytest

import oracle_lib as OL

C = OL.C
S = OL.PKG.scenes
APP = os.path.join(OL.ROOT, "tests", "cxx", "app.cpp")


def build_app(tmpdir):
    exe = os.path.join(tmpdir, "app")
    lib_dir = os.path.dirname(C.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(OL.ROOT, "include"), APP, "-o", exe,
                    "-L" + lib_dir, "-lexposurerender", "-Wl,-rpath," + lib_dir], check=True)
    return exe


def test_app_compiles_and_links(tmp_path):
    assert os.path.exists(build_app(str(tmp_path)))


@pytest.mark.gpu
def test_app_renders_like_the_oracle(tmp_path, oracle):
    exe = build_app(str(tmp_path))
    res = 24
    vol = S.blob_volume((res, res, res), n_blobs=6, seed=3)
    vol_path = os.path.join(str(tmp_path), "vol.raw")
    vol.tofile(vol_path)
    out_path = os.path.join(str(tmp_path), "out.rgba")
    r = subprocess.run([exe, vol_path, str(res), "3", out_path], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(out_path, np.uint8).reshape(32, 40, 4)
    # the same scene through the oracle: 3 frames of the reference pipeline
    sc = S.scene_tiny(res=res, film=(40, 32), seed=3)
    sc.volume = vol
    m = [[-1.0, 0.0, 0.0, 0.0], [0.0, 1.0, 0.0, 0.0], [0.0, 0.0, -1.0, 1.0], [0.0, 0.0, 0.0, 1.0]]
    C.set_matrix(sc.lights[0].shape.tm, m)     # the application's light frame (positive zeros)
    C.set_matrix(sc.lights[0].shape.inv_tm, m)
    h = OL.SceneHandle(oracle, sc)
    W, H = 40, 32
    lanes = OL.initial_lanes(1, W, H)
    running = np.zeros((H, W, 4), np.float32)
    rgba = np.zeros((H, W, 4), np.uint8)
    for n in range(3):
        frame = h.render_frame(lanes, nthreads=4)
        oracle.post_frame(OL.ptr(frame), OL.ptr(running), OL.ptr(rgba), W, H, n, 1.0)
    assert np.array_equal(got, rgba)
