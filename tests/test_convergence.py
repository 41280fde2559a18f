"""Image-RMSE helpers and the FP64 reference fixtures (CPU only)."""
import os

import numpy as np
import pytest

import convergence as CV
import oracle_lib as OL

S = OL.PKG.scenes



def test_spp_to_rmse_interpolates_inverse_sqrt():
    spp = [1, 2, 4, 8, 16, 32, 64]
    err = [0.08 / np.sqrt(n) for n in spp]
    got = CV.spp_to_rmse(spp, err, 1e-2)
    assert got == pytest.approx(64.0, rel=1e-9)
    assert CV.spp_to_rmse(spp, err, 1e-3) is None
    assert CV.spp_to_rmse([4], [0.005], 1e-2) == pytest.approx(1.0)


def test_tonemap_matches_oracle_bytes():
    """tonemap_rgb is the float tone map of the oracle before 8-bit quantisation"""
    orc = OL.load_oracle()
    rng = np.random.default_rng(3)
    xyza = rng.uniform(0.0, 2.0, size=(256, 4)).astype(np.float32)
    rgba = np.zeros((256, 4), dtype=np.uint8)
    orc.tonemap(256, OL.ptr(xyza), 1.0, OL.ptr(rgba))
    tm = CV.tonemap_rgb(xyza.astype(np.float64), 1.0)
    # truncation to 8 bits: 255 * c rounds down, float vs double may differ by one step
    assert np.all(np.abs(np.floor(255.0 * tm) - rgba[:, :3]) <= 1)


@pytest.mark.parametrize("name", ["c1", "c1p", "c3v0", "c3v1", "c3v2", "c2", "c5v0"])
def test_fp64_reference_fixture(name):
    p = os.path.join(CV.GOLDEN, f"fp64_{name}.npz")
    assert os.path.exists(p), "run tests/golden/make_fp64.py"
    ref = CV.load_reference(name)
    assert ref["mean_xyz"].dtype == np.float64 and ref["mean_xyz"].shape == (128, 128, 3)
    assert int(ref["spp"]) >= 8192
    assert 0.0 < float(ref["noise2"]) < (2e-3) ** 2          # the reference's own noise is well below 1e-2
    assert CV.rmse(ref["mean_xyz"], ref) == 0.0               # noise-corrected distance to itself


def test_fp64_oracle_agrees_with_float_oracle():
    """the binary64 build and the float build estimate the same image:
    64 spp of each from independent streams differ by noise only"""
    f64, f32 = OL.load_fp64(), OL.load_oracle()
    sc = S.scene_tiny(res=24, film=(24, 20), seed=5)
    sc.tracer.settings.free_flight = 1
    sc.tracer.settings.mis = 1
    h1, h2 = OL.SceneHandle(f64, sc), OL.SceneHandle(f32, sc)
    a, a2 = h1.render_moments(256, view=1, nthreads=4)
    b, b2 = h2.render_moments(256, view=2, nthreads=4)
    h1.close()
    h2.close()
    n = 256
    ma, mb = (a / n)[..., :3], (b / n)[..., :3].astype(np.float64)
    va = (a2 / n)[..., :3] - ma ** 2                                  # per-sample variances
    vb = (b2 / n)[..., :3].astype(np.float64) - mb ** 2
    v = np.maximum(va, 0.0) + np.maximum(vb, 0.0)
    noisy = v > 1e-9 * (1.0 + ma ** 2)
    # constant pixels (empty background, directly visible light) agree to float rounding
    assert np.all(np.abs(ma - mb)[~noisy] <= 1e-5 * (1.0 + np.abs(ma[~noisy])))
    z = (ma - mb)[noisy] / np.sqrt(v[noisy] / n)
    assert noisy.sum() > 100
    assert np.mean(z * z) < 1.5                                       # chi-square per degree of freedom ~ 1
