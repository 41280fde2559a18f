"""The autotuner (er_autotune_tracer): candidate sweep, tuning cache, and
bit-exact renders with the tuned settings."""
import importlib
import os

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


@pytest.fixture()
def cache(tmp_path, monkeypatch):
    p = tmp_path / "tune" / "autotune.txt"
    monkeypatch.setenv("ER_TUNE_CACHE", str(p))
    return p


def test_autotune_delta_sweep_and_cache(torch, lib, runtime, oracle, cache):
    sc = S.scene_tiny(seed=11)
    sc.tracer.settings.free_flight = C.FREE_FLIGHT_DELTA
    r = runtime.Renderer(sc, lib)
    try:
        first = r.autotune(2)
        assert first["majorant_brick"] in (1, 2, 4, 8, 16)
        assert first["tune_primary"] in (2, 3, 4, 6, 8) and first["tune_shadow"] in (2, 3, 4, 6, 8)
        assert first["tune_shade"] in (2, 3, 4, 6)
        assert first["tune_stages"] & 3 in (C.PERSISTENT_SHADOW, C.PERSISTENT_BOTH, C.PERSISTENT_NONE, C.PERSISTENT_PRIMARY)
        assert first["tune_stages"] & ~(3 | C.TUNE_NO_SKIP) == 0
        # five brick sizes (the empty-space jump always on), eleven occupancy pairs under the four
        # persistent-lane modes, four shade variants
        assert first["candidates"] == 5 + 4 * 11 + 4 and not first["from_cache"] and first["msamples_per_s"] > 0
        assert cache.exists() and len(cache.read_text().splitlines()) == 1
        again = r.autotune(2)
        assert again["from_cache"] and again["candidates"] == 0
        for k in ("majorant_brick", "tune_primary", "tune_shadow", "tune_shade", "tune_stages"):
            assert again[k] == first[k]
        s = C.er_render_settings()
        C.check(lib.er_get_render_settings(r.tracer_id, s))
        assert s.majorant_brick == first["majorant_brick"] and s.tune_primary == first["tune_primary"]
        # the tuned tracer renders bit-exactly what the oracle renders with the same settings
        d = torch.zeros((r.height, r.width, 4), dtype=torch.float32, device="cuda")
        r.trace_sum_device(d.data_ptr(), 3, 0, 0, 0, None)
        torch.cuda.synchronize()
        sc.tracer.settings.majorant_brick = first["majorant_brick"]
        h = OL.SceneHandle(oracle, sc)
        ref = h.render_sum(3)
        h.close()
        assert np.array_equal(bits(d.cpu().numpy()), bits(ref))
    finally:
        r.close()


def test_autotune_march_skips_bricks(torch, lib, runtime, cache):
    sc = S.scene_tiny(seed=12)
    r = runtime.Renderer(sc, lib)
    try:
        res = r.autotune(1)
        assert res["candidates"] == 1 + 11 + 4     # the brick does not matter to the march
        assert res["majorant_brick"] == 8
    finally:
        r.close()


def test_autotune_cache_off(torch, lib, runtime, monkeypatch, tmp_path):
    monkeypatch.setenv("ER_TUNE_CACHE", "off")
    monkeypatch.setenv("HOME", str(tmp_path))
    sc = S.scene_tiny(seed=13)
    sc.tracer.settings.free_flight = C.FREE_FLIGHT_DELTA
    r = runtime.Renderer(sc, lib)
    try:
        a = r.autotune(1)
        b = r.autotune(1)
        assert not a["from_cache"] and not b["from_cache"]
        assert not os.listdir(tmp_path)
    finally:
        r.close()


def test_autotune_arguments(torch, lib):
    res = C.er_tune_result()
    assert lib.er_autotune_tracer(4321, 2, res) == C.ER_ERR_INVALID_ID
    assert lib.er_get_render_settings(4321, C.er_render_settings()) == C.ER_ERR_INVALID_ID
