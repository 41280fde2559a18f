"""Partial re-upload of a bound volume (er_update_volume_region and its
device-pointer variant): after an edit, renders equal a fresh bind of the
edited volume bit for bit (corner quads, maximum voxel, gradient-magnitude
range, sigma table and majorant grid all follow the edit), and equal the
oracle of the edited volume."""
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
def env():
    import torch
    assert torch.cuda.is_available()
    lib = C.load_library()
    C.check(lib.er_set_device(0))
    rt = importlib.import_module("exposure-render_gb300.runtime")
    yield torch, lib, rt
    lib.er_reset()


def gpu_sum(torch, r, spp):
    d = torch.zeros((r.height, r.width, 4), dtype=torch.float32, device="cuda")
    r.trace_sum_device(d.data_ptr(), spp, 0, 0, 0, None)
    torch.cuda.synchronize()
    return d.cpu().numpy()


def edited_scene(box, seed):
    """the tiny scene with delta tracking, the hybrid shader (gradient-magnitude
    range) and full MIS; returns (scene, edited scene, offset, size, region)"""
    a = S.scene_tiny(res=32, seed=3)
    a.tracer.settings.free_flight = C.FREE_FLIGHT_DELTA
    a.tracer.settings.mis = C.MIS_FULL
    a.tracer.settings.apply_shading_type = 1
    a.tracer.settings.shading_type = C.SHADING_HYBRID
    a.tracer.settings.majorant_brick = 4
    (x0, y0, z0), (sx, sy, sz) = box
    rng = np.random.default_rng(seed)
    # values above the volume's maximum grow the sigma table
    region = rng.integers(0, int(a.volume.max()) + 3000, size=(sz, sy, sx), dtype=np.uint16)
    b = S.scene_tiny(res=32, seed=3)
    ctypes.memmove(ctypes.byref(b.tracer), ctypes.byref(a.tracer), ctypes.sizeof(a.tracer))
    b.volume = a.volume.copy()
    b.volume[z0:z0 + sz, y0:y0 + sy, x0:x0 + sx] = region
    return a, b, (x0, y0, z0), (sx, sy, sz), np.ascontiguousarray(region)


def i3(v):
    return (ctypes.c_int32 * 3)(*v)


@pytest.mark.parametrize("box", [((5, 7, 9), (11, 6, 4)), ((0, 0, 0), (32, 32, 1)), ((31, 20, 3), (1, 12, 29))],
                         ids=["inside", "bottom-slice", "edge-column"])
def test_region_update_equals_fresh_bind(env, oracle, box):
    torch, lib, rt = env
    a, b, off, size, region = edited_scene(box, seed=sum(box[0]))
    ra = rt.Renderer(a, lib)
    rb = rt.Renderer(b, lib)
    try:
        before = gpu_sum(torch, ra, 3)
        fresh = gpu_sum(torch, rb, 3)
        C.check(lib.er_update_volume_region(ra.volume_id, i3(off), i3(size), region.ctypes.data))
        edited = gpu_sum(torch, ra, 3)
        assert np.array_equal(bits(edited), bits(fresh))
        assert not np.array_equal(bits(edited), bits(before))
        h = OL.SceneHandle(oracle, b)
        assert np.array_equal(bits(edited), bits(h.render_sum(3, nthreads=4)))
        h.close()
        # back to the original voxels from device memory
        orig = np.ascontiguousarray(a.volume[off[2]:off[2] + size[2], off[1]:off[1] + size[1], off[0]:off[0] + size[0]])
        d = torch.from_numpy(orig.view(np.int16).copy()).cuda()
        C.check(lib.er_update_volume_region_device(ra.volume_id, i3(off), i3(size), d.data_ptr(), None))
        assert np.array_equal(bits(gpu_sum(torch, ra, 3)), bits(before))
    finally:
        ra.close()
        rb.close()


def test_rebind_in_place_and_errors(env):
    torch, lib, rt = env
    a, b, off, size, region = edited_scene(((4, 4, 4), (8, 8, 8)), seed=1)
    ra = rt.Renderer(a, lib)
    rb = rt.Renderer(b, lib)
    try:
        fresh = gpu_sum(torch, rb, 2)
        gpu_sum(torch, ra, 2)
        vd = b.volume_desc()
        vid = ctypes.c_int32(ra.volume_id)
        C.check(lib.er_bind_volume(ctypes.byref(vd), ctypes.byref(vid)))      # same ID, same resolution
        assert vid.value == ra.volume_id
        assert np.array_equal(bits(gpu_sum(torch, ra, 2)), bits(fresh))
        bad = [((30, 0, 0), (4, 1, 1)), ((0, -1, 0), (1, 1, 1)), ((0, 0, 0), (0, 1, 1))]
        for o, s in bad:
            assert lib.er_update_volume_region(ra.volume_id, i3(o), i3(s), region.ctypes.data) == C.ER_ERR_INVALID_ARGUMENT
        assert lib.er_update_volume_region(12345, i3(off), i3(size), region.ctypes.data) == C.ER_ERR_INVALID_ID
    finally:
        ra.close()
        rb.close()
