"""The C ABI library loads without a GPU and exports every entry point that
include/er_capi.h declares; the ctypes mirrors have the C layout."""
import ctypes
import os
import subprocess
import tempfile

import pytest

import oracle_lib as OL

C = OL.C


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(C.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return ctypes.CDLL(C.LIB_PATH)


def test_exports_every_declared_symbol(lib):
    names = C.exported_symbols()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_loader_declares_every_symbol():
    lib = C.load_library()
    for n in C.exported_symbols():
        assert getattr(lib, n).argtypes is not None or n in ("er_abi_version", "er_last_error_message", "er_synchronize", "er_reset"), n


def test_host_only_calls(lib):
    L = C.load_library()
    assert L.er_abi_version() == 1
    s = C.er_render_settings()
    L.er_default_render_settings(ctypes.byref(s))
    ref = C.default_render_settings()
    for f, _ in C.er_render_settings._fields_:
        if f in ("reserved",):
            continue
        assert getattr(s, f) == getattr(ref, f), f
    p = C.er_plf()
    L.er_plf_init(ctypes.byref(p))
    for i in range(130):
        L.er_plf_add_node(ctypes.byref(p), float(i), float(i) * 0.5)
    q = C.plf_init(C.er_plf())
    for i in range(130):
        C.plf_add_node(q, float(i), float(i) * 0.5)
    assert p.count == 127 == q.count                      # Source/plf.h:53 cap
    assert bytes(p) == bytes(q)


def test_struct_layout_matches_c():
    structs = ["er_plf", "er_color_tf", "er_shape", "er_light_desc", "er_procedural", "er_texture_desc", "er_volume_desc",
               "er_bitmap_desc", "er_object_desc", "er_clipping_object_desc", "er_camera_desc", "er_render_settings",
               "er_tracer_desc", "er_batch_view", "er_tune_result", "er_medium_desc"]
    src = '#include <stdio.h>\n#include <stddef.h>\n#include "er_capi.h"\nint main(void){\n'
    for s in structs:
        src += f'printf("{s} %zu\\n", sizeof({s}));\n'
    src += 'printf("settings.seed %zu\\n", offsetof(er_render_settings, seed));\n'
    src += 'printf("tracer.volume_id %zu\\n", offsetof(er_tracer_desc, volume_id));\n'
    src += 'printf("settings.stratify %zu\\n", offsetof(er_render_settings, stratify));\n'
    src += 'printf("settings.tune_stages %zu\\n", offsetof(er_render_settings, tune_stages));\n'
    src += 'printf("tune.tune_stages %zu\\n", offsetof(er_tune_result, tune_stages));\n'
    src += 'printf("batch.d_sum %zu\\n", offsetof(er_batch_view, d_sum_xyza));\nreturn 0;}\n'
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "s.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "s")
        subprocess.run(["gcc", "-I" + os.path.join(OL.ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = dict(line.split() for line in out if line)
    for s in structs:
        assert int(got[s]) == ctypes.sizeof(getattr(C, s)), s
    assert int(got["settings.seed"]) == C.er_render_settings.seed.offset
    assert int(got["tracer.volume_id"]) == C.er_tracer_desc.volume_id.offset
    assert int(got["batch.d_sum"]) == C.er_batch_view.d_sum_xyza.offset
    assert int(got["settings.stratify"]) == C.er_render_settings.stratify.offset
    assert int(got["settings.tune_stages"]) == C.er_render_settings.tune_stages.offset
    assert int(got["tune.tune_stages"]) == C.er_tune_result.tune_stages.offset


@pytest.mark.parametrize("case", ["null", "resolution", "spacing-zero", "spacing-negative", "spacing-nan", "spacing-inf"])
def test_bind_volume_rejects_degenerate_descriptors(case):
    """er_bind_volume refuses, before any device work, a descriptor whose box
    would be degenerate: a zero, negative or non-finite spacing.
    normalize_size = 0 is accepted as the reference accepts it (its box then
    has no extent, Source/volume.h:106-114; tests/test_gpu_clipping.py)."""
    import numpy as np
    L = C.load_library()
    vox = np.zeros((4, 4, 4), dtype=np.uint16)
    d = C.er_volume_desc()
    for i in range(3):
        d.resolution[i] = 4
        d.spacing[i] = 1.0
    d.normalize_size = 1
    d.voxels = vox.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))
    if case == "null":
        d.voxels = None
    elif case == "resolution":
        d.resolution[1] = 0
    else:
        d.spacing[2] = {"spacing-zero": 0.0, "spacing-negative": -1.0, "spacing-nan": float("nan"),
                        "spacing-inf": float("inf")}[case]
    vid = ctypes.c_int32(-1)
    assert L.er_bind_volume(ctypes.byref(d), ctypes.byref(vid)) == C.ER_ERR_INVALID_ARGUMENT
    assert vid.value == -1
    msg = L.er_last_error_message().decode()
    assert {"null": "NULL", "resolution": "resolution"}.get(case, "spacing") in msg


@pytest.mark.parametrize("case", ["step-primary-zero", "step-shadow-nan", "density-zero", "density-inf", "film-zero",
                                  "film-huge", "lights-negative"])
def test_bind_tracer_rejects_invalid_settings(case):
    """er_bind_tracer refuses, before any device work, settings under which a
    march would take steps of zero or NaN length, and out-of-range films and
    light counts"""
    L = C.load_library()
    t = OL.PKG.scenes.c1_tracer((16, 16))
    s = t.settings
    if case == "step-primary-zero":
        s.step_factor_primary = 0.0
    elif case == "step-shadow-nan":
        s.step_factor_shadow = float("nan")
    elif case == "density-zero":
        s.density_scale = 0.0
    elif case == "density-inf":
        s.density_scale = float("inf")
    elif case == "film-zero":
        t.camera.film_size[0] = 0
    elif case == "film-huge":
        t.camera.film_size[1] = 40000
    else:
        t.light_count = -1
    tid = ctypes.c_int32(-1)
    assert L.er_bind_tracer(ctypes.byref(t), ctypes.byref(tid)) == C.ER_ERR_INVALID_ARGUMENT
    assert tid.value == -1
    msg = L.er_last_error_message().decode()
    assert {"step": "step factors", "density": "density_scale", "film": "film size",
            "lights": "light_count"}[case.split("-")[0]] in msg
