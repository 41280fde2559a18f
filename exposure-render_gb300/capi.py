"""ctypes mirror of include/er_capi.h and the loader of libexposurerender.so.

The structures below are field-for-field copies of the C descriptors, which
themselves mirror the reference's ErTracer/ErVolume/ErLight/ErTexture types
(Source/ertracer.h:33-117, Source/ervolume.h:28-74, Source/erlight.h:27-66,
Source/ertexture.h:27-82).
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, Structure, c_char_p, c_float, c_int32, c_uint8, c_uint16, c_uint32, c_void_p

import numpy as np

ER_MAX_TF_NODES = 128
ER_MAX_ITEMS_PER_LIST = 31
ER_MAX_INDICES = 256

ER_OK = 0
(ER_ERR_INVALID_ID, ER_ERR_INVALID_ARGUMENT, ER_ERR_LIST_FULL, ER_ERR_CUDA, ER_ERR_OUT_OF_MEMORY, ER_ERR_UNSUPPORTED,
 ER_ERR_NO_DEVICE, ER_ERR_TIMEOUT) = range(1, 9)
STATUS_NAMES = {
    0: "ER_OK",
    1: "ER_ERR_INVALID_ID",
    2: "ER_ERR_INVALID_ARGUMENT",
    3: "ER_ERR_LIST_FULL",
    4: "ER_ERR_CUDA",
    5: "ER_ERR_OUT_OF_MEMORY",
    6: "ER_ERR_UNSUPPORTED",
    7: "ER_ERR_NO_DEVICE",
    8: "ER_ERR_TIMEOUT",
}

SHAPE_PLANE, SHAPE_DISK, SHAPE_RING, SHAPE_BOX, SHAPE_SPHERE, SHAPE_CYLINDER, SHAPE_CONE = range(7)
PROCEDURAL_UNIFORM, PROCEDURAL_CHECKER, PROCEDURAL_GRADIENT = range(3)
TEXTURE_PROCEDURAL, TEXTURE_BITMAP = range(2)
PERSISTENT_SHADOW, PERSISTENT_BOTH, PERSISTENT_NONE, PERSISTENT_PRIMARY = range(4)
TUNE_NO_SKIP_PRIMARY, TUNE_NO_SKIP_SHADOW = 4, 8
TUNE_NO_SKIP = TUNE_NO_SKIP_PRIMARY | TUNE_NO_SKIP_SHADOW
SHADING_BRDF_ONLY, SHADING_PHASE_ONLY, SHADING_HYBRID, SHADING_MODULATION, SHADING_THRESHOLD, SHADING_GRADIENT_MAGNITUDE = range(6)
GRADIENT_FORWARD, GRADIENT_CENTRAL, GRADIENT_FILTERED = range(3)
UNIT_POWER, UNIT_LUX, UNIT_INTENSITY = range(3)
FREE_FLIGHT_MARCH, FREE_FLIGHT_DELTA = range(2)
MIS_LIGHT_ONLY, MIS_FULL = range(2)

FLT_MAX = float(np.finfo(np.float32).max)
FLT_MIN = float(np.finfo(np.float32).tiny)


class er_plf(Structure):
    _fields_ = [
        ("count", c_int32),
        ("node_range", c_float * 2),
        ("position", c_float * ER_MAX_TF_NODES),
        ("value", c_float * ER_MAX_TF_NODES),
    ]


class er_color_tf(Structure):
    _fields_ = [("plf", er_plf * 3)]


class er_shape(Structure):
    _fields_ = [
        ("tm", (c_float * 4) * 4),
        ("inv_tm", (c_float * 4) * 4),
        ("one_sided", c_int32),
        ("type", c_int32),
        ("size", c_float * 3),
        ("area", c_float),
        ("inner_radius", c_float),
        ("outer_radius", c_float),
    ]


class er_light_desc(Structure):
    _fields_ = [
        ("visible", c_int32),
        ("shape", er_shape),
        ("texture_id", c_int32),
        ("multiplier", c_float),
        ("unit", c_int32),
    ]


class er_procedural(Structure):
    _fields_ = [
        ("type", c_int32),
        ("uniform_color", c_float * 3),
        ("checker_color1", c_float * 3),
        ("checker_color2", c_float * 3),
        ("gradient", er_color_tf),
    ]


class er_texture_desc(Structure):
    _fields_ = [
        ("type", c_int32),
        ("output_level", c_float),
        ("bitmap_id", c_int32),
        ("procedural", er_procedural),
        ("offset", c_float * 2),
        ("repeat", c_float * 2),
        ("flip", c_int32 * 2),
    ]


class er_volume_desc(Structure):
    _fields_ = [
        ("resolution", c_int32 * 3),
        ("spacing", c_float * 3),
        ("normalize_size", c_int32),
        ("voxels", POINTER(c_uint16)),
    ]


class er_bitmap_desc(Structure):
    _fields_ = [("resolution", c_int32 * 2), ("pixels", POINTER(c_uint8))]


class er_object_desc(Structure):
    _fields_ = [
        ("shape", er_shape),
        ("diffuse_texture_id", c_int32),
        ("specular_texture_id", c_int32),
        ("glossiness_texture_id", c_int32),
        ("ior", c_float),
    ]


class er_clipping_object_desc(Structure):
    _fields_ = [("shape", er_shape), ("invert", c_int32)]


class er_camera_desc(Structure):
    _fields_ = [
        ("film_size", c_int32 * 2),
        ("pos", c_float * 3),
        ("target", c_float * 3),
        ("up", c_float * 3),
        ("focal_distance", c_float),
        ("aperture_size", c_float),
        ("clip_near", c_float),
        ("clip_far", c_float),
        ("exposure", c_float),
        ("gamma", c_float),
        ("fov", c_float),
    ]


class er_render_settings(Structure):
    _fields_ = [
        ("step_factor_primary", c_float),
        ("step_factor_shadow", c_float),
        ("shadows", c_int32),
        ("max_shadow_distance", c_float),
        ("shading_type", c_int32),
        ("density_scale", c_float),
        ("opacity_modulated", c_int32),
        ("gradient_computation", c_int32),
        ("gradient_threshold", c_float),
        ("gradient_factor", c_float),
        ("apply_shading_type", c_int32),
        ("free_flight", c_int32),
        ("mis", c_int32),
        ("volume_ior", c_float),
        ("frame_filter", c_int32),
        ("bilateral", c_int32),
        ("bilateral_radius", c_int32),
        ("bilateral_sigma_d", c_float),
        ("bilateral_sigma_r", c_float),
        ("seed", c_uint32),
        ("majorant_brick", c_int32),
        ("engine", c_int32),
        ("tune_primary", c_int32),
        ("tune_shadow", c_int32),
        ("tune_shade", c_int32),
        ("stratify", c_int32),
        ("tune_stages", c_int32),
    ]


class er_tracer_desc(Structure):
    _fields_ = [
        ("opacity", er_plf),
        ("diffuse", er_color_tf),
        ("specular", er_color_tf),
        ("glossiness", er_plf),
        ("emission", er_color_tf),
        ("camera", er_camera_desc),
        ("settings", er_render_settings),
        ("volume_id", c_int32),
        ("light_count", c_int32),
        ("light_ids", c_int32 * ER_MAX_INDICES),
        ("object_count", c_int32),
        ("object_ids", c_int32 * ER_MAX_INDICES),
        ("clipping_object_count", c_int32),
        ("clipping_object_ids", c_int32 * ER_MAX_INDICES),
    ]


class er_medium_desc(Structure):
    _fields_ = [
        ("d_density", c_void_p),
        ("d_opacity", c_void_p),
        ("n_opacity", c_int32),
        ("scale", c_float),
        ("albedo", c_float * 3),
        ("nee_probability", c_float),
        ("d_majorant", c_void_p),
        ("brick", c_int32),
        ("model", c_int32),
        ("gradient_magnitude_inv", c_float),
    ]


ER_MEDIUM_SPLINE, ER_MEDIUM_TRACER = 0, 1


class er_tune_result(Structure):
    _fields_ = [
        ("majorant_brick", c_int32),
        ("tune_primary", c_int32),
        ("tune_shadow", c_int32),
        ("from_cache", c_int32),
        ("msamples_per_s", c_float),
        ("candidates", c_int32),
        ("tune_shade", c_int32),
        ("tune_stages", c_int32),
    ]


class er_batch_view(Structure):
    _fields_ = [
        ("tracer_id", c_int32),
        ("spp", c_int32),
        ("view", c_uint32),
        ("first_sample", c_uint32),
        ("d_sum_xyza", c_void_p),
        ("accumulate", c_int32),
        ("display", c_int32),
        ("camera", POINTER(er_camera_desc)),
    ]


ER_BATCH_GRAPH = 1


# ---------------------------------------------------------------------------
# helpers that mirror the reference's host-side builders
# ---------------------------------------------------------------------------

def plf_init(p: er_plf) -> er_plf:
    """PiecewiseFunction() (Source/pf.h:39-46): empty, NodeRange = (FLT_MAX, FLT_MIN)."""
    p.count = 0
    p.node_range[0] = FLT_MAX
    p.node_range[1] = FLT_MIN
    for i in range(ER_MAX_TF_NODES):
        p.position[i] = 0.0
        p.value[i] = 0.0
    return p


def plf_add_node(p: er_plf, position: float, value: float) -> None:
    """PiecewiseLinearFunction::AddNode (Source/plf.h:51-66), float32 semantics."""
    if p.count + 1 >= ER_MAX_TF_NODES:
        return
    pos = np.float32(position)
    p.position[p.count] = float(pos)
    p.value[p.count] = float(np.float32(value))
    if pos < np.float32(p.node_range[0]):
        p.node_range[0] = float(pos)
    if pos > np.float32(p.node_range[1]):
        p.node_range[1] = float(pos)
    p.count += 1


def make_plf(nodes) -> er_plf:
    p = plf_init(er_plf())
    for pos, val in nodes:
        plf_add_node(p, pos, val)
    return p


def make_color_tf(nodes_rgb) -> er_color_tf:
    """nodes_rgb: list of (position, (v0, v1, v2)); each channel gets the same positions."""
    t = er_color_tf()
    for c in range(3):
        plf_init(t.plf[c])
        for pos, vals in nodes_rgb:
            plf_add_node(t.plf[c], pos, vals[c])
    return t


def identity4():
    return [[1.0 if i == j else 0.0 for j in range(4)] for i in range(4)]


def set_matrix(dst, m) -> None:
    for i in range(4):
        for j in range(4):
            dst[i][j] = float(m[i][j])


def default_render_settings() -> er_render_settings:
    """RenderSettings() defaults (Source/rendersettings.h:33-39, :69-77)."""
    s = er_render_settings()
    s.step_factor_primary = 0.1
    s.step_factor_shadow = 0.1
    s.shadows = 1
    s.max_shadow_distance = 1.0
    s.shading_type = 0
    s.density_scale = 100.0
    s.opacity_modulated = 1
    s.gradient_computation = 1
    s.gradient_threshold = 0.5
    s.gradient_factor = 0.5
    s.apply_shading_type = 0
    s.free_flight = FREE_FLIGHT_MARCH
    s.mis = MIS_LIGHT_ONLY
    s.volume_ior = 15.0
    s.frame_filter = 1
    s.bilateral = 0
    s.bilateral_radius = 2
    s.bilateral_sigma_d = 1.5
    s.bilateral_sigma_r = 20.0
    s.seed = 1
    s.majorant_brick = 8
    return s


def new_tracer_desc() -> er_tracer_desc:
    t = er_tracer_desc()
    plf_init(t.opacity)
    plf_init(t.glossiness)
    for tf in (t.diffuse, t.specular, t.emission):
        for c in range(3):
            plf_init(tf.plf[c])
    t.settings = default_render_settings()
    for i in range(ER_MAX_INDICES):
        t.light_ids[i] = -1       # Indices() fills -1 (Source/vector.h:557-563)
        t.object_ids[i] = -1
        t.clipping_object_ids[i] = -1
    return t


def new_texture_desc() -> er_texture_desc:
    """ErTexture() defaults (Source/ertexture.h:30-40)."""
    t = er_texture_desc()
    t.type = TEXTURE_PROCEDURAL
    t.output_level = 1.0
    t.bitmap_id = -1
    t.procedural.type = PROCEDURAL_UNIFORM
    for c in range(3):
        plf_init(t.procedural.gradient.plf[c])
    return t


# ---------------------------------------------------------------------------
# library loading
# ---------------------------------------------------------------------------

_PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG_DIR, "_build", "libexposurerender.so")


class ErError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_lib = None


def load_library(path: str | None = None):
    """Loads libexposurerender.so (raises if it was not built: there is no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(f"{p} is missing: run __graft_entry__.build() to compile the CUDA library")
    lib = ctypes.CDLL(p)
    _declare(lib)
    if path is None:
        _lib = lib
    return lib


def _declare(lib) -> None:
    i32p = POINTER(c_int32)
    sig = {
        "er_abi_version": (c_int32, []),
        "er_last_error_message": (c_char_p, []),
        "er_set_device": (c_int32, [c_int32]),
        "er_set_stream": (c_int32, [c_void_p]),
        "er_synchronize": (c_int32, []),
        "er_reset": (c_int32, []),
        "er_default_render_settings": (None, [POINTER(er_render_settings)]),
        "er_plf_init": (None, [POINTER(er_plf)]),
        "er_plf_add_node": (None, [POINTER(er_plf), c_float, c_float]),
        "er_bind_tracer": (c_int32, [POINTER(er_tracer_desc), i32p]),
        "er_unbind_tracer": (c_int32, [c_int32]),
        "er_bind_volume": (c_int32, [POINTER(er_volume_desc), i32p]),
        "er_unbind_volume": (c_int32, [c_int32]),
        "er_update_volume_region": (c_int32, [c_int32, POINTER(c_int32), POINTER(c_int32), c_void_p]),
        "er_update_volume_region_device": (c_int32, [c_int32, POINTER(c_int32), POINTER(c_int32), c_void_p, c_void_p]),
        "er_bind_light": (c_int32, [POINTER(er_light_desc), i32p]),
        "er_unbind_light": (c_int32, [c_int32]),
        "er_bind_object": (c_int32, [POINTER(er_object_desc), i32p]),
        "er_unbind_object": (c_int32, [c_int32]),
        "er_bind_clipping_object": (c_int32, [POINTER(er_clipping_object_desc), i32p]),
        "er_unbind_clipping_object": (c_int32, [c_int32]),
        "er_bind_texture": (c_int32, [POINTER(er_texture_desc), i32p]),
        "er_unbind_texture": (c_int32, [c_int32]),
        "er_bind_bitmap": (c_int32, [POINTER(er_bitmap_desc), i32p]),
        "er_unbind_bitmap": (c_int32, [c_int32]),
        "er_render_estimate": (c_int32, [c_int32]),
        "er_get_estimate": (c_int32, [c_int32, c_void_p]),
        "er_get_auto_focus_distance": (c_int32, [c_int32, c_int32, c_int32, POINTER(c_float)]),
        "er_get_no_iterations": (c_int32, [c_int32, i32p]),
        "er_render_spp": (c_int32, [c_int32, c_int32]),
        "er_reset_accumulation": (c_int32, [c_int32]),
        "er_get_frame_estimate": (c_int32, [c_int32, c_void_p]),
        "er_get_running_estimate": (c_int32, [c_int32, c_void_p]),
        "er_get_seeds": (c_int32, [c_int32, c_void_p]),
        "er_set_seeds": (c_int32, [c_int32, c_void_p]),
        "er_get_film_size": (c_int32, [c_int32, i32p, i32p]),
        "er_trace_sum_device": (c_int32, [c_int32, c_int32, c_uint32, c_uint32, c_void_p, c_int32, c_void_p]),
        "er_batch_create": (c_int32, [POINTER(er_batch_view), c_int32, c_int32, c_int32, i32p]),
        "er_batch_launch": (c_int32, [c_int32, c_void_p]),
        "er_batch_advance": (c_int32, [c_int32, c_uint32, c_void_p]),
        "er_batch_set_tuning": (c_int32, [c_int32, c_int32, c_int32]),
        "er_batch_info": (c_int32, [c_int32, i32p, i32p, POINTER(ctypes.c_int64)]),
        "er_batch_set_stages": (c_int32, [c_int32, c_int32]),
        "er_batch_autotune": (c_int32, [c_int32, c_void_p, i32p, POINTER(c_float)]),
        "er_batch_destroy": (c_int32, [c_int32]),
        "er_autotune_tracer": (c_int32, [c_int32, c_int32, POINTER(er_tune_result)]),
        "er_get_render_settings": (c_int32, [c_int32, POINTER(er_render_settings)]),
        "er_profile_enable": (c_int32, [c_int32]),
        "er_medium_majorant": (c_int32, [c_int32, POINTER(er_medium_desc), c_float, c_float, c_void_p, c_void_p]),
        "er_medium_render": (c_int32, [c_int32, POINTER(er_medium_desc), c_int32, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p]),
        "er_medium_render_f64": (c_int32, [c_int32, POINTER(er_medium_desc), c_int32, c_uint32, c_uint32, c_void_p, c_void_p,
                                           c_void_p]),
        "er_medium_adjoint": (c_int32, [c_int32, POINTER(er_medium_desc), c_int32, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p,
                                        c_void_p, c_void_p]),
        "er_profile_read": (c_int32, [c_void_p, c_void_p]),
        "er_trace_frame_device": (c_int32, [c_int32, c_void_p, c_void_p, c_void_p]),
        "er_post_frame_device": (c_int32, [c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_int32, c_float, c_int32, c_void_p]),
        "er_tonemap_device": (c_int32, [c_void_p, c_float, c_void_p, c_int32, c_int32, c_float, c_void_p]),
        "er_bilateral_device": (c_int32, [c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_int32, c_float, c_float, c_void_p]),
        "er_gradient_magnitude": (c_int32, [c_int32, c_void_p, POINTER(c_float)]),
        "er_math_eval_device": (c_int32, [c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p]),
        "er_build_majorant_device": (c_int32, [c_void_p, POINTER(c_int32), c_int32, c_void_p, c_int32, c_float, c_void_p, c_void_p]),
        "er_build_majorant_device_noalloc": (c_int32, [c_void_p, POINTER(c_int32), c_int32, c_void_p, c_int32, c_float, c_void_p,
                                                       c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def check(status: int) -> None:
    if status != ER_OK:
        msg = _lib.er_last_error_message().decode() if _lib is not None else ""
        raise ErError(status, msg)


def exported_symbols() -> list[str]:
    """Every function name include/er_capi.h declares (parsed from the header)."""
    import re
    here = os.path.dirname(_PKG_DIR)
    hdr = os.path.join(here, "include", "er_capi.h")
    names = re.findall(r"ER_API\s+[\w\s\*]+?\b(er_\w+)\s*\(", open(hdr).read())
    return names
