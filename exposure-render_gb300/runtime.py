"""Python host side over the C ABI: binds a scenes.Scene the way a reference
application binds its Er* objects (BindTexture, BindLight, BindVolume,
BindTracer - Source/exposurerender.h:32-38) and exposes the render calls.

Every call goes through libexposurerender.so; a missing library raises.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_float, c_int32

import numpy as np

from . import capi as C


class Renderer:
    """One bound scene (texture/light/volume/tracer IDs) in the library context."""

    def __init__(self, scene, lib=None):
        self.lib = lib or C.load_library()
        self.scene = scene
        self.texture_ids = []
        self.light_ids = []
        # BindBitmap (Source/exposurerender.h:38): bitmap i of the scene
        self.bitmap_ids = []
        for px in getattr(scene, "bitmaps", []):
            px = np.ascontiguousarray(px, dtype=np.uint8)
            b = C.er_bitmap_desc()
            b.resolution[0], b.resolution[1] = px.shape[1], px.shape[0]
            b.pixels = px.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
            i = c_int32(-1)
            C.check(self.lib.er_bind_bitmap(byref(b), byref(i)))
            self.bitmap_ids.append(i.value)
        for t in scene.textures:
            tc = C.er_texture_desc()
            ctypes.memmove(byref(tc), byref(t), ctypes.sizeof(t))
            if tc.type == C.TEXTURE_BITMAP:
                k = tc.bitmap_id
                tc.bitmap_id = self.bitmap_ids[k] if 0 <= k < len(self.bitmap_ids) else -1
            i = c_int32(-1)
            C.check(self.lib.er_bind_texture(byref(tc), byref(i)))
            self.texture_ids.append(i.value)
        for L in scene.lights:
            Lc = C.er_light_desc()
            ctypes.memmove(byref(Lc), byref(L), ctypes.sizeof(L))
            if Lc.texture_id >= 0:
                Lc.texture_id = self.texture_ids[Lc.texture_id]
            i = c_int32(-1)
            C.check(self.lib.er_bind_light(byref(Lc), byref(i)))
            self.light_ids.append(i.value)
        # BindObject (Source/exposurerender.h:35): object i of the scene is the
        # i-th bound object, the order IntersectObjects walks (Source/objects.h:52)
        self.object_ids = []
        for o in getattr(scene, "objects", []):
            oc = C.er_object_desc()
            ctypes.memmove(byref(oc), byref(o), ctypes.sizeof(o))
            for f in ("diffuse_texture_id", "specular_texture_id", "glossiness_texture_id"):
                k = getattr(oc, f)
                setattr(oc, f, self.texture_ids[k] if 0 <= k < len(self.texture_ids) else -1)
            i = c_int32(-1)
            C.check(self.lib.er_bind_object(byref(oc), byref(i)))
            self.object_ids.append(i.value)
        # BindClippingObject (Source/exposurerender.h:36): clipping object i of
        # the scene; the tracer's clipping_object_ids index this list
        self.clipping_ids = []
        for k in getattr(scene, "clipping_objects", []):
            i = c_int32(-1)
            C.check(self.lib.er_bind_clipping_object(byref(k), byref(i)))
            self.clipping_ids.append(i.value)
        vd = scene.volume_desc()
        vid = c_int32(-1)
        C.check(self.lib.er_bind_volume(byref(vd), byref(vid)))
        self.volume_id = vid.value
        t = C.er_tracer_desc()
        ctypes.memmove(byref(t), byref(scene.tracer), ctypes.sizeof(t))
        t.volume_id = self.volume_id
        for k in range(t.light_count):
            src = scene.tracer.light_ids[k]
            t.light_ids[k] = self.light_ids[src] if 0 <= src < len(self.light_ids) else -1
        for k in range(t.object_count):
            src = scene.tracer.object_ids[k]
            t.object_ids[k] = self.object_ids[src] if 0 <= src < len(self.object_ids) else -1
        for k in range(max(0, min(t.clipping_object_count, C.ER_MAX_INDICES))):
            src = scene.tracer.clipping_object_ids[k]
            t.clipping_object_ids[k] = self.clipping_ids[src] if 0 <= src < len(self.clipping_ids) else -1
        self.tracer_desc = t
        tid = c_int32(-1)
        C.check(self.lib.er_bind_tracer(byref(t), byref(tid)))
        self.tracer_id = tid.value

    @property
    def width(self) -> int:
        return self.scene.width

    @property
    def height(self) -> int:
        return self.scene.height

    def rebind_tracer(self) -> None:
        tid = c_int32(self.tracer_id)
        C.check(self.lib.er_bind_tracer(byref(self.tracer_desc), byref(tid)))

    def render_estimate(self) -> None:
        C.check(self.lib.er_render_estimate(self.tracer_id))

    def render_spp(self, spp: int) -> None:
        C.check(self.lib.er_render_spp(self.tracer_id, spp))

    def get_estimate(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 4), dtype=np.uint8)
        C.check(self.lib.er_get_estimate(self.tracer_id, out.ctypes.data))
        return out

    def get_running_estimate(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 4), dtype=np.float32)
        C.check(self.lib.er_get_running_estimate(self.tracer_id, out.ctypes.data))
        return out

    def get_frame_estimate(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 4), dtype=np.float32)
        C.check(self.lib.er_get_frame_estimate(self.tracer_id, out.ctypes.data))
        return out

    def get_seeds(self) -> np.ndarray:
        out = np.empty(2 * self.width * self.height, dtype=np.uint32)
        C.check(self.lib.er_get_seeds(self.tracer_id, out.ctypes.data))
        return out

    def no_iterations(self) -> int:
        n = c_int32(0)
        C.check(self.lib.er_get_no_iterations(self.tracer_id, byref(n)))
        return n.value

    def trace_sum_device(self, d_sum_ptr: int, spp: int, view: int = 0, first: int = 0, accumulate: int = 0, stream=None) -> None:
        C.check(self.lib.er_trace_sum_device(self.tracer_id, spp, view, first, d_sum_ptr, accumulate, stream))

    def trace_frame_device(self, d_lanes_ptr: int, d_frame_ptr: int, stream=None) -> None:
        C.check(self.lib.er_trace_frame_device(self.tracer_id, d_lanes_ptr, d_frame_ptr, stream))

    def autotune(self, probe_spp: int = 2) -> dict:
        """er_autotune_tracer; the chosen settings are copied into tracer_desc so
        that a later rebind_tracer keeps them"""
        r = C.er_tune_result()
        C.check(self.lib.er_autotune_tracer(self.tracer_id, probe_spp, byref(r)))
        s = self.tracer_desc.settings
        s.majorant_brick, s.tune_primary, s.tune_shadow = r.majorant_brick, r.tune_primary, r.tune_shadow
        s.tune_shade = r.tune_shade
        s.tune_stages = r.tune_stages
        return {"majorant_brick": r.majorant_brick, "tune_primary": r.tune_primary, "tune_shadow": r.tune_shadow,
                "tune_shade": r.tune_shade, "tune_stages": r.tune_stages,
                "from_cache": bool(r.from_cache), "msamples_per_s": r.msamples_per_s, "candidates": r.candidates}

    def gradient_magnitude(self, d_gm_ptr=None) -> float:
        m = c_float(0.0)
        C.check(self.lib.er_gradient_magnitude(self.volume_id, d_gm_ptr, byref(m)))
        return m.value

    def close(self) -> None:
        lib = self.lib
        lib.er_unbind_tracer(self.tracer_id)
        lib.er_unbind_volume(self.volume_id)
        for i in self.object_ids:
            lib.er_unbind_object(i)
        for i in self.light_ids:
            lib.er_unbind_light(i)
        for i in self.texture_ids:
            lib.er_unbind_texture(i)
        for i in self.bitmap_ids:
            lib.er_unbind_bitmap(i)
        for i in getattr(self, "clipping_ids", []):
            lib.er_unbind_clipping_object(i)
        self.bitmap_ids, self.clipping_ids = [], []
        self.light_ids, self.texture_ids, self.object_ids = [], [], []


class Batch:
    """Many views rendered by one submission (er_batch_create / er_batch_launch).

    `views` holds (tracer_id, spp, d_sum_ptr, camera or None) tuples or
    er_batch_view records; `first`, `view` and `accumulate` default to 0 and
    view index i.  The plan is made at construction; binding anything
    re-plans it at the next launch."""

    def __init__(self, views, flags=C.ER_BATCH_GRAPH, window_items=0, lib=None, accumulate=0, display=0):
        self.lib = lib or C.load_library()
        n = len(views)
        arr = (C.er_batch_view * n)()
        self._cams = []
        for i, v in enumerate(views):
            if isinstance(v, C.er_batch_view):
                arr[i] = v
                continue
            tid, spp, d_sum, cam = v
            b = arr[i]
            b.tracer_id = tid
            b.spp = spp
            b.view = i
            b.first_sample = 0
            b.d_sum_xyza = d_sum
            b.accumulate = accumulate
            b.display = display
            if cam is not None:
                c = C.er_camera_desc()
                ctypes.memmove(byref(c), byref(cam), ctypes.sizeof(c))
                self._cams.append(c)
                b.camera = ctypes.pointer(c)
        self.views = arr
        bid = c_int32(-1)
        C.check(self.lib.er_batch_create(arr, n, flags, window_items, byref(bid)))
        self.batch_id = bid.value

    def launch(self, stream=None) -> None:
        C.check(self.lib.er_batch_launch(self.batch_id, stream))

    def advance(self, samples: int, stream=None) -> None:
        C.check(self.lib.er_batch_advance(self.batch_id, samples, stream))

    def set_tuning(self, primary: int = 0, shadow: int = 0) -> None:
        C.check(self.lib.er_batch_set_tuning(self.batch_id, primary, shadow))

    def set_stages(self, tune_stages: int) -> None:
        C.check(self.lib.er_batch_set_stages(self.batch_id, tune_stages))

    def autotune(self, stream=None) -> dict:
        """er_batch_autotune: the fastest tune_stages for this batch, timed on
        whole launches (the views' sums are rendered into)"""
        st, m = c_int32(0), ctypes.c_float(0.0)
        C.check(self.lib.er_batch_autotune(self.batch_id, stream, byref(st), byref(m)))
        return {"tune_stages": st.value, "msamples_per_s": m.value}

    def info(self) -> dict:
        w, s, q = c_int32(0), c_int32(0), ctypes.c_int64(0)
        C.check(self.lib.er_batch_info(self.batch_id, byref(w), byref(s), byref(q)))
        return {"windows": w.value, "segments": s.value, "queue_bytes": q.value}

    def close(self) -> None:
        if self.batch_id >= 0:
            self.lib.er_batch_destroy(self.batch_id)
            self.batch_id = -1
