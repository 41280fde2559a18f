"""ctypes loader of the CPU oracle (test infrastructure).

`or_` = oracle/_build/liberoracle.so, the C restatement of the reference path;
`fp64_` = oracle/_build/liberfp64.so, the same restatement in binary64;
`ref_` = oracle/_ref/liberref.so, the reference's own code built for this host
(present only where the reference sources were available at build time).
"""
from __future__ import annotations

import ctypes
import importlib
import os
import subprocess
import sys
from ctypes import POINTER, c_double, c_float, c_int32, c_uint32, c_void_p

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
PKG = importlib.import_module("exposure-render_gb300")
C = PKG.capi

ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "liberoracle.so")
FP64_SO = os.path.join(ROOT, "oracle", "_build", "liberfp64.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "liberref.so")


def build_oracle() -> None:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True)


class Oracle:
    def __init__(self, path: str, prefix: str):
        self.lib = ctypes.CDLL(path)
        self.p = prefix
        f = self.fn
        f("scene_create", c_void_p, [POINTER(C.er_tracer_desc), POINTER(C.er_volume_desc), c_void_p, c_int32, c_void_p, c_int32])
        f("scene_destroy", None, [c_void_p])
        f("scene_set_objects", None, [c_void_p, c_void_p, c_int32])
        f("scene_set_bitmaps", None, [c_void_p, c_void_p, c_int32])
        if prefix != "ref_":
            f("segments_hit_shape", None, [POINTER(C.er_shape), c_int32, c_void_p, c_void_p])
            f("scene_set_clipping_objects", None, [c_void_p, c_void_p, c_int32])
        f("render_frame", None, [c_void_p, c_void_p, c_void_p, c_int32])
        f("render_sum", None, [c_void_p, c_int32, c_uint32, c_uint32, c_int32, c_int32, c_int32, c_int32, c_void_p, c_int32])
        if prefix != "ref_":
            f("autofocus", c_float if prefix == "or_" else c_double, [c_void_p, c_int32, c_int32, c_uint32, c_uint32])
            f("render_stats", None, [c_void_p])
            f("render_moments", None, [c_void_p, c_int32, c_uint32, c_uint32, c_int32, c_int32, c_int32, c_int32, c_void_p,
                                       c_void_p, c_int32])
        if prefix != "ref_":
            f("dm_attach", None, [c_void_p, c_void_p, c_void_p, c_int32, self._real_c(prefix), c_void_p,
                                  self._real_c(prefix), c_void_p, c_int32])
            f("dm_set_model", None, [c_void_p, c_int32, self._real_c(prefix)])
            f("dm_render", None, [c_void_p, c_int32, c_uint32, c_uint32, c_void_p, c_void_p, c_int32])
            f("dm_adjoint", None, [c_void_p, c_int32, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p, c_int32])
        # the FP64 build takes double buffers wherever the float build takes float
        self.real = np.float64 if prefix == "fp64_" else np.float32
        f("post_frame", None, [c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_int32, c_float])
        f("lookups_per_sample", c_double, [])
        f("rng_draws", None, [c_uint32, c_uint32, c_int32, c_void_p])
        f("rng_get2_get3", None, [c_uint32, c_uint32, c_void_p])
        f("plf_evaluate", None, [POINTER(C.er_plf), c_int32, c_void_p, c_void_p])
        f("get_intensity", None, [c_void_p, c_int32, c_void_p, c_void_p])
        f("normalized_gradient", None, [c_void_p, c_int32, c_void_p, c_void_p])
        f("gradient_magnitude", None, [c_void_p, c_int32, c_void_p, c_void_p])
        f("intersect_volume_box", None, [c_void_p, c_int32, c_void_p, c_void_p])
        f("concentric_sample_disk", None, [c_int32, c_void_p, c_void_p])
        f("tonemap", None, [c_int32, c_void_p, c_float, c_void_p])
        f("camera_ray", None, [c_void_p, c_int32, c_int32, c_void_p, c_void_p])
        f("camera_frame", None, [c_void_p, c_void_p])
        f("volume_frame", None, [c_void_p, c_void_p])
        if prefix == "or_":
            f("bilateral", None, [c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_int32, c_float, c_float])
            f("gradient_magnitude_volume", c_float, [c_void_p, c_void_p])
            f("math_eval", None, [c_int32, c_int32, c_void_p, c_void_p, c_void_p])
            f("majorant_grid", None, [c_void_p, c_void_p, c_int32, c_void_p, c_int32, c_float, c_void_p])
            f("dda_walk", None, [c_void_p, c_int32, c_void_p, c_int32, c_int32, c_void_p, c_void_p])
            f("brick_bound", None, [c_void_p, c_int32, c_void_p, c_void_p, c_void_p])

    @staticmethod
    def _real_c(prefix):
        return c_double if prefix == "fp64_" else c_float

    def fn(self, name, res, args):
        h = getattr(self.lib, self.p + name)
        h.restype = res
        h.argtypes = args
        setattr(self, name, h)


STAT_NAMES = ("free_flight_lookups", "majorant_reads", "shadow_lookups", "shadow_majorant_reads", "events", "shadow_rays",
              "normal_lookups")


def render_stats(orc: Oracle) -> dict:
    """Work counters per sample of the oracle's last render, plus the total
    lookups per sample."""
    out = np.zeros(len(STAT_NAMES), dtype=np.float64)
    orc.render_stats(out.ctypes.data_as(c_void_p))
    d = dict(zip(STAT_NAMES, out.tolist()))
    d["lookups"] = float(orc.lookups_per_sample())
    return d


def ptr(a: np.ndarray):
    return a.ctypes.data_as(c_void_p)


class SceneHandle:
    """An oracle scene built from a scenes.Scene; keeps the inputs alive."""

    def __init__(self, orc: Oracle, scene):
        self.orc = orc
        self.scene = scene
        self.vd = scene.volume_desc()
        self.la = scene.light_array()
        self.ta = scene.texture_array()
        self.h = orc.scene_create(ctypes.byref(scene.tracer), ctypes.byref(self.vd), ctypes.cast(self.la, c_void_p),
                                  len(scene.lights), ctypes.cast(self.ta, c_void_p), len(scene.textures))
        bms = getattr(scene, "bitmaps", [])
        if bms:
            self.bitmap_pixels = [np.ascontiguousarray(b, dtype=np.uint8) for b in bms]
            self.ba = (C.er_bitmap_desc * len(bms))()
            for i, px in enumerate(self.bitmap_pixels):
                self.ba[i].resolution[0] = px.shape[1]
                self.ba[i].resolution[1] = px.shape[0]
                self.ba[i].pixels = px.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
            orc.scene_set_bitmaps(self.h, ctypes.cast(self.ba, c_void_p), len(bms))
        objs = getattr(scene, "objects", [])
        if objs:
            self.oa = (C.er_object_desc * len(objs))(*objs)
            orc.scene_set_objects(self.h, ctypes.cast(self.oa, c_void_p), len(objs))
        clips = getattr(scene, "clipping_objects", [])
        if clips:
            if orc.p == "ref_":
                raise ValueError("the reference build does not apply clipping objects")
            self.ca = (C.er_clipping_object_desc * len(clips))(*clips)
            orc.scene_set_clipping_objects(self.h, ctypes.cast(self.ca, c_void_p), len(clips))

    def close(self):
        if self.h:
            self.orc.scene_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def render_frame(self, lanes: np.ndarray, nthreads: int = 8) -> np.ndarray:
        W, H = self.scene.width, self.scene.height
        frame = np.zeros((H, W, 4), dtype=np.float32)
        self.orc.render_frame(self.h, ptr(lanes), ptr(frame), nthreads)
        return frame

    def render_sum(self, spp: int, view: int = 0, first: int = 0, rect=None, nthreads: int = 8) -> np.ndarray:
        W, H = self.scene.width, self.scene.height
        x0, y0, w, h = rect if rect is not None else (0, 0, W, H)
        out = np.zeros((h, w, 4), dtype=self.orc.real)
        self.orc.render_sum(self.h, spp, view, first, x0, y0, w, h, ptr(out), nthreads)
        return out

    def render_moments(self, spp: int, view: int = 0, first: int = 0, rect=None, nthreads: int = 8):
        """(sum, sum of squares) per pixel and component"""
        W, H = self.scene.width, self.scene.height
        x0, y0, w, h = rect if rect is not None else (0, 0, W, H)
        out = np.zeros((h, w, 4), dtype=self.orc.real)
        out2 = np.zeros((h, w, 4), dtype=self.orc.real)
        self.orc.render_moments(self.h, spp, view, first, x0, y0, w, h, ptr(out), ptr(out2), nthreads)
        return out, out2


class MediumHandle(SceneHandle):
    """An oracle scene with a differentiable medium attached: `rho` (Z, Y, X)
    float density, `tf` opacity B-spline values (model 0) or the values of
    the tracer's opacity nodes (model 1, the tracer's transfer functions and
    shading), fixed `majorant` grid."""

    def __init__(self, orc: Oracle, scene, rho, tf, scale, albedo, q, majorant, brick, model=0, gm_inv=0.0):
        super().__init__(orc, scene)
        r = orc.real
        self.rho = np.ascontiguousarray(rho, dtype=r)
        self.tf = np.ascontiguousarray(tf, dtype=r)
        self.albedo = np.ascontiguousarray(albedo, dtype=r)
        self.maj = np.ascontiguousarray(majorant, dtype=r)
        orc.dm_attach(self.h, ptr(self.rho), ptr(self.tf), len(self.tf), scale, ptr(self.albedo), q, ptr(self.maj), brick)
        orc.dm_set_model(self.h, model, gm_inv)

    def render(self, spp, view=0, first=0, keep_samples=False, nthreads=8):
        W, H = self.scene.width, self.scene.height
        r = self.orc.real
        out = np.zeros((H, W, 3), dtype=r)
        smp = np.zeros((spp, H, W, 3), dtype=r) if keep_samples else None
        self.orc.dm_render(self.h, spp, view, first, ptr(out), ptr(smp) if keep_samples else None, nthreads)
        return (out, smp) if keep_samples else out

    def adjoint(self, spp, dimg, samples, view=0, first=0, nthreads=8):
        r = self.orc.real
        g_rho = np.zeros(self.rho.shape, dtype=r)
        g_tf = np.zeros(self.tf.shape, dtype=r)
        d = np.ascontiguousarray(dimg, dtype=r)
        f = np.ascontiguousarray(samples, dtype=r)
        self.orc.dm_adjoint(self.h, spp, view, first, ptr(d), ptr(f), ptr(g_rho), ptr(g_tf), nthreads)
        return g_rho, g_tf


def initial_lanes(seed: int, width: int, height: int) -> np.ndarray:
    """Per-pixel RNG lanes of a fresh tracer: er_seed_lanes(seed, 0, pixel, 0xffffffff)."""
    n = width * height
    lanes = np.empty(2 * n, dtype=np.uint32)
    for p in range(n):
        a, b = seed_lanes(seed, 0, p, 0xFFFFFFFF)
        lanes[p] = a
        lanes[n + p] = b
    return lanes


def _hash32(x):
    x &= 0xFFFFFFFF
    x ^= x >> 16
    x = (x * 0x7FEB352D) & 0xFFFFFFFF
    x ^= x >> 15
    x = (x * 0x846CA68B) & 0xFFFFFFFF
    x ^= x >> 16
    return x


def seed_lanes(seed, view, pixel, sample):
    """Python restatement of er_seed_lanes (include/er_math.h)."""
    h = _hash32((seed * 0x9E3779B9 + 0x632BE5AB) & 0xFFFFFFFF)
    h = _hash32(h ^ ((view * 0x85EBCA6B) & 0xFFFFFFFF))
    h = _hash32((h + pixel) & 0xFFFFFFFF)
    h = _hash32(h ^ ((sample * 0xC2B2AE35) & 0xFFFFFFFF))
    a = h
    b = _hash32(h ^ 0x68E31DA4)
    if a in (0, 0x9068FFFF):
        a = 0x2545F491
    if b in (0, 0x464FFFFF):
        b = 0x4F6CDD1D
    return a, b


def load_oracle() -> Oracle:
    if not os.path.exists(ORACLE_SO):
        build_oracle()
    return Oracle(ORACLE_SO, "or_")


def load_fp64() -> Oracle:
    """The FP64 oracle (oracle/_build/liberfp64.so): converged reference images."""
    if not os.path.exists(FP64_SO):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "fp64"], check=True)
    return Oracle(FP64_SO, "fp64_")


def load_ref() -> Oracle | None:
    if not os.path.exists(REF_SO):
        return None
    return Oracle(REF_SO, "ref_")
