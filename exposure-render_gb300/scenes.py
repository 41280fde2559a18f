"""Seeded synthetic scenes with the shapes, sizes and value ranges of the
workloads the renderer is measured on.

The reference ships no datasets (its GUI example used a CT scan that is not
distributed with it); every volume here is generated from a fixed seed, so a
scene is fully described by its name and parameters.

    c1  128^3 uint16 sum of 12 anisotropic Gaussian blobs (amplitude U[500,4000])
        plus uniform noise U[0,50]; 4-node opacity/albedo transfer function;
        one square area light; pinhole camera; 256^2; 64 spp.
    c2  512^3 uint16 nested spherical shells (~1000/1400/2500 with Gaussian
        noise sigma 30) in a soft-tissue ellipsoid; 16-node transfer function,
        hybrid phase/BRDF (roughness 0.3); two area lights plus an environment
        sphere light; 1024^2; 256 spp; bilateral filter and tone map.
    c3  batched forward: 64 random orbit views over three blob volumes of
        96^3, 256^3 and 384x384x256 (x, y, z); films drawn from
        {128, 256, 384, 512}^2; 32-128 spp per view; delta tracking, full MIS.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import capi as C


@dataclass
class Scene:
    name: str
    volume: np.ndarray                      # uint16, shape (Z, Y, X), x fastest
    spacing: tuple = (1.0, 1.0, 1.0)
    normalize_size: int = 1
    tracer: C.er_tracer_desc = None
    lights: list = field(default_factory=list)      # er_light_desc, light i has ID i
    textures: list = field(default_factory=list)    # er_texture_desc, texture i has ID i
    spp: int = 1
    objects: list = field(default_factory=list)     # er_object_desc, object i has ID i
    bitmaps: list = field(default_factory=list)     # uint8 (H, W, 4) RGBA arrays, bitmap i has ID i
    clipping_objects: list = field(default_factory=list)   # er_clipping_object_desc, clipping object i has ID i

    @property
    def width(self) -> int:
        return int(self.tracer.camera.film_size[0])

    @property
    def height(self) -> int:
        return int(self.tracer.camera.film_size[1])

    def volume_desc(self) -> C.er_volume_desc:
        v = np.ascontiguousarray(self.volume, dtype=np.uint16)
        self.volume = v
        d = C.er_volume_desc()
        d.resolution[0] = v.shape[2]
        d.resolution[1] = v.shape[1]
        d.resolution[2] = v.shape[0]
        for i in range(3):
            d.spacing[i] = self.spacing[i]
        d.normalize_size = self.normalize_size
        d.voxels = v.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))
        return d

    def light_array(self):
        arr = (C.er_light_desc * max(1, len(self.lights)))()
        for i, l in enumerate(self.lights):
            arr[i] = l
        return arr

    def texture_array(self):
        arr = (C.er_texture_desc * max(1, len(self.textures)))()
        for i, t in enumerate(self.textures):
            arr[i] = t
        return arr


# ---------------------------------------------------------------------------
# geometry helpers
# ---------------------------------------------------------------------------

def look_at_tm(pos, target, up):
    """Shape transform whose local +z axis points from pos towards target.

    Returns (TM, InvTM) as float32-rounded 4x4 lists (rows), the layout of
    Matrix44::NN (Source/matrix.h:55) used by TransformPoint
    (Source/geometry.h:43-52)."""
    p = np.asarray(pos, dtype=np.float64)
    n = np.asarray(target, dtype=np.float64) - p
    n /= np.linalg.norm(n)
    u = np.cross(np.asarray(up, dtype=np.float64), n)
    if np.linalg.norm(u) < 1e-9:
        u = np.cross(np.array([1.0, 0.0, 0.0]), n)
    u /= np.linalg.norm(u)
    v = np.cross(n, u)
    tm = np.eye(4)
    tm[:3, 0], tm[:3, 1], tm[:3, 2], tm[:3, 3] = u, v, n, p
    inv = np.linalg.inv(tm)
    return tm.astype(np.float32).tolist(), inv.astype(np.float32).tolist()


def make_shape(shape_type, tm_inv, size=(1.0, 1.0, 1.0), inner=0.0, outer=1.0, one_sided=0) -> C.er_shape:
    s = C.er_shape()
    tm, inv = tm_inv
    C.set_matrix(s.tm, tm)
    C.set_matrix(s.inv_tm, inv)
    s.one_sided = one_sided
    s.type = shape_type
    for i in range(3):
        s.size[i] = size[i]
    s.inner_radius = inner
    s.outer_radius = outer
    s.area = 0.0
    return s


def uniform_texture(color=(1.0, 1.0, 1.0), level=1.0) -> C.er_texture_desc:
    t = C.new_texture_desc()
    t.procedural.type = C.PROCEDURAL_UNIFORM
    for i in range(3):
        t.procedural.uniform_color[i] = color[i]
    t.output_level = level
    return t


def gradient_texture(nodes_rgb, level=1.0, repeat=(1.0, 1.0)) -> C.er_texture_desc:
    t = C.new_texture_desc()
    t.procedural.type = C.PROCEDURAL_GRADIENT
    t.procedural.gradient = C.make_color_tf(nodes_rgb)
    t.output_level = level
    t.repeat[0], t.repeat[1] = repeat
    return t


def make_camera(film, pos, target, up=(0.0, 0.0, 1.0), fov=35.0, exposure=1.0) -> C.er_camera_desc:
    c = C.er_camera_desc()
    c.film_size[0], c.film_size[1] = film
    for i in range(3):
        c.pos[i] = pos[i]
        c.target[i] = target[i]
        c.up[i] = up[i]
    c.focal_distance = -1.0
    c.aperture_size = 0.0
    c.clip_near = 0.0
    c.clip_far = 1000.0
    c.exposure = exposure
    c.gamma = 2.2
    c.fov = fov
    return c


def orbit_camera(rng, film, radius=2.0, fov=35.0, exposure=1.0) -> C.er_camera_desc:
    """Random orbit camera looking at the volume centre."""
    theta = rng.uniform(0.0, 2.0 * np.pi)
    z = rng.uniform(-0.5, 0.5)
    r = np.sqrt(1.0 - z * z)
    pos = (radius * r * np.cos(theta), radius * r * np.sin(theta), radius * z)
    return make_camera(film, pos, (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), fov, exposure)


# ---------------------------------------------------------------------------
# volumes
# ---------------------------------------------------------------------------

def blob_volume(shape_zyx, n_blobs=12, seed=1, amp=(500.0, 4000.0), sigma=(0.04, 0.14), noise=50.0) -> np.ndarray:
    """Sum of `n_blobs` axis-aligned anisotropic Gaussians plus uniform noise,
    truncated to uint16 (x fastest)."""
    Z, Y, X = shape_zyx
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.2, 0.8, size=(n_blobs, 3)) * np.array([X, Y, Z])
    sig = rng.uniform(sigma[0], sigma[1], size=(n_blobs, 3)) * np.array([X, Y, Z])
    amps = rng.uniform(amp[0], amp[1], size=n_blobs)
    xs = np.arange(X, dtype=np.float32)
    ys = np.arange(Y, dtype=np.float32)
    vol = np.zeros((Z, Y, X), dtype=np.float32)
    for k in range(n_blobs):
        gx = np.exp(-0.5 * ((xs - centres[k, 0]) / sig[k, 0]) ** 2).astype(np.float32)
        gy = np.exp(-0.5 * ((ys - centres[k, 1]) / sig[k, 1]) ** 2).astype(np.float32)
        gxy = (gy[:, None] * gx[None, :]) * np.float32(amps[k])
        for z in range(Z):
            gz = np.float32(np.exp(-0.5 * ((z - centres[k, 2]) / sig[k, 2]) ** 2))
            if gz > 1e-7:
                vol[z] += gxy * gz
    for z in range(Z):
        vol[z] += rng.uniform(0.0, noise, size=(Y, X)).astype(np.float32)
    return np.clip(np.floor(vol), 0, 65535).astype(np.uint16)


def shell_volume(n=512, seed=2, noise_sigma=30.0) -> np.ndarray:
    """Nested spherical shells in a soft-tissue ellipsoid (CT-like), uint16."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, n, n), dtype=np.uint16)
    c = (n - 1) / 2.0
    xs = (np.arange(n, dtype=np.float32) - c) / n
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    for zi in range(n):
        z = np.float32((zi - c) / n)
        ell = (X / 0.46) ** 2 + (Y / 0.40) ** 2 + (z / 0.36) ** 2 <= 1.0
        r = np.sqrt(X * X + Y * Y + z * z)
        v = np.where(ell, 1000.0, 0.0).astype(np.float32)
        v = np.where((r >= 0.26) & (r < 0.30), 1400.0, v)
        v = np.where((r >= 0.15) & (r < 0.19), 2500.0, v)
        v = np.where(r < 0.07, 1400.0, v)
        v = v + np.where(ell, rng.normal(0.0, noise_sigma, size=v.shape), 0.0).astype(np.float32)
        out[zi] = np.clip(np.floor(v), 0, 65535).astype(np.uint16)
    return out


# ---------------------------------------------------------------------------
# configurations
# ---------------------------------------------------------------------------

def c1_tracer(film=(256, 256), phase=False) -> C.er_tracer_desc:
    t = C.new_tracer_desc()
    # 4-node opacity; the last node sits between integers so no reachable
    # intensity equals it (PLF::Evaluate returns 0 exactly at the last node,
    # Source/plf.h:79-90)
    t.opacity = C.make_plf([(0.0, 0.0), (400.0, 0.0), (1500.0, 0.6), (4000.5, 1.0)])
    t.diffuse = C.make_color_tf([(0.0, (0.8, 0.8, 0.8)), (400.0, (0.8, 0.75, 0.7)),
                                 (1500.0, (0.85, 0.7, 0.6)), (4000.5, (0.9, 0.85, 0.8))])
    t.specular = C.make_color_tf([(0.0, (0.2, 0.2, 0.2)), (4000.5, (0.2, 0.2, 0.2))])
    t.glossiness = C.make_plf([(0.0, 0.6), (4000.5, 0.6)])
    t.emission = C.make_color_tf([(0.0, (0.0, 0.0, 0.0)), (4000.5, (0.0, 0.0, 0.0))])
    t.camera = make_camera(film, (0.0, -2.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 35.0, 1.0)
    t.settings.seed = 1
    if phase:
        t.settings.apply_shading_type = 1
        t.settings.shading_type = C.SHADING_PHASE_ONLY
    t.volume_id = 0
    t.light_count = 1
    t.light_ids[0] = 0
    return t


def c1_lights():
    # 0.5 x 0.5 plane light at z = +1 facing down, multiplier 20, uniform texture 0
    L = C.er_light_desc()
    L.visible = 1
    L.shape = make_shape(C.SHAPE_PLANE, look_at_tm((0.0, 0.0, 1.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0)),
                         size=(0.5, 0.5, 0.0))
    L.texture_id = 0
    L.multiplier = 20.0
    L.unit = C.UNIT_POWER
    return [L], [uniform_texture()]


def scene_c1(res=128, film=(256, 256), spp=64, phase=False) -> Scene:
    vol = blob_volume((res, res, res), seed=1)
    lights, textures = c1_lights()
    return Scene("c1", vol, tracer=c1_tracer(film, phase), lights=lights, textures=textures, spp=spp)


def scene_tiny(res=32, film=(48, 40), spp=4, seed=3) -> Scene:
    """Small C1-shaped scene for fast CPU/GPU parity tests."""
    vol = blob_volume((res, res, res), n_blobs=6, seed=seed)
    lights, textures = c1_lights()
    t = c1_tracer(film)
    return Scene("tiny", vol, tracer=t, lights=lights, textures=textures, spp=spp)


def c2_tracer(film=(1024, 1024)) -> C.er_tracer_desc:
    t = C.new_tracer_desc()
    t.opacity = C.make_plf([
        (0.0, 0.0), (600.0, 0.0), (850.0, 0.0), (950.0, 0.02), (1050.0, 0.04), (1150.0, 0.02),
        (1250.0, 0.05), (1350.0, 0.2), (1450.0, 0.35), (1600.0, 0.3), (1900.0, 0.3), (2200.0, 0.6),
        (2400.0, 0.9), (2600.0, 1.0), (3000.0, 1.0), (65535.5, 1.0)])
    t.diffuse = C.make_color_tf([
        (0.0, (0.6, 0.4, 0.3)), (1000.0, (0.75, 0.45, 0.35)), (1400.0, (0.8, 0.6, 0.45)),
        (2500.0, (0.92, 0.9, 0.85)), (65535.5, (0.92, 0.9, 0.85))])
    t.specular = C.make_color_tf([(0.0, (0.1, 0.1, 0.1)), (2500.0, (0.4, 0.4, 0.4)), (65535.5, (0.4, 0.4, 0.4))])
    t.glossiness = C.make_plf([(0.0, 0.7), (65535.5, 0.7)])          # roughness 0.3
    t.emission = C.make_color_tf([(0.0, (0.0, 0.0, 0.0)), (65535.5, (0.0, 0.0, 0.0))])
    t.camera = make_camera(film, (0.3, -1.9, 0.5), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 35.0, 1.0)
    t.settings.seed = 2
    t.settings.apply_shading_type = 1
    t.settings.shading_type = C.SHADING_HYBRID
    t.settings.mis = C.MIS_FULL
    t.settings.bilateral = 1
    t.volume_id = 0
    t.light_count = 3
    for i in range(3):
        t.light_ids[i] = i
    return t


def c2_lights():
    key = C.er_light_desc()
    key.visible = 1
    key.shape = make_shape(C.SHAPE_PLANE, look_at_tm((0.8, -0.8, 1.0), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0)), size=(0.6, 0.6, 0.0))
    key.texture_id = 0
    key.multiplier = 25.0
    key.unit = C.UNIT_POWER
    fill = C.er_light_desc()
    fill.visible = 1
    fill.shape = make_shape(C.SHAPE_PLANE, look_at_tm((-1.0, -0.6, -0.2), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0)), size=(0.8, 0.8, 0.0))
    fill.texture_id = 1
    fill.multiplier = 8.0
    fill.unit = C.UNIT_POWER
    env = C.er_light_desc()
    env.visible = 1
    tm = np.eye(4).tolist()
    env.shape = make_shape(C.SHAPE_SPHERE, (tm, tm), outer=5.0)
    env.texture_id = 2
    env.multiplier = 0.6
    env.unit = C.UNIT_POWER
    textures = [
        uniform_texture((1.0, 0.97, 0.9)),
        uniform_texture((0.7, 0.8, 1.0)),
        gradient_texture([(0.0, (0.25, 0.22, 0.2)), (0.5, (0.5, 0.55, 0.6)), (1.0, (0.9, 0.95, 1.0))]),
    ]
    return [key, fill, env], textures


def scene_c2(res=512, film=(1024, 1024), spp=256) -> Scene:
    vol = shell_volume(res, seed=2)
    lights, textures = c2_lights()
    return Scene("c2", vol, tracer=c2_tracer(film), lights=lights, textures=textures, spp=spp)


# ---------------------------------------------------------------------------
# batched forward (c3)
# ---------------------------------------------------------------------------

C3_FILMS = (128, 256, 384, 512)
C3_VOLUMES = ((96, 96, 96), (256, 256, 256), (256, 384, 384))   # (z, y, x)


def c3_scenes(volumes=C3_VOLUMES, seed=30) -> list:
    """One C1-style scene (4-node transfer function, one area light) per blob
    volume, delta-tracked free flight, full MIS and stratified light samples
    (the unbiased estimator);
    each scene's tracer is the template of the views that look at its
    volume."""
    out = []
    for k, shp in enumerate(volumes):
        vol = blob_volume(shp, seed=seed + k)
        lights, textures = c1_lights()
        t = c1_tracer((C3_FILMS[0], C3_FILMS[0]))
        t.settings.free_flight = C.FREE_FLIGHT_DELTA
        t.settings.mis = C.MIS_FULL
        t.settings.stratify = 1
        out.append(Scene(f"c3v{k}", vol, tracer=t, lights=lights, textures=textures, spp=32))
    return out


def c3_views(n_views=64, n_volumes=3, seed=7, films=C3_FILMS, spp=(32, 128)) -> list:
    """(volume index, orbit camera, spp) of each view, from a fixed seed."""
    rng = np.random.default_rng(seed)
    views = []
    for _ in range(n_views):
        k = int(rng.integers(0, n_volumes))
        f = int(films[int(rng.integers(0, len(films)))])
        cam = orbit_camera(rng, (f, f), radius=float(rng.uniform(1.8, 2.6)))
        views.append((k, cam, int(rng.integers(spp[0], spp[1] + 1))))
    return views


# ---------------------------------------------------------------------------
# large batched forward + adjoint (c5)
# ---------------------------------------------------------------------------

C5_SHAPE = (512, 1024, 1024)     # (z, y, x): 1024 x 1024 x 512 voxels, 1 GiB of uint16


def c5_volume(shape_zyx=C5_SHAPE, seed=5, noise_sigma=30.0, n_blobs=24) -> np.ndarray:
    """Shells in a soft-tissue ellipsoid (the c2 design on a 2:2:1 grid) plus
    `n_blobs` Gaussian blobs of amplitude 500-4000 inside it, with Gaussian
    noise inside the ellipsoid; uint16, x fastest.  Built slab by slab in
    float32."""
    Z, Y, X = shape_zyx
    rng = np.random.default_rng(seed)
    ext = np.array([X, Y, Z], dtype=np.float64)
    centres = rng.uniform(0.3, 0.7, size=(n_blobs, 3)) * ext
    sig = rng.uniform(0.02, 0.06, size=(n_blobs, 3)) * ext
    amps = rng.uniform(500.0, 4000.0, size=n_blobs)
    xs = np.arange(X, dtype=np.float32)
    ys = np.arange(Y, dtype=np.float32)
    gx = [np.exp(-0.5 * ((xs - centres[k, 0]) / sig[k, 0]) ** 2).astype(np.float32) for k in range(n_blobs)]
    gy = [np.exp(-0.5 * ((ys - centres[k, 1]) / sig[k, 1]) ** 2).astype(np.float32) * np.float32(amps[k]) for k in range(n_blobs)]
    # each blob's support (values above 1e-4 of its amplitude)
    boxes = []
    for k in range(n_blobs):
        ry = np.nonzero(gy[k] > 1e-4 * amps[k])[0]
        rx = np.nonzero(gx[k] > 1e-4)[0]
        boxes.append(((int(ry[0]), int(ry[-1]) + 1), (int(rx[0]), int(rx[-1]) + 1)))
    out = np.empty((Z, Y, X), dtype=np.uint16)
    # normalised coordinates: the longest axis spans [-0.5, 0.5]
    L = float(max(X, Y, Z))
    nx = (xs - (X - 1) / 2.0) / np.float32(L)
    ny = (ys - (Y - 1) / 2.0) / np.float32(L)
    PX, PY = np.meshgrid(nx, ny, indexing="xy")
    base = (PX / 0.46) ** 2 + (PY / 0.40) ** 2
    rxy = PX * PX + PY * PY
    for zi in range(Z):
        z = np.float32((zi - (Z - 1) / 2.0) / L)
        ell = base + (z / 0.22) ** 2 <= 1.0
        r = np.sqrt(rxy + z * z)
        v = np.where(ell, np.float32(1000.0), np.float32(0.0)).astype(np.float32)
        v = np.where((r >= 0.16) & (r < 0.19), np.float32(1400.0), v)
        v = np.where((r >= 0.08) & (r < 0.11), np.float32(2500.0), v)
        for k in range(n_blobs):
            gz = np.float32(np.exp(-0.5 * ((zi - centres[k, 2]) / sig[k, 2]) ** 2))
            if gz > 1e-4:
                (y0, y1), (x0, x1) = boxes[k]
                v[y0:y1, x0:x1] += (gy[k][y0:y1, None] * gx[k][None, x0:x1]) * gz
        v = v + np.where(ell, rng.standard_normal(size=v.shape, dtype=np.float32) * np.float32(noise_sigma), np.float32(0.0))
        out[zi] = np.clip(np.floor(v), 0, 65535).astype(np.uint16)
    return out


def scene_c5(volume=None, film=(2048, 2048), spp=64) -> Scene:
    """The c5 volume under the c2 tracer (16-node transfer function, hybrid
    shader, full MIS, two area lights and an environment sphere) with delta
    tracking; the views override its camera."""
    vol = c5_volume() if volume is None else volume
    lights, textures = c2_lights()
    t = c2_tracer(film)
    t.settings.free_flight = C.FREE_FLIGHT_DELTA
    t.settings.stratify = 1
    t.settings.bilateral = 0
    t.settings.seed = 5
    return Scene("c5", vol, tracer=t, lights=lights, textures=textures, spp=spp)


def c5_views(n_views=16, film=2048, spp=64, seed=11) -> list:
    """(volume index 0, orbit camera, spp) of the c5 views"""
    rng = np.random.default_rng(seed)
    return [(0, orbit_camera(rng, (film, film), radius=float(rng.uniform(1.6, 2.2))), spp) for _ in range(n_views)]


def density_subblock(volume, size=256, lo=800.0, hi=3000.0) -> np.ndarray:
    """The centred size^3 block of a uint16 volume as a float density in
    [0, 1] (a linear window from lo to hi), the parameter grid of the c5
    adjoint."""
    Z, Y, X = volume.shape
    z0, y0, x0 = (Z - size) // 2, (Y - size) // 2, (X - size) // 2
    b = volume[z0:z0 + size, y0:y0 + size, x0:x0 + size].astype(np.float32)
    return np.ascontiguousarray(np.clip((b - lo) / (hi - lo), 0.0, 1.0), dtype=np.float32)


# ---------------------------------------------------------------------------
# views with converged FP64 references (image RMSE measurements)
# ---------------------------------------------------------------------------

def rmse_views(film=128, names=None) -> list:
    """(name, Scene) of the views whose converged images the FP64 oracle
    provides: the c1 scene with the BRDF at every volume event (the
    reference's live shading) and with the isotropic phase function (c1p,
    the c1 workload's shading), the first view of each c3 volume, c2, and -
    only when named, as its volume is 1 GiB - the first c5 view (c5v0); all
    at a film of `film`^2 with each workload's camera and settings.  `names`
    restricts the list (and the volumes generated)."""
    want = set(names) if names else {"c1", "c1p", "c3v0", "c3v1", "c3v2", "c2"}
    out = []
    if "c1" in want:
        out.append(("c1", scene_c1(res=128, film=(film, film))))
    if "c1p" in want:
        out.append(("c1p", scene_c1(res=128, film=(film, film), phase=True)))
    c3 = [k for k in range(3) if f"c3v{k}" in want]
    if c3:
        views = c3_views()
        for k in c3:
            sc = c3_scenes(volumes=(C3_VOLUMES[k],), seed=30 + k)[0]
            sc.name = f"c3v{k}"
            cam = C.er_camera_desc.from_buffer_copy([c for (kk, c, _) in views if kk == k][0])
            cam.film_size[0] = cam.film_size[1] = film
            sc.tracer.camera = cam
            out.append((f"c3v{k}", sc))
    if "c2" in want:
        out.append(("c2", scene_c2(res=512, film=(film, film))))
    if "c5v0" in want:
        sc = scene_c5(film=(film, film))
        sc.name = "c5v0"
        cam = C.er_camera_desc.from_buffer_copy(c5_views()[0][1])
        cam.film_size[0] = cam.film_size[1] = film
        sc.tracer.camera = cam
        out.append(("c5v0", sc))
    return out


# ---------------------------------------------------------------------------
# differentiable medium (c4)
# ---------------------------------------------------------------------------

def blob_density(shape_zyx, n_blobs=10, seed=40) -> np.ndarray:
    """float32 density in [0, 1]: a clipped sum of anisotropic Gaussians"""
    Z, Y, X = shape_zyx
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.25, 0.75, size=(n_blobs, 3)) * np.array([X, Y, Z])
    sig = rng.uniform(0.06, 0.16, size=(n_blobs, 3)) * np.array([X, Y, Z])
    amps = rng.uniform(0.3, 0.9, size=n_blobs)
    z, y, x = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    rho = np.zeros((Z, Y, X), dtype=np.float64)
    for k in range(n_blobs):
        rho += amps[k] * np.exp(-0.5 * (((x - centres[k, 0]) / sig[k, 0]) ** 2 + ((y - centres[k, 1]) / sig[k, 1]) ** 2
                                        + ((z - centres[k, 2]) / sig[k, 2]) ** 2))
    return np.clip(rho, 0.0, 1.0).astype(np.float32)


def ramp_opacity(n=64, lo=0.15, hi=0.7) -> np.ndarray:
    """opacity B-spline values: 0 below `lo`, rising linearly to 1 at `hi`
    (control i sits at density (i - 2) / (n - 5))"""
    u = (np.arange(n) - 2.0) / (n - 5.0)
    return np.clip((u - lo) / (hi - lo), 0.0, 1.0).astype(np.float32)


def spline_majorant(rho, tf, scale, brick=8, margin=1.25, floor=1e-3) -> np.ndarray:
    """per-brick upper bound of sigma = scale * alpha(rho): the largest
    B-spline control value over the spline segments that the brick's density
    range (with a 1-voxel apron) covers (convex-hull property), times
    `margin`, plus `floor` * scale.  Shape (nbz, nby, nbx), float32."""
    n = len(tf)
    Z, Y, X = rho.shape
    nb = [(d + brick - 1) // brick for d in (Z, Y, X)]
    out = np.zeros(nb, dtype=np.float32)
    for bz in range(nb[0]):
        for by in range(nb[1]):
            for bx in range(nb[2]):
                sl = rho[max(bz * brick - 1, 0):min((bz + 1) * brick + 1, Z),
                         max(by * brick - 1, 0):min((by + 1) * brick + 1, Y),
                         max(bx * brick - 1, 0):min((bx + 1) * brick + 1, X)]
                u0 = np.clip(2.0 + float(sl.min()) * (n - 5), 1.0, n - 2.0)
                u1 = np.clip(2.0 + float(sl.max()) * (n - 5), 1.0, n - 2.0)
                i0 = min(int(np.floor(u0)), n - 3)
                i1 = min(int(np.floor(u1)), n - 3)
                vmax = float(np.max(tf[i0 - 1:i1 + 3]))
                out[bz, by, bx] = scale * (vmax * margin + floor)
    return out


def medium_scene(res=(128, 128, 128), film=(256, 256), seed=40) -> Scene:
    """the c1 camera and light around a zero intensity volume of the medium's
    resolution (the tracer's volume gives the medium its placement)"""
    lights, textures = c1_lights()
    t = c1_tracer(film)
    return Scene("medium", np.zeros(res, dtype=np.uint16), tracer=t, lights=lights, textures=textures, spp=32)


# ---------------------------------------------------------------------------
# surface objects (SampleRay's third event type)
# ---------------------------------------------------------------------------

def checker_texture(c1, c2, level=1.0, repeat=(1.0, 1.0)) -> C.er_texture_desc:
    t = C.new_texture_desc()
    t.procedural.type = C.PROCEDURAL_CHECKER
    for i in range(3):
        t.procedural.checker_color1[i] = c1[i]
        t.procedural.checker_color2[i] = c2[i]
    t.output_level = level
    t.repeat[0], t.repeat[1] = repeat
    return t


def make_object(shape, diffuse=-1, specular=-1, glossiness=-1, ior=5.0) -> C.er_object_desc:
    o = C.er_object_desc()
    o.shape = shape
    o.diffuse_texture_id = diffuse
    o.specular_texture_id = specular
    o.glossiness_texture_id = glossiness
    o.ior = ior
    return o


def scene_objects(res=32, film=(48, 40), spp=4, seed=3) -> Scene:
    """The tiny blob scene on a textured floor plane with a sphere beside it:
    volume, light and object events in one image, objects shadowing the
    volume and the volume shadowing the floor."""
    vol = blob_volume((res, res, res), n_blobs=6, seed=seed)
    lights, textures = c1_lights()
    textures = textures + [uniform_texture((0.7, 0.5, 0.3)), checker_texture((0.3, 0.3, 0.3), (0.05, 0.05, 0.05), repeat=(4.0, 4.0)),
                           uniform_texture((0.6, 0.6, 0.6))]
    floor = make_shape(C.SHAPE_PLANE, look_at_tm((0.0, 0.0, -0.6), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0)), size=(3.0, 3.0, 0.0))
    ball = make_shape(C.SHAPE_SPHERE, look_at_tm((0.55, -0.1, 0.25), (0.55, -0.1, 1.25), (0.0, 1.0, 0.0)), outer=0.2)
    objects = [make_object(floor, 1, 2, 3), make_object(ball, 1, 1, 3)]
    t = c1_tracer(film)
    t.object_count = 2
    t.object_ids[0], t.object_ids[1] = 0, 1
    return Scene("objects", vol, tracer=t, lights=lights, textures=textures, spp=spp, objects=objects)


# ---------------------------------------------------------------------------
# bitmap textures (ErTexture of type Bitmap over a bound ErBitmap)
# ---------------------------------------------------------------------------

def bitmap_texture(bitmap_id, level=1.0, repeat=(1.0, 1.0), offset=(0.0, 0.0), flip=(0, 0)) -> C.er_texture_desc:
    t = C.new_texture_desc()
    t.type = C.TEXTURE_BITMAP
    t.bitmap_id = bitmap_id
    t.output_level = level
    t.repeat[0], t.repeat[1] = repeat
    t.offset[0], t.offset[1] = offset
    t.flip[0], t.flip[1] = flip
    return t


def scene_bitmaps(res=32, film=(48, 40), spp=4, seed=3) -> Scene:
    """The objects scene with bitmap textures.  The reference's bitmap lookup
    (Source/buffer2d.h:227-254) carries its bilinear weights in unsigned char,
    so it returns the floor texel where the scaled coordinate is an integer
    and black elsewhere: texture 4 (repeat 0, offsets on the texel grid of a
    4x2 bitmap) reads texel (1, 1) everywhere and lights the scene; texture 5
    (a repeated 16x16 bitmap) shows the black case on the sphere."""
    sc = scene_objects(res=res, film=film, spp=spp, seed=seed)
    rng = np.random.default_rng(seed + 100)
    sc.bitmaps = [rng.integers(0, 256, size=(2, 4, 4), dtype=np.uint8),
                  rng.integers(0, 256, size=(16, 16, 4), dtype=np.uint8)]
    sc.textures = sc.textures + [bitmap_texture(0, level=1.5, repeat=(0.0, 0.0), offset=(0.25, 0.5)),
                                 bitmap_texture(1, repeat=(3.0, 3.0), flip=(1, 0))]
    sc.objects[0].diffuse_texture_id = 4
    sc.objects[1].specular_texture_id = 5
    sc.lights[0].texture_id = 4
    return sc


# ---------------------------------------------------------------------------
# clipping objects (ErClippingObject: a shape that removes part of the volume)
# ---------------------------------------------------------------------------

def make_clipping_object(shape, invert=0) -> C.er_clipping_object_desc:
    k = C.er_clipping_object_desc()
    k.shape = shape
    k.invert = invert
    return k


def scene_clipped(res=32, film=(48, 40), spp=4, seed=3) -> Scene:
    """The tiny blob scene cut by three clipping objects: a tilted plane
    (the half-space on its +z side is removed), a sphere with Invert set
    (only the volume inside it is kept) and a box that removes a corner."""
    sc = scene_tiny(res=res, film=film, spp=spp, seed=seed)
    plane = make_shape(C.SHAPE_PLANE, look_at_tm((0.05, 0.0, 0.1), (0.35, 0.2, 1.1), (0.0, 1.0, 0.0)), size=(1.0, 1.0, 0.0))
    ball = make_shape(C.SHAPE_SPHERE, look_at_tm((0.0, 0.05, -0.05), (0.0, 0.05, 0.95), (0.0, 1.0, 0.0)), outer=0.42)
    box = make_shape(C.SHAPE_BOX, look_at_tm((-0.3, -0.25, -0.3), (0.2, 0.25, 0.7), (0.0, 0.0, 1.0)), size=(0.35, 0.3, 0.4))
    sc.clipping_objects = [make_clipping_object(plane), make_clipping_object(ball, invert=1), make_clipping_object(box)]
    sc.tracer.clipping_object_count = 3
    for i in range(3):
        sc.tracer.clipping_object_ids[i] = i
    return sc


def lattice_volume(shape_zyx, period=96.0, seed=13, noise=40.0) -> np.ndarray:
    """A volume filled everywhere: 1200 + 900 sin(2 pi x / p) sin(2 pi y / p)
    sin(2 pi z / p) plus uniform noise in [0, noise), uint16, x fastest (the
    large-index tests need voxels that matter in every slice).  Built slab by
    slab in float32."""
    Z, Y, X = shape_zyx
    rng = np.random.default_rng(seed)
    sx = np.sin(2.0 * np.pi * np.arange(X, dtype=np.float32) / np.float32(period)).astype(np.float32)
    sy = np.sin(2.0 * np.pi * np.arange(Y, dtype=np.float32) / np.float32(period)).astype(np.float32)
    sxy = (sy[:, None] * sx[None, :]) * np.float32(900.0)
    out = np.empty((Z, Y, X), dtype=np.uint16)
    for z in range(Z):
        sz = np.float32(np.sin(2.0 * np.pi * z / period))
        v = np.float32(1200.0) + sxy * sz + rng.random(size=(Y, X), dtype=np.float32) * np.float32(noise)
        out[z] = v.astype(np.uint16)
    return out


# ---------------------------------------------------------------------------
# the differentiable product estimator: the tracer's transfer functions and
# shading over a float intensity grid (medium model 1)
# ---------------------------------------------------------------------------

def tf_medium_tracer(film=(256, 256), n_nodes=64, shading=C.SHADING_HYBRID, glossiness=0.3, emission=0.0):
    """The c1 camera and light with transfer functions over intensities in
    [0, 1]: an n-node opacity PLF (positions i / (n - 1), a ramp from 0.15 to
    0.7 as the values), a diffuse colour ramp, a constant specular colour and
    glossiness (exponent 1e6 g^7), an optional emission bump, and the given
    shader (BRDF, phase or hybrid, opacity-modulated)."""
    t = c1_tracer(film)
    pos = np.arange(n_nodes, dtype=np.float64) / (n_nodes - 1)
    vals = np.clip((pos - 0.15) / (0.7 - 0.15), 0.0, 1.0)
    t.opacity = C.make_plf([(float(p), float(v)) for p, v in zip(pos, vals)])
    t.diffuse = C.make_color_tf([(0.0, (0.9, 0.5, 0.3)), (0.4, (0.8, 0.7, 0.5)), (1.0, (0.6, 0.8, 0.9))])
    t.specular = C.make_color_tf([(0.0, (0.25, 0.25, 0.25)), (1.0, (0.35, 0.3, 0.3))])
    t.glossiness = C.make_plf([(0.0, glossiness), (1.0, glossiness)])
    t.emission = C.make_color_tf([(0.0, (0.0, 0.0, 0.0)), (0.45, (0.0, 0.0, 0.0)), (0.6, (emission, 0.6 * emission, 0.2 * emission)),
                                  (0.75, (0.0, 0.0, 0.0)), (1.0, (0.0, 0.0, 0.0))])
    t.settings.apply_shading_type = 1
    t.settings.shading_type = shading
    t.settings.opacity_modulated = 1
    return t


def tf_medium_scene(res=(128, 128, 128), film=(256, 256), n_nodes=64, shading=C.SHADING_HYBRID, glossiness=0.3, emission=0.0,
                    two_lights=True) -> Scene:
    """tf_medium_tracer around a zero volume of the grid's resolution (the
    volume gives the grid its placement), with the c1 area light and, with
    two_lights, a small sphere light beside the volume"""
    lights, textures = c1_lights()
    t = tf_medium_tracer(film, n_nodes, shading, glossiness, emission)
    if two_lights:
        L = C.er_light_desc()
        L.visible = 0
        L.shape = make_shape(C.SHAPE_SPHERE, look_at_tm((-0.9, -0.6, 0.3), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0)), outer=0.15)
        L.texture_id = 0
        L.multiplier = 6.0
        L.unit = C.UNIT_POWER
        lights.append(L)
        t.light_count = 2
        t.light_ids[1] = 1
    return Scene("tf_medium", np.zeros(res, dtype=np.uint16), tracer=t, lights=lights, textures=textures, spp=32)


def plf_node_values(plf) -> np.ndarray:
    return np.array([plf.value[i] for i in range(plf.count)], dtype=np.float32)


def plf_majorant(rho, plf, values, scale, brick=8, margin=1.25, floor=1e-3) -> np.ndarray:
    """per-brick upper bound of sigma = scale * PLF(rho) with the node
    values `values` at the positions of `plf`: the PLF's maximum over the
    brick's density range (1-voxel apron) - its values at both ends and at
    the nodes inside - times `margin`, plus `floor` * scale.  Shape
    (nbz, nby, nbx), float32."""
    n = plf.count
    pos = np.array([plf.position[i] for i in range(n)], dtype=np.float64)
    vals = np.asarray(values, dtype=np.float64)

    def ev(x):
        if x < pos[0]:
            return vals[0]
        if x > pos[-1]:
            return vals[-1]
        return float(np.interp(x, pos, vals))
    Z, Y, X = rho.shape
    nb = [(d + brick - 1) // brick for d in (Z, Y, X)]
    out = np.zeros(nb, dtype=np.float32)
    for bz in range(nb[0]):
        for by in range(nb[1]):
            for bx in range(nb[2]):
                sl = rho[max(bz * brick - 1, 0):min((bz + 1) * brick + 1, Z),
                         max(by * brick - 1, 0):min((by + 1) * brick + 1, Y),
                         max(bx * brick - 1, 0):min((bx + 1) * brick + 1, X)]
                lo, hi = float(sl.min()), float(sl.max())
                inside = vals[(pos >= lo) & (pos <= hi)]
                vmax = max(ev(lo), ev(hi), float(inside.max()) if inside.size else -np.inf)
                out[bz, by, bx] = scale * (max(vmax, 0.0) * margin + floor)
    return out


def gradient_magnitude_range(rho, spacing=(1.0, 1.0, 1.0)) -> float:
    """1 / the largest central-difference gradient magnitude of a float grid
    at its voxel centres (the hybrid shader's normalisation), with the
    normalised volume's spacing (longest axis 1)"""
    Z, Y, X = rho.shape
    phys = np.array([X * spacing[0], Y * spacing[1], Z * spacing[2]], dtype=np.float64)
    sp = np.array(spacing, dtype=np.float64) / phys.max()
    r = np.pad(rho.astype(np.float64), 1, mode="edge")
    gx = (r[1:-1, 1:-1, :-2] - r[1:-1, 1:-1, 2:]) * 0.5 / sp[0]
    gy = (r[1:-1, :-2, 1:-1] - r[1:-1, 2:, 1:-1]) * 0.5 / sp[1]
    gz = (r[:-2, 1:-1, 1:-1] - r[2:, 1:-1, 1:-1]) * 0.5 / sp[2]
    m = float(np.sqrt(gx * gx + gy * gy + gz * gz).max())
    return 1.0 / m if m > 0.0 else 0.0
