"""Clipping objects in the CPU oracle (ErClippingObject,
Source/erclippingobject.h:27-58, bound by BindClippingObject,
Source/core.cu:96-104, and named by the tracer's ClippingObjectIDs,
Source/ertracer.h:100-116).  The reference binds them and never reads them;
the restatement removes the volume inside each clipping shape (outside it
with Invert), using the reference's Inside* predicates."""
import copy

import numpy as np
import pytest

import oracle_lib as OL

C = OL.C
S = OL.PKG.scenes


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def render(orc, sc, spp=3, free_flight=0):
    sc = copy.copy(sc)
    sc.tracer = C.er_tracer_desc.from_buffer_copy(sc.tracer)
    sc.tracer.settings.free_flight = free_flight
    sc.tracer.settings.majorant_brick = 4
    h = OL.SceneHandle(orc, sc)
    try:
        out = h.render_sum(spp, nthreads=8)
        return out, OL.render_stats(orc)
    finally:
        h.close()


def with_environment(sc):
    """adds a visible environment sphere light (gradient texture), so that
    every camera ray that leaves the volume sees a light"""
    tm = np.eye(4).tolist()
    env = C.er_light_desc()
    env.visible = 1
    env.shape = S.make_shape(C.SHAPE_SPHERE, (tm, tm), outer=4.0)
    env.texture_id = len(sc.textures)
    env.multiplier = 0.7
    sc.lights.append(env)
    sc.textures.append(S.gradient_texture([(0.0, (0.2, 0.2, 0.3)), (0.5, (0.5, 0.5, 0.6)), (1.0, (1.0, 1.0, 1.0))]))
    sc.tracer.light_ids[sc.tracer.light_count] = len(sc.lights) - 1
    sc.tracer.light_count += 1
    return sc


def far_sphere(invert):
    """a small sphere well outside the unit volume"""
    return S.make_clipping_object(S.make_shape(C.SHAPE_SPHERE, S.look_at_tm((3.0, 3.0, 3.0), (3.0, 3.0, 4.0), (0.0, 1.0, 0.0)),
                                               outer=0.05), invert=invert)


@pytest.mark.parametrize("free_flight", [0, 1])
def test_clipping_everything_renders_the_lights_only(oracle, free_flight):
    """An inverted clipping sphere far outside the volume removes all of it:
    the render equals that of the volume without NormalizeSize (zero-size
    box), which shows only the visible light, bit for bit, and makes no
    volume lookup"""
    sc = with_environment(S.scene_tiny(res=20, film=(24, 20), seed=5))
    sc.clipping_objects = [far_sphere(1)]
    sc.tracer.clipping_object_count = 1
    sc.tracer.clipping_object_ids[0] = 0
    clipped, st = render(oracle, sc, free_flight=free_flight)
    assert st["lookups"] == 0.0
    empty = with_environment(S.scene_tiny(res=20, film=(24, 20), seed=5))
    empty.normalize_size = 0
    ref, _ = render(oracle, empty, free_flight=free_flight)
    assert np.array_equal(bits(clipped), bits(ref))
    assert ref[..., :3].all(-1).all()     # every pixel sees the environment light
    full, _ = render(oracle, with_environment(S.scene_tiny(res=20, film=(24, 20), seed=5)), free_flight=free_flight)
    assert not np.array_equal(bits(full), bits(ref))


@pytest.mark.parametrize("free_flight", [0, 1])
def test_clipping_nothing_changes_nothing(oracle, free_flight):
    """A clipping sphere far outside the volume (no Invert) removes nothing,
    and an unbound clipping ID is skipped: the render is the unclipped one,
    bit for bit"""
    sc = S.scene_tiny(res=20, film=(24, 20), seed=5)
    base, st0 = render(oracle, sc, free_flight=free_flight)
    sc.clipping_objects = [far_sphere(0)]
    sc.tracer.clipping_object_count = 2
    sc.tracer.clipping_object_ids[0] = 0
    sc.tracer.clipping_object_ids[1] = 7
    got, st1 = render(oracle, sc, free_flight=free_flight)
    assert np.array_equal(bits(got), bits(base))
    assert st0["lookups"] == st1["lookups"]


def test_clipping_removes_volume(oracle):
    """The three clipping objects of scenes.scene_clipped remove most of the
    blobs: fewer than half the lookups and less alpha, but not all of it"""
    sc = S.scene_clipped(res=20, film=(24, 20))
    got, st = render(oracle, sc, free_flight=1)
    base, st0 = render(oracle, S.scene_tiny(res=20, film=(24, 20)), free_flight=1)
    assert st["lookups"] < 0.5 * st0["lookups"]
    assert got[..., 3].sum() < base[..., 3].sum()
    assert got[..., 3].sum() > 0.0


def test_clipping_invert_is_the_complement(oracle):
    """Clipping only lowers the extinction along a ray: with the fixed-step
    march and the same random numbers, a sample that found no event without
    clipping finds none with a clipping box, nor with the same box inverted;
    each of the two keeps part of the volume"""
    box = S.make_shape(C.SHAPE_BOX, S.look_at_tm((0.1, -0.05, 0.0), (0.1, -0.05, 1.0), (0.0, 1.0, 0.0)), size=(0.5, 0.6, 0.7))
    outs = []
    for inv in (0, 1):
        sc = S.scene_tiny(res=20, film=(24, 20), seed=5)
        for L in sc.lights:
            L.visible = 0
        sc.clipping_objects = [S.make_clipping_object(box, invert=inv)]
        sc.tracer.clipping_object_count = 1
        sc.tracer.clipping_object_ids[0] = 0
        outs.append(render(oracle, sc, spp=2)[0])
    sc = S.scene_tiny(res=20, film=(24, 20), seed=5)
    for L in sc.lights:
        L.visible = 0
    full, _ = render(oracle, sc, spp=2)
    none = full[..., 3] == 0.0
    assert (outs[0][..., 3][none] == 0.0).all() and (outs[1][..., 3][none] == 0.0).all()
    assert outs[0][..., 3].sum() > 0.0 and outs[1][..., 3].sum() > 0.0
