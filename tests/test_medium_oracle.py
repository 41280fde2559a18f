"""Differentiable medium in the CPU oracle: the float adjoint (path replay)
against central finite differences of the binary64 forward with the same
random numbers, and the float forward against the binary64 one.

The differences use h = 1e-3 and h/2 combined by Richardson extrapolation:
on this small, optically thick medium the loss is curved enough in the
low-density opacity values that a plain central difference at h = 1e-3 is
itself 1.5e-3 off (it converges to the adjoint as h -> 0)."""
import numpy as np
import pytest

import oracle_lib as OL

S = OL.PKG.scenes
RES, N, SCALE, SPP, BRICK, Q = (16, 16, 16), 16, 30.0, 4, 4, 0.5
ALB = np.array([0.8, 0.7, 0.6])


@pytest.fixture(scope="module")
def setup():
    rho = S.blob_density(RES, n_blobs=4, seed=3)
    tf = S.ramp_opacity(N)
    maj = S.spline_majorant(rho, tf, SCALE, brick=BRICK)
    sc = S.medium_scene(res=RES, film=(24, 20))
    return rho, tf, maj, sc


def render(orc, sc, rho, tf, maj, keep=False):
    h = OL.MediumHandle(orc, sc, rho, tf, SCALE, ALB, Q, maj, BRICK)
    out = h.render(SPP, keep_samples=keep, nthreads=4)
    if keep:
        return h, out
    h.close()
    return out


def central(loss, f64, sc, maj, kind, i, r64, t64, h):
    lp, lm, tp, tm = r64.copy(), r64.copy(), t64.copy(), t64.copy()
    if kind == "tf":
        tp[i] += h
        tm[i] -= h
    else:
        lp.ravel()[i] += h
        lm.ravel()[i] -= h
    return (loss(render(f64, sc, lp, tp, maj)) - loss(render(f64, sc, lm, tm, maj))) / (2 * h)


def richardson(d, h):
    """fourth-order derivative estimate from central differences at h and h/2"""
    return (4.0 * d(h / 2) - d(h)) / 3.0


def test_forward_float_matches_binary64(setup):
    rho, tf, maj, sc = setup
    a = render(OL.load_oracle(), sc, rho, tf, maj)
    b = render(OL.load_fp64(), sc, rho, tf, maj)
    assert np.abs(a - b).max() <= 1e-4 * np.abs(b).max()


def test_adjoint_matches_finite_differences(setup):
    rho, tf, maj, sc = setup
    f64 = OL.load_fp64()
    target = render(f64, sc, rho, tf, maj) / SPP * 0.9 + 0.01

    def loss(img):
        return float(np.sum((img / SPP - target) ** 2))

    h, (img, smp) = render(OL.load_oracle(), sc, rho, tf, maj, keep=True)
    g_rho, g_tf = h.adjoint(SPP, 2.0 * (img / SPP - target) / SPP, smp, nthreads=4)
    h.close()
    hstep = 1e-3
    params = [("tf", i) for i in (3, 5, 6, 7)] + [("rho", int(i)) for i in np.argsort(-np.abs(g_rho).ravel())[:4]]
    for kind, i in params:
        r64, t64 = rho.astype(np.float64), tf.astype(np.float64)
        adj = g_tf[i] if kind == "tf" else g_rho.ravel()[i]
        fd = richardson(lambda d: central(loss, f64, sc, maj, kind, i, r64, t64, d), hstep)
        assert abs(adj - fd) <= 1e-3 * abs(fd), (kind, i, adj, fd)
