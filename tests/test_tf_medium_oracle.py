"""The differentiable tracer model (medium model 1, ER_MEDIUM_TRACER) in the
CPU oracle: the tracer's opacity PLF with its node values as parameters,
its diffuse / specular / glossiness / emission transfer functions over a
float intensity grid, and its BRDF, phase or hybrid shading.

The brute-force reference gradient: central differences of the binary64
forward, with the same random numbers, over every parameter of a small
scene (every voxel of a 10^3 grid and every opacity node).  h = 1e-6: the
transfer functions are piecewise linear in the intensity, so a difference
quotient whose step crosses a node position is off by the kink; at 1e-6 no
step of this scene crosses one (at 1e-4 a few voxels' did, and converged to
the adjoint as h shrank).  The binary64 adjoint must agree to 1e-7 of the
largest gradient, the float adjoint to 1e-3 relative plus 1e-5 of the
largest gradient (float sums of contributions that cancel)."""
import numpy as np
import pytest

import oracle_lib as OL

S = OL.PKG.scenes
C = OL.C
RES, FILM, SPP, N, SCALE, BRICK, Q = (10, 10, 10), (12, 10), 2, 12, 30.0, 4, 0.5


@pytest.fixture(scope="module")
def grid():
    return S.blob_density(RES, n_blobs=4, seed=3)


def scene(shading):
    return S.tf_medium_scene(res=RES, film=FILM, n_nodes=N, shading=shading, emission=0.8)


def handle(orc, sc, rho, vals, rho0):
    maj = S.plf_majorant(rho0, sc.tracer.opacity, S.plf_node_values(sc.tracer.opacity), SCALE, brick=BRICK)
    return OL.MediumHandle(orc, sc, rho, vals, SCALE, np.array([0.8, 0.7, 0.6]), Q, maj, BRICK, model=1,
                           gm_inv=S.gradient_magnitude_range(rho0))


def render(orc, sc, rho, vals, rho0, keep=False):
    h = handle(orc, sc, rho, vals, rho0)
    out = h.render(SPP, keep_samples=keep, nthreads=4)
    if keep:
        return h, out
    h.close()
    return out


@pytest.mark.parametrize("shading", [C.SHADING_BRDF_ONLY, C.SHADING_PHASE_ONLY, C.SHADING_HYBRID])
def test_forward_float_matches_binary64(grid, shading):
    sc = scene(shading)
    vals = S.plf_node_values(sc.tracer.opacity)
    a = render(OL.load_oracle(), sc, grid, vals, grid)
    b = render(OL.load_fp64(), sc, grid, vals, grid)
    assert np.abs(a - b).max() <= 1e-4 * np.abs(b).max()
    assert np.abs(b).max() > 0.0


@pytest.mark.parametrize("shading,stride", [(C.SHADING_HYBRID, 1), (C.SHADING_BRDF_ONLY, 5), (C.SHADING_PHASE_ONLY, 5)])
def test_adjoint_matches_brute_force_gradient(grid, shading, stride):
    """every opacity node and every `stride`-th voxel (all voxels for the
    hybrid shader)"""
    sc = scene(shading)
    vals = S.plf_node_values(sc.tracer.opacity)
    f64, orc = OL.load_fp64(), OL.load_oracle()
    r64, v64 = grid.astype(np.float64), vals.astype(np.float64)
    target = render(f64, sc, r64, v64, grid) / SPP * 0.9 + 0.01

    def loss(img):
        return float(np.sum((img / SPP - target) ** 2))

    def adjoint(o, r, v):
        h, (img, smp) = render(o, sc, r, v, grid, keep=True)
        g = h.adjoint(SPP, 2.0 * (img / SPP - target) / SPP, smp, nthreads=4)
        h.close()
        return g

    g_rho, g_tf = adjoint(orc, grid, vals)
    G_rho, G_tf = adjoint(f64, r64, v64)
    hstep = 1e-6
    fd_tf = np.zeros(N)
    for i in range(N):
        p, m = v64.copy(), v64.copy()
        p[i] += hstep
        m[i] -= hstep
        fd_tf[i] = (loss(render(f64, sc, r64, p, grid)) - loss(render(f64, sc, r64, m, grid))) / (2 * hstep)
    idx = np.arange(0, grid.size, stride)
    fd_rho = np.zeros(len(idx))
    for n, i in enumerate(idx):
        p, m = r64.copy(), r64.copy()
        p.ravel()[i] += hstep
        m.ravel()[i] -= hstep
        fd_rho[n] = (loss(render(f64, sc, p, v64, grid)) - loss(render(f64, sc, m, v64, grid))) / (2 * hstep)
    for name, fd, G, g in (("opacity nodes", fd_tf, G_tf, g_tf), ("voxels", fd_rho, G_rho.ravel()[idx], g_rho.ravel()[idx])):
        big = np.abs(fd).max()
        assert big > 0.0, name
        assert np.abs(G - fd).max() <= 1e-7 * big, (name, "binary64 adjoint", np.abs(G - fd).max() / big)
        err = np.abs(g - fd) / (1e-3 * np.abs(fd) + 1e-5 * big)
        assert err.max() <= 1.0, (name, "float adjoint", int(err.argmax()), float(g[err.argmax()]), float(fd[err.argmax()]))
    # the voxels the image depends on are many: the gradient is not a few
    # isolated entries
    assert (fd_rho != 0.0).sum() > len(idx) // 4
