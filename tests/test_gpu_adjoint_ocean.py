"""Hand-written adjoint of the ocean app's tracer RK4 step (GPU): thickness and
velocity prescribed, FCT advection and del2 mixing differentiated on the
forward's branch; checked by the dot-product identity against the complex-step
tangent of the CPU restatement, by central differences of the CUDA forward, and
for independence from the checkpoint interval (and the stored window)."""
import numpy as np
import pytest

import mpaso
from mpaso.initial import ocean_state
from mpaso.setup import fct_statics

pytestmark = pytest.mark.gpu


def make(L, T, opts, level=3, seed=7, noise=True):
    import mpaso.gpu as G
    mesh = mpaso.Mesh.icosa(level)
    f = fct_statics(mesh, L)
    h, hE, u, tr = ocean_state(mesh, seed, L, T, clip=False)
    if noise:  # cell noise on top: local extrema everywhere, so the limiter's active branch is exercised
        tr = 0.7 * tr + 0.3 * tr.max() * np.random.default_rng(seed).uniform(0.0, 1.0, tr.shape)
    dm = G.DeviceMesh(mesh, fct=f)
    st = G.State(dm, app=G.APP_OCEAN, nlev=L, ntr=T, **opts)
    st.set(G.FIELD_H, h)
    st.set(G.FIELD_U, u)
    st.set(G.FIELD_LAYER_THICKNESS_EDGE, hE)
    return mesh, f, st, (h, hE, u, tr)


@pytest.mark.parametrize("opts", [dict(fct=True, hmix=True, kappa=1e5), dict(fct=True), dict(hmix=True, kappa=1e5)])
def test_ocean_adjoint_dot_product_against_complex_step(opts):
    import mpaso.gpu as G
    from sw_complex import SwComplex
    L, T, dt, n = 2, 2, 600.0, 4
    mesh, f, st, (h, hE, u, tr) = make(L, T, opts)
    rng = np.random.default_rng(3)
    w = rng.standard_normal(tr.shape)
    st.set(G.FIELD_TRACERS, tr)
    st.forward(dt, n, 2)
    gh, gu, gt = st.vjp_tracers(np.zeros(h.shape), np.zeros(u.shape), w)
    assert not gh.any() and not gu.any()  # prescribed fields: zeros
    from mpaso._lib import MpasoError
    with pytest.raises(MpasoError, match="prescribed"):
        st.vjp(np.zeros(h.shape), np.zeros(u.shape))
    C = SwComplex(mesh, L, fct=f, centred=not opts.get("fct", False), T=T, hmix=opts.get("hmix", False),
                  kappa=opts.get("kappa", 0.0))
    for _ in range(2):
        v = rng.standard_normal(tr.shape)
        jv = C.ocean_jvp(h, hE, u, tr, v, dt, n)
        lhs, rhs = float((w * jv).sum()), float((gt * v).sum())
        assert abs(lhs - rhs) <= 1e-10 * np.abs(w * jv).sum(), (lhs, rhs)


@pytest.mark.parametrize("level", [2, 4])
def test_ocean_adjoint_sixty_levels(level):
    """The benchmark's column (60 levels x 3 tracers, dt = 450 s, kappa 1e4)
    on a small sphere: the dot-product identity against the complex-step
    tangent at 1e-10.  The initial temperature is not clipped to [0, 30]:
    on a clipped plateau the limiter quotient (trmax - upw) / (tmax_new - upw
    + 1e-10) divides rounding-level differences by ~1e-10, its branch
    derivative reaches ~1e4 and the branch itself follows rounding, so no
    restatement that is not bit-exact can check it there."""
    import mpaso.gpu as G
    from sw_complex import SwComplex
    L, T, dt, n = 60, 3, 450.0, 3
    mesh, f, st, (h, hE, u, tr) = make(L, T, dict(fct=True, hmix=True, kappa=1e4), level=level, seed=1234,
                                       noise=False)
    rng = np.random.default_rng(4)
    w = rng.standard_normal(tr.shape)
    st.set(G.FIELD_TRACERS, tr)
    st.forward(dt, n, 2)
    gt = st.vjp_tracers(np.zeros(h.shape), np.zeros(u.shape), w)[2]
    C = SwComplex(mesh, L, fct=f, T=T, hmix=True, kappa=1e4)
    v = rng.standard_normal(tr.shape)
    jv = C.ocean_jvp(h, hE, u, tr, v, dt, n)
    lhs, rhs = float((w * jv).sum()), float((gt * v).sum())
    assert abs(lhs - rhs) <= 1e-10 * np.abs(w * jv).sum(), (lhs, rhs)


def test_ocean_adjoint_one_lane_per_cell_level():
    """At a million cell-levels and more the tracer gather runs one thread per
    cell-level instead of two: 1700 levels on a level-3 sphere (1.09M
    cell-levels) hold that path to the same 1e-10 dot-product bar."""
    import mpaso.gpu as G
    from sw_complex import SwComplex
    L, T, dt, n = 1700, 1, 450.0, 2
    mesh, f, st, (h, hE, u, tr) = make(L, T, dict(fct=True, hmix=True, kappa=1e4), level=3, seed=1234,
                                       noise=False)
    assert mesh.nCells * L >= 1 << 20
    rng = np.random.default_rng(4)
    w = rng.standard_normal(tr.shape)
    st.set(G.FIELD_TRACERS, tr)
    st.forward(dt, n, 1)
    gt = st.vjp_tracers(np.zeros(h.shape), np.zeros(u.shape), w)[2]
    C = SwComplex(mesh, L, fct=f, T=T, hmix=True, kappa=1e4)
    v = rng.standard_normal(tr.shape)
    jv = C.ocean_jvp(h, hE, u, tr, v, dt, n)
    lhs, rhs = float((w * jv).sum()), float((gt * v).sum())
    assert abs(lhs - rhs) <= 1e-10 * np.abs(w * jv).sum(), (lhs, rhs)


def test_ocean_adjoint_fd_checkpoints_and_stored_window():
    import mpaso.gpu as G
    L, T, dt, n = 1, 3, 600.0, 5
    mesh, f, st, (h, hE, u, tr) = make(L, T, dict(fct=True, hmix=True, kappa=1e5), level=2)
    rng = np.random.default_rng(5)
    w = rng.standard_normal(tr.shape)
    zh, zu = np.zeros(h.shape), np.zeros(u.shape)
    grads = []
    for k in (1, 2, 5, 0):
        st.set(G.FIELD_TRACERS, tr)
        st.forward(dt, n, k)
        grads.append(st.vjp_tracers(zh, zu, w)[2])
    for g in grads[1:]:
        assert np.array_equal(g, grads[0])

    def J(x):
        st.set(G.FIELD_TRACERS, x)
        st.step(dt, n)
        return float((w * st.get(G.FIELD_TRACERS)).sum())

    for _ in range(3):
        v = rng.standard_normal(tr.shape) * 1e-3
        eps = 1e-3
        fd = (J(tr + eps * v) - J(tr - eps * v)) / (2 * eps)
        ad = float((grads[0] * v).sum())
        assert abs(fd - ad) <= 1e-6 * np.abs(grads[0] * v).sum(), (fd, ad)


def test_ocean_adjoint_central_differences_away_from_extrema():
    """Central differences of the CUDA forward against the adjoint along 8
    directions at the benchmark's column (60 levels x 3 tracers, FCT + del2;
    level-5 sphere, 2 steps of 900 s): each direction is supported on one cell
    and its neighbours, at one level and tracer, at least 6 rings from every
    local extremum of that tracer.  Near an extremum with no antidiffusive
    inflow the limiter's quotient (max - upwind) / (0 + 1e-10) changes branch
    under rounding-level perturbations, so no difference quotient checks the
    branch derivative there; away from extrema the limiter keeps its branch and
    the two agree to 1e-5 relative."""
    import mpaso.gpu as G
    from helpers import extremum_distance
    L, T, dt, n = 60, 3, 900.0, 2
    mesh, f, st, (h, hE, u, tr) = make(L, T, dict(fct=True, hmix=True, kappa=1e4), level=5, noise=False)
    area = mesh.fields["areaCell"]
    w = (area / area.sum())[:, None, None]
    target = tr[::-1].copy()

    def final(x):
        st.set(G.FIELD_TRACERS, x)
        st.step(dt, n)
        return st.get(G.FIELD_TRACERS)
    st.set(G.FIELD_TRACERS, tr)
    st.forward(dt, n, 1)
    gN = w * (st.get(G.FIELD_TRACERS) - target)
    gt = st.vjp_tracers(np.zeros(h.shape), np.zeros(u.shape), gN)[2]
    rng = np.random.default_rng(11)
    coc = mesh.fields["cellsOnCell"] - 1
    nE = mesh.fields["nEdgesOnCell"]
    errs, draws = [], 0
    while len(errs) < 8:
        draws += 1
        assert draws < 500, "no cell far enough from the extrema"
        k, t = int(rng.integers(L)), int(rng.integers(T))
        dist = extremum_distance(mesh, tr[:, k, t])
        centres = np.flatnonzero(dist >= 6)
        if centres.size == 0:
            continue
        c0 = int(rng.choice(centres))
        patch = np.concatenate([[c0], coc[c0, :nE[c0]]])
        v = np.zeros_like(tr)
        v[patch, k, t] = rng.standard_normal(patch.size)
        d = 1e-6 * np.abs(tr[:, k, t]).max()
        ap, am = final(tr + d * v), final(tr - d * v)
        fd = float((w * (ap - am) * (ap + am - 2.0 * target)).sum()) / (4 * d)
        ad = float((gt * v).sum())
        errs.append(abs(fd - ad) / abs(ad))
    assert max(errs) < 1e-5, errs
