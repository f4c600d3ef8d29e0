"""The CPU oracle, pinned (CPU): the C restatement reproduces the reference's own
task sources bit for bit, on the committed golden fixtures and, where the
reference checkout was available, against the shim-compiled reference itself."""
import numpy as np
import pytest

from helpers import Golden, golden_names
from oracle import Oracle, ref_available


@pytest.mark.parametrize("name", golden_names())
def test_restatement_matches_reference_goldens(name):
    g = Golden(name)
    S = Oracle("restatement")
    cfg = S.config(g.L, g.T, **g.opts)
    st = S.static(g.mesh, g.fct)
    for n in g.steps:
        if g.app == "sw":
            h, u, tr = S.sw_run(g.mesh, st, cfg, g.dt, n, g["h0"], g["u0"], g["tr0"])
            assert np.array_equal(h, g[f"h_{n}"]) and np.array_equal(u, g[f"u_{n}"])
            assert np.array_equal(tr, g[f"tr_{n}"])
        else:
            tr = S.ocean_run(g.mesh, st, cfg, g.dt, n, g["h0"], g["hE0"], g["u0"], g["tr0"])
            assert np.array_equal(tr, g[f"tr_{n}"])


@pytest.mark.parametrize("name", ["sw_fct_icosa3_L1T1", "ocean_icosa3_L3T2", "sw_fct_icosa2_L5T5"])
def test_restatement_fct_statics_match_reference(name):
    g = Golden(name)
    S = Oracle("restatement")
    out = S.fct_statics(g.mesh, g.L, cfg=S.config(g.L, g.T))
    for k, v in g.fct.items():
        assert np.array_equal(out[k], v), k


@pytest.mark.parametrize("L,T", [(1, 1), (3, 2)])
def test_restatement_matches_live_reference(L, T):
    if not ref_available(L, T):
        pytest.skip("reference checkout not built here (oracle/_ref)")
    import mpaso
    from mpaso.initial import sw_state
    mesh = mpaso.Mesh.icosa(2)
    R, S = Oracle("ref", L, T), Oracle("restatement")
    fr = R.fct_statics(mesh, L, cfg=R.config(L, T))
    fs = S.fct_statics(mesh, L, cfg=S.config(L, T))
    for k in fr:
        assert np.array_equal(fr[k], fs[k]), k
    h, u, tr = sw_state(mesh, 99, L, T)
    opts = dict(fct=True, hmix=True, kappa=3e4, nu=2e4)
    a = R.sw_run(mesh, R.static(mesh, fr), R.config(L, T, **opts), 450.0, 4, h, u, tr)
    b = S.sw_run(mesh, S.static(mesh, fs), S.config(L, T, **opts), 450.0, 4, h, u, tr)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_oracle_detects_planted_error():
    """A mistake planted in the oracle's inputs is caught by the bit-exact comparison."""
    g = Golden("sw_fct_icosa3_L1T1")
    S = Oracle("restatement")
    fct = dict(g.fct)
    fct["advCoef"] = fct["advCoef"].copy()
    fct["advCoef"][17, 3] *= 1.0 + 1e-6
    h, u, tr = S.sw_run(g.mesh, S.static(g.mesh, fct), S.config(g.L, g.T, **g.opts), g.dt, 1,
                        g["h0"], g["u0"], g["tr0"])
    assert not np.array_equal(tr, g["tr_1"])


@pytest.mark.parametrize("kind", ["icosa3", "hex16"])
@pytest.mark.parametrize("nu", [0.0, 2e5])
def test_complex_step_restatement(kind, nu):
    """The complex-step restatement of the sw (h, u) step reproduces the oracle's
    real step to rounding, and its tangent agrees with central differences of the
    oracle to the differences' truncation error."""
    import mpaso
    from mpaso.initial import sw_state
    from sw_complex import SwComplex
    mesh = mpaso.Mesh.icosa(3) if kind == "icosa3" else mpaso.Mesh.hex(16, 16, 10e3)
    dt, L, n = (300.0 if kind == "icosa3" else 30.0), 2, 3
    S = Oracle("restatement")
    h, u, tr = sw_state(mesh, 3, L, 1)
    run = lambda hh, uu: S.sw_run(mesh, S.static(mesh), S.config(L, 1, nu=nu), dt, n, hh, uu, tr)  # noqa: E731
    hr, ur, _ = run(h, u)
    C = SwComplex(mesh, L, nu=nu)
    hc, uc = C.step(h, u, dt, n)
    assert np.abs(hc.ravel() - hr.ravel()).max() <= 1e-13 * np.abs(hr).max()
    assert np.abs(uc.ravel() - ur.ravel()).max() <= 1e-13 * np.abs(ur).max()
    rng = np.random.default_rng(0)
    vh, vu = rng.standard_normal(h.shape), rng.standard_normal(u.shape) * 1e-3
    jh, ju = C.jvp(h, u, vh, vu, dt, n)
    eps = 1e-3
    hp, up, _ = run(h + eps * vh, u + eps * vu)
    hm, um, _ = run(h - eps * vh, u - eps * vu)
    fh, fu = (hp - hm) / (2 * eps), (up - um) / (2 * eps)
    assert np.abs(jh.ravel() - fh.ravel()).max() <= 1e-8 * np.abs(fh).max()
    assert np.abs(ju.ravel() - fu.ravel()).max() <= 1e-8 * np.abs(fu).max()


@pytest.mark.parametrize("fct,hmix", [(True, True), (True, False), (False, True)])
def test_complex_step_restatement_with_tracers(fct, hmix):
    """The tracer part of the complex-step restatement (FCT advection, del2
    mixing, thickness-weighted RK) reproduces the oracle's real step to
    rounding, and its tangent, taken on the branch the real step takes,
    agrees with central differences of the oracle along a direction small
    enough to keep every limiter branch."""
    import mpaso
    from mpaso.initial import sw_state
    from sw_complex import SwComplex
    mesh = mpaso.Mesh.icosa(3)
    dt, L, T, n, kappa = 300.0, 2, 2, 3, 2e6
    S = Oracle("restatement")
    h, u, tr = sw_state(mesh, 3, L, T)
    tr = 0.7 * tr + 0.3 * np.random.default_rng(103).uniform(0.0, 1.0, tr.shape)
    f = S.fct_statics(mesh, L)
    cfg = S.config(L, T, fct=fct, hmix=hmix, kappa=kappa)
    run = lambda a, b, c: S.sw_run(mesh, S.static(mesh, f), cfg, dt, n, a, b, c)  # noqa: E731
    ref = run(h, u, tr)
    C = SwComplex(mesh, L, fct=f, centred=not fct, T=T, hmix=hmix, kappa=kappa)
    got = C.step(h, u, dt, n, tr=tr)
    for x, y in zip(got, ref):
        assert np.abs(x.ravel() - y.ravel()).max() <= 1e-13 * np.abs(y).max()
    rng = np.random.default_rng(0)
    v = (rng.standard_normal(h.shape), rng.standard_normal(u.shape) * 1e-3, rng.standard_normal(tr.shape))
    jv = C.jvp_tracers(h, u, tr, *v, dt, n)
    eps = 1e-6
    P = run(*[a + eps * b for a, b in zip((h, u, tr), v)])
    M = run(*[a - eps * b for a, b in zip((h, u, tr), v)])
    fd_tr = (P[2] - M[2]) / (2 * eps)
    assert np.abs(jv[2].ravel() - fd_tr.ravel()).max() <= 1e-7 * np.abs(jv[2]).max()


@pytest.mark.parametrize("fct,hmix", [(True, True), (True, False), (False, True)])
def test_complex_step_restatement_ocean(fct, hmix):
    """The ocean app's tracer step in the complex-step restatement (prescribed
    thickness, edge thickness and velocity; no thickness weighting in the RK
    sums) reproduces the oracle's ocean run to rounding, and its tangent
    agrees with central differences of the oracle."""
    import mpaso
    from mpaso.initial import ocean_state
    from sw_complex import SwComplex
    mesh = mpaso.Mesh.icosa(3)
    dt, L, T, n, kappa = 600.0, 2, 2, 3, 1e5
    S = Oracle("restatement")
    h, hE, u, tr = ocean_state(mesh, 7, L, T, clip=False)
    tr = 0.7 * tr + 0.3 * tr.max() * np.random.default_rng(7).uniform(0.0, 1.0, tr.shape)
    f = S.fct_statics(mesh, L)
    cfg = S.config(L, T, fct=fct, hmix=hmix, kappa=kappa)
    run = lambda t: S.ocean_run(mesh, S.static(mesh, f), cfg, dt, n, h, hE, u, t)  # noqa: E731
    ref = run(tr)
    C = SwComplex(mesh, L, fct=f, centred=not fct, T=T, hmix=hmix, kappa=kappa)
    got = C.ocean_step(h, hE, u, tr, dt, n)
    assert np.abs(got.ravel() - ref.ravel()).max() <= 1e-12 * np.abs(ref).max()
    v = np.random.default_rng(1).standard_normal(tr.shape)
    jv = C.ocean_jvp(h, hE, u, tr, v, dt, n)
    eps = 1e-6
    fd = (run(tr + eps * v) - run(tr - eps * v)) / (2 * eps)
    assert np.abs(jv.ravel() - fd.ravel()).max() <= 1e-5 * np.abs(jv).max()


@pytest.mark.skipif(not __import__("oracle").cstep_available(), reason="reference checkout absent")
@pytest.mark.parametrize("kind", ["icosa3", "hex"])
def test_complex_step_restatement_pinned_to_reference_code(kind):
    """The reference's own sw tasks evaluated on complex state (shim complex-step
    build, an FP64 tape over the reference step) give the same real step as the
    restatement, bit for bit, and the same tangent as the array restatement that
    the GPU adjoint test uses, to rounding."""
    import mpaso
    from mpaso.initial import sw_state
    from oracle import RefComplexStep
    from sw_complex import SwComplex
    mesh = mpaso.Mesh.icosa(3) if kind == "icosa3" else mpaso.Mesh.hex(12, 10, 20e3)
    dt = 300.0 if kind == "icosa3" else 30.0
    R = RefComplexStep()
    h, u, _ = sw_state(mesh, 5, R.L, 1)
    rng = np.random.default_rng(1)
    dh, du = rng.standard_normal(h.shape), rng.standard_normal(u.shape) * 1e-3
    (hr, ur), (jh, ju) = R.jvp(mesh, dt, 4, h, u, dh, du)
    S = Oracle("restatement")
    h2, u2, _ = S.sw_run(mesh, S.static(mesh), S.config(R.L, 1), dt, 4, h, u, np.zeros((mesh.nCells, R.L, 1)))
    assert np.array_equal(hr, h2) and np.array_equal(ur, u2)
    ch, cu = SwComplex(mesh, R.L).jvp(h, u, dh, du, dt, 4)
    assert np.abs(jh.ravel() - ch.ravel()).max() <= 1e-14 * np.abs(ch).max()
    assert np.abs(ju.ravel() - cu.ravel()).max() <= 1e-14 * np.abs(cu).max()
