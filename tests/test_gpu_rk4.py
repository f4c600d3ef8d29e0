"""Fused RK4 path against the reference (GPU).

Tolerances (relative max-norm, max|x-y| / max|y|): 1e-12 after one step and
1e-9 after 100 steps, the parity bar of this path; the fused kernels
reassociate sums and use fast reciprocals, so they agree to rounding, not bit
for bit.  Goldens come from the reference's own task sources."""
import numpy as np
import pytest

import mpaso
from helpers import Golden, golden_names, rel_max
from mpaso.initial import sw_state
from oracle import Oracle

pytestmark = pytest.mark.gpu
TOL1, TOL100 = 1e-12, 1e-9


def make_state(g, reorder=True):
    import mpaso.gpu as G
    dm = G.DeviceMesh(g.mesh, fct=g.fct, reorder=reorder)
    o = g.opts
    app = G.APP_SW if g.app == "sw" else G.APP_OCEAN
    st = G.State(dm, app=app, nlev=g.L, ntr=g.T, gravity=9.80616, fct=o.get("fct", False),
                 hmix=o.get("hmix", False), kappa=o.get("kappa", 0.0), nu=o.get("nu", 0.0))
    st.set(G.FIELD_H, g["h0"])
    st.set(G.FIELD_U, g["u0"])
    st.set(G.FIELD_TRACERS, g["tr0"])
    if g.app == "ocean":
        st.set(G.FIELD_LAYER_THICKNESS_EDGE, g["hE0"])
    return dm, st


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("graph", [False, True])
def test_fused_matches_reference_goldens(name, graph):
    import mpaso.gpu as G
    g = Golden(name)
    dm, st = make_state(g)
    done = 0
    for n in g.steps:
        (st.step_graph if graph else st.step)(g.dt, n - done)
        done = n
        tol = TOL1 if n == 1 else TOL1 * 10 * n
        tr = st.get(G.FIELD_TRACERS)
        assert rel_max(tr, g[f"tr_{n}"]) < tol, (n, rel_max(tr, g[f"tr_{n}"]))
        if g.app == "sw":
            assert rel_max(st.get(G.FIELD_H), g[f"h_{n}"]) < tol
            assert rel_max(st.get(G.FIELD_U), g[f"u_{n}"]) < tol
    st.close()
    dm.close()


def test_fused_100_steps_against_oracle():
    import mpaso.gpu as G
    mesh = mpaso.Mesh.icosa(4)
    S = Oracle("restatement")
    fct = S.fct_statics(mesh, 1)
    h, u, tr = sw_state(mesh, 11, 1, 1)
    opts = dict(fct=True, hmix=True, kappa=1e4, nu=1e4)
    dt = 240.0
    h1, u1, tr1 = S.sw_run(mesh, S.static(mesh, fct), S.config(1, 1, **opts), dt, 1, h, u, tr)
    h100, u100, tr100 = S.sw_run(mesh, S.static(mesh, fct), S.config(1, 1, **opts), dt, 100, h, u, tr)
    dm = G.DeviceMesh(mesh, fct=fct)
    st = G.State(dm, nlev=1, ntr=1, **opts)
    for f, a in ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_TRACERS, tr)):
        st.set(f, a)
    st.step_graph(dt, 1)
    assert rel_max(st.get(G.FIELD_H), h1) < TOL1
    assert rel_max(st.get(G.FIELD_U), u1) < TOL1
    assert rel_max(st.get(G.FIELD_TRACERS), tr1) < TOL1
    st.step_graph(dt, 99)
    assert rel_max(st.get(G.FIELD_H), h100) < TOL100
    assert rel_max(st.get(G.FIELD_U), u100) < TOL100
    assert rel_max(st.get(G.FIELD_TRACERS), tr100) < TOL100


def test_conservation_and_bounds():
    """Total mass and tracer content are conserved to roundoff; FCT tracers stay bounded."""
    import mpaso.gpu as G
    g = Golden("sw_fct_icosa3_L1T1")
    dm, st = make_state(g)
    area = g.mesh.fields["areaCell"][:, None]
    h0, tr0 = g["h0"], g["tr0"][:, :, 0]
    mass0, trm0 = (h0 * area).sum(), (h0 * tr0 * area).sum()
    st.step(g.dt, 50)
    h, tr = st.get(G.FIELD_H), st.get(G.FIELD_TRACERS)[:, :, 0]
    assert abs((h * area).sum() / mass0 - 1) < 1e-13
    assert abs((h * tr * area).sum() / trm0 - 1) < 1e-12
    assert tr.min() > -1e-3 and tr.max() < 1 + 1e-3


def test_unreordered_context_agrees():
    import mpaso.gpu as G
    g = Golden("sw_scalar_icosa3_L3T2")
    _, a = make_state(g, reorder=True)
    _, b = make_state(g, reorder=False)
    a.step(g.dt, 3)
    b.step(g.dt, 3)
    for f in (G.FIELD_H, G.FIELD_U, G.FIELD_TRACERS):
        assert rel_max(a.get(f), b.get(f)) < 1e-13


def test_host_boundary_call_matches():
    import mpaso.gpu as G
    g = Golden("sw_fct_icosa3_L1T1")
    dm, st = make_state(g)
    h, u, tr = g["h0"].copy(), g["u0"].copy(), g["tr0"].copy()
    st.step_host(g.dt, 1, h, u, tr)
    assert rel_max(h, g["h_1"]) < TOL1 and rel_max(u, g["u_1"]) < TOL1 and rel_max(tr, g["tr_1"]) < TOL1


def _run_both(mesh, fct, state, L, T, dt, n, **opts):
    """(gpu fields, oracle fields) after n steps from `state` = (h, u, tr)."""
    import mpaso.gpu as G
    S = Oracle("restatement")
    want = S.sw_run(mesh, S.static(mesh, fct), S.config(L, T, **opts), dt, n, *state)
    dm = G.DeviceMesh(mesh, fct=fct)
    st = G.State(dm, nlev=L, ntr=T, **opts)
    st.set(G.FIELD_H, state[0])
    st.set(G.FIELD_U, state[1])
    if T:
        st.set(G.FIELD_TRACERS, state[2])
    st.step_graph(dt, n)
    got = (st.get(G.FIELD_H), st.get(G.FIELD_U), st.get(G.FIELD_TRACERS) if T else state[2])
    st.close()
    dm.close()
    return got, want


def test_planar_64x64_plain_method_100_steps():
    """The reference's CPU-runnable configuration: 64 x 64 doubly periodic hex
    mesh (dc = 10 km, f = 1e-4, g = 9.81, H0 = 1000 m, bumps of 10 m, peak u 1 m/s),
    FP64 shallow water with del2 viscosity 1e3, dt = 30 s: 1e-12 after one step and
    1e-9 after 100 against the oracle."""
    mesh = mpaso.Mesh.hex(64, 64, 10e3, 1e-4)
    h, u, _ = sw_state(mesh, 7, 1, 0)
    state = (h, u, np.zeros((mesh.nCells, 1, 0)))
    opts = dict(gravity=9.81, nu=1e3)
    for n, tol in ((1, TOL1), (100, TOL100)):
        got, want = _run_both(mesh, None, state, 1, 0, 30.0, n, **opts)
        assert rel_max(got[0], want[0]) < tol and rel_max(got[1], want[1]) < tol, n


def test_sw_case1_on_device():
    """Williamson case 1 through the CUDA path: the reference's 0.0015 bound after its
    ctest (5 steps of 40 s on a 240 km sphere), matching the oracle's h."""
    from mpaso.testcases import sw_case1, sw_case1_error
    mesh = mpaso.Mesh.icosa(5)
    h, u = sw_case1(mesh)
    got, want = _run_both(mesh, None, (h, u, np.zeros((mesh.nCells, 1, 0))), 1, 0, 40.0, 5, pin_u=True)
    assert np.array_equal(got[1], u)
    assert rel_max(got[0], want[0]) < TOL1 * 10 * 5
    assert sw_case1_error(mesh, got[0], 200.0) <= 0.0015


def test_del2_mode_decay_on_device():
    from mpaso.testcases import del2_mode
    mesh = mpaso.Mesh.hex(32, 32, 10e3, 0.0)
    h, u, pattern, k2 = del2_mode(mesh)
    nu, dt, n = 1e5, 30.0, 100
    got, want = _run_both(mesh, None, (h, u, np.zeros((mesh.nCells, 1, 0))), 1, 0, dt, n, nu=nu)
    a = float((got[1][:, 0] * pattern).sum() / (pattern * pattern).sum()) / 1e-6
    assert abs(-np.log(a) / (nu * dt * n) / k2 - 1) < 0.01
    assert rel_max(got[1], want[1]) < TOL100


def test_host_boundary_call_with_page_locked_buffers():
    """Page-locked (mapped) host buffers take the zero-copy path of mpaso_rk4_step_host;
    it must give exactly what the staged path gives for pageable buffers."""
    torch = pytest.importorskip("torch")
    import mpaso.gpu as G
    g = Golden("sw_fct_icosa3_L1T1")
    _, st = make_state(g)
    h, u, tr = g["h0"].copy(), g["u0"].copy(), g["tr0"].copy()
    st.step_host(g.dt, 2, h, u, tr)
    _, st2 = make_state(g)
    hp, up, tp = (torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in (g["h0"], g["u0"], g["tr0"]))
    st2.step_host(g.dt, 2, hp, up, tp)
    assert np.array_equal(hp.numpy(), h) and np.array_equal(up.numpy(), u) and np.array_equal(tp.numpy(), tr)


@pytest.mark.parametrize("offset", [0, 1])
def test_page_locked_exchange_odd_sizes_and_unaligned_buffers(offset):
    """The one-pass exchange of mapped page-locked buffers (16-byte host accesses
    where the field's size and the buffer's alignment allow, 8-byte ones
    otherwise) equals the staged path of pageable buffers bit for bit, with
    buffers on a 16-byte boundary and 8 bytes past one (the 8-byte form), on a
    15 x 14 periodic hex mesh."""
    torch = pytest.importorskip("torch")
    import mpaso.gpu as G
    from mpaso.initial import sw_state
    mesh = mpaso.Mesh.hex(15, 14, 10e3, 1e-4)
    h, u, tr = sw_state(mesh, 7, 1, 1)

    def state():
        dm = G.DeviceMesh(mesh)
        return dm, G.State(dm, nlev=1, ntr=1, nu=1e3)

    def pinned(a):
        buf = torch.empty(a.size + offset, dtype=torch.float64).pin_memory()
        v = buf[offset:].view(a.shape)
        v.copy_(torch.from_numpy(np.ascontiguousarray(a)))
        return v

    _, st = state()
    hh, uu, tt = h.copy(), u.copy(), tr.copy()
    st.step_host(30.0, 2, hh, uu, tt)
    _, st2 = state()
    hp, up, tp = pinned(h), pinned(u), pinned(tr)
    assert (hp.data_ptr() % 16 == 8) == (offset == 1)
    st2.step_host(30.0, 2, hp, up, tp)
    assert not np.array_equal(hh, h)
    for a, b in ((hp, hh), (up, uu), (tp, tt)):
        assert np.array_equal(a.numpy(), b)


def test_ocean_host_exchange_matches_goldens():
    """The ocean app through the host-buffer call: thickness, velocity and
    tracers in from page-locked buffers (the one-pass exchange kernels), one
    step at a time, equal to the reference's goldens value for value after 1
    and 10 steps (the ocean kernels keep the reference's rounding)."""
    torch = pytest.importorskip("torch")
    g = Golden("ocean_icosa3_L3T2")
    _, st = make_state(g)
    hp, up, tp = (torch.from_numpy(np.ascontiguousarray(g[k])).pin_memory() for k in ("h0", "u0", "tr0"))
    done = 0
    for n in g.steps:
        for _ in range(n - done):
            st.step_host(g.dt, 1, hp, up, tp)
        done = n
        assert np.array_equal(tp.numpy(), g[f"tr_{n}"])
        assert np.array_equal(hp.numpy(), g["h0"]) and np.array_equal(up.numpy(), g["u0"])  # prescribed


def test_async_host_boundary_calls_in_a_loop():
    """Queued one-step exchanges on the same page-locked buffers (each copying in
    what the previous one copied out) end where the same number of blocking
    calls ends, bit for bit; pageable buffers are refused for the queued form."""
    torch = pytest.importorskip("torch")
    g = Golden("sw_fct_icosa3_L1T1")
    _, st = make_state(g)
    h, u, tr = (torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in (g["h0"], g["u0"], g["tr0"]))
    for _ in range(5):
        st.step_host(g.dt, 1, h, u, tr)
    _, st2 = make_state(g)
    ha, ua, ta = (torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in (g["h0"], g["u0"], g["tr0"]))
    for _ in range(5):
        st2.step_host_async(g.dt, 1, ha, ua, ta)
    st2.sync()
    for a, b in ((h, ha), (u, ua), (tr, ta)):
        assert np.array_equal(a.numpy(), b.numpy())
    with pytest.raises(mpaso.MpasoError, match="page-locked"):
        st2.step_host_async(g.dt, 1, g["h0"].copy(), g["u0"].copy(), g["tr0"].copy())


def test_history_snapshots_while_stepping():
    """Snapshots taken between graph-replayed steps, copied out asynchronously while
    later steps run, equal the state read synchronously at the same points."""
    torch = pytest.importorskip("torch")
    import mpaso.gpu as G
    g = Golden("sw_fct_icosa3_L1T1")
    _, st = make_state(g)
    _, ref = make_state(g)
    snaps, want = [], []
    for n in range(4):
        st.step_graph(g.dt, 2)
        hp = torch.empty(g["h0"].shape, dtype=torch.float64).pin_memory()
        tp = torch.empty(g["tr0"].shape, dtype=torch.float64).pin_memory()
        snaps.append((st.snapshot(G.FIELD_H, hp), st.snapshot(G.FIELD_TRACERS, tp)))
        ref.step_graph(g.dt, 2)
        want.append((ref.get(G.FIELD_H), ref.get(G.FIELD_TRACERS)))
    st.snapshot_wait()
    for (hp, tp), (h, tr) in zip(snaps, want):
        assert np.array_equal(hp.numpy(), h) and np.array_equal(tp.numpy(), tr)


def test_ocean_without_fct_mixes_but_does_not_advect():
    """The ocean app advects tracers only through FCT (apps/ocean/run.cc:20-38):
    with fct = 0 and del2 mixing on, a nonzero velocity leaves only the mixing."""
    import mpaso.gpu as G
    from mpaso.initial import ocean_state
    mesh = mpaso.Mesh.icosa(3)
    L, T, dt = 2, 2, 600.0
    S = Oracle("restatement")
    f = S.fct_statics(mesh, L)
    h, hE, u, tr = ocean_state(mesh, 5, L, T, clip=False)
    cfg = S.config(L, T, hmix=True, kappa=1e5)
    want1 = S.ocean_run(mesh, S.static(mesh, f), cfg, dt, 1, h, hE, u, tr)
    want20 = S.ocean_run(mesh, S.static(mesh, f), cfg, dt, 20, h, hE, u, tr)
    dm = G.DeviceMesh(mesh, fct=f)
    st = G.State(dm, app=G.APP_OCEAN, nlev=L, ntr=T, hmix=True, kappa=1e5)
    for fld, a in ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_TRACERS, tr), (G.FIELD_LAYER_THICKNESS_EDGE, hE)):
        st.set(fld, a)
    st.step_graph(dt, 1)
    assert rel_max(st.get(G.FIELD_TRACERS), want1) < TOL1
    st.step_graph(dt, 19)
    assert rel_max(st.get(G.FIELD_TRACERS), want20) < TOL100


@pytest.mark.parametrize("app,opts", [
    ("sw", dict(fct=True)), ("sw", dict(hmix=True, kappa=1e5)), ("sw", dict(fct=True, nu=1e5)),
    ("sw", dict(hmix=True, kappa=1e5, nu=1e5)),
    ("ocean", dict(fct=True)), ("ocean", dict()), ("ocean", dict(fct=True, hmix=True, kappa=1e5))])
def test_every_option_combination_against_oracle(app, opts):
    """Each combination of FCT advection, del2 tracer mixing and del2 momentum the
    two apps accept, on the fused path against the oracle after 1 and 10 steps."""
    import mpaso.gpu as G
    from mpaso.initial import ocean_state
    mesh = mpaso.Mesh.icosa(3)
    L, T, dt, n = 2, 2, 450.0, 10
    S = Oracle("restatement")
    f = S.fct_statics(mesh, L)
    cfg = S.config(L, T, **opts)
    dm = G.DeviceMesh(mesh, fct=f)
    if app == "sw":
        h, u, tr = sw_state(mesh, 21, L, T)
        run = lambda k: S.sw_run(mesh, S.static(mesh, f), cfg, dt, k, h, u, tr)  # noqa: E731
        st = G.State(dm, nlev=L, ntr=T, **opts)
        fields = ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_TRACERS, tr))
        out = (G.FIELD_H, G.FIELD_U, G.FIELD_TRACERS)
    else:
        h, hE, u, tr = ocean_state(mesh, 21, L, T, clip=False)
        run = lambda k: (S.ocean_run(mesh, S.static(mesh, f), cfg, dt, k, h, hE, u, tr),)  # noqa: E731
        st = G.State(dm, app=G.APP_OCEAN, nlev=L, ntr=T, **opts)
        fields = ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_TRACERS, tr), (G.FIELD_LAYER_THICKNESS_EDGE, hE))
        out = (G.FIELD_TRACERS,)
    for fld, a in fields:
        st.set(fld, a)
    st.step_graph(dt, 1)
    for fld, want in zip(out, run(1)):
        assert rel_max(st.get(fld), want) < TOL1
    st.step_graph(dt, n - 1)
    for fld, want in zip(out, run(n)):
        assert rel_max(st.get(fld), want) < TOL100
