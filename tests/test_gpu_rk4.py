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
