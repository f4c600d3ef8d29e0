"""The benchmark workloads at their full sizes (GPU): the level-7 sphere
shallow-water step with an FCT + del2 tracer against the oracle after 1 and 100
steps (relative max-norm 1e-12 / 1e-9), then 1000 steps checked through
size-independent properties (mass and tracer mass conserved to roundoff,
tracers inside their initial range); and the level-7 ocean step with 60 levels
and 3 tracers against the oracle after one step.  The oracle takes about a
minute here: these are the slowest GPU tests."""
import numpy as np
import pytest

import mpaso
from helpers import rel_max
from mpaso.initial import ocean_state, sw_state
from mpaso.setup import fct_statics
from oracle import Oracle

pytestmark = pytest.mark.gpu

SW = dict(fct=True, hmix=True, kappa=1e4, nu=1e4)  # the level-7 benchmark workload, dt = 60 s


def test_sw_level7_parity_and_invariants():
    import mpaso.gpu as G
    mesh = mpaso.Mesh.icosa(7)
    f = fct_statics(mesh, 1)
    h, u, tr = sw_state(mesh, 1000, 1, 1)
    S = Oracle("restatement")
    st_o, cfg = S.static(mesh, f), S.config(1, 1, **SW)
    want1 = S.sw_run(mesh, st_o, cfg, 60.0, 1, h, u, tr)
    want100 = S.sw_run(mesh, st_o, cfg, 60.0, 100, h, u, tr)
    dm = G.DeviceMesh(mesh, fct=f)
    st = G.State(dm, nlev=1, ntr=1, **SW)
    for fld, a in ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_TRACERS, tr)):
        st.set(fld, a)
    st.step_graph(60.0, 1)
    got = (st.get(G.FIELD_H), st.get(G.FIELD_U), st.get(G.FIELD_TRACERS))
    for a, b in zip(got, want1):
        assert rel_max(a, b) < 1e-12
    st.step_graph(60.0, 99)
    got = (st.get(G.FIELD_H), st.get(G.FIELD_U), st.get(G.FIELD_TRACERS))
    for a, b in zip(got, want100):
        assert rel_max(a, b) < 1e-9
    st.step_graph(60.0, 900)  # the workload's 1000 steps
    area = mesh.fields["areaCell"][:, None]
    hN, trN = st.get(G.FIELD_H), st.get(G.FIELD_TRACERS)[:, :, 0]
    assert abs((hN * area).sum() / (h * area).sum() - 1) < 1e-13
    assert abs((hN * trN * area).sum() / (h * tr[:, :, 0] * area).sum() - 1) < 1e-12
    assert trN.min() >= tr.min() - 1e-6 and trN.max() <= tr.max() + 1e-6


@pytest.mark.parametrize("clip", [False, True])
def test_ocean_level7_60_levels_one_step(clip):
    """One ocean step at level 7 with 60 levels and 3 tracers.  Unclipped fields:
    1e-12.  The benchmark's fields clip temperature to [0, 30], leaving plateaus
    where the limiter's quotient (max - upwind) / (dt flxIn / hProv + eps)
    cancels: there the reference's own output moves by 3.8e-11 when the velocity
    moves by one ulp (measured on the oracle), and the fused path, which rounds
    differently, agrees to 1e-8; tracer content and bounds hold exactly as well."""
    import mpaso.gpu as G
    mesh = mpaso.Mesh.icosa(7)
    L, T, dt = 60, 3, 300.0
    f = fct_statics(mesh, L)
    h, hE, u, tr = ocean_state(mesh, 1000, L, T, clip=clip)
    S = Oracle("restatement")
    want = S.ocean_run(mesh, S.static(mesh, f), S.config(L, T, fct=True, hmix=True, kappa=1e4), dt, 1,
                       h, hE, u, tr)
    dm = G.DeviceMesh(mesh, fct=f)
    st = G.State(dm, app=G.APP_OCEAN, nlev=L, ntr=T, fct=True, hmix=True, kappa=1e4)
    for fld, a in ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_TRACERS, tr), (G.FIELD_LAYER_THICKNESS_EDGE, hE)):
        st.set(fld, a)
    st.step_graph(dt, 1)
    got = st.get(G.FIELD_TRACERS)
    assert rel_max(got, want) < (1e-8 if clip else 1e-12)
    area = mesh.fields["areaCell"][:, None, None]
    content = lambda x: (x * h[:, :, None] * area).sum(axis=(0, 1))  # noqa: E731
    assert np.all(np.abs(content(got) / content(tr) - 1) < 1e-12)
