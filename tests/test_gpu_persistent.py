"""The persistent RK4 step (GPU): the whole run in one cooperative launch with
grid barriers between the phases of each stage.  It advances a state as the
graph-replayed three-kernel stages do -- on one mesh and on an ensemble of
uneven meshes -- and every barrier wait is bounded: a wait made to run out
(arrivals that never come) ends the launch with MPASO_ERR_TIMEOUT and leaves
the context usable."""
import numpy as np
import pytest

import mpaso
from helpers import rel_max
from mpaso.initial import sw_state
from mpaso.setup import fct_statics

pytestmark = pytest.mark.gpu

OPTS = dict(fct=True, hmix=True, kappa=1e4, nu=1e4)


def _pair(dm, fields, T):
    import mpaso.gpu as G
    out = []
    for _ in range(2):
        st = G.State(dm, nlev=1, ntr=T, **(OPTS if T else dict(nu=1e4)))
        for f, a in fields:
            st.set(f, a)
        out.append(st)
    return out


@pytest.mark.parametrize("T", [0, 1])
def test_persistent_matches_graph_steps(T):
    import mpaso.gpu as G
    mesh = mpaso.Mesh.icosa(5)
    h, u, tr = sw_state(mesh, 3, 1, max(T, 1))
    dm = G.DeviceMesh(mesh, fct=fct_statics(mesh, 1) if T else None)
    fields = [(G.FIELD_H, h), (G.FIELD_U, u)] + ([(G.FIELD_TRACERS, tr)] if T else [])
    a, b = _pair(dm, fields, T)
    a.step_graph(120.0, 25)
    b.step_persistent(120.0, 25)
    for f in [G.FIELD_H, G.FIELD_U] + ([G.FIELD_TRACERS] if T else []):
        assert rel_max(b.get(f), a.get(f)) < 1e-14
    b.step_persistent(120.0, 5)  # a second launch continues the same trajectory
    a.step_graph(120.0, 5)
    assert rel_max(b.get(G.FIELD_H), a.get(G.FIELD_H)) < 1e-14


def test_persistent_ensemble_matches_graph_steps():
    import mpaso.gpu as G
    members = [mpaso.Mesh.hex(32, 32, 10e3, 1e-4), mpaso.Mesh.icosa(4), mpaso.Mesh.hex(48, 48, 10e3, 1e-4)]
    fcts = [fct_statics(m, 1) for m in members]
    states = [sw_state(m, 10 + i, 1, 1) for i, m in enumerate(members)]
    dm = G.DeviceMesh.ensemble(members, fcts)
    fields = [(f, np.concatenate([s[k] for s in states])) for f, k in
              ((G.FIELD_H, 0), (G.FIELD_U, 1), (G.FIELD_TRACERS, 2))]
    a, b = _pair(dm, fields, 1)
    a.step_graph(30.0, 20)
    b.step_persistent(30.0, 20)
    for f in (G.FIELD_H, G.FIELD_U, G.FIELD_TRACERS):
        assert rel_max(b.get(f), a.get(f)) < 1e-14


def test_persistent_barrier_bound_runs_out():
    """Every barrier waits for one arrival more than the grid makes: each wait
    gives up after its poll bound, the launch ends, the call returns
    MPASO_ERR_TIMEOUT (6), and the context and state still work afterwards."""
    import mpaso.gpu as G
    from mpaso._lib import MpasoError
    mesh = mpaso.Mesh.icosa(3)
    h, u, _ = sw_state(mesh, 4, 1, 1)
    dm = G.DeviceMesh(mesh)
    st = G.State(dm, nlev=1, ntr=0)
    st.set(G.FIELD_H, h), st.set(G.FIELD_U, u)
    with pytest.raises(MpasoError) as e:
        st.step_persistent(60.0, 3, spin_limit=2000, extra_arrivals=1)
    assert e.value.code == 6 and "gave up" in str(e.value)
    st.set(G.FIELD_H, h), st.set(G.FIELD_U, u)
    st.step_persistent(60.0, 3)
    ref = G.State(dm, nlev=1, ntr=0)
    ref.set(G.FIELD_H, h), ref.set(G.FIELD_U, u)
    ref.step_graph(60.0, 3)
    assert rel_max(st.get(G.FIELD_H), ref.get(G.FIELD_H)) < 1e-14
