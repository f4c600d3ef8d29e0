"""Ensemble contexts (GPU): one context over uneven members (mpaso_mesh_create_ensemble)
advances each member exactly as a context of that member alone does, and as the
reference does (oracle restatement, per member, at the fused path's parity bar)."""
import numpy as np
import pytest

import mpaso
from helpers import rel_max
from mpaso.initial import sw_state
from mpaso.setup import fct_statics
from oracle import Oracle

pytestmark = pytest.mark.gpu
OPTS = dict(fct=True, hmix=True, kappa=1e3, nu=1e3)
LAUNCH = ([1, 1, 1], [128, 128, 128], [0, 0, 0])


def members():
    ms = [mpaso.Mesh.hex(8, 6, 20e3, 1e-4), mpaso.Mesh.icosa(2), mpaso.Mesh.hex(12, 10, 15e3, 1e-4),
          mpaso.Mesh.icosa(3)]
    return ms, [fct_statics(m, 1) for m in ms], [sw_state(m, 10 + i, 1, 1) for i, m in enumerate(ms)]


def test_member_offsets():
    import mpaso.gpu as G
    ms, fcts, _ = members()
    dm = G.DeviceMesh.ensemble(ms, fcts)
    offs = dm.members()
    want = np.cumsum([[0, 0, 0]] + [[m.nCells, m.nEdges, m.nVertices] for m in ms], axis=0)
    assert np.array_equal(offs, want)
    single = G.DeviceMesh(ms[1])
    assert np.array_equal(single.members(), [[0, 0, 0], [ms[1].nCells, ms[1].nEdges, ms[1].nVertices]])
    dm.close()
    single.close()


def test_ensemble_matches_members_alone_and_reference():
    import mpaso.gpu as G
    ms, fcts, states = members()
    dt, n = 30.0, 3
    dm = G.DeviceMesh.ensemble(ms, fcts)
    st = G.State(dm, nlev=1, ntr=1, **OPTS)
    st.set_launch_config(*LAUNCH)
    for f, k in ((G.FIELD_H, 0), (G.FIELD_U, 1), (G.FIELD_TRACERS, 2)):
        st.set(f, np.concatenate([s[k] for s in states]))
    st.step_graph(dt, n)
    H, U, TR = st.get(G.FIELD_H), st.get(G.FIELD_U), st.get(G.FIELD_TRACERS)
    offs = dm.members()
    S = Oracle("restatement")
    for i, (m, f, s0) in enumerate(zip(ms, fcts, states)):
        c0, c1, e0, e1 = offs[i][0], offs[i + 1][0], offs[i][1], offs[i + 1][1]
        d1 = G.DeviceMesh(m, fct=f)
        s1 = G.State(d1, nlev=1, ntr=1, **OPTS)
        s1.set_launch_config(*LAUNCH)
        for fld, k in ((G.FIELD_H, 0), (G.FIELD_U, 1), (G.FIELD_TRACERS, 2)):
            s1.set(fld, s0[k])
        s1.step_graph(dt, n)
        # same member order and arithmetic as the member's own context
        assert np.array_equal(H[c0:c1], s1.get(G.FIELD_H))
        assert np.array_equal(U[e0:e1], s1.get(G.FIELD_U))
        assert np.array_equal(TR[c0:c1], s1.get(G.FIELD_TRACERS))
        h, u, tr = S.sw_run(m, S.static(m, f), S.config(1, 1, **OPTS), dt, n, *s0)
        tol = 1e-12 * 10 * n
        assert rel_max(H[c0:c1], h) < tol and rel_max(U[e0:e1], u) < tol and rel_max(TR[c0:c1], tr) < tol
        s1.close()
        d1.close()
    st.close()
    dm.close()


def test_ensemble_rejects_mixed_fct():
    import mpaso.gpu as G
    ms, fcts, _ = members()
    with pytest.raises(mpaso.MpasoError):
        G.DeviceMesh.ensemble(ms[:2], [fcts[0], None])
