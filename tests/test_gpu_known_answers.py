"""The ocean app's three test cases and sw cases 5 and 6 through the CUDA path
(GPU): the state after the full run agrees with the oracle's run to the
100-step parity bar, and the analytic error norms and conserved quantities meet
the bounds the CPU known-answer tests set."""
import numpy as np
import pytest

from helpers import rel_max
from mpaso.setup import fct_statics
from mpaso.testcases import ocean_case, ocean_case_error, sw_invariants
from test_known_answers import OCEAN_RUN, ocean_run, sw_case_run

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", [1, 2, 3])
def test_ocean_case_on_device(case):
    import mpaso.gpu as G
    level = 4
    m, tr0, want, t = ocean_run(level, case)
    h, u, tr = ocean_case(m, case)
    dm = G.DeviceMesh(m, fct=fct_statics(m, 1))
    st = G.State(dm, app=G.APP_OCEAN, nlev=1, ntr=1, fct=case != 3, hmix=case == 3,
                 kappa=1e7 if case == 3 else 0.0)
    st.set(G.FIELD_H, h)
    st.set(G.FIELD_U, u)
    st.set(G.FIELD_TRACERS, tr)
    st.set(G.FIELD_LAYER_THICKNESS_EDGE, np.ones((m.nEdges, 1)))
    dt, days = OCEAN_RUN[case][level]
    st.step_graph(dt, int(round(days * 86400.0 / dt)))
    got = st.get(G.FIELD_TRACERS)
    assert rel_max(got, want) < 1e-9
    l2, mx = ocean_case_error(m, case, got, t)
    if case == 3:
        assert l2 < 4e-6 and mx < 4e-4
    else:
        assert got.max() <= tr0.max() and got.min() > 50.0 * (1 - 2e-3)
        assert l2 < (5e-4 if case == 1 else 2.5e-3)


@pytest.mark.parametrize("case", [5, 6])
def test_sw_case_on_device(case):
    import mpaso.gpu as G
    m, (h, u, tr, hs), want = sw_case_run(case)
    T = 0 if case == 6 else 2
    dm = G.DeviceMesh(m, fct=fct_statics(m, 1) if T else None, bottomDepth=hs)
    st = G.State(dm, nlev=1, ntr=T, fct=bool(T))
    st.set(G.FIELD_H, h)
    st.set(G.FIELD_U, u)
    if T:
        st.set(G.FIELD_TRACERS, tr)
    st.step_graph(600.0, 144)
    got = (st.get(G.FIELD_H), st.get(G.FIELD_U)) + ((st.get(G.FIELD_TRACERS),) if T else ())
    for a, b in zip(got, want):
        assert rel_max(a, b) < 1e-9
    i0 = sw_invariants(m, h, u, tr if T else None, hs)
    i1 = sw_invariants(m, got[0], got[1], got[2] if T else None, hs)
    assert abs(i1["mass"] / i0["mass"] - 1) < 1e-14
    assert abs(i1["energy"] / i0["energy"] - 1) < (1e-7 if T else 1e-6)
    if T:
        assert np.all(np.abs(i1["tracer_mass"] / i0["tracer_mass"] - 1) < 1e-13)
