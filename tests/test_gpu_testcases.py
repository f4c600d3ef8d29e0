"""Test-case initialisers and error norms on the device (GPU): the sw app's
Williamson cases 1, 5, 6 and the ocean app's cases 1-3
(apps/sw/tasks/testcase.cc:37-227, apps/ocean/tasks/testcase.cc:96-294) set
up by mpaso_state_setup_case against the host restatements of the same
formulas (mpaso/testcases.py), and their error norms
(apps/sw/tasks/solve.cc:404-436, calc_error_case_1/2/3) by
mpaso_state_case_error against the host norms on the same fields.  Device
sin / cos / asin / pow / exp may differ from the host's in the last place, so
fields agree to 1e-12 relative; the slotted cylinder's two values agree
exactly."""
import numpy as np
import pytest

import mpaso
from helpers import rel_max
from mpaso.setup import fct_statics
from mpaso.testcases import (ocean_case, ocean_case_error, sw_case1, sw_case1_error, sw_case5,
                             sw_case6)

pytestmark = pytest.mark.gpu


def _sw(mesh, T=0, fct=None, **kw):
    import mpaso.gpu as G
    dm = G.DeviceMesh(mesh, fct=fct, **kw)
    dm.set_geometry(mesh)
    return dm, G.State(dm, nlev=1, ntr=T, fct=fct is not None)


@pytest.mark.parametrize("case", [1, 5, 6])
def test_sw_case_fields_match_host(case):
    import mpaso.gpu as G
    mesh = mpaso.Mesh.icosa(4)
    T = 2 if case == 5 else 0
    dm, st = _sw(mesh, T, fct_statics(mesh, 1) if T else None)
    st.setup_case(case)
    if case == 1:
        h, u = sw_case1(mesh)
    elif case == 5:
        h, u, hs, tr = sw_case5(mesh)
        assert rel_max(st.get(G.FIELD_TRACERS), tr) < 1e-12
    else:
        h, u = sw_case6(mesh)
    assert rel_max(st.get(G.FIELD_H), h) < 1e-12
    assert rel_max(st.get(G.FIELD_U), u) < 1e-12
    if case == 5:
        # the mountain lives in the state: one step from the device set-up equals
        # one step from the host fields on a mesh built with that bottom depth
        st.step_graph(600.0, 3)
        dm2 = G.DeviceMesh(mesh, fct=fct_statics(mesh, 1), bottomDepth=hs)
        st2 = G.State(dm2, nlev=1, ntr=2, fct=True)
        for f, a in ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_TRACERS, tr)):
            st2.set(f, a)
        st2.step_graph(600.0, 3)
        for f in (G.FIELD_H, G.FIELD_U, G.FIELD_TRACERS):
            assert rel_max(st.get(f), st2.get(f)) < 1e-11


def test_sw_case1_error_norm_matches_host():
    """The reference's ctest: case 1, 5 steps of 40 s; the device norm of the
    stepped state equals the host norm of the same fields and meets the
    reference's 0.0015 bound (apps/sw/finalize.cc:24-25)."""
    import mpaso.gpu as G
    mesh = mpaso.Mesh.icosa(5)
    dm = G.DeviceMesh(mesh)
    dm.set_geometry(mesh)
    st = G.State(dm, nlev=1, ntr=0, pin_u=True)
    st.setup_case(1)
    assert st.case_error(1, 0.0)[0] < 1e-15
    st.step_graph(40.0, 5)
    l2, mx = st.case_error(1, 200.0)
    hN = st.get(G.FIELD_H)
    want = sw_case1_error(mesh, hN, 200.0)
    assert abs(l2 / want - 1) < 1e-10
    assert l2 <= 0.0015
    # the largest pointwise relative error sits where the bell reaches zero at
    # its rim (the reference's bell, apps/sw/tasks/testcase.cc:71-76), the
    # same cell on the host
    f = mesh.fields
    from mpaso.testcases import _bell
    ht = _bell(f["latCell"], f["lonCell"], 3 * np.pi / 2 + 2 * np.pi * (200.0 / 86400 / 12), mpaso.EARTH_RADIUS)
    assert abs(mx / (np.abs(hN[:, 0] - ht) / ht).max() - 1) < 1e-9


@pytest.mark.parametrize("case", [1, 2, 3])
def test_ocean_case_fields_and_norms_match_host(case):
    import mpaso.gpu as G
    mesh = mpaso.Mesh.icosa(4)
    coef = 1e7
    dm = G.DeviceMesh(mesh, fct=fct_statics(mesh, 1))
    dm.set_geometry(mesh)
    st = G.State(dm, app=G.APP_OCEAN, nlev=1, ntr=1, fct=case != 3, hmix=case == 3,
                 kappa=coef if case == 3 else 0.0)
    st.setup_case(case, coef)
    h, u, tr = ocean_case(mesh, case, coef)
    assert np.array_equal(st.get(G.FIELD_H), h)
    assert np.array_equal(st.get(G.FIELD_LAYER_THICKNESS_EDGE), np.ones((mesh.nEdges, 1)))
    assert rel_max(st.get(G.FIELD_U), u) < 1e-12 if case != 3 else not st.get(G.FIELD_U).any()
    got = st.get(G.FIELD_TRACERS)
    if case == 2:
        assert np.array_equal(got, tr)
    else:
        assert rel_max(got, tr) < 1e-12
    dt = 900.0
    st.step_graph(dt, 8)
    l2, mx = st.case_error(case, 8 * dt, coef)
    hl2, hmx = ocean_case_error(mesh, case, st.get(G.FIELD_TRACERS), 8 * dt, coef)
    assert abs(l2 / hl2 - 1) < 1e-9 and abs(mx / hmx - 1) < 1e-9


def test_ensemble_setup_matches_members():
    """On an ensemble context the geometry is the members' concatenated and
    every member is set up as it would be alone."""
    import mpaso.gpu as G
    members = [mpaso.Mesh.icosa(3), mpaso.Mesh.icosa(4)]
    dm = G.DeviceMesh.ensemble(members)
    dm.set_geometry(members)
    st = G.State(dm, nlev=1, ntr=0)
    st.setup_case(6)
    h = np.concatenate([sw_case6(m)[0] for m in members])
    u = np.concatenate([sw_case6(m)[1] for m in members])
    assert rel_max(st.get(G.FIELD_H), h) < 1e-12
    assert rel_max(st.get(G.FIELD_U), u) < 1e-12


def test_setup_without_geometry_is_refused():
    import mpaso.gpu as G
    from mpaso._lib import MpasoError
    mesh = mpaso.Mesh.icosa(2)
    dm = G.DeviceMesh(mesh)
    st = G.State(dm, nlev=1, ntr=0)
    with pytest.raises(MpasoError) as e:
        st.setup_case(1)
    assert "set_geometry" in str(e.value)
    dm.set_geometry(mesh)
    with pytest.raises(MpasoError):
        st.setup_case(2)  # not a sw case
