"""Checkpoint / resume (GPU): a run stopped after n steps, written with
write_restart, read into a fresh state and continued gives the uninterrupted
run's fields bit for bit (sw with FCT tracers; the ocean app)."""
import numpy as np
import pytest

import mpaso
from mpaso.setup import fct_statics

pytestmark = pytest.mark.gpu


def sw_state(L=2, T=2):
    import mpaso.gpu as G
    from mpaso.initial import sw_state as init
    mesh = mpaso.Mesh.icosa(3)
    dm = G.DeviceMesh(mesh, fct=fct_statics(mesh, L))
    make = lambda: G.State(dm, nlev=L, ntr=T, fct=True, hmix=True, kappa=1e4, nu=1e4)  # noqa: E731
    h, u, tr = init(mesh, 5, L, T)
    return make, ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_TRACERS, tr)), 90.0


def ocean_state(L=3, T=2):
    import mpaso.gpu as G
    from mpaso.initial import ocean_state as init
    mesh = mpaso.Mesh.icosa(3)
    dm = G.DeviceMesh(mesh, fct=fct_statics(mesh, L))
    make = lambda: G.State(dm, app=G.APP_OCEAN, nlev=L, ntr=T, fct=True, hmix=True, kappa=1e4)  # noqa: E731
    h, hE, u, tr = init(mesh, 5, L, T)
    return make, ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_LAYER_THICKNESS_EDGE, hE),
                  (G.FIELD_TRACERS, tr)), 450.0


@pytest.mark.parametrize("case", [sw_state, ocean_state])
def test_resume_from_restart_is_bitwise(case, tmp_path):
    import mpaso.gpu as G
    from mpaso.mpas_io import read_restart, write_restart
    make, fields, dt = case()
    a = make()
    for f, x in fields:
        a.set(f, x)
    a.step(dt, 10)
    want = {f: a.get(f) for f, _ in fields}
    b = make()
    for f, x in fields:
        b.set(f, x)
    b.step(dt, 4)
    path = str(tmp_path / "restart.nc")
    write_restart(path, b, time=4 * dt)
    b.close()
    c = make()
    assert read_restart(path, c) == 4 * dt
    c.step(dt, 6)
    for f, _ in fields:
        assert np.array_equal(c.get(f), want[f]), f
    assert G.FIELD_H in want


def test_restart_mismatch_is_rejected(tmp_path):
    import mpaso.gpu as G
    from mpaso.mpas_io import read_restart, write_restart
    make, fields, dt = sw_state()
    a = make()
    for f, x in fields:
        a.set(f, x)
    path = str(tmp_path / "restart.nc")
    write_restart(path, a)
    mesh = mpaso.Mesh.icosa(3)
    other = G.State(G.DeviceMesh(mesh), nlev=3, ntr=2)
    with pytest.raises(ValueError, match="nVertLevels"):
        read_restart(path, other)
    fewer = G.State(G.DeviceMesh(mesh, fct=fct_statics(mesh, 2)), nlev=2, ntr=1)
    with pytest.raises(ValueError, match="tracer count"):
        read_restart(path, fewer)
