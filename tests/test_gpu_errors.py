"""Failure detection at the C ABI (GPU): faults are injected on the host only
(corrupted connectivity, out-of-range parameters, NaN written into the state,
calls out of order) and every one must come back as a status code with a
message, leaving the device context usable.  Nothing here faults, traps or
hangs a GPU: malformed meshes are rejected before any upload, and the NaN
check is a read-only scan."""
import types

import numpy as np
import pytest

import mpaso
from mpaso._lib import MpasoError
from mpaso.setup import fct_statics

pytestmark = pytest.mark.gpu


def corrupted(mesh, name, edit):
    """A stand-in for `mesh` whose CRS connectivity `name` is edited by edit(off, idx)."""
    crs = dict(mesh.crs())
    off, idx = crs[name]
    off, idx = off.copy(), idx.copy()
    edit(off, idx)
    crs[name] = (off, idx)
    return types.SimpleNamespace(crs=lambda: crs, fields=mesh.fields, nCells=mesh.nCells, nEdges=mesh.nEdges,
                                 nVertices=mesh.nVertices, on_sphere=mesh.on_sphere)


def expect_mesh_error(fake, match):
    import mpaso.gpu as G
    with pytest.raises(MpasoError, match=match) as e:
        G.DeviceMesh(fake)
    assert "[mpaso error 2]" in str(e.value)  # MPASO_ERR_MESH


def test_corrupted_meshes_are_rejected():
    mesh = mpaso.Mesh.icosa(2)
    nC, nE = mesh.nCells, mesh.nEdges

    def cell_out_of_range(off, idx):
        idx[5] = nC + 3

    def offsets_decrease(off, idx):
        off[4] = off[5] + 1

    def edge_index_out_of_range(off, idx):
        idx[0] = nE

    expect_mesh_error(corrupted(mesh, "c2c", cell_out_of_range), "c2c: index out of range")
    expect_mesh_error(corrupted(mesh, "c2v", offsets_decrease), "offsets decrease")
    expect_mesh_error(corrupted(mesh, "c2e", edge_index_out_of_range), "c2e: index out of range")

    # a cell lists another cell's edge in place of its own: one edge is left with one cell
    def edge_with_one_cell(off, idx):
        c0 = set(idx[off[0]:off[1]].tolist())
        other = next(e for e in idx[off[1]:] if e not in c0)
        idx[off[0]] = other

    expect_mesh_error(corrupted(mesh, "c2e", edge_with_one_cell), "exactly two cells")

    # edgesOnEdge of edge 0 names an edge whose own list does not name edge 0
    def not_symmetric(off, idx):
        crs = mesh.crs()
        eo, ei = crs["e2e"]
        near = set(ei[eo[0]:eo[1]].tolist()) | {0}
        far = next(e for e in range(nE) if e not in near and 0 not in ei[eo[e]:eo[e + 1]])
        idx[off[0]] = far

    expect_mesh_error(corrupted(mesh, "e2e", not_symmetric), "edgesOnEdge is not symmetric")


def test_state_parameters_are_checked():
    import mpaso.gpu as G
    mesh = mpaso.Mesh.icosa(2)
    plain = G.DeviceMesh(mesh)
    with_fct = G.DeviceMesh(mesh, fct=fct_statics(mesh, 2))
    cases = [
        (plain, dict(nlev=0, ntr=1), "nlev out of range"),
        (plain, dict(nlev=1, ntr=9), "ntr out of range"),
        (plain, dict(nlev=1, ntr=1, fct=True), "no FCT statics"),
        (with_fct, dict(nlev=3, ntr=1, fct=True), "another level count"),
        (plain, dict(app=G.APP_OCEAN, nlev=1, ntr=0), "ocean app needs tracers"),
    ]
    for dm, kw, match in cases:
        with pytest.raises(MpasoError, match=match):
            G.State(dm, **kw)
    # the context still works after the rejected calls
    st = G.State(with_fct, nlev=2, ntr=1, fct=True)
    st.set(G.FIELD_H, np.full((mesh.nCells, 2), 1000.0))
    st.step(60.0, 1)
    st.check_finite()


def test_nan_in_the_state_is_found_and_located():
    import mpaso.gpu as G
    from mpaso.initial import sw_state
    mesh = mpaso.Mesh.icosa(3)
    L, T = 2, 2
    st = G.State(G.DeviceMesh(mesh, fct=fct_statics(mesh, L)), nlev=L, ntr=T, fct=True)
    h, u, tr = sw_state(mesh, 1, L, T)
    for f, a in ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_TRACERS, tr)):
        st.set(f, a)
    st.check_finite()  # clean state passes
    bad = h.copy()
    bad[17, 1] = np.nan
    st.set(G.FIELD_H, bad)
    with pytest.raises(MpasoError, match=r"non-finite layer thickness at cell 17 level 1") as e:
        st.check_finite()
    assert "[mpaso error 7]" in str(e.value)  # MPASO_ERR_NUMERIC
    st.set(G.FIELD_H, h)
    badt = tr.copy()
    badt[40, 0, 1] = np.inf
    st.set(G.FIELD_TRACERS, badt)
    with pytest.raises(MpasoError, match=r"non-finite tracer at cell 40 level 0 tracer 1"):
        st.check_finite()
    # a NaN injected into the velocity spreads through the step and is caught after it
    st.set(G.FIELD_TRACERS, tr)
    badu = u.copy()
    badu[3, 0] = np.nan
    st.set(G.FIELD_U, badu)
    st.step(60.0, 2)
    with pytest.raises(MpasoError, match="non-finite"):
        st.check_finite()
    # restoring the fields restores the state
    for f, a in ((G.FIELD_H, h), (G.FIELD_U, u), (G.FIELD_TRACERS, tr)):
        st.set(f, a)
    st.step(60.0, 2)
    st.check_finite()


def test_calls_out_of_order_and_null_handles():
    import ctypes

    import mpaso.gpu as G
    from mpaso._lib import lib
    mesh = mpaso.Mesh.icosa(2)
    st = G.State(G.DeviceMesh(mesh), nlev=1, ntr=0)
    st.set(G.FIELD_H, np.full((mesh.nCells, 1), 1000.0))
    with pytest.raises(MpasoError, match="preceding mpaso_rk4_forward"):
        st.vjp(np.zeros((mesh.nCells, 1)), np.zeros((mesh.nEdges, 1)))
    assert lib().mpaso_rk4_step(None, ctypes.c_double(60.0), 1) == 1  # MPASO_ERR_ARG
    assert b"null" in lib().mpaso_last_error() or b"bad argument" in lib().mpaso_last_error()
    assert lib().mpaso_state_check_finite(None) == 1
    st.step(60.0, 1)  # the state is still usable
    st.check_finite()


def test_mesh_destroyed_before_its_state():
    """A mesh context outlives its destroy call while states use it (Python may
    finalise a state and its mesh in either order when they die in a cycle):
    the state keeps stepping, and tearing both down leaves no CUDA error
    behind for the next call."""
    import mpaso.gpu as G
    mesh = mpaso.Mesh.icosa(2)
    dm = G.DeviceMesh(mesh, fct=fct_statics(mesh, 1))
    st = G.State(dm, nlev=1, ntr=1, fct=True)
    st.set(G.FIELD_H, np.full((mesh.nCells, 1), 1000.0))
    dm.close()
    st.step(60.0, 3)
    st.check_finite()
    st.close()
    fct_statics(mesh, 1, device=0)  # a later call's own error check sees nothing stale
