"""History output of a device state (GPU): the sw diagnostics exposed as state
fields against the oracle's compute_solve_diagnostics, and the MPAS-layout
history file (netCDF classic) written from asynchronous snapshots while the
state keeps stepping."""
import numpy as np
import pytest

from helpers import Golden, rel_max
from oracle import Oracle
from test_gpu_rk4 import make_state

pytestmark = pytest.mark.gpu


def _oracle_diag(g, h, u):
    S = Oracle("restatement")
    L, nC, nE, nV = g.L, g.mesh.nCells, g.mesh.nEdges, g.mesh.nVertices
    out = {k: np.zeros((n, L)) for k, n in (("h_edge", nE), ("h_vertex", nV), ("circulation", nV),
                                             ("vorticity", nV), ("ke", nC), ("pv_edge", nE), ("pv_vertex", nV))}
    S.call("sw_compute_solve_diagnostics", S.mesh(g.mesh), S.static(g.mesh, g.fct), S.config(L, g.T),
           np.ascontiguousarray(h), np.ascontiguousarray(u), out["h_edge"], out["h_vertex"], out["circulation"],
           out["vorticity"], out["ke"], out["pv_edge"], out["pv_vertex"])
    return out


@pytest.mark.parametrize("name", ["sw_fct_icosa3_L1T1", "sw_scalar_icosa3_L3T2"])
def test_diagnostic_fields_match_oracle(name):
    import mpaso.gpu as G
    g = Golden(name)
    _, st = make_state(g)
    for steps in (0, 3):  # initial diagnostics, then those the steps leave current
        if steps:
            st.step_graph(g.dt, steps)
        h, u = st.get(G.FIELD_H), st.get(G.FIELD_U)
        want = _oracle_diag(g, h, u)
        assert rel_max(st.get(G.FIELD_VORTICITY), want["vorticity"]) < 1e-12
        assert rel_max(st.get(G.FIELD_PV_VERTEX), want["pv_vertex"]) < 1e-12
    with pytest.raises(Exception):
        st.set(G.FIELD_VORTICITY, np.zeros((g.mesh.nVertices, g.L)))


def test_history_file_records_while_stepping(tmp_path):
    import mpaso.gpu as G
    from mpaso.mpas_io import History, NcFile
    g = Golden("sw_fct_icosa3_L1T1")
    _, st = make_state(g)
    path = str(tmp_path / "history.nc")
    want = []
    with History(path, g.mesh, g.L, g.T, version=2) as hist:
        for _ in range(4):
            hist.write(st)  # record of the current state; copied out while the next steps run
            want.append({k: st.get(k) for k in (G.FIELD_H, G.FIELD_VORTICITY, G.FIELD_PV_VERTEX,
                                                  G.FIELD_TRACERS)})
            st.step_graph(g.dt, 2)
    with NcFile(path) as f:
        assert f.numrecs == 4 and f.get_att("on_a_sphere") == "YES"
        assert f.var_dims("h") == ["Time", "nCells", "nVertLevels"]
        assert f.var_dims("tracers") == ["Time", "nCells", "nVertLevels", "nTracers"]
        assert np.array_equal(f.get_var("areaCell"), g.mesh.fields["areaCell"])
        assert np.array_equal(f.get_var("cellsOnVertex"), g.mesh.fields["cellsOnVertex"])
        for r, w in enumerate(want):
            assert np.array_equal(f.get_rec("h", r), w[G.FIELD_H])
            assert np.array_equal(f.get_rec("vorticity", r), w[G.FIELD_VORTICITY])
            assert np.array_equal(f.get_rec("potential_vorticity", r), w[G.FIELD_PV_VERTEX])
            assert np.array_equal(f.get_rec("tracers", r), w[G.FIELD_TRACERS])
    sp = pytest.importorskip("scipy.io")
    with sp.netcdf_file(path, "r", mmap=False) as f:  # an independent reader sees the same file
        assert f.variables["h"].shape == (4, g.mesh.nCells, g.L)
        assert np.array_equal(f.variables["h"][3], want[3][G.FIELD_H])
