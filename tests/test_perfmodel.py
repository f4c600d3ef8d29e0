"""The byte model of the roofline (CPU): the minimal fused dataflow, every
array read or written once per RK stage, from the mesh's own sums of the
ragged counts.  On the level-7 sphere with one level and one FCT tracer it
is 1.0695 GB per RK4 step (6,528 B per cell-update), the figure the bench
line's roofline divides by the step time."""
import numpy as np

import mpaso
from mpaso.perfmodel import dataflow_bytes
from mpaso.setup import fct_statics


def test_dataflow_bytes_level7_one_tracer():
    mesh = mpaso.Mesh.icosa(7)
    f = fct_statics(mesh, 1)
    b = dataflow_bytes(mesh, 1, 1, f)
    assert abs(b - 1.069541056e9) < 1.0
    assert abs(b / mesh.nCells - 6527.88) < 0.01


def test_dataflow_bytes_by_hand_on_a_small_mesh():
    """The same count written out term by term on a level-3 sphere, with the
    level and tracer terms scaling as L and L x T."""
    mesh = mpaso.Mesh.icosa(3)
    f = fct_statics(mesh, 2)
    fl = mesh.fields
    nC, nE, nV = mesh.nCells, mesh.nEdges, mesh.nVertices
    s_eoe, s_eoc, s_adv = fl["nEdgesOnEdge"].sum(), fl["nEdgesOnCell"].sum(), f["nAdvCellsForEdge"].sum()
    static = 36 * nE + 12 * s_eoe + 20 * nC + 4 * s_eoc + 64 * nV
    fct_static = 4 * nE + 20 * s_adv + 4 * s_eoc + 4 * nC + 8 * nE
    L, T = 2, 3
    per_stage = static + fct_static + L * (40 * (nC + nE) + 16 * (nV + nC)) + L * T * (40 * nC + 32 * nC + 16 * nE)
    assert dataflow_bytes(mesh, L, T, f) == 4 * per_stage
    # no tracers: the tracer rows drop out
    assert dataflow_bytes(mesh, L, 0, f) == 4 * (static + L * (40 * (nC + nE) + 16 * (nV + nC)))
    assert np.isclose(dataflow_bytes(mesh, 1, 1, f, fct=False, hmix=False),
                      4 * (static + 40 * (nC + nE) + 16 * (nV + nC) + 40 * nC))
