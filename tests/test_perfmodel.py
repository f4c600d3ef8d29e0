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


def test_fp64_instruction_counts_match_the_profiler():
    """The FP64 instruction counts behind the bench line's `fp64` objects, at
    the sizes the committed ncu captures were taken on: the sw stage kernels on
    the level-7 sphere with one FCT tracer (per launch, within 2% of ncu's
    DFMA + DADD + DMUL counts), and the ocean's edge and final kernels on the
    level-6 sphere with 60 levels and 3 tracers (equal to ncu's counts)."""
    from mpaso.perfmodel import Dims, ocean_kernels, sw_kernels
    m7 = mpaso.Mesh.icosa(7)
    sw = sw_kernels(Dims.of(m7, 1, 1, fct_statics(m7, 1)), True, True, True)
    ncu_sw = {"sw_edge_pre": 9830399, "sw_tend": 20152406, "sw_final": 10977361}  # profiles/*_sw_l7.txt
    for k, v in ncu_sw.items():
        assert abs(sw[k][1] / v - 1) < 0.025, (k, sw[k][1], v)
    m6 = mpaso.Mesh.icosa(6)
    oc = ocean_kernels(Dims.of(m6, 60, 3, fct_statics(m6, 60)))
    assert int(oc["oc_edges"][1]) == 648806400  # profiles/oc_edges_ocean_l6.txt: 648,806,401
    assert int(oc["oc_final"][1]) == 250676640  # profiles/oc_final_ocean_l6.txt: 250,676,640
    assert abs(oc["oc_cells"][1] / 291282365 - 1) < 0.05  # the guarded divisions, averaged
