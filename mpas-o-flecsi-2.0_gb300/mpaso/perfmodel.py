"""Algorithmic traffic and FP64 work of the fused RK4 kernels.

Bytes: every array a launch touches counted once (reads + writes), at its
real size on the mesh (8 B per double, 4 B per index), the compulsory traffic
of the dataflow -- repeated gathers of a neighbour's value are not counted
again.  FP64 work: DADD / DMUL / DFMA thread instructions per launch (a
reciprocal by rcp_nr is 4 on the FP64 pipe plus the approximation on the
special-function unit; the limiter's two guarded quotients run only where a
bound is active, counted as a quarter of the cells); min/max/select/sign work
runs on the integer pipe and is not counted.  ncu's counts for the same
launches are in profiles/ (within about 10% of these).

One cell-update = one cell x one level advanced by one full RK4 step.

Two byte models are kept.  `dataflow_bytes` is the model of record for the
roofline: the minimal fused dataflow, each array counted once per RK stage.
`sw_kernels` / `ocean_kernels` count what each launch touches, re-reads across
the three kernels of a stage included; they explain per-kernel traffic.
"""
from dataclasses import dataclass


@dataclass
class Dims:
    nC: int
    nE: int
    nV: int
    L: int
    T: int
    maxEoE: int  # edgesOnEdge slots (padded)
    maxAdv: int  # advection cells per edge (padded)
    avgEoC: float  # mean edges per cell

    @classmethod
    def of(cls, mesh, L, T, fct_statics=None):
        f = mesh.fields
        maxEoE = int(f["nEdgesOnEdge"].max())
        maxAdv = int(fct_statics["nAdvCellsForEdge"].max()) if fct_statics is not None else 1
        return cls(mesh.nCells, mesh.nEdges, mesh.nVertices, L, T, maxEoE, maxAdv,
                   float(f["nEdgesOnCell"].mean()))


def dataflow_bytes(mesh, L, T, fct_statics=None, fct=True, hmix=True):
    """Algorithmic bytes of one RK4 step in the minimal fused dataflow: every
    array read or written once per RK stage (FP64 = 8 B, index = 4 B), from
    the mesh's own sums of the ragged counts.

    Per stage:
      shallow-water statics -- edges: cellsOnEdge 8, verticesOnEdge 8, dvEdge 8,
        dcEdge 8, nEdgesOnEdge 4, per edgesOnEdge slot index 4 + weight 8;
        cells: areaCell 8, bottom depth 8, nEdgesOnCell 4, per edge slot 4
        (edge signs follow from cellsOnEdge); vertices: cellsOnVertex 12,
        kites 24, areaTriangle 8, fVertex 8, edgesOnVertex 12;
      shallow water per level -- h and u: stage input, step start, accumulator
        read + write, next stage input (5 x 8 B per cell and edge); the
        compulsory intermediates pv (vertices) and ke (cells), write + read
        (del2 momentum adds no array: its divergence folds into the cell
        function ke - nu div that the gradient already reads);
      FCT + del2 tracer statics -- nAdvCellsForEdge 4 and per stencil slot
        index 4 + advCoef 8 + advCoef_3rd 8 per edge; cellsOnCell (4 per slot
        + 4 per cell); meshScalingDel2 8 per edge;
      per level and tracer -- the tracer state as h and u (5 x 8 per cell),
        the limiter factors R+ and R- write + read (32 per cell), the
        anti-diffusive flux write + read (16 per edge).
    Without tracers the tracer rows drop out."""
    f = mesh.fields
    nC, nE, nV = mesh.nCells, mesh.nEdges, mesh.nVertices
    s_eoe = float(f["nEdgesOnEdge"].sum())
    s_eoc = float(f["nEdgesOnCell"].sum())
    stage = 36 * nE + 12 * s_eoe + 20 * nC + 4 * s_eoc + 64 * nV
    stage += L * (40 * (nC + nE) + 16 * (nV + nC))
    if T:
        if fct:
            s_adv = (float(fct_statics["nAdvCellsForEdge"].sum()) if fct_statics is not None
                     else 10.0 * nE)
            stage += 4 * nE + 20 * s_adv + 4 * s_eoc + 4 * nC
        if hmix:
            stage += 8 * nE
        stage += L * T * (40 * nC + (32 * nC + 16 * nE if fct else 0))
    return 4 * stage


def sw_kernels(d: Dims, fct=True, hmix=True, visc=True):
    """Per-launch (bytes, fp64 instructions) of the three sw stage kernels,
    averaged over the four RK stages."""
    nC, nE, nV, L, T = d.nC, d.nE, d.nV, d.L, d.T
    Ne, Na, Nc = d.maxEoE, d.maxAdv, d.avgEoC
    cl, el, vl = nC * L, nE * L, nV * L
    slot_c = Nc * nC  # ragged cell slots
    # ---- K1 edge pre-pass
    b1 = 8 * nE * 2 + 8 * cl + 8 * el + 8 * vl + 24 * el
    f1 = 4 * el  # h1 + h2, u hs, pv_a + pv_b, F Pv
    if T:
        b1 += 8 * cl * T + 8 * nE
        f1 += el
        if fct:
            # advCells + the one coefficient the flux sign selects (the {cp, cm} pair the kernel
            # loads is 8 B more per slot), hoMask, LO, A
            b1 += 12 * Na * nE + 4 * el + 16 * el * T
            # per tracer the stencil sum, LO and A (the centred flux of unmasked edges
            # sits behind a branch and is rare)
            f1 += el * T * (Na + 2)
        else:
            b1 += 8 * el * T
            f1 += el * (1 + 2 * T)
        if hmix:
            b1 += 8 * nE + 8 * el * T
            f1 += el * (1 + 2 * T)
    # ---- K2 edges + cells
    # TRiSK stencil (eoe, W/8), {F, F Pv} gathers, Pv, invDc, ke - nu div, h, dhs, coe; u update
    b2 = 12 * Ne * nE + 16 * el + 8 * el + 8 * nE + 8 * cl + 8 * cl + 8 * nE + 8 * nE
    b2 += 8 * el + 16 * el + 8 * el * 0.75
    f2 = el * (2 * Ne + 6 + 1.75)  # 2 per slot, q, thickness and kdiv differences, 2 FMA, update
    if visc:
        b2 += 8 * vl + 16 * nE  # vorticity gather, nu / dv, voe
        f2 += 2 * el
    b2 += 4 * nC + 12 * slot_c + 8 * nC + 8 * cl + 16 * cl + 8 * cl * 0.75
    f2 += cl * (Nc + 1.75)
    if T:
        b2 += 8 * slot_c
        if fct:
            b2 += 4 * slot_c + 8 * cl * T + 16 * el * T + 24 * cl * T
            # 1/hProv (5), dt/area, dt/(area hProv); per tracer 2 sums per edge (the upwind
            # sum, and flxIn or flxOut by the flux sign), trUp (3), numerators / denominators
            # (4); the two quotients are divided only strictly inside (0, 1), rarely (about
            # half an instruction per cell on average, from ncu's count)
            f2 += cl * (7 + T * (2 * Nc + 7 + 0.5))
        else:
            b2 += 8 * el * T + 8 * cl * T
            f2 += cl * T * Nc
    # ---- K3 cells + vertices
    b3 = 8 * nE + 8 * el + 8 * nC + 8 * cl  # kw, u_next, invArea, kdiv
    f3 = cl * (2 * Nc + 1)
    if visc:
        b3 += 8 * slot_c + 8 * nC  # sdv, nu / area
        f3 += cl * Nc
    if T:
        b3 += 4 * nC + 12 * slot_c + 8 * nE + 8 * cl * 2 + 8 * cl * T * 2 + 16 * cl * T + 8 * cl * T * 0.75
        if fct:
            b3 += 8 * el * T + 16 * cl * T
        if hmix:
            b3 += 8 * el * T
        # per slot: a r - DF contracts to one FMA, plus the accumulation
        f3 += cl * (4 + T * (Nc * (1 + int(fct)) + 4.75))
    b3 += 8 * nV * (3 + 1.5 + 3 + 1.5 + 3) + 8 * vl + 16 * vl
    f3 += vl * 13  # circulation and kite sums (6), vorticity, f A + circ, 1/hs (4), pv
    return {"sw_edge_pre": (b1, f1), "sw_tend": (b2, f2), "sw_final": (b3, f3)}


def ocean_kernels(d: Dims, fct=True, hmix=True):
    """Per-launch (bytes, fp64 instructions) of the three ocean stage kernels.
    They keep the reference's rounding (no contracted multiply-adds), so every
    stencil term is a multiply and an add."""
    nC, nE, L, T = d.nC, d.nE, d.L, d.T
    Na, Nc = d.maxAdv, d.avgEoC
    cl, el = nC * L, nE * L
    slot_c = Nc * nC
    b1 = 8 * nE + 8 * el * T  # coe, tr_in (two cells)
    f1 = 0
    if fct:
        # F, advCells + one coefficient pair per slot, hoMask, dv, LO, A
        b1 += 8 * el + 20 * Na * nE + 4 * el + 8 * nE + 16 * el * T
        # a weight per slot, per tracer a multiply and an add per slot, LO (2) and
        # A (1); the mask weight is a select, the centred flux of unmasked edges rare
        f1 += el * (Na + T * (2 * Na + 3))
    if hmix:
        b1 += 8 * nE + 8 * el + 8 * el * T  # rho, hE, DF
        f1 += el * 3 * T
    b2 = 4 * nC + 12 * slot_c + 8 * nC + 8 * cl * 2 + 4 * slot_c + 8 * slot_c + 8 * cl * T
    b2 += 16 * el * T + 24 * cl * T
    # per slot and tracer: LO and A scaled by 1/area and summed (4); trUp (4), the
    # new max / min (6), numerators and denominators (6); the two quotients are
    # divided only strictly inside (0, 1), rarely (~1 instruction per cell-level
    # and tracer on average, from ncu's DFMA count)
    f2 = cl * T * (4 * Nc + 16 + 1) if fct else 0
    b3 = 4 * nC + 12 * slot_c + 8 * nC + 16 * cl * T + 8 * cl * T * 3 + 16 * cl * T
    b3 += 8 * el * T * (int(fct) + int(hmix))
    # per slot and tracer: the limited flux, its 1/area scaling and sum (3), the
    # del2 term (2); step_tracers_forward (4)
    f3 = cl * T * ((3 * Nc if fct else 0) + (2 * Nc if hmix else 0) + 4)
    return {"oc_edges": (b1, f1), "oc_cells": (b2, f2), "oc_final": (b3, f3)}


def per_step(kernels):
    """Bytes and FP64 instructions of one RK4 step (four stages)."""
    return (4 * sum(b for b, _ in kernels.values()), 4 * sum(f for _, f in kernels.values()))
