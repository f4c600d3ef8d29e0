"""Ensembles of uneven meshes advanced together.

Members are independent, so their disjoint union is itself a valid MPAS mesh:
concatenating the datasets with index offsets gives one mesh context whose
kernels advance every member in the same launch (one graph-captured RK4 step
for the whole ensemble).  Each member is first regenerated in Hilbert order,
and the union keeps members contiguous (the context is built without global
renumbering), so every member keeps its own locality.

All members of one ensemble share dt, gravity and the diffusion
coefficients; the Coriolis parameter is mesh data, so f-plane and spherical
members mix freely.
"""
import numpy as np

from .mesh import Mesh
from .setup import fct_statics

_CELL_REFS = ("cellsOnCell", "cellsOnEdge", "cellsOnVertex")
_EDGE_REFS = ("edgesOnCell", "edgesOnEdge", "edgesOnVertex")
_VERT_REFS = ("verticesOnCell", "verticesOnEdge")


def union(meshes, fcts=None):
    """Disjoint union of meshes (and their FCT statics); returns (mesh, fct, offsets)
    with offsets[i] = (cell, edge, vertex) start of member i."""
    offs = [(0, 0, 0)]
    for m in meshes:
        c, e, v = offs[-1]
        offs.append((c + m.nCells, e + m.nEdges, v + m.nVertices))
    u = Mesh()
    u.nCells, u.nEdges, u.nVertices = offs[-1]
    u.on_sphere = all(m.on_sphere for m in meshes)
    u.radius, u.Lx, u.Ly = meshes[0].radius, 0.0, 0.0
    u.fields = {}
    for name in meshes[0].fields:
        parts = []
        for m, (c, e, v) in zip(meshes, offs[:-1]):
            a = m.fields[name]
            shift = c if name in _CELL_REFS else e if name in _EDGE_REFS else v if name in _VERT_REFS else None
            if shift is not None:
                a = np.where(a != 0, a + shift, 0).astype(np.int32)  # 1-based, 0 = unused slot
            parts.append(a)
        u.fields[name] = np.concatenate(parts)
    fct = None
    if fcts is not None:
        fct = {}
        for name in fcts[0]:
            parts = []
            for f, m, (c, e, v) in zip(fcts, meshes, offs[:-1]):
                a = f[name]
                if name == "advCellsForEdge":
                    n = f["nAdvCellsForEdge"]
                    a = np.where(np.arange(a.shape[1])[None, :] < n[:, None], a + c, 0).astype(np.int32)
                parts.append(a)
            fct[name] = np.concatenate(parts)
    return u, fct, np.array(offs, np.int64)


def build(specs, nlev=1, with_fct=True, return_member_fct=False):
    """specs: list of ("hex", nx, ny, dc, f0) or ("icosa", level).  Returns
    (union mesh, union FCT statics, offsets, member meshes[, member FCT statics])."""
    members = []
    for s in specs:
        m = Mesh.hex(s[1], s[2], s[3], s[4]) if s[0] == "hex" else Mesh.icosa(s[1])
        members.append(m.reordered()[0])
    fcts = [fct_statics(m, nlev) for m in members] if with_fct else None
    u, fct, offs = union(members, fcts)
    if return_member_fct:
        return u, fct, offs, members, fcts
    return u, fct, offs, members
