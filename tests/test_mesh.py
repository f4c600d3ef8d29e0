"""Mesh generation and the reference's connectivity semantics (CPU)."""
import numpy as np
import pytest

import mpaso


@pytest.fixture(scope="module")
def hexmesh():
    return mpaso.Mesh.hex(16, 12, 10e3)


@pytest.fixture(scope="module")
def sphere():
    return mpaso.Mesh.icosa(3)


def test_counts():
    for lev, nc in [(0, 12), (2, 162), (5, 10242)]:
        m = mpaso.Mesh.icosa(lev)
        assert (m.nCells, m.nEdges, m.nVertices) == (nc, 3 * (nc - 2), 2 * (nc - 2))
    h = mpaso.Mesh.hex(64, 64, 10e3)
    assert (h.nCells, h.nEdges, h.nVertices) == (4096, 12288, 8192)


def test_areas_close(sphere, hexmesh):
    f = sphere.fields
    total = 4 * np.pi * sphere.radius ** 2
    assert abs(f["areaCell"].sum() / total - 1) < 1e-12
    assert abs(f["areaTriangle"].sum() / total - 1) < 1e-12
    assert np.allclose(f["kiteAreasOnVertex"].sum(1), f["areaTriangle"], rtol=1e-13)
    g = hexmesh.fields
    assert abs(g["areaCell"].sum() / (hexmesh.Lx * hexmesh.Ly) - 1) < 1e-12


def test_orientation_conventions(sphere):
    f = sphere.fields
    coe = f["cellsOnEdge"] - 1
    assert np.all(coe[:, 0] < coe[:, 1])  # c1 < c2 so the transposed e2c keeps file orientation
    cov = f["cellsOnVertex"]
    assert np.all(np.diff(cov, axis=1) > 0)  # sorted, as the reference's v2c pairing assumes
    # cellsOnCell[j] lies across edgesOnCell[j]
    eoc, coc, n = f["edgesOnCell"] - 1, f["cellsOnCell"] - 1, f["nEdgesOnCell"]
    for c in range(0, sphere.nCells, 37):
        for j in range(n[c]):
            assert set(coe[eoc[c, j]]) == {c, coc[c, j]}


def _trisk_tangential(m, u):
    f = m.fields
    eoe, W, ne = f["edgesOnEdge"] - 1, f["weightsOnEdge"], f["nEdgesOnEdge"]
    mask = np.arange(16)[None, :] < ne[:, None]
    return (W * np.where(mask, u[np.maximum(eoe, 0)], 0.0)).sum(1)


def test_trisk_uniform_flow_on_hex(hexmesh):
    f = hexmesh.fields
    ang = f["angleEdge"]
    U = np.array([0.7, -0.3])
    u = np.cos(ang) * U[0] + np.sin(ang) * U[1]
    ut = -np.sin(ang) * U[0] + np.cos(ang) * U[1]
    assert np.abs(_trisk_tangential(hexmesh, u) - ut).max() < 1e-13


def test_trisk_antisymmetry(sphere):
    f = sphere.fields
    eoe, W, ne = f["edgesOnEdge"] - 1, f["weightsOnEdge"], f["nEdgesOnEdge"]
    dc, dv = f["dcEdge"], f["dvEdge"]
    worst = 0.0
    for e in range(0, sphere.nEdges, 7):
        for j in range(ne[e]):
            ep = eoe[e, j]
            jj = list(eoe[ep, :ne[ep]]).index(e)
            worst = max(worst, abs(dc[e] * dv[e] * W[e, j] + dc[ep] * dv[ep] * W[ep, jj]) / (dc[e] * dv[e]))
    assert worst < 1e-14


def test_crs_semantics(sphere):
    crs = sphere.crs()
    off, idx = crs["e2c"]
    assert np.all(np.diff(off) == 2)
    assert np.all(idx[0::2] < idx[1::2])  # transposition yields ascending ids
    off, idx = crs["v2c"]
    assert np.all(np.diff(idx.reshape(-1, 3), axis=1) > 0)
    off, idx = crs["c2e"]
    f = sphere.fields
    assert np.array_equal(idx[off[5]:off[6]], f["edgesOnCell"][5, :f["nEdgesOnCell"][5]] - 1)


def test_sfc_reorder_is_permutation(sphere):
    r, (pc, pe, pv) = sphere.reordered()
    for p, n in ((pc, sphere.nCells), (pe, sphere.nEdges), (pv, sphere.nVertices)):
        assert np.array_equal(np.sort(p), np.arange(n))
    f, g = sphere.fields, r.fields
    assert np.array_equal(g["xCell"], f["xCell"][pc])
    assert np.allclose(g["areaCell"], f["areaCell"][pc], rtol=1e-13)


def test_crs_is_cached_until_a_connectivity_array_is_replaced():
    """Mesh.crs() is built once and shared; replacing one of the file's
    connectivity arrays rebuilds it from the new array."""
    m = mpaso.Mesh.icosa(2)
    a = m.crs()
    assert m.crs() is a
    coc = m.fields["cellsOnCell"].copy()
    coc[0, [0, 1]] = coc[0, [1, 0]]  # swap two neighbours of cell 0
    m.fields["cellsOnCell"] = coc
    b = m.crs()
    assert b is not a
    off, idx = b["c2c"]
    assert np.array_equal(idx[off[0]:off[0] + 2], a["c2c"][1][[1, 0]])
    assert np.array_equal(b["e2e"][1], a["e2e"][1])
