"""Product-side FCT / del2 static setup (CPU): bit-identical to the reference
on the sphere (apps/ocean/tasks/init_functions.cc), exact for quadratics on the
periodic plane (a branch the reference does not have)."""
import numpy as np
import pytest

import mpaso
from helpers import Golden
from mpaso.setup import fct_statics
from oracle import Oracle


@pytest.mark.parametrize("name", ["sw_fct_icosa3_L1T1", "ocean_icosa3_L3T2", "sw_fct_icosa2_L5T5"])
def test_sphere_statics_equal_reference(name):
    g = Golden(name)
    out = fct_statics(g.mesh, g.L)
    for k, v in g.fct.items():
        assert np.array_equal(out[k], v), k


def test_sphere_statics_equal_oracle_level4_with_boundaries():
    mesh = mpaso.Mesh.icosa(4)
    rng = np.random.default_rng(0)
    bc = (rng.random((mesh.nCells, 2)) < 0.05).astype(np.int32)
    a = fct_statics(mesh, 2, boundaryCell=bc)
    b = Oracle("restatement").fct_statics(mesh, 2, boundaryCell=bc)
    for k in b:
        assert np.array_equal(a[k], b[k]), k
    assert (a["highOrderAdvMask"] == 0).any()


def test_planar_second_derivative_exact_for_quadratics():
    m = mpaso.Mesh.hex(12, 10, 5e3)
    s = fct_statics(m, 1)
    f = m.fields
    coe, coc, eoc = f["cellsOnEdge"] - 1, f["cellsOnCell"] - 1, f["edgesOnCell"] - 1
    voe = f["verticesOnEdge"] - 1
    wrap = lambda d, L: d - L * np.round(d / L)  # noqa: E731
    a, b, c = 0.3, -1.1, 0.7  # f = a x^2 + b x y + c y^2 around each cell
    for cell in range(0, m.nCells, 7):
        for j in range(f["nEdgesOnCell"][cell]):
            e = eoc[cell, j]
            side = 0 if coe[e, 0] == cell else 1
            pts = [cell] + list(coc[cell, :f["nEdgesOnCell"][cell]])
            dx = np.array([wrap(f["xCell"][p] - f["xCell"][cell], m.Lx) for p in pts])
            dy = np.array([wrap(f["yCell"][p] - f["yCell"][cell], m.Ly) for p in pts])
            vals = a * dx ** 2 + b * dx * dy + c * dy ** 2
            got = (s["derivTwo"][e, :len(pts), side] * vals).sum()
            xm = 0.5 * sum(wrap(f["xVertex"][v] - f["xCell"][cell], m.Lx) for v in voe[e])
            ym = 0.5 * sum(wrap(f["yVertex"][v] - f["yCell"][cell], m.Ly) for v in voe[e])
            t = np.arctan2(ym, xm)
            exact = 2 * a * np.cos(t) ** 2 + 2 * b * np.cos(t) * np.sin(t) + 2 * c * np.sin(t) ** 2
            assert abs(got - exact) < 1e-9 * (abs(a) + abs(b) + abs(c))
    # advection coefficients of an edge sum to dv (consistency: a constant tracer gives F dv)
    n = s["nAdvCellsForEdge"]
    tot = np.array([s["advCoef"][e, :n[e]].sum() for e in range(m.nEdges)])
    assert np.allclose(tot, f["dvEdge"], rtol=1e-9)


def test_batched_device_setup_validates_members_on_the_host():
    """mpaso_fct_setup_device_many checks every member's offsets and indices
    before any device work, so a corrupted member is refused, by number, even
    on a host without a GPU."""
    import types

    import mpaso
    from mpaso._lib import MpasoError
    from mpaso.setup import fct_statics_many
    good = mpaso.Mesh.icosa(1)
    bad_src = mpaso.Mesh.icosa(1)
    crs = dict(bad_src.crs())
    off, idx = crs["c2c"]
    idx = idx.copy()
    idx[3] = bad_src.nCells + 1
    crs["c2c"] = (off, idx)
    bad = types.SimpleNamespace(crs=lambda: crs, fields=bad_src.fields, nCells=bad_src.nCells,
                                nEdges=bad_src.nEdges, nVertices=bad_src.nVertices, on_sphere=True)
    with pytest.raises(MpasoError, match="member 1: cell index out of range"):
        fct_statics_many([good, bad], 1, device=0)
