"""FCT / del2 static setup on the GPU (mpaso_fct_setup_device) against the host
setup, which equals the reference's init_functions.cc output bit for bit on
the sphere: integer outputs identical; coefficients closer to the host's than
the host's own move under a one-ulp perturbation of the cell coordinates (the
reference's fit takes acos of dot products of nearly parallel unit vectors,
so on the sphere a last-place change of an input moves derivTwo by ~1e-6 of
its scale, and CUDA's acos / sin / cos differ from the C library's in the last
place); and the same RK4 trajectory to rounding when a state runs on either
set."""
import types

import numpy as np
import pytest

import mpaso
from mpaso.setup import fct_statics

pytestmark = pytest.mark.gpu

INTS = ("maxLevelEdgeTop", "nAdvCellsForEdge", "advCellsForEdge", "highOrderAdvMask", "edgeSignOnCell",
        "meshScalingDel2")
FLOATS = ("derivTwo", "advCoef", "advCoef_3rd")


def meshes():
    return [("icosa3", mpaso.Mesh.icosa(3)), ("icosa5", mpaso.Mesh.icosa(5)),
            ("hex32", mpaso.Mesh.hex(32, 32, 10e3, 1e-4)), ("hex48x40", mpaso.Mesh.hex(48, 40, 25e3, 1e-4))]


def ulp_sensitivity(mesh, L):
    """How far the host setup's coefficients move (relative to their scale)
    when every cell coordinate is perturbed by at most one ulp."""
    rng = np.random.default_rng(0)
    f = dict(mesh.fields)
    for k in ("xCell", "yCell", "zCell"):
        f[k] = f[k] * (1 + rng.choice([-1, 0, 1], f[k].shape) * 2.0 ** -52)
    fake = types.SimpleNamespace(crs=mesh.crs, fields=f, nCells=mesh.nCells, nEdges=mesh.nEdges,
                                 nVertices=mesh.nVertices, on_sphere=mesh.on_sphere,
                                 Lx=getattr(mesh, "Lx", 0.0), Ly=getattr(mesh, "Ly", 0.0))
    h, p = fct_statics(mesh, L), fct_statics(fake, L)
    return {k: np.abs(h[k] - p[k]).max() / np.abs(h[k]).max() for k in FLOATS}


@pytest.mark.parametrize("i", range(4))
def test_device_setup_matches_host(i):
    name, mesh = meshes()[i]
    L = 3
    rng = np.random.default_rng(i)
    mlc = rng.integers(1, L + 1, mesh.nCells).astype(np.int32)
    bc = (rng.uniform(size=(mesh.nCells, L)) < 0.05).astype(np.int32)
    bar = ulp_sensitivity(mesh, L)
    for kw in (dict(), dict(maxLevelCell=mlc, boundaryCell=bc)):
        h = fct_statics(mesh, L, **kw)
        d = fct_statics(mesh, L, device=0, **kw)
        for k in INTS:
            assert np.array_equal(h[k], d[k]), (name, k)
        for k in FLOATS:
            rel = np.abs(h[k] - d[k]).max() / np.abs(h[k]).max()
            assert rel <= max(bar[k], 1e-14), (name, k, rel, bar[k])


def test_batched_device_setup_matches_one_at_a_time():
    """mpaso_fct_setup_device_many over sphere and plane members gives each
    member exactly what the single-mesh device call gives it."""
    from mpaso.setup import fct_statics_many
    ms = [m for _, m in meshes()] + [mpaso.Mesh.icosa(2)]
    many = fct_statics_many(ms, 2, device=0)
    for m, got in zip(ms, many):
        one = fct_statics(m, 2, device=0)
        for k in INTS + FLOATS:
            assert np.array_equal(one[k], got[k]), k


def test_device_setup_gives_the_same_trajectory():
    import mpaso.gpu as G
    from mpaso.initial import sw_state
    mesh = mpaso.Mesh.icosa(4)
    h0, u0, tr0 = sw_state(mesh, 3, 1, 1)
    out = []
    for dev in (None, 0):
        f = fct_statics(mesh, 1, device=dev)
        st = G.State(G.DeviceMesh(mesh, fct=f), nlev=1, ntr=1, fct=True, hmix=True, kappa=1e4, nu=1e4)
        st.set(G.FIELD_H, h0), st.set(G.FIELD_U, u0), st.set(G.FIELD_TRACERS, tr0)
        st.step(90.0, 20)
        out.append([st.get(x) for x in (G.FIELD_H, G.FIELD_U, G.FIELD_TRACERS)])
    for a, b in zip(*out):
        assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()


def test_device_setup_rejects_bad_indices_on_the_host():
    """An out-of-range neighbour index is caught before any device work."""
    from mpaso._lib import MpasoError
    mesh = mpaso.Mesh.icosa(2)
    crs = mesh.crs()
    off, idx = crs["c2c"]
    idx = idx.copy()
    idx[7] = mesh.nCells + 5
    bad = dict(crs, c2c=(off, idx))
    fake = types.SimpleNamespace(crs=lambda: bad, fields=mesh.fields, nCells=mesh.nCells, nEdges=mesh.nEdges,
                                 nVertices=mesh.nVertices, on_sphere=mesh.on_sphere)
    with pytest.raises(MpasoError, match="cell index out of range"):
        fct_statics(fake, 1, device=0)
