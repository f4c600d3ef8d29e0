"""Seeded synthetic initial states for the benchmark configurations.

The reference initialises its states from analytic test cases
(apps/sw/tasks/testcase.cc:37-227, apps/ocean/tasks/testcase.cc:96-173);
its mesh files are not available, so these generators build comparable
smooth seeded states on the generated meshes:

- sphere: random combinations of monomials x^a y^b z^c (a+b+c <= degree) on the
  unit sphere, which span the spherical harmonics up to that degree;
- plane: sums of periodic Gaussian bumps.

Velocity is the rotational field of a streamfunction psi sampled at vertices,
u = -(psi(v2) - psi(v1)) / dvEdge, the construction of
apps/sw/tasks/testcase.cc:61-66.
"""
import numpy as np

from .mesh import EARTH_RADIUS


def splitmix64(x):
    """SplitMix64 step (Steele, Lea & Flood 2014): derives per-member seeds."""
    x = (x + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = x
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return z ^ (z >> 31)


def _sphere_field(rng, xyz, degree):
    """Random smooth field on the unit sphere: polynomial of the given degree."""
    x, y, z = xyz
    px, py, pz = [np.ones_like(x)], [np.ones_like(x)], [np.ones_like(x)]
    for _ in range(degree):
        px.append(px[-1] * x), py.append(py[-1] * y), pz.append(pz[-1] * z)
    out = np.zeros_like(x)
    for a in range(degree + 1):
        for b in range(degree + 1 - a):
            xy = px[a] * py[b]
            for c in range(degree + 1 - a - b):
                out += rng.standard_normal() * (xy * pz[c])
    return out


def _plane_field(rng, xy, Lx, Ly, nbumps, rmin, rmax):
    x, y = xy
    out = np.zeros_like(x)
    for _ in range(nbumps):
        cx, cy = rng.uniform(0, Lx), rng.uniform(0, Ly)
        r = rng.uniform(rmin, rmax)
        dx = (x - cx + Lx / 2) % Lx - Lx / 2
        dy = (y - cy + Ly / 2) % Ly - Ly / 2
        out += rng.choice([-1.0, 1.0]) * np.exp(-(dx * dx + dy * dy) / (r * r))
    return out


def _unit_xyz(mesh, kind):
    f = mesh.fields
    p = np.stack([f["x" + kind], f["y" + kind], f["z" + kind]])
    return p / np.linalg.norm(p, axis=0)


def _velocity(mesh, psi_v):
    f = mesh.fields
    v = f["verticesOnEdge"] - 1
    return -(psi_v[v[:, 1]] - psi_v[v[:, 0]]) / f["dvEdge"]


def sw_state(mesh, seed, nlev=1, ntr=1, h0=None, h_amp=None, u_peak=None, degree=8):
    """Shallow-water state (h [nC][L], u [nE][L], tracers [nC][L][T]).

    Sphere defaults: h = 8000 m + degree-8 perturbation of max 100 m, u from a
    degree-8 streamfunction with peak 30 m/s, tracers in [0, 1].  Plane
    defaults: h = 1000 m + Gaussian bumps of 10 m (radius 50-200 km), peak u
    1 m/s.  Each level and tracer gets its own seeded field.
    """
    rng = np.random.default_rng(seed)
    nC, nE = mesh.nCells, mesh.nEdges
    h = np.empty((nC, nlev))
    u = np.empty((nE, nlev))
    tr = np.empty((nC, nlev, ntr))
    if mesh.on_sphere:
        h0 = 8000.0 if h0 is None else h0
        h_amp = 100.0 if h_amp is None else h_amp
        u_peak = 30.0 if u_peak is None else u_peak
        pc, pv = _unit_xyz(mesh, "Cell"), _unit_xyz(mesh, "Vertex")
        for k in range(nlev):
            p = _sphere_field(rng, pc, degree)
            h[:, k] = h0 + h_amp * p / np.abs(p).max()
            uu = _velocity(mesh, _sphere_field(rng, pv, degree))
            u[:, k] = u_peak * uu / np.abs(uu).max()
            for t in range(ntr):
                q = _sphere_field(rng, pc, degree)
                tr[:, k, t] = (q - q.min()) / (q.max() - q.min())
    else:
        h0 = 1000.0 if h0 is None else h0
        h_amp = 10.0 if h_amp is None else h_amp
        u_peak = 1.0 if u_peak is None else u_peak
        f = mesh.fields
        xy_c = (f["xCell"], f["yCell"])
        xy_v = (f["xVertex"], f["yVertex"])
        nb = 12
        for k in range(nlev):
            p = _plane_field(rng, xy_c, mesh.Lx, mesh.Ly, nb, 50e3, 200e3)
            h[:, k] = h0 + h_amp * p / max(np.abs(p).max(), 1e-300)
            uu = _velocity(mesh, _plane_field(rng, xy_v, mesh.Lx, mesh.Ly, nb, 50e3, 200e3))
            u[:, k] = u_peak * uu / max(np.abs(uu).max(), 1e-300)
            for t in range(ntr):
                q = _plane_field(rng, xy_c, mesh.Lx, mesh.Ly, nb, 50e3, 200e3)
                tr[:, k, t] = (q - q.min()) / max(q.max() - q.min(), 1e-300)
    return h, u, tr


def ocean_state(mesh, seed, nlev=60, ntr=3, layer_thickness=None, u_peak=0.3, degree=8, clip=True):
    """Multi-layer ocean tracer state for the FCT/del2 tracer app.

    Layer thickness: uniform per level (default 100 m); velocity per level from
    a seeded streamfunction (peak `u_peak` m/s, decaying with depth);
    tracers: temperature 0-30 C decreasing linearly with depth, salinity
    34-36 psu, passive tracer 0-1, each with seeded smooth noise.
    Temperature is clipped to [0, 30] (clip=True), which leaves plateaus at
    exactly 0 and 30 where the FCT limiter is ill-conditioned.
    Returns (h [nC][L], hEdge [nE][L], u [nE][L], tracers [nC][L][T]).
    """
    rng = np.random.default_rng(seed)
    nC, nE = mesh.nCells, mesh.nEdges
    dz = 100.0 if layer_thickness is None else layer_thickness
    h = np.full((nC, nlev), dz)
    hE = np.full((nE, nlev), dz)
    u = np.empty((nE, nlev))
    tr = np.empty((nC, nlev, ntr))
    if mesh.on_sphere:
        pc, pv = _unit_xyz(mesh, "Cell"), _unit_xyz(mesh, "Vertex")
        field_c = lambda: _sphere_field(rng, pc, degree)  # noqa: E731
        field_v = lambda: _sphere_field(rng, pv, degree)  # noqa: E731
    else:
        f = mesh.fields
        field_c = lambda: _plane_field(rng, (f["xCell"], f["yCell"]), mesh.Lx, mesh.Ly, 12, 50e3, 200e3)  # noqa
        field_v = lambda: _plane_field(rng, (f["xVertex"], f["yVertex"]), mesh.Lx, mesh.Ly, 12, 50e3, 200e3)  # noqa
    base_psi = field_v()
    for k in range(nlev):
        depth_frac = (k + 0.5) / nlev
        uu = _velocity(mesh, base_psi + 0.3 * field_v())
        u[:, k] = u_peak * (1.0 - 0.8 * depth_frac) * uu / np.abs(uu).max()
        n0 = field_c()
        n0 = n0 / np.abs(n0).max()
        tr[:, k, 0] = 30.0 * (1.0 - depth_frac) + 1.0 * n0 if ntr > 0 else 0
        if ntr > 1:
            n1 = field_c()
            tr[:, k, 1] = 35.0 + 0.9 * n1 / np.abs(n1).max()
        if ntr > 2:
            q = field_c()
            tr[:, k, 2] = (q - q.min()) / (q.max() - q.min())
        for t in range(3, ntr):
            q = field_c()
            tr[:, k, t] = (q - q.min()) / (q.max() - q.min())
    if ntr > 0 and clip:
        tr[:, :, 0] = np.clip(tr[:, :, 0], 0.0, 30.0)
    return h, hE, u, tr
