"""Analytic test cases and error norms of the sw app, as known answers.

- `sw_case1`: Williamson et al. (1992) case 1, a cosine bell advected by solid
  body rotation with a pinned wind (apps/sw/tasks/testcase.cc:37-80: u0 =
  2 pi a / 12 days, alpha = 0, h0 = 1000 m, bell of radius a/3 centred at
  (0, 3 pi / 2)); u is the rotational field of the streamfunction at
  vertices, as the reference builds it.
- `sw_case1_error`: the reference's normalised l2 error of h against the bell
  rotated by the elapsed time (apps/sw/tasks/solve.cc:404-436); its ctest
  (apps/sw/CMakeLists.txt:28-31, 5 steps of the default dt = 40 s on a
  240 km quasi-uniform sphere) requires <= 0.0015 (apps/sw/finalize.cc:24-25).
- `sw_case5`, `sw_case6`: Williamson cases 5 (zonal flow over an isolated
  mountain, with the reference's two cone tracers) and 6 (Rossby-Haurwitz wave
  of wavenumber 4), as apps/sw/tasks/testcase.cc:80-227 sets them up; the
  reference runs them as stability runs, and `sw_invariants` gives the
  discrete mass, tracer mass and energy whose conservation the tests check.
- `ocean_case`, `ocean_case_error`: the ocean app's three test cases
  (apps/ocean/tasks/testcase.cc:16-173) -- a Gaussian hill (1) and a slotted
  cylinder (2) carried once round the sphere in a day by solid-body rotation
  with unit thickness (FCT advection), and a spherical harmonic of degree 2
  (3) decaying under del2 mixing at exp(-6 kappa t / a^2) -- with their error
  norms (:175-294): the root of the summed squared pointwise relative errors
  over nCells, and the largest relative error.  (The reference's running
  maximum compares |error| with a signed value, so it can report a smaller
  one; the true maximum is returned here.)
- `del2_mode`: a divergence-free planar Fourier mode u = curl(A sin(2 pi x /
  Lx)) on an f = 0 doubly periodic mesh with uniform h, whose only dynamics at
  small amplitude is viscous decay exp(-nu k^2 t) (k = 2 pi / Lx): the known
  answer for the del2 momentum term, which the reference does not have.
"""
import numpy as np

from .mesh import EARTH_RADIUS, OMEGA

GRAVITY = 9.80616  # mpasoflecsi/common/constants.hh:30-31


def sphere_distance(lat1, lon1, lat2, lon2, radius):
    """Great-circle distance (haversine form, mpasoflecsi/eqns/metrics.hh:16-21)."""
    arg = np.sqrt(np.sin(0.5 * (lat2 - lat1)) ** 2 +
                  np.cos(lat1) * np.cos(lat2) * np.sin(0.5 * (lon2 - lon1)) ** 2)
    return 2 * radius * np.arcsin(arg)


def _bell(lat, lon, lon_c, a, h0=1000.0):
    r = sphere_distance(0.0, lon_c, lat, lon, a)
    return np.where(r < a / 3.0, (h0 / 2.0) * (1.0 + np.cos(np.pi * r * 3.0 / a)), h0 / 2.0)


def sw_case1(mesh, a=EARTH_RADIUS):
    """(h [nC][1], u [nE][1]) of test case 1 on a generated sphere."""
    f = mesh.fields
    u0 = 2.0 * np.pi * a / (12.0 * 86400.0)
    alpha = 0.0
    latv, lonv = f["latVertex"], f["lonVertex"]
    psi = -a * u0 * (np.sin(latv) * np.cos(alpha) - np.cos(lonv) * np.cos(latv) * np.sin(alpha))
    v = f["verticesOnEdge"] - 1
    u = -1.0 * (psi[v[:, 1]] - psi[v[:, 0]]) / f["dvEdge"]
    h = _bell(f["latCell"], f["lonCell"], 3.0 * np.pi / 2.0, a)
    return h[:, None].copy(), u[:, None].copy()


def sw_case1_error(mesh, h, elapsed, a=EARTH_RADIUS):
    """Normalised l2 error of h (level 0) against the rotated bell."""
    f = mesh.fields
    rot = 3 * np.pi / 2.0 + 2 * np.pi * (elapsed / 86400 / 12)
    lat, lon, area = f["latCell"], f["lonCell"], f["areaCell"]
    ht = _bell(lat, lon, rot, a)
    w = np.cos(lat) / area
    num = np.sum((np.asarray(h).reshape(mesh.nCells, -1)[:, 0] - ht) ** 2 * w) / (4 * np.pi)
    den = np.sum(ht ** 2 * w) / (4 * np.pi)
    return float(np.sqrt(num) / np.sqrt(den))


def _psi_to_u(mesh, psi_vertex):
    """Normal velocity of a streamfunction at vertices, as the reference builds it."""
    v = mesh.fields["verticesOnEdge"] - 1
    return -(psi_vertex[v[:, 1]] - psi_vertex[v[:, 0]]) / mesh.fields["dvEdge"]


def sw_case5(mesh, a=EARTH_RADIUS, omega=OMEGA, g=GRAVITY):
    """(h [nC][1], u [nE][1], h_s [nC], tracers [nC][1][2]) of Williamson case 5
    (apps/sw/tasks/testcase.cc:80-168): alpha = 0, so f keeps its usual form."""
    f = mesh.fields
    u0, gh0, hs0 = 20.0, 5960.0 * g, 2000.0
    theta_c, lambda_c, rr = np.pi / 6.0, 3.0 * np.pi / 2.0, np.pi / 9.0
    u = _psi_to_u(mesh, -a * u0 * np.sin(f["latVertex"]))
    lat, lon = f["latCell"], np.where(f["lonCell"] < 0, f["lonCell"] + 2.0 * np.pi, f["lonCell"])
    r = np.sqrt(np.minimum(rr ** 2, (lon - lambda_c) ** 2 + (lat - theta_c) ** 2))
    hs = hs0 * (1.0 - r / rr)
    r2 = np.sqrt(np.minimum(rr ** 2, (lon - lambda_c) ** 2 + (lat - theta_c - np.pi / 6.0) ** 2))
    tr = np.stack([1.0 - r / rr, 1.0 - r2 / rr], axis=1)[:, None, :]
    h = (gh0 - (a * omega * u0 + 0.5 * u0 ** 2) * np.sin(lat) ** 2) / g - hs
    return h[:, None].copy(), u[:, None].copy(), hs, np.ascontiguousarray(tr)


def sw_case6(mesh, a=EARTH_RADIUS, omega=OMEGA, g=GRAVITY):
    """(h [nC][1], u [nE][1]) of the Rossby-Haurwitz wave, Williamson case 6
    (apps/sw/tasks/testcase.cc:171-225)."""
    f = mesh.fields
    h0, w, K, R = 8000.0, 7.848e-6, 7.848e-6, 4.0
    latv, lonv = f["latVertex"], f["lonVertex"]
    psi = -a * a * w * np.sin(latv) + a * a * K * np.cos(latv) ** R * np.sin(latv) * np.cos(R * lonv)
    u = _psi_to_u(mesh, psi)
    th, lon = f["latCell"], f["lonCell"]
    c = np.cos(th)
    A = (0.5 * w * (2.0 * omega + w) * c ** 2 +
         0.25 * K ** 2 * c ** (2 * R) * ((R + 1.0) * c ** 2 + 2.0 * R ** 2 - R - 2.0 - 2.0 * R ** 2 * c ** -2))
    B = (2.0 * (omega + w) * K / ((R + 1.0) * (R + 2.0))) * c ** R * ((R ** 2 + 2.0 * R + 2.0) - ((R + 1.0) * c) ** 2)
    C = 0.25 * K ** 2 * c ** (2.0 * R) * ((R + 1.0) * c ** 2 - R - 2.0)
    h = (g * h0 + a * a * A + a * a * B * np.cos(R * lon) + a * a * C * np.cos(2.0 * R * lon)) / g
    return h[:, None].copy(), u[:, None].copy()


def sw_invariants(mesh, h, u, tracers=None, h_s=None, g=GRAVITY):
    """Discrete mass sum(A h), tracer masses sum(A h tr) and total energy
    sum_c A (h K + g h (h/2 + h_s)), K the cell kinetic energy of
    compute_solve_diagnostics (apps/sw/tasks/solve.cc:62-77), level 0."""
    f = mesh.fields
    A = f["areaCell"]
    hh = np.asarray(h).reshape(mesh.nCells, -1)[:, 0]
    uu = np.asarray(u).reshape(mesh.nEdges, -1)[:, 0]
    e = f["edgesOnCell"] - 1
    n = f["nEdgesOnCell"]
    valid = np.arange(e.shape[1])[None, :] < n[:, None]
    w = (0.25 * f["dcEdge"] * f["dvEdge"])[np.where(valid, e, 0)] * valid
    ke = (w * uu[np.where(valid, e, 0)] ** 2).sum(axis=1) / A
    hs = np.zeros(mesh.nCells) if h_s is None else np.asarray(h_s)
    out = {"mass": float((A * hh).sum()),
           "energy": float((A * (hh * ke + g * hh * (0.5 * hh + hs))).sum())}
    if tracers is not None:
        tr = np.asarray(tracers).reshape(mesh.nCells, -1, np.asarray(tracers).shape[-1])[:, 0, :]
        out["tracer_mass"] = (A[:, None] * hh[:, None] * tr).sum(axis=0)
    return out


def del2_mode(mesh, amp=1e-6, h0=1000.0):
    """(h, u, pattern, k^2) of the planar viscous-decay mode; `pattern` is u / amp."""
    f = mesh.fields
    k = 2 * np.pi / mesh.Lx
    psi = np.sin(k * f["xVertex"]) / k
    v = f["verticesOnEdge"] - 1
    pattern = -(psi[v[:, 1]] - psi[v[:, 0]]) / f["dvEdge"]
    u = amp * pattern
    h = np.full((mesh.nCells, 1), h0)
    return h, u[:, None].copy(), pattern, k * k


# ---------------------------------------------------------------- ocean app
_DAY = 86400.0


def ocean_rotation_velocity(mesh, a=EARTH_RADIUS):
    """Normal velocity of solid-body rotation with a one-day period
    (apps/ocean/tasks/testcase.cc:16-22): u0 cos(latEdge) cos(angleEdge)."""
    f = mesh.fields
    u0 = 2.0 * np.pi * a / _DAY
    return u0 * np.cos(f["latEdge"]) * np.cos(f["angleEdge"])


def _gaussian(x, a):
    maxg = 21983.7698959881  # :28-31
    return 50.0 + (20.0 / maxg) * np.exp(10.0 * x / a)


def _slotted_cylinder(x, y, z, lat, lon, a):
    """apps/ocean/tasks/testcase.cc:36-60 (arc length as mpasoflecsi/eqns/metrics.hh:75-90)."""
    r = np.sqrt(x * x + y * y + z * z)
    c = np.sqrt((a - x) ** 2 + y ** 2 + z ** 2)
    dist = r * 2.0 * np.arcsin(c / (2.0 * r))
    lon = np.where(lon > np.pi, lon - 2.0 * np.pi, lon)
    slot = (a * lat > -a / 3.0) & (a * lat < a / 2.0) & (a * np.abs(lon) < a / 12.0)
    return np.where(dist > a / 2.0, 50.0, np.where(slot, 50.0, 100.0))


def _harmonic(lat, lon, coef, t, a):
    """apps/ocean/tasks/testcase.cc:62-73."""
    return 50.0 + 20.0 * np.cos(lat) ** 2 * np.cos(2.0 * lon) * np.exp(-6.0 * coef * t / (a * a))


def ocean_case(mesh, case, coef=1e7, a=EARTH_RADIUS):
    """(h [nC][1], u [nE][1], tracers [nC][1][1]) of ocean test case 1, 2 or 3
    (setup_case_1/2/3, apps/ocean/tasks/testcase.cc:96-173); case 3 is at rest."""
    f = mesh.fields
    h = np.ones((mesh.nCells, 1))
    u = ocean_rotation_velocity(mesh, a)[:, None] if case in (1, 2) else np.zeros((mesh.nEdges, 1))
    if case == 1:
        tr = _gaussian(f["xCell"], a)
    elif case == 2:
        tr = _slotted_cylinder(f["xCell"], f["yCell"], f["zCell"], f["latCell"], f["lonCell"], a)
    elif case == 3:
        tr = _harmonic(f["latCell"], f["lonCell"], coef, 0.0, a)
    else:
        raise ValueError("ocean test cases are 1, 2 and 3")
    return h, u, np.ascontiguousarray(tr[:, None, None])


def ocean_case_exact(mesh, case, elapsed, coef=1e7, a=EARTH_RADIUS):
    """The analytic tracer of case 1, 2 or 3 after `elapsed` seconds
    (calc_error_case_1/2/3, apps/ocean/tasks/testcase.cc:175-294)."""
    f = mesh.fields
    rot = 2.0 * np.pi * elapsed / _DAY
    x, y = f["xCell"], f["yCell"]
    if case == 1:
        return _gaussian(x * np.cos(-rot) - y * np.sin(-rot), a)
    if case == 2:
        xp = x * np.cos(rot) + y * np.sin(rot)
        yp = -x * np.sin(rot) + y * np.cos(rot)
        return _slotted_cylinder(xp, yp, f["zCell"], f["latCell"], f["lonCell"] - rot, a)
    return _harmonic(f["latCell"], f["lonCell"], coef, elapsed, a)


def ocean_case_error(mesh, case, tracers, elapsed, coef=1e7, a=EARTH_RADIUS):
    """(l2, max) of the pointwise relative error of tracer 0, level 0, against the
    analytic solution: l2 = sqrt(sum err^2) / nCells as the reference reports it."""
    tr = np.asarray(tracers).reshape(mesh.nCells, -1)[:, 0]
    exact = ocean_case_exact(mesh, case, elapsed, coef, a)
    err = (tr - exact) / exact
    return float(np.sqrt(np.sum(err * err)) / mesh.nCells), float(np.abs(err).max())
