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
- `del2_mode`: a divergence-free planar Fourier mode u = curl(A sin(2 pi x /
  Lx)) on an f = 0 doubly periodic mesh with uniform h, whose only dynamics at
  small amplitude is viscous decay exp(-nu k^2 t) (k = 2 pi / Lx): the known
  answer for the del2 momentum term, which the reference does not have.
"""
import numpy as np

from .mesh import EARTH_RADIUS


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
