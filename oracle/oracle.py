"""TEST INFRASTRUCTURE ONLY: ctypes binding of the CPU oracle (oracle.h).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  `Oracle("restatement")` loads the plain-C restatement;
`Oracle("ref", L, T)` loads the reference's own task sources built through
the header shim (present only where the reference checkout was available).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MAXE, MAXE2 = 8, 16
CNX = ["c2v", "c2e", "c2c", "e2v", "e2e", "v2c", "e2c", "v2e"]

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_lp = ctypes.POINTER(ctypes.c_int64)


class OrcMesh(ctypes.Structure):
    _fields_ = [("nC", ctypes.c_int64), ("nE", ctypes.c_int64), ("nV", ctypes.c_int64),
                ("off", _lp * 8), ("idx", _ip * 8)]


class OrcStatic(ctypes.Structure):
    _fields_ = [(n, _dp) for n in ("areaCell", "dvEdge", "dcEdge", "areaTriangle",
                                   "kiteAreasOnVertex", "fVertex", "weightsOnEdge", "bottomDepth")] + \
               [(n, _ip) for n in ("maxLevelCell", "maxLevelEdgeTop", "nAdvCellsForEdge",
                                   "advCellsForEdge", "highOrderAdvMask")] + \
               [(n, _dp) for n in ("edgeSignOnCell", "advCoef", "advCoef_3rd", "meshScalingDel2")]


class OrcConfig(ctypes.Structure):
    _fields_ = [("nlev", ctypes.c_int32), ("ntr", ctypes.c_int32), ("gravity", ctypes.c_double),
                ("fct", ctypes.c_int32), ("hmix", ctypes.c_int32), ("kappa", ctypes.c_double),
                ("nu", ctypes.c_double), ("pin_u", ctypes.c_int32)]


class OrcGeom(ctypes.Structure):
    _fields_ = [(n, _dp) for n in ("angleEdge", "dcEdge", "dvEdge", "xCell", "yCell", "zCell",
                                   "xVertex", "yVertex", "zVertex", "meshDensity")] + \
               [("maxLevelCell", _ip), ("boundaryCell", _ip)]


class OrcSetupOut(ctypes.Structure):
    _fields_ = [(n, _ip) for n in ("maxLevelEdgeTop", "nAdvCellsForEdge", "advCellsForEdge",
                                   "highOrderAdvMask")] + \
               [(n, _dp) for n in ("meshScalingDel2", "edgeSignOnCell", "derivTwo", "advCoef",
                                   "advCoef_3rd")]


def _ptr(a):
    if a is None:
        return None
    if a.dtype == np.float64:
        return a.ctypes.data_as(_dp)
    if a.dtype == np.int32:
        return a.ctypes.data_as(_ip)
    if a.dtype == np.int64:
        return a.ctypes.data_as(_lp)
    raise TypeError(a.dtype)


def lib_path(kind, L=None, T=None):
    if kind == "restatement":
        return os.path.join(HERE, "_build", "liboracle.so")
    return os.path.join(HERE, "_ref", f"libref_L{L}_T{T}.so")


def ref_available(L, T):
    return os.path.exists(lib_path("ref", L, T))


class Oracle:
    def __init__(self, kind="restatement", L=None, T=None):
        path = lib_path(kind, L, T)
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library {path} not built (python oracle/build.py)")
        self.kind = kind
        self.lib = ctypes.CDLL(path)
        self.lib.orc_last_error.restype = ctypes.c_char_p
        self._keep = []

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("oracle: " + self.lib.orc_last_error().decode())

    # ---- argument structs ----
    def mesh(self, mesh):
        crs = mesh.crs()
        m = OrcMesh(mesh.nCells, mesh.nEdges, mesh.nVertices)
        keep = []
        for k, name in enumerate(CNX):
            off, idx = crs[name]
            off = np.ascontiguousarray(off, np.int64)
            idx = np.ascontiguousarray(idx, np.int32)
            keep += [off, idx]
            m.off[k] = _ptr(off)
            m.idx[k] = _ptr(idx)
        m._keep = keep
        return m

    @staticmethod
    def static(mesh, fct=None, bottomDepth=None):
        f = mesh.fields
        arrays = {n: np.ascontiguousarray(f[n], np.float64) for n in
                  ("areaCell", "dvEdge", "dcEdge", "areaTriangle", "kiteAreasOnVertex", "fVertex",
                   "weightsOnEdge")}
        arrays["bottomDepth"] = (np.zeros(mesh.nCells) if bottomDepth is None
                                 else np.ascontiguousarray(bottomDepth, np.float64))
        if fct is not None:
            for n in ("maxLevelCell", "maxLevelEdgeTop", "nAdvCellsForEdge", "advCellsForEdge",
                      "highOrderAdvMask"):
                arrays[n] = np.ascontiguousarray(fct[n], np.int32)
            for n in ("edgeSignOnCell", "advCoef", "advCoef_3rd", "meshScalingDel2"):
                arrays[n] = np.ascontiguousarray(fct[n], np.float64)
        s = OrcStatic(**{k: _ptr(v) for k, v in arrays.items()})
        s._keep = arrays
        return s

    @staticmethod
    def config(L, T, gravity=9.80616, fct=False, hmix=False, kappa=0.0, nu=0.0, pin_u=False):
        return OrcConfig(L, T, gravity, int(fct), int(hmix), kappa, nu, int(pin_u))

    # ---- static setup ----
    def fct_statics(self, mesh, L, maxLevelCell=None, boundaryCell=None, cfg=None):
        f = mesh.fields
        nC, nE = mesh.nCells, mesh.nEdges
        mlc = (np.full(nC, L, np.int32) if maxLevelCell is None
               else np.ascontiguousarray(maxLevelCell, np.int32))
        bc = (np.zeros((nC, L), np.int32) if boundaryCell is None
              else np.ascontiguousarray(boundaryCell, np.int32))
        geom_arrays = {n: np.ascontiguousarray(f[n], np.float64) for n in
                       ("angleEdge", "dcEdge", "dvEdge", "xCell", "yCell", "zCell", "xVertex",
                        "yVertex", "zVertex", "meshDensity")}
        g = OrcGeom(**{k: _ptr(v) for k, v in geom_arrays.items()}, maxLevelCell=_ptr(mlc),
                    boundaryCell=_ptr(bc))
        out = {
            "maxLevelEdgeTop": np.zeros(nE, np.int32),
            "nAdvCellsForEdge": np.zeros(nE, np.int32),
            "advCellsForEdge": np.zeros((nE, MAXE2), np.int32),
            "highOrderAdvMask": np.zeros((nE, L), np.int32),
            "meshScalingDel2": np.zeros(nE),
            "edgeSignOnCell": np.zeros((nC, MAXE)),
            "derivTwo": np.zeros((nE, MAXE2, 2)),
            "advCoef": np.zeros((nE, MAXE2)),
            "advCoef_3rd": np.zeros((nE, MAXE2)),
        }
        o = OrcSetupOut(**{k: _ptr(v) for k, v in out.items()})
        cfg = cfg or self.config(L, 1 if self.kind == "restatement" else self._compiled()[1])
        self._check(self.lib.orc_init_fct_statics(ctypes.byref(self.mesh(mesh)), ctypes.byref(cfg),
                                                   ctypes.byref(g), ctypes.byref(o)))
        out["maxLevelCell"] = mlc
        return out

    def _compiled(self):
        L = ctypes.c_int32()
        T = ctypes.c_int32()
        g = ctypes.c_double()
        self.lib.orc_compiled_levels(ctypes.byref(L), ctypes.byref(T), ctypes.byref(g))
        return L.value, T.value, g.value

    # ---- drivers ----
    def sw_run(self, mesh, static, cfg, dt, nsteps, h, u, tracers):
        h = np.ascontiguousarray(h, np.float64).copy()
        u = np.ascontiguousarray(u, np.float64).copy()
        tr = np.ascontiguousarray(tracers, np.float64).copy()
        om = mesh if isinstance(mesh, OrcMesh) else self.mesh(mesh)
        self._check(self.lib.orc_sw_run(ctypes.byref(om), ctypes.byref(static), ctypes.byref(cfg),
                                        ctypes.c_double(dt), ctypes.c_int32(nsteps), _ptr(h), _ptr(u),
                                        _ptr(tr)))
        return h, u, tr

    def ocean_run(self, mesh, static, cfg, dt, nsteps, h, hEdge, u, tracers):
        tr = np.ascontiguousarray(tracers, np.float64).copy()
        om = mesh if isinstance(mesh, OrcMesh) else self.mesh(mesh)
        args = [np.ascontiguousarray(a, np.float64) for a in (h, hEdge, u)]
        self._check(self.lib.orc_ocean_run(ctypes.byref(om), ctypes.byref(static), ctypes.byref(cfg),
                                           ctypes.c_double(dt), ctypes.c_int32(nsteps),
                                           *[_ptr(a) for a in args], _ptr(tr)))
        return tr

    def call(self, name, *args):
        """Calls orc_<name> with numpy arrays / structs / floats converted."""
        conv = []
        for a in args:
            if isinstance(a, np.ndarray):
                conv.append(_ptr(a))
            elif isinstance(a, ctypes.Structure):
                conv.append(ctypes.byref(a))
            elif isinstance(a, float):
                conv.append(ctypes.c_double(a))
            else:
                conv.append(a)
        self._check(getattr(self.lib, "orc_" + name)(*conv))


def cstep_path():
    return os.path.join(HERE, "_ref", "libref_cstep_L2.so")


def cstep_available():
    return os.path.exists(cstep_path())


class RefComplexStep:
    """Complex-step tangent of the reference's own sw RK4 step (ref_cstep.cc):
    the reference tasks evaluated on complex state, nu = 0, wind not pinned,
    passive zero tracers, levels fixed by the build (2)."""

    def __init__(self):
        if not cstep_available():
            raise FileNotFoundError(f"{cstep_path()} not built (python oracle/build.py)")
        self.lib = ctypes.CDLL(cstep_path())
        self.lib.orc_cstep_last_error.restype = ctypes.c_char_p
        L = ctypes.c_int32()
        self.lib.orc_cstep_levels(ctypes.byref(L))
        self.L = L.value
        self._o = Oracle("restatement")  # for the mesh / static argument structs

    def jvp(self, mesh, dt, nsteps, h, u, dh, du, eps=1e-30):
        """((h_N, u_N), (dh_N, du_N)) of nsteps steps from (h, u) along (dh, du)."""
        arrs = [np.ascontiguousarray(a, np.float64).copy() for a in (h, u, dh, du)]
        om, st = self._o.mesh(mesh), Oracle.static(mesh)
        rc = self.lib.orc_cstep_sw_run(ctypes.byref(om), ctypes.byref(st), ctypes.c_double(dt),
                                       ctypes.c_int32(nsteps), ctypes.c_double(eps), *[_ptr(a) for a in arrs])
        if rc != 0:
            raise RuntimeError("oracle: " + self.lib.orc_cstep_last_error().decode())
        return (arrs[0], arrs[1]), (arrs[2], arrs[3])
