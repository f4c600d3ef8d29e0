"""FCT / del2 static coefficients (libmpaso's mpaso_fct_setup, or
mpaso_fct_setup_device on a GPU).

The setup of apps/ocean/tasks/init_functions.cc:18-447, bit-identical to the
reference on the sphere when run on the host; on a periodic plane it fits the
same polynomial in plane coordinates (the reference leaves that branch
empty).  On the GPU the integer outputs are identical and the coefficients
agree to the last-place differences of CUDA's trigonometric functions."""
import ctypes

import numpy as np

from ._lib import check, lib

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_lp = ctypes.POINTER(ctypes.c_int64)


class _In(ctypes.Structure):
    _fields_ = ([("nCells", ctypes.c_int64), ("nEdges", ctypes.c_int64), ("nVertices", ctypes.c_int64)]
                + [(n, _lp) for n in ("c2e_off", "c2c_off", "e2v_off")]
                + [(n, _ip) for n in ("c2e", "c2c", "e2v")]
                + [(n, _dp) for n in ("dcEdge", "dvEdge", "xCell", "yCell", "zCell", "xVertex",
                                      "yVertex", "zVertex", "meshDensity")]
                + [("on_sphere", ctypes.c_int32), ("Lx", ctypes.c_double), ("Ly", ctypes.c_double),
                   ("nlev", ctypes.c_int32), ("maxLevelCell", _ip), ("boundaryCell", _ip)])


class _Out(ctypes.Structure):
    _fields_ = [("maxLevelEdgeTop", _ip), ("meshScalingDel2", _dp), ("edgeSignOnCell", _dp),
                ("derivTwo", _dp), ("nAdvCellsForEdge", _ip), ("advCellsForEdge", _ip),
                ("highOrderAdvMask", _ip), ("advCoef", _dp), ("advCoef_3rd", _dp)]


def fct_statics(mesh, nlev, maxLevelCell=None, boundaryCell=None, device=None):
    """Returns the FCT statics as a dict of numpy arrays (reference layouts);
    device = a CUDA device index computes them on that GPU."""
    i, o, out, keep = _setup_args(mesh, nlev, maxLevelCell, boundaryCell)
    if device is None:
        check(lib().mpaso_fct_setup(ctypes.byref(i), ctypes.byref(o)))
    else:
        check(lib().mpaso_fct_setup_device(ctypes.byref(i), ctypes.byref(o), ctypes.c_int32(int(device))))
    return out


def fct_statics_many(meshes, nlev, device=0):
    """FCT statics of every mesh in one device call (mpaso_fct_setup_device_many)."""
    args = [_setup_args(m, nlev, None, None) for m in meshes]
    ins = (_In * len(args))(*[a[0] for a in args])
    outs = (_Out * len(args))(*[a[1] for a in args])
    check(lib().mpaso_fct_setup_device_many(ins, outs, ctypes.c_int32(len(args)), ctypes.c_int32(int(device))))
    return [a[2] for a in args]


def _setup_args(mesh, nlev, maxLevelCell, boundaryCell):
    crs = mesh.crs()
    f = mesh.fields
    nC, nE = mesh.nCells, mesh.nEdges
    keep = []

    def P(a, dtype, kind):
        a = np.ascontiguousarray(a, dtype)
        keep.append(a)
        return a.ctypes.data_as(kind)

    mlc = (np.full(nC, nlev, np.int32) if maxLevelCell is None
           else np.ascontiguousarray(maxLevelCell, np.int32))
    i = _In()
    i.nCells, i.nEdges, i.nVertices = nC, nE, mesh.nVertices
    for n in ("c2e", "c2c", "e2v"):
        setattr(i, n + "_off", P(crs[n][0], np.int64, _lp))
        setattr(i, n, P(crs[n][1], np.int32, _ip))
    for n in ("dcEdge", "dvEdge", "xCell", "yCell", "zCell", "xVertex", "yVertex", "zVertex", "meshDensity"):
        setattr(i, n, P(f[n], np.float64, _dp))
    i.on_sphere = 1 if mesh.on_sphere else 0
    i.Lx, i.Ly = (0.0, 0.0) if mesh.on_sphere else (mesh.Lx, mesh.Ly)
    i.nlev = nlev
    i.maxLevelCell = P(mlc, np.int32, _ip)
    if boundaryCell is not None:
        i.boundaryCell = P(boundaryCell, np.int32, _ip)
    out = {
        "maxLevelEdgeTop": np.zeros(nE, np.int32), "meshScalingDel2": np.zeros(nE),
        "edgeSignOnCell": np.zeros((nC, 8)), "derivTwo": np.zeros((nE, 16, 2)),
        "nAdvCellsForEdge": np.zeros(nE, np.int32), "advCellsForEdge": np.zeros((nE, 16), np.int32),
        "highOrderAdvMask": np.zeros((nE, nlev), np.int32), "advCoef": np.zeros((nE, 16)),
        "advCoef_3rd": np.zeros((nE, 16)),
    }
    o = _Out(**{k: v.ctypes.data_as(_dp if v.dtype == np.float64 else _ip) for k, v in out.items()})
    out["maxLevelCell"] = mlc
    return i, o, out, keep
