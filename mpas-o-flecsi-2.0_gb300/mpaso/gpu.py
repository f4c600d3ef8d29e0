"""ctypes binding of the device path (include/mpaso.h).

Arrays may be numpy arrays (host memory) or any object with `data_ptr()` /
`__cuda_array_interface__` pointing at device memory (e.g. torch CUDA
tensors); the library detects which.  All arrays use the reference's entity
numbering and per-entity AoS rows.
"""
import ctypes

import numpy as np

from ._lib import check, lib

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_lp = ctypes.POINTER(ctypes.c_int64)

CELLS, EDGES, VERTICES = 0, 1, 2
APP_SW, APP_OCEAN = 0, 1
FIELD_H, FIELD_U, FIELD_TRACERS, FIELD_LAYER_THICKNESS_EDGE = 0, 1, 2, 3
FIELD_VORTICITY, FIELD_PV_VERTEX = 4, 5  # sw diagnostics of the current state, read-only


class MeshDesc(ctypes.Structure):
    _fields_ = ([("nCells", ctypes.c_int64), ("nEdges", ctypes.c_int64), ("nVertices", ctypes.c_int64)]
                + [(n, _lp) for n in ("c2v_off", "c2e_off", "c2c_off", "e2v_off", "e2e_off")]
                + [(n, _ip) for n in ("c2v", "c2e", "c2c", "e2v", "e2e")]
                + [(n, _dp) for n in ("areaCell", "dvEdge", "dcEdge", "areaTriangle",
                                      "kiteAreasOnVertex", "fVertex", "weightsOnEdge", "bottomDepth",
                                      "xCell", "yCell", "zCell")]
                + [("reorder", ctypes.c_int32), ("fct_nlev", ctypes.c_int32)]
                + [(n, _ip) for n in ("maxLevelCell", "maxLevelEdgeTop", "nAdvCellsForEdge",
                                      "advCellsForEdge", "highOrderAdvMask")]
                + [(n, _dp) for n in ("edgeSignOnCell", "advCoef", "advCoef_3rd", "meshScalingDel2")])


class Geometry(ctypes.Structure):
    _fields_ = [(n, _dp) for n in ("latCell", "lonCell", "latVertex", "lonVertex", "latEdge", "lonEdge",
                                   "angleEdge", "xCell", "yCell", "zCell")]


class Params(ctypes.Structure):
    _fields_ = [("app", ctypes.c_int32), ("nlev", ctypes.c_int32), ("ntr", ctypes.c_int32),
                ("gravity", ctypes.c_double), ("fct", ctypes.c_int32), ("hmix", ctypes.c_int32),
                ("kappa", ctypes.c_double), ("nu", ctypes.c_double), ("pin_u", ctypes.c_int32)]


def _np_ptr(a, kind):
    return a.ctypes.data_as(kind)


def _ptr(a):
    """Raw address of a numpy array or a device tensor."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous")
        return ctypes.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):
        if hasattr(a, "is_contiguous") and not a.is_contiguous():
            raise ValueError("tensors must be contiguous")
        return ctypes.c_void_p(a.data_ptr())
    if hasattr(a, "__cuda_array_interface__"):
        return ctypes.c_void_p(a.__cuda_array_interface__["data"][0])
    raise TypeError(f"unsupported array type {type(a)}")


def device_count():
    n = ctypes.c_int32()
    check(lib().mpaso_device_count(ctypes.byref(n)))
    return n.value


def _mesh_desc(mesh, fct, bottomDepth, reorder, keep):
    """mpaso_mesh_desc of a generated mesh; the arrays it points at go into `keep`."""
    crs = mesh.crs()
    f = mesh.fields

    def arr(a, dtype):
        a = np.ascontiguousarray(a, dtype)
        keep.append(a)
        return _np_ptr(a, _dp if dtype == np.float64 else (_ip if dtype == np.int32 else _lp))

    d = MeshDesc()
    d.nCells, d.nEdges, d.nVertices = mesh.nCells, mesh.nEdges, mesh.nVertices
    for n in ("c2v", "c2e", "c2c", "e2v", "e2e"):
        off, idx = crs[n]
        setattr(d, n + "_off", arr(off, np.int64))
        setattr(d, n, arr(idx, np.int32))
    for n in ("areaCell", "dvEdge", "dcEdge", "areaTriangle", "kiteAreasOnVertex", "fVertex",
              "weightsOnEdge", "xCell", "yCell", "zCell"):
        setattr(d, n, arr(f[n], np.float64))
    if bottomDepth is not None:
        d.bottomDepth = arr(bottomDepth, np.float64)
    d.reorder = int(reorder)  # True -> 1 (Hilbert), False -> 0, or an explicit mode 0..3
    if fct is not None:
        d.fct_nlev = fct["highOrderAdvMask"].shape[1]
        for n in ("maxLevelCell", "maxLevelEdgeTop", "nAdvCellsForEdge", "advCellsForEdge",
                  "highOrderAdvMask"):
            setattr(d, n, arr(fct[n], np.int32))
        for n in ("edgeSignOnCell", "advCoef", "advCoef_3rd", "meshScalingDel2"):
            setattr(d, n, arr(fct[n], np.float64))
    return d


class DeviceMesh:
    """Device mesh context built from a generated mpaso.Mesh (reference semantics)."""

    def __init__(self, mesh, fct=None, bottomDepth=None, reorder=True, device=0):
        if mesh is None:  # filled in by a classmethod
            return
        keep = []
        d = _mesh_desc(mesh, fct, bottomDepth, reorder, keep)
        self._h = ctypes.c_void_p()
        check(lib().mpaso_mesh_create(ctypes.byref(d), int(device), ctypes.byref(self._h)))
        self.mesh = mesh
        self.nC, self.nE, self.nV = mesh.nCells, mesh.nEdges, mesh.nVertices

    @classmethod
    def ensemble(cls, meshes, fcts=None, bottomDepths=None, reorder=True, device=0):
        """One context over the disjoint union of the member meshes
        (mpaso_mesh_create_ensemble); fields are the members' concatenated."""
        keep = []
        descs = (MeshDesc * len(meshes))()
        for i, m in enumerate(meshes):
            descs[i] = _mesh_desc(m, None if fcts is None else fcts[i],
                                  None if bottomDepths is None else bottomDepths[i], reorder, keep)
        self = cls(None)
        self._h = ctypes.c_void_p()
        check(lib().mpaso_mesh_create_ensemble(descs, len(meshes), int(device), ctypes.byref(self._h)))
        self.mesh = None
        self.nC = sum(m.nCells for m in meshes)
        self.nE = sum(m.nEdges for m in meshes)
        self.nV = sum(m.nVertices for m in meshes)
        return self

    def members(self):
        """(n + 1, 3) int64: first cell, edge, vertex of each member, then the totals."""
        n = ctypes.c_int32()
        check(lib().mpaso_mesh_members(self._h, ctypes.byref(n), None))
        out = np.empty((n.value + 1, 3), np.int64)
        check(lib().mpaso_mesh_members(self._h, ctypes.byref(n), _np_ptr(out, _lp)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().mpaso_mesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def permutation(self, entity):
        n = (self.nC, self.nE, self.nV)[entity]
        out = np.empty(n, np.int32)
        check(lib().mpaso_mesh_permutation(self._h, int(entity), _np_ptr(out, _ip)))
        return out

    def set_gravity(self, g):
        check(lib().mpaso_mesh_set_gravity(self._h, ctypes.c_double(g)))

    def device_bytes(self):
        b = ctypes.c_int64()
        check(lib().mpaso_mesh_device_bytes(self._h, ctypes.byref(b)))
        return b.value

    def set_geometry(self, meshes):
        """Geometry of the device test cases (mpaso_mesh_set_geometry) from one
        mesh's fields, or from a list of members' (concatenated)."""
        ms = meshes if isinstance(meshes, (list, tuple)) else [meshes]
        names = ("latCell", "lonCell", "latVertex", "lonVertex", "latEdge", "lonEdge", "angleEdge",
                 "xCell", "yCell", "zCell")
        arrs = [np.ascontiguousarray(np.concatenate([m.fields[n] for m in ms]), np.float64) for n in names]
        g = Geometry(*[_np_ptr(a, _dp) for a in arrs])
        check(lib().mpaso_mesh_set_geometry(self._h, ctypes.byref(g)))

    # ---- per-task entries: return outputs as new numpy arrays ----
    def _call(self, name, *args):
        conv = [self._h]
        for a in args:
            if isinstance(a, float):
                conv.append(ctypes.c_double(a))
            elif isinstance(a, int):
                conv.append(ctypes.c_int32(a))
            else:
                conv.append(_ptr(a))
        conv.append(None)  # stream: the context's own
        check(getattr(lib(), "mpaso_" + name)(*conv))

    def sw_compute_solve_diagnostics(self, L, h, u, out=None):
        o = out or {k: np.zeros((n, L)) for k, n in (("h_edge", self.nE), ("h_vertex", self.nV),
                                                     ("circulation", self.nV), ("vorticity", self.nV),
                                                     ("ke", self.nC), ("pv_edge", self.nE),
                                                     ("pv_vertex", self.nV))}
        self._call("sw_compute_solve_diagnostics", L, h, u, o["h_edge"], o["h_vertex"],
                   o["circulation"], o["vorticity"], o["ke"], o["pv_edge"], o["pv_vertex"])
        return o

    def sw_compute_tend(self, L, h_edge, h, u, ke, pv_edge):
        th, tu = np.zeros((self.nC, L)), np.zeros((self.nE, L))
        self._call("sw_compute_tend", L, h_edge, h, u, ke, pv_edge, th, tu)
        return th, tu

    def sw_compute_scalar_tend(self, L, T, h_edge, u, tracers):
        out = np.zeros((self.nC, L, T))
        self._call("sw_compute_scalar_tend", L, T, h_edge, u, tracers, out)
        return out

    def call(self, name, *args):
        """Generic per-task call: mpaso_<name>(mesh, *args, stream=NULL)."""
        self._call(name, *args)


class State:
    """Device-resident state of the fused RK4 path."""

    def __init__(self, dmesh, app=APP_SW, nlev=1, ntr=1, gravity=9.80616, fct=False, hmix=False,
                 kappa=0.0, nu=0.0, pin_u=False):
        self.dmesh = dmesh
        self.L, self.T, self.app = nlev, ntr, app
        p = Params(app, nlev, ntr, gravity, int(fct), int(hmix), kappa, nu, int(pin_u))
        self._h = ctypes.c_void_p()
        check(lib().mpaso_state_create(dmesh.handle, ctypes.byref(p), ctypes.byref(self._h)))

    def close(self):
        if getattr(self, "_h", None):
            lib().mpaso_state_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _shape(self, field):
        dm = self.dmesh
        return {FIELD_H: (dm.nC, self.L), FIELD_U: (dm.nE, self.L),
                FIELD_TRACERS: (dm.nC, self.L, self.T),
                FIELD_LAYER_THICKNESS_EDGE: (dm.nE, self.L), FIELD_VORTICITY: (dm.nV, self.L),
                FIELD_PV_VERTEX: (dm.nV, self.L)}[field]

    def set(self, field, data):
        if isinstance(data, np.ndarray):
            data = np.ascontiguousarray(data, np.float64)
            if data.size != int(np.prod(self._shape(field))):
                raise ValueError("field size mismatch")
        check(lib().mpaso_state_set(self._h, int(field), _ptr(data)))

    def check_finite(self):
        """Raises MpasoError (MPASO_ERR_NUMERIC) naming the first NaN / infinity
        in h, u, the tracers or the ocean's edge thickness."""
        check(lib().mpaso_state_check_finite(self._h))

    def get(self, field, out=None):
        out = np.empty(self._shape(field)) if out is None else out
        check(lib().mpaso_state_get(self._h, int(field), _ptr(out)))
        return out

    def step(self, dt, nsteps=1):
        check(lib().mpaso_rk4_step(self._h, ctypes.c_double(dt), int(nsteps)))

    def step_graph(self, dt, nsteps=1):
        check(lib().mpaso_rk4_step_graph(self._h, ctypes.c_double(dt), int(nsteps)))

    def step_host(self, dt, nsteps, h, u, tracers):
        """One boundary call with host buffers (copied in and back out, in place)."""
        check(lib().mpaso_rk4_step_host(self._h, ctypes.c_double(dt), int(nsteps), _ptr(h), _ptr(u),
                                        _ptr(tracers)))

    def step_host_async(self, dt, nsteps, h, u, tracers):
        """The same exchange queued without waiting (page-locked buffers; read them after sync())."""
        check(lib().mpaso_rk4_step_host_async(self._h, ctypes.c_double(dt), int(nsteps), _ptr(h), _ptr(u),
                                              _ptr(tracers)))

    def sync(self):
        check(lib().mpaso_state_sync(self._h))

    def snapshot(self, field, out):
        """Asynchronous copy of a field into `out` (page-locked for overlap); valid after
        snapshot_wait()."""
        check(lib().mpaso_state_snapshot(self._h, int(field), _ptr(out)))
        return out

    def snapshot_wait(self):
        check(lib().mpaso_state_snapshot_wait(self._h))

    def stream(self):
        s = ctypes.c_void_p()
        check(lib().mpaso_state_stream(self._h, ctypes.byref(s)))
        return s.value

    def step_persistent(self, dt, nsteps, spin_limit=0, extra_arrivals=0):
        """nsteps RK4 steps in one persistent launch (mpaso_rk4_step_persistent)."""
        check(lib().mpaso_rk4_step_persistent(self._h, ctypes.c_double(dt), int(nsteps),
                                              ctypes.c_int64(spin_limit), int(extra_arrivals)))

    def setup_case(self, case, coef=0.0):
        """The reference test case's initial fields, written on the device
        (mpaso_state_setup_case; the mesh needs set_geometry first)."""
        check(lib().mpaso_state_setup_case(self._h, int(case), ctypes.c_double(coef)))

    def case_error(self, case, elapsed, coef=0.0):
        """(reference norm, largest pointwise relative error) of the state
        against the case's analytic solution (mpaso_state_case_error)."""
        err = (ctypes.c_double * 2)()
        check(lib().mpaso_state_case_error(self._h, int(case), ctypes.c_double(elapsed), ctypes.c_double(coef),
                                           err))
        return float(err[0]), float(err[1])

    def profile(self, dt, nsteps):
        """Mean ms per launch of each stage kernel kind: dict name -> ms."""
        ms = (ctypes.c_double * 8)()
        n = ctypes.c_int32()
        names = ctypes.create_string_buffer(256)
        check(lib().mpaso_state_profile(self._h, ctypes.c_double(dt), int(nsteps), ms, ctypes.byref(n),
                                        names, 256))
        return dict(zip(names.value.decode().split(","), list(ms)[:n.value]))

    # ---- launch configuration of the three stage kernels ----
    @staticmethod
    def _cfg_dict(c):
        return {"unroll": [int(x) for x in c[:3]], "threads": [int(x) for x in c[3:6]],
                "capped": [int(x) for x in c[6:9]], "l2": int(c[9]), "overlap": int(c[10]),
                "split": int(c[11]), "lanes": int(c[12])}

    def launch_config(self):
        """{'unroll', 'threads', 'capped'}: one value per stage kernel; 'l2': the
        static array kept resident in L2 (0 none, 1 advection coefficients, 2 TRiSK weights);
        'overlap': programmatic dependent launch between stage kernels; 'split': the
        four-launch schedule (sw with tracers); 'lanes': threads per edge-level of the
        TRiSK loop (1, 2 or 4)."""
        c = (ctypes.c_int32 * 13)()
        check(lib().mpaso_state_launch_config_ex(self._h, c, 13))
        return self._cfg_dict(c)

    def set_launch_config(self, unroll, threads, capped=(0, 0, 0), l2=0, overlap=0, split=0, lanes=1):
        c = (ctypes.c_int32 * 13)(*[int(x) for x in list(unroll) + list(threads) + list(capped) +
                                    [l2, overlap, split, lanes]])
        check(lib().mpaso_state_set_launch_config_ex(self._h, c, 13))

    def autotune(self, dt, nsteps=3):
        """Times every launch variant of each stage kernel on this mesh and keeps
        the fastest; (h, u, tracers) are restored afterwards.  Returns the choice."""
        c = (ctypes.c_int32 * 12)()
        check(lib().mpaso_state_autotune(self._h, ctypes.c_double(dt), int(nsteps), c))
        return self.launch_config()

    # ---- differentiation (sw app: h and u) ----
    def forward(self, dt, nsteps, ckpt_every):
        """Advances nsteps from the current (h, u), keeping a checkpoint every ckpt_every steps
        (0: the whole window is stored and the vjp recomputes nothing)."""
        check(lib().mpaso_rk4_forward(self._h, ctypes.c_double(dt), int(nsteps), int(ckpt_every)))

    def vjp(self, gh, gu, out=None):
        """Cotangents of the initial (h, u) from cotangents of the final (h, u) of the last forward."""
        gh0, gu0 = out if out is not None else (np.empty(self._shape(FIELD_H)), np.empty(self._shape(FIELD_U)))
        gh = np.ascontiguousarray(gh, np.float64) if isinstance(gh, np.ndarray) else gh
        gu = np.ascontiguousarray(gu, np.float64) if isinstance(gu, np.ndarray) else gu
        check(lib().mpaso_rk4_vjp(self._h, _ptr(gh), _ptr(gu), _ptr(gh0), _ptr(gu0)))
        return gh0, gu0

    def vjp_tracers(self, gh, gu, gtr, out=None):
        """Cotangents of the initial (h, u, tracers) from cotangents of the final (h, u, tracers)
        of the last forward; the FCT limiter is differentiated on the branch the forward took.
        On an ocean state h and u are prescribed: gh / gu are ignored and the returned
        gh0 / gu0 are zero."""
        gh0, gu0, gtr0 = out if out is not None else (
            np.empty(self._shape(FIELD_H)), np.empty(self._shape(FIELD_U)), np.empty(self._shape(FIELD_TRACERS)))
        gh, gu, gtr = (np.ascontiguousarray(x, np.float64) if isinstance(x, np.ndarray) else x
                       for x in (gh, gu, gtr))
        check(lib().mpaso_rk4_vjp_tracers(self._h, _ptr(gh), _ptr(gu), _ptr(gtr), _ptr(gh0), _ptr(gu0),
                                          _ptr(gtr0)))
        return gh0, gu0, gtr0

    def adjoint_device_bytes(self):
        b = ctypes.c_int64()
        check(lib().mpaso_adjoint_device_bytes(self._h, ctypes.byref(b)))
        return b.value

    def launches_per_step(self):
        n = ctypes.c_int32()
        check(lib().mpaso_state_launches_per_step(self._h, ctypes.byref(n)))
        return n.value

    def device_bytes(self):
        b = ctypes.c_int64()
        check(lib().mpaso_state_device_bytes(self._h, ctypes.byref(b)))
        return b.value


# ---------------------------------------------------------------- ordering tuner
ORDERINGS = {0: "file order", 1: "Hilbert cells, edges/vertices after their cells",
             2: "Hilbert curve per entity (cells, edge midpoints, vertex centroids)",
             3: "Morton cells, edges/vertices after their cells"}


def tune_ordering(mesh, fields, dt, fct=None, bottomDepth=None, state_kwargs=None, nsteps=50,
                  modes=(1, 2, 3, 0), device=0):
    """The ordering half of the per-mesh autotuner: builds the device mesh in each
    numbering of `modes`, autotunes the state's launch configuration on it
    (State.autotune) and times `nsteps` graph-replayed steps; returns
    (best mode, {mode: ms per step}, (DeviceMesh, State) of the best mode, its
    launch configuration).  `fields` maps FIELD_* ids to arrays in the reference
    numbering; the returned state holds them, unstepped."""
    import time
    state_kwargs = dict(state_kwargs or {})
    ms, best = {}, None
    for mode in modes:
        dm = DeviceMesh(mesh, fct=fct, bottomDepth=bottomDepth, reorder=mode, device=device)
        st = State(dm, **state_kwargs)
        for f, a in fields.items():
            st.set(f, a)
        cfg = st.autotune(dt, 3)
        st.step_graph(dt, 2)  # capture + warm-up
        st.sync()
        t0 = time.perf_counter()
        st.step_graph(dt, nsteps)
        st.sync()
        ms[mode] = (time.perf_counter() - t0) * 1e3 / nsteps
        if best is None or ms[mode] < ms[best[0]]:
            if best is not None:
                best[1].close(), best[2].close()
            best = (mode, st, dm, cfg)
        else:
            st.close(), dm.close()
    mode, st, dm, cfg = best
    for f, a in fields.items():  # back to the initial fields
        st.set(f, a)
    return mode, ms, (dm, st), cfg
