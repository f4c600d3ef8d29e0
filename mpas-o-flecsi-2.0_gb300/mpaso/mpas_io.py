"""MPAS-format mesh and history files (netCDF classic, CDF-1/2/5) through libmpaso.

`NcFile` wraps the mpaso_nc_* C ABI (include/mpaso_io.h).  On top of it:

- `read_mesh(path)`: an MPAS mesh file as an `mpaso.Mesh`, keeping the file's
  conventions (1-based connectivity, 0 = no neighbour); `Mesh.crs()` then
  applies the reference's read semantics (1-based -> 0-based, zero slots
  dropped; mpasoflecsi/specialization/definition.hh:693-718, 1055-1106).
  The datasets are the ones read_entities, read_mesh_fields and
  read_ocean_mesh_fields read (definition.hh:1070-1101,
  mpasoflecsi/tasks/io.cc:14-158).
- `write_mesh(mesh, path)`: the same datasets under MPAS names and dimensions.
- `History`: the sw history file of mpaso_state runs, laid out as the
  reference's output task writes it (mesh_output_init,
  mpasoflecsi/tasks/io.cc:160-247; output_fields, apps/sw/state.hh:66-70;
  write_timestep, mpasoflecsi/io/helpers.hh:127-151): mesh datasets, then
  one record per output time of h, h_s, vorticity, potential_vorticity and
  tracers along the Time dimension.  Records are read from the device with
  the state's asynchronous snapshots, so writing record n overlaps stepping.
- `write_restart(path, state, time)` / `read_restart(path, state)`: the
  prognostic state (h, u, tracers; the ocean's edge thickness) in one file,
  so a run resumes where it stopped.  The reference has no restart read
  (its only file output is the history above); resuming from this file
  continues the trajectory bit for bit.
"""
import ctypes

import numpy as np

from ._lib import check, lib
from .mesh import MAX_EDGES, MAX_EDGES2, VERTEX_DEGREE, Mesh

NC_BYTE, NC_CHAR, NC_SHORT, NC_INT, NC_FLOAT, NC_DOUBLE, NC_INT64 = 1, 2, 3, 4, 5, 6, 10
_NP = {NC_BYTE: np.int8, NC_CHAR: np.uint8, NC_SHORT: np.int16, NC_INT: np.int32, NC_FLOAT: np.float32,
       NC_DOUBLE: np.float64, NC_INT64: np.int64}
_NC = {np.dtype(v): k for k, v in _NP.items()}


def _buf(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class NcFile:
    """A netCDF classic file (read, create, or append records)."""

    def __init__(self, path, mode="r", version=5):
        self._h = ctypes.c_void_p()
        self.path = path
        if mode == "w":
            check(lib().mpaso_nc_create(path.encode(), int(version), ctypes.byref(self._h)))
        elif mode in ("r", "a"):
            check(lib().mpaso_nc_open(path.encode(), 1 if mode == "a" else 0, ctypes.byref(self._h)))
        else:
            raise ValueError("mode is 'r', 'w' or 'a'")

    def close(self):
        if self._h:
            h, self._h = self._h, None
            check(lib().mpaso_nc_close(h))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- define mode ----
    def def_dim(self, name, length):
        check(lib().mpaso_nc_def_dim(self._h, name.encode(), ctypes.c_int64(int(length))))

    def def_var(self, name, nc_type, dims):
        arr = (ctypes.c_char_p * max(len(dims), 1))(*[d.encode() for d in dims])
        check(lib().mpaso_nc_def_var(self._h, name.encode(), int(nc_type), len(dims), arr))

    def put_att(self, name, value, var=None):
        if isinstance(value, str):
            a, t = np.frombuffer(value.encode(), np.uint8).copy(), NC_CHAR
        else:
            a = np.atleast_1d(np.asarray(value))
            if a.dtype.kind == "f":
                a = a.astype(np.float64)
            elif a.dtype.kind in "iu":
                a = a.astype(np.int32)
            t = _NC[a.dtype]
        check(lib().mpaso_nc_put_att(self._h, var.encode() if var else None, name.encode(), t,
                                     ctypes.c_int64(a.size), _buf(a)))

    def enddef(self):
        check(lib().mpaso_nc_enddef(self._h))

    # ---- data ----
    def put_var(self, name, data):
        a = np.ascontiguousarray(data)
        if a.dtype not in _NC:
            a = a.astype(np.float64 if a.dtype.kind == "f" else np.int32)
        check(lib().mpaso_nc_put_var(self._h, name.encode(), _NC[a.dtype], _buf(a)))

    def put_rec(self, name, rec, data):
        a = np.ascontiguousarray(data)
        if a.dtype not in _NC:
            a = a.astype(np.float64 if a.dtype.kind == "f" else np.int32)
        check(lib().mpaso_nc_put_rec(self._h, name.encode(), ctypes.c_int64(int(rec)), _NC[a.dtype], _buf(a)))

    def var_info(self, name):
        """(nc_type, shape, is_record) of a variable."""
        t, nd, rec = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        shape = (ctypes.c_int64 * 8)()
        check(lib().mpaso_nc_inq_var(self._h, name.encode(), ctypes.byref(t), ctypes.byref(nd), shape,
                                     ctypes.byref(rec)))
        return t.value, tuple(int(shape[i]) for i in range(nd.value)), bool(rec.value)

    def get_var(self, name, dtype=None):
        t, shape, _ = self.var_info(name)
        out = np.empty(shape, dtype or _NP[t])
        check(lib().mpaso_nc_get_var(self._h, name.encode(), _NC[out.dtype], _buf(out)))
        return out

    def get_rec(self, name, rec, dtype=None):
        t, shape, isrec = self.var_info(name)
        if not isrec:
            raise ValueError(f"{name} is not a record variable")
        out = np.empty(shape[1:], dtype or _NP[t])
        check(lib().mpaso_nc_get_rec(self._h, name.encode(), ctypes.c_int64(int(rec)), _NC[out.dtype], _buf(out)))
        return out

    # ---- queries ----
    def inq(self):
        v, nr, nd, nv, na = (ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32(),
                             ctypes.c_int32())
        check(lib().mpaso_nc_inq(self._h, ctypes.byref(v), ctypes.byref(nr), ctypes.byref(nd), ctypes.byref(nv),
                                 ctypes.byref(na)))
        return {"version": v.value, "numrecs": nr.value, "ndims": nd.value, "nvars": nv.value,
                "ngatts": na.value}

    @property
    def numrecs(self):
        return self.inq()["numrecs"]

    def dims(self):
        buf = ctypes.create_string_buffer(4097)
        n = ctypes.c_int64()
        out = {}
        for i in range(self.inq()["ndims"]):
            check(lib().mpaso_nc_dim_name(self._h, i, buf, 4097, ctypes.byref(n)))
            out[buf.value.decode()] = n.value
        return out

    def variables(self):
        buf = ctypes.create_string_buffer(4097)
        out = []
        for i in range(self.inq()["nvars"]):
            check(lib().mpaso_nc_var_name(self._h, i, buf, 4097))
            out.append(buf.value.decode())
        return out

    def var_dims(self, name):
        buf = ctypes.create_string_buffer(4097)
        return [self._dim_name(name, i, buf) for i in range(len(self.var_info(name)[1]))]

    def _dim_name(self, var, i, buf):
        check(lib().mpaso_nc_var_dim_name(self._h, var.encode(), i, buf, 4097))
        return buf.value.decode()

    def get_att(self, name, var=None, default=None):
        t, n = ctypes.c_int32(), ctypes.c_int64()
        vb = var.encode() if var else None
        rc = lib().mpaso_nc_get_att(self._h, vb, name.encode(), ctypes.byref(t), ctypes.byref(n), None,
                                    ctypes.c_int64(0))
        if rc != 0:
            if default is not None or rc == 5:  # MPASO_ERR_NOTFOUND
                return default
            check(rc)
        out = np.empty(n.value, _NP[t.value])
        check(lib().mpaso_nc_get_att(self._h, vb, name.encode(), ctypes.byref(t), ctypes.byref(n), _buf(out),
                                     ctypes.c_int64(out.nbytes)))
        if t.value == NC_CHAR:
            return out.tobytes().split(b"\0")[0].decode(errors="replace")
        return out[0] if out.size == 1 else out

    def attributes(self, var=None):
        buf = ctypes.create_string_buffer(4097)
        out = {}
        i = 0
        vb = var.encode() if var else None
        while lib().mpaso_nc_att_name(self._h, vb, i, buf, 4097) == 0:
            name = buf.value.decode()
            out[name] = self.get_att(name, var)
            i += 1
        return out


# MPAS dimension names of every mesh dataset: (entity dimension, second dimension)
_MESH_VARS = {
    "nEdgesOnCell": ("nCells", None), "edgesOnCell": ("nCells", "maxEdges"),
    "cellsOnCell": ("nCells", "maxEdges"), "verticesOnCell": ("nCells", "maxEdges"),
    "cellsOnEdge": ("nEdges", "TWO"), "verticesOnEdge": ("nEdges", "TWO"),
    "nEdgesOnEdge": ("nEdges", None), "edgesOnEdge": ("nEdges", "maxEdges2"),
    "weightsOnEdge": ("nEdges", "maxEdges2"), "cellsOnVertex": ("nVertices", "vertexDegree"),
    "edgesOnVertex": ("nVertices", "vertexDegree"), "kiteAreasOnVertex": ("nVertices", "vertexDegree"),
}
_ENTITY = {"Cell": "nCells", "Edge": "nEdges", "Vertex": "nVertices", "Triangle": "nVertices"}
_INT_VARS = {"nEdgesOnCell", "edgesOnCell", "cellsOnCell", "verticesOnCell", "cellsOnEdge", "verticesOnEdge",
             "nEdgesOnEdge", "edgesOnEdge", "cellsOnVertex", "edgesOnVertex"}
# datasets the path needs, and the ones read when present (read_mesh_fields /
# read_ocean_mesh_fields)
_REQUIRED = ("nEdgesOnCell", "edgesOnCell", "cellsOnCell", "verticesOnCell", "cellsOnEdge", "verticesOnEdge",
             "nEdgesOnEdge", "edgesOnEdge", "weightsOnEdge", "cellsOnVertex", "edgesOnVertex", "areaCell",
             "areaTriangle", "kiteAreasOnVertex", "dcEdge", "dvEdge", "xCell", "yCell", "zCell", "xVertex",
             "yVertex", "zVertex")
_OPTIONAL = ("angleEdge", "xEdge", "yEdge", "zEdge", "latCell", "lonCell", "latEdge", "lonEdge", "latVertex",
             "lonVertex", "fCell", "fEdge", "fVertex", "meshDensity", "bottomDepth")


_CELL_FIELDS = {"meshDensity", "mDensity", "bottomDepth", "bottomDepthObserved", "maxLevelCell"}


def _entity_dim(name):
    if name in _MESH_VARS:
        return _MESH_VARS[name][0]
    if name in _CELL_FIELDS:
        return "nCells"
    for suffix, dim in _ENTITY.items():
        if name.endswith(suffix):
            return dim
    raise KeyError(name)


def read_mesh(path):
    """An MPAS mesh file (netCDF classic) as an mpaso.Mesh in the file's conventions."""
    with NcFile(path) as f:
        dims = f.dims()
        have = set(f.variables())
        missing = [n for n in _REQUIRED if n not in have]
        if missing:
            raise ValueError(f"{path}: MPAS mesh datasets missing: {', '.join(missing)}")
        m = Mesh()
        m.nCells, m.nEdges, m.nVertices = dims["nCells"], dims["nEdges"], dims["nVertices"]
        m.fields = {}
        for n in _REQUIRED + tuple(x for x in _OPTIONAL if x in have):
            a = f.get_var(n, np.int32 if n in _INT_VARS else np.float64)
            if a.ndim == 2:  # the compiled-in widths (mpasoflecsi/common/constants.hh:11-14)
                width = {"maxEdges": MAX_EDGES, "maxEdges2": MAX_EDGES2, "TWO": 2,
                         "vertexDegree": VERTEX_DEGREE}[_MESH_VARS[n][1]]
                if a.shape[1] > width:
                    if np.any(a[:, width:] != 0):
                        raise ValueError(f"{path}: {n} has {a.shape[1]} columns in use; the path holds {width}")
                    a = a[:, :width]
                elif a.shape[1] < width:
                    a = np.concatenate([a, np.zeros((a.shape[0], width - a.shape[1]), a.dtype)], axis=1)
            m.fields[n] = np.ascontiguousarray(a)
        sphere = str(f.get_att("on_a_sphere", default="YES")).strip().upper().startswith("Y")
        m.on_sphere = sphere
        if sphere:
            r = f.get_att("sphere_radius", default=0.0)
            if not r:  # no attribute: the radius the cell centres lie on
                r = float(np.sqrt(m.fields["xCell"][0] ** 2 + m.fields["yCell"][0] ** 2 + m.fields["zCell"][0] ** 2))
            m.radius = float(r)
            m.Lx = m.Ly = 0.0
        else:
            m.radius = 1.0
            m.Lx = float(f.get_att("x_period", default=0.0))
            m.Ly = float(f.get_att("y_period", default=0.0))
        if "fVertex" not in m.fields:
            m.fields["fVertex"] = np.zeros(m.nVertices)
        if "meshDensity" not in m.fields:
            m.fields["meshDensity"] = np.ones(m.nCells)
        if "angleEdge" not in m.fields:
            m.fields["angleEdge"] = np.zeros(m.nEdges)
        return m


def write_mesh(mesh, path, version=5, extra=None):
    """Writes mesh.fields (plus `extra` {name: array}) under MPAS names and dimensions."""
    with NcFile(path, "w", version) as f:
        _define_mesh(f, mesh, list(mesh.fields) + list(extra or {}), extra)
        f.enddef()
        for n, a in list(mesh.fields.items()) + list((extra or {}).items()):
            f.put_var(n, a)


def _define_mesh(f, mesh, names, extra=None):
    f.def_dim("nCells", mesh.nCells)
    f.def_dim("nEdges", mesh.nEdges)
    f.def_dim("nVertices", mesh.nVertices)
    f.def_dim("maxEdges", MAX_EDGES)
    f.def_dim("maxEdges2", MAX_EDGES2)
    f.def_dim("TWO", 2)
    f.def_dim("vertexDegree", VERTEX_DEGREE)
    f.put_att("on_a_sphere", "YES" if mesh.on_sphere else "NO")
    if mesh.on_sphere:
        f.put_att("sphere_radius", float(mesh.radius))
    else:
        f.put_att("sphere_radius", 0.0)
        f.put_att("is_periodic", "YES")
        f.put_att("x_period", float(mesh.Lx))
        f.put_att("y_period", float(mesh.Ly))
    f.put_att("source", "mpaso (GB300 path of MPAS-O-FleCSI)")
    allf = dict(mesh.fields, **(extra or {}))
    for n in names:
        a = np.asarray(allf[n])
        dims = [_entity_dim(n)]
        if a.ndim == 2:
            dims.append(_MESH_VARS[n][1])
        f.def_var(n, NC_INT if a.dtype.kind in "iu" else NC_DOUBLE, dims)


class History:
    """sw history output of a device state, one record per `write()` call.

    The file holds the datasets mesh_output_init writes (areaCell, x/y/zCell,
    lat/lonCell, lat/lonVertex, mDensity, dvEdge, dcEdge, cellsOnVertex; global
    attribute on_a_sphere) and, per record, the output fields of the sw app:
    h [Time][nCells][nVertLevels], h_s [Time][nCells], vorticity and
    potential_vorticity [Time][nVertices][nVertLevels], tracers
    [Time][nCells][nVertLevels][nTracers].  `write(state)` takes the state's
    snapshots asynchronously (mpaso_state_snapshot) and writes the previous
    record to the file meanwhile; `close()` drains.
    """

    def __init__(self, path, mesh, nlev, ntr, bottomDepth=None, version=5):
        self.mesh, self.L, self.T = mesh, nlev, ntr
        self.f = NcFile(path, "w", version)
        f = self.f
        m = mesh
        for d, n in (("nCells", m.nCells), ("nEdges", m.nEdges), ("nVertices", m.nVertices),
                     ("vertexDegree", VERTEX_DEGREE), ("nVertLevels", nlev), ("nTracers", max(ntr, 1))):
            f.def_dim(d, n)
        f.def_dim("Time", 0)
        f.put_att("on_a_sphere", "YES" if m.on_sphere else "NO")
        fl = m.fields
        self._static = {
            "areaCell": fl["areaCell"], "xCell": fl["xCell"], "yCell": fl["yCell"], "zCell": fl["zCell"],
            "latCell": fl.get("latCell", np.zeros(m.nCells)), "lonCell": fl.get("lonCell", np.zeros(m.nCells)),
            "latVertex": fl.get("latVertex", np.zeros(m.nVertices)),
            "lonVertex": fl.get("lonVertex", np.zeros(m.nVertices)),
            "mDensity": fl.get("meshDensity", np.ones(m.nCells)), "dvEdge": fl["dvEdge"], "dcEdge": fl["dcEdge"],
            "cellsOnVertex": fl["cellsOnVertex"]}
        for n, a in self._static.items():
            ent = _entity_dim(n)
            f.def_var(n, NC_INT if np.asarray(a).dtype.kind in "iu" else NC_DOUBLE,
                      [ent] + (["vertexDegree"] if np.asarray(a).ndim == 2 else []))
        f.def_var("h", NC_DOUBLE, ["Time", "nCells", "nVertLevels"])
        f.def_var("h_s", NC_DOUBLE, ["Time", "nCells"])
        f.def_var("vorticity", NC_DOUBLE, ["Time", "nVertices", "nVertLevels"])
        f.def_var("potential_vorticity", NC_DOUBLE, ["Time", "nVertices", "nVertLevels"])
        f.def_var("tracers", NC_DOUBLE, ["Time", "nCells", "nVertLevels", "nTracers"])
        f.enddef()
        for n, a in self._static.items():
            f.put_var(n, a)
        self.h_s = np.zeros(m.nCells) if bottomDepth is None else np.asarray(bottomDepth, np.float64)
        self.nrec = 0
        self._pending = None
        self._bufs = None

    def _alloc(self):
        import mpaso.gpu as G
        shapes = {G.FIELD_H: (self.mesh.nCells, self.L), G.FIELD_VORTICITY: (self.mesh.nVertices, self.L),
                  G.FIELD_PV_VERTEX: (self.mesh.nVertices, self.L)}
        if self.T:
            shapes[G.FIELD_TRACERS] = (self.mesh.nCells, self.L, self.T)
        return [{k: self._pinned(s) for k, s in shapes.items()} for _ in range(2)]

    def _pinned(self, shape):
        """Page-locked host buffer (so the snapshot copies overlap the steps), as numpy."""
        try:
            import torch
            t = torch.empty(shape, dtype=torch.float64).pin_memory()
            self._keep = getattr(self, "_keep", []) + [t]
            return t.numpy()
        except Exception:  # no torch / no CUDA runtime for pinning: pageable memory still works
            return np.empty(shape)

    def _flush(self):
        if self._pending is None:
            return
        import mpaso.gpu as G
        st, b = self._pending
        st.snapshot_wait()
        f, r = self.f, self.nrec
        f.put_rec("h", r, b[G.FIELD_H])
        f.put_rec("h_s", r, self.h_s)
        f.put_rec("vorticity", r, b[G.FIELD_VORTICITY])
        f.put_rec("potential_vorticity", r, b[G.FIELD_PV_VERTEX])
        tr = b[G.FIELD_TRACERS] if self.T else np.zeros((self.mesh.nCells, self.L, 1))
        f.put_rec("tracers", r, tr)
        self.nrec += 1
        self._pending = None

    def write(self, state):
        """Queues the state's current fields as the next record (returns before they reach the file)."""
        if self._bufs is None:
            self._bufs = self._alloc()
        self._flush()
        b = self._bufs[self.nrec % 2]
        for field, buf in b.items():
            state.snapshot(field, buf)
        self._pending = (state, b)

    def close(self):
        if self.f is not None:
            self._flush()
            self.f.close()
            self.f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


_RESTART_VARS = (  # (variable, field attribute of mpaso.gpu, entity dimension, ocean only)
    ("h", "FIELD_H", "nCells", False),
    ("u", "FIELD_U", "nEdges", False),
    ("layerThicknessEdge", "FIELD_LAYER_THICKNESS_EDGE", "nEdges", True),
)


def write_restart(path, state, time=0.0, version=5):
    """Writes the state's prognostic fields (reference numbering) and the model time."""
    import mpaso.gpu as G
    dm = state.dmesh
    ocean = state.app == G.APP_OCEAN
    with NcFile(path, "w", version) as f:
        for d, n in (("nCells", dm.nC), ("nEdges", dm.nE), ("nVertLevels", state.L),
                     ("nTracers", max(state.T, 1))):
            f.def_dim(d, n)
        f.put_att("app", "ocean" if ocean else "sw")
        f.put_att("nTracersInState", int(state.T))
        f.put_att("model_time_s", float(time))
        for name, _, ent, oc in _RESTART_VARS:
            if oc and not ocean:
                continue
            f.def_var(name, NC_DOUBLE, [ent, "nVertLevels"])
        if state.T:
            f.def_var("tracers", NC_DOUBLE, ["nCells", "nVertLevels", "nTracers"])
        f.enddef()
        for name, field, _, oc in _RESTART_VARS:
            if oc and not ocean:
                continue
            f.put_var(name, state.get(getattr(G, field)))
        if state.T:
            f.put_var("tracers", state.get(G.FIELD_TRACERS))


def read_restart(path, state):
    """Sets the state from a restart file (its mesh sizes, levels, tracers and
    app must match); returns the model time stored with it."""
    import mpaso.gpu as G
    dm = state.dmesh
    ocean = state.app == G.APP_OCEAN
    with NcFile(path) as f:
        dims = f.dims()
        want = {"nCells": dm.nC, "nEdges": dm.nE, "nVertLevels": state.L}
        for d, n in want.items():
            if dims.get(d) != n:
                raise ValueError(f"restart file has {d} = {dims.get(d)}, the state {n}")
        if f.get_att("app") is None or f.get_att("nTracersInState") is None:
            raise ValueError(f"{path} is not a restart file")
        if f.get_att("app") != ("ocean" if ocean else "sw") or int(f.get_att("nTracersInState")) != state.T:
            raise ValueError("restart file was written by another app or tracer count")
        for name, field, _, oc in _RESTART_VARS:
            if oc and not ocean:
                continue
            state.set(getattr(G, field), f.get_var(name))
        if state.T:
            state.set(G.FIELD_TRACERS, f.get_var("tracers"))
        return float(f.get_att("model_time_s"))
