"""MPAS meshes in memory: generation (libmpaso) and the reference's read semantics.

`Mesh.fields` holds every MPAS dataset under its MPAS name, in the MPAS file
conventions (connectivity int32, 1-based, 0-padded).  `Mesh.crs()` converts the
connectivity the way the reference's reader and mesh specialization do:

- 1-based -> 0-based and zero slots dropped into CRS
  (mpasoflecsi/specialization/definition.hh:693-718);
- c2v, c2e, c2c, e2v, e2e kept in file order
  (mpasoflecsi/specialization/mesh.cc:67-89, 93-105);
- v2c, e2c, v2e built by transposition, i.e. ascending ids
  (mpasoflecsi/specialization/mesh.cc:108-116).
"""
import ctypes

import numpy as np

from ._lib import check, lib

EARTH_RADIUS = 6371000.0  # mpasoflecsi/common/constants.hh:28
OMEGA = 7.29212e-5  # mpasoflecsi/common/constants.hh:32-33

MAX_EDGES = 8
MAX_EDGES2 = 16
VERTEX_DEGREE = 3


class Mesh:
    def __init__(self, handle=None):
        self._h = handle
        if handle is None:
            return
        L = lib()
        dims = (ctypes.c_int64 * 3)()
        flags = (ctypes.c_int32 * 1)()
        geom = (ctypes.c_double * 3)()
        check(L.mpaso_genmesh_dims(handle, dims, flags, geom))
        self.nCells, self.nEdges, self.nVertices = int(dims[0]), int(dims[1]), int(dims[2])
        self.on_sphere = bool(flags[0])
        self.radius, self.Lx, self.Ly = float(geom[0]), float(geom[1]), float(geom[2])
        self.fields = {}
        for name in L.mpaso_genmesh_names().decode().split(","):
            dt = ctypes.c_int32()
            rows = ctypes.c_int64()
            cols = ctypes.c_int64()
            check(L.mpaso_genmesh_field(handle, name.encode(), ctypes.byref(dt),
                                        ctypes.byref(rows), ctypes.byref(cols)))
            arr = np.empty((rows.value, cols.value), dtype=np.int32 if dt.value == 0 else np.float64)
            check(L.mpaso_genmesh_copy(handle, name.encode(), arr.ctypes.data_as(ctypes.c_void_p)))
            self.fields[name] = arr[:, 0].copy() if cols.value == 1 else arr

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                lib().mpaso_genmesh_free(h)
            except Exception:
                pass
            self._h = None

    # ---- (de)serialisation ----
    def to_dict(self):
        d = {"mesh_" + k: v for k, v in self.fields.items()}
        d["mesh_dims"] = np.array([self.nCells, self.nEdges, self.nVertices], np.int64)
        d["mesh_geom"] = np.array([float(self.on_sphere), self.radius, self.Lx, self.Ly])
        return d

    @classmethod
    def from_dict(cls, d):
        m = cls()
        m.nCells, m.nEdges, m.nVertices = (int(x) for x in d["mesh_dims"])
        g = d["mesh_geom"]
        m.on_sphere, m.radius, m.Lx, m.Ly = bool(g[0]), float(g[1]), float(g[2]), float(g[3])
        m.fields = {k[5:]: np.asarray(v) for k, v in d.items()
                    if k.startswith("mesh_") and k not in ("mesh_dims", "mesh_geom")}
        return m

    # ---- constructors ----
    @classmethod
    def icosa(cls, level, radius=EARTH_RADIUS, omega=OMEGA):
        h = ctypes.c_void_p()
        check(lib().mpaso_genmesh_icosa(int(level), ctypes.c_double(radius), ctypes.c_double(omega),
                                        ctypes.byref(h)))
        return cls(h)

    @classmethod
    def hex(cls, nx, ny, dc, f0=1e-4):
        h = ctypes.c_void_p()
        check(lib().mpaso_genmesh_hex(int(nx), int(ny), ctypes.c_double(dc), ctypes.c_double(f0),
                                      ctypes.byref(h)))
        return cls(h)

    def reordered(self):
        """Same mesh regenerated in Hilbert-curve order; returns (mesh, (pc, pe, pv)) with
        perm[new] = old for cells, edges and vertices."""
        if self._h is None:
            raise ValueError("only generated meshes can be regenerated in curve order")
        h = ctypes.c_void_p()
        pc = np.empty(self.nCells, np.int32)
        pe = np.empty(self.nEdges, np.int32)
        pv = np.empty(self.nVertices, np.int32)
        i32p = ctypes.POINTER(ctypes.c_int32)
        check(lib().mpaso_genmesh_reorder_sfc(self._h, ctypes.byref(h), pc.ctypes.data_as(i32p),
                                              pe.ctypes.data_as(i32p), pv.ctypes.data_as(i32p)))
        return Mesh(h), (pc, pe, pv)

    # ---- reference read semantics ----
    _CRS_SOURCES = ("verticesOnCell", "edgesOnCell", "cellsOnCell", "verticesOnEdge", "edgesOnEdge")

    def crs(self):
        """Connectivity as the reference's mesh holds it: dict name -> (offsets, indices).
        Built once and kept while the five file connectivity arrays are the same
        objects (the result is shared: treat it as read-only)."""
        f = self.fields
        src = tuple(f.get(n) for n in self._CRS_SOURCES)
        cached = getattr(self, "_crs_cache", None)
        if cached is not None and all(a is b for a, b in zip(cached[0], src)):
            return cached[1]
        out = self._build_crs()
        self._crs_cache = (src, out)
        return out

    def _build_crs(self):
        f = self.fields

        def from_file(name):
            a = f[name]
            if a.ndim == 1:
                a = a[:, None]
            mask = a != 0
            counts = mask.sum(axis=1)
            off = np.zeros(a.shape[0] + 1, np.int64)
            np.cumsum(counts, out=off[1:])
            idx = (a[mask] - 1).astype(np.int32)  # row-major: keeps file order within rows
            return off, idx

        def transpose(cnx, n_to):
            off, idx = cnx
            n_from = off.size - 1
            src = np.repeat(np.arange(n_from, dtype=np.int32), np.diff(off))
            order = np.argsort(idx, kind="stable")  # stable: ascending source id per target
            counts = np.bincount(idx, minlength=n_to)
            toff = np.zeros(n_to + 1, np.int64)
            np.cumsum(counts, out=toff[1:])
            return toff, src[order].astype(np.int32)

        c2v = from_file("verticesOnCell")
        c2e = from_file("edgesOnCell")
        c2c = from_file("cellsOnCell")
        e2v = from_file("verticesOnEdge")
        e2e = from_file("edgesOnEdge")
        return {
            "c2v": c2v, "c2e": c2e, "c2c": c2c, "e2v": e2v, "e2e": e2e,
            "v2c": transpose(c2v, self.nVertices),
            "e2c": transpose(c2e, self.nEdges),
            "v2e": transpose(e2v, self.nVertices),
        }
