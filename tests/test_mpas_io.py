"""MPAS-format files without HDF5 (host code, no GPU): the netCDF classic
reader/writer against scipy's independent implementation of CDF-1/2 in both
directions, CDF-5 round trips, and MPAS mesh files read with the reference's
semantics (1-based, zero-padded connectivity; definition.hh:1055-1106)."""
import os

import numpy as np
import pytest

import mpaso
from mpaso._lib import MpasoError
from mpaso.mpas_io import NcFile, read_mesh, write_mesh

netcdf_file = pytest.importorskip("scipy.io").netcdf_file


def _sample(rng):
    return {
        "i32": rng.integers(-2**31, 2**31 - 1, size=(7, 3), dtype=np.int64).astype(np.int32),
        "f64": rng.standard_normal((7, 5)),
        "f32": rng.standard_normal(7).astype(np.float32),
        "i16": rng.integers(-30000, 30000, size=(3, 5)).astype(np.int16),
        "i8": rng.integers(-100, 100, size=5).astype(np.int8),
        "rec": rng.standard_normal((4, 7, 3)),
        "rec_i": rng.integers(0, 1000, size=(4, 5)).astype(np.int32),
    }


_DIMS = {"i32": ("n", "m"), "f64": ("n", "k"), "f32": ("n",), "i16": ("m", "k"), "i8": ("k",),
         "rec": ("Time", "n", "m"), "rec_i": ("Time", "k")}


@pytest.mark.parametrize("version", [1, 2])
def test_reads_files_written_by_scipy(tmp_path, version):
    rng = np.random.default_rng(version)
    data = _sample(rng)
    path = str(tmp_path / "s.nc")
    with netcdf_file(path, "w", version=version) as f:
        f.createDimension("Time", None)  # scipy wants the record dimension first
        f.createDimension("n", 7), f.createDimension("m", 3), f.createDimension("k", 5)
        f.title = "written by scipy"
        f.answer = np.int32(42)
        for name, a in data.items():
            v = f.createVariable(name, a.dtype, _DIMS[name])
            v[:] = a
            v.units = "m s-1"
    with NcFile(path) as g:
        assert g.inq()["version"] == version and g.numrecs == 4
        assert g.dims() == {"Time": 4, "n": 7, "m": 3, "k": 5}
        assert g.get_att("title") == "written by scipy" and g.get_att("answer") == 42
        for name, a in data.items():
            got = g.get_var(name)
            assert got.dtype == a.dtype and np.array_equal(got, a), name
            assert g.get_att("units", var=name) == "m s-1"
            assert g.var_dims(name) == list(_DIMS[name])
        for r in range(4):
            assert np.array_equal(g.get_rec("rec", r), data["rec"][r])
        # conversions on read
        assert np.array_equal(g.get_var("i16", np.float64), data["i16"].astype(np.float64))
        assert np.array_equal(g.get_var("f32", np.float64), data["f32"].astype(np.float64))


@pytest.mark.parametrize("version", [1, 2])
def test_files_written_here_read_by_scipy(tmp_path, version):
    rng = np.random.default_rng(10 + version)
    data = _sample(rng)
    path = str(tmp_path / "o.nc")
    with NcFile(path, "w", version) as f:
        f.def_dim("n", 7), f.def_dim("m", 3), f.def_dim("k", 5), f.def_dim("Time", 0)
        f.put_att("title", "written here")
        f.put_att("values", np.array([1.5, 2.5]))
        for name, a in data.items():
            f.def_var(name, {np.dtype(np.int32): 4, np.dtype(np.float64): 6, np.dtype(np.float32): 5,
                             np.dtype(np.int16): 3, np.dtype(np.int8): 1}[a.dtype], list(_DIMS[name]))
        f.enddef()
        for name, a in data.items():
            if name.startswith("rec"):
                for r in range(a.shape[0]):
                    f.put_rec(name, r, a[r])
            else:
                f.put_var(name, a)
    with netcdf_file(path, "r", mmap=False) as g:
        assert g.version_byte == version
        assert g.title == b"written here" and np.array_equal(g.values, [1.5, 2.5])
        for name, a in data.items():
            assert np.array_equal(g.variables[name][:], a), name


def test_cdf5_round_trip_and_header(tmp_path):
    rng = np.random.default_rng(5)
    path = str(tmp_path / "c5.nc")
    big = rng.integers(-2**62, 2**62, size=11, dtype=np.int64)
    a = rng.standard_normal((11, 2))
    with NcFile(path, "w", 5) as f:
        f.def_dim("n", 11), f.def_dim("two", 2), f.def_dim("Time", 0)
        f.def_var("big", 10, ["n"]), f.def_var("a", 6, ["n", "two"]), f.def_var("r", 6, ["Time", "two"])
        f.enddef()
        f.put_var("big", big), f.put_var("a", a)
        for r in range(3):
            f.put_rec("r", r, np.array([r, -r], float))
    raw = open(path, "rb").read()
    assert raw[:4] == b"CDF\x05" and int.from_bytes(raw[4:12], "big") == 3  # 8-byte record count
    with NcFile(path) as g:
        assert np.array_equal(g.get_var("big"), big) and np.array_equal(g.get_var("a"), a)
        assert np.array_equal(g.get_var("r"), [[0, 0], [1, -1], [2, -2]])
    # appending records to an existing file
    with NcFile(path, "a") as g:
        g.put_rec("r", 3, np.array([7.0, 8.0]))
    with NcFile(path) as g:
        assert g.numrecs == 4 and np.array_equal(g.get_rec("r", 3), [7.0, 8.0])


def test_errors(tmp_path):
    p = str(tmp_path / "x.h5")
    with open(p, "wb") as f:
        f.write(b"\x89HDF\r\n\x1a\n" + bytes(100))
    with pytest.raises(MpasoError) as e:
        NcFile(p)
    assert e.value.code == 9 and "netCDF-4" in str(e.value)
    with pytest.raises(MpasoError):
        NcFile(str(tmp_path / "missing.nc"))
    q = str(tmp_path / "v1.nc")
    with NcFile(q, "w", 1) as f:
        f.def_dim("n", 2)
        with pytest.raises(MpasoError):
            f.def_var("x", 10, ["n"])  # int64 needs CDF-5
        with pytest.raises(MpasoError):
            f.def_var("y", 6, ["nope"])
        f.def_var("z", 4, ["n"])
        f.enddef()
        with pytest.raises(MpasoError):
            f.put_var("z", np.array([1e12, 0.0]))  # does not fit an int
    with NcFile(q) as g:
        with pytest.raises(MpasoError) as e:
            g.get_var("nothere")
        assert e.value.code == 5


@pytest.mark.parametrize("version", [1, 2, 5])
def test_corrupt_header_counts_refused_before_allocating(tmp_path, version):
    """Counts in a header (dimensions, variables, attributes, attribute
    lengths) that the rest of the file could not hold are refused as a
    malformed file, without sizing anything by them."""
    nn = 8 if version == 5 else 4
    be = lambda v, n=nn: int(v).to_bytes(n, "big")  # noqa: E731
    head = b"CDF" + bytes([version]) + be(0)
    cases = {
        "dims": head + be(10, 4) + be(2**31 - 1),                      # NC_DIMENSION, huge count
        "gatts": head + be(0, 4) + be(0) + be(12, 4) + be(2**31 - 1),  # NC_ATTRIBUTE, huge count
        "vars": head + be(0, 4) + be(0) + be(0, 4) + be(0) + be(11, 4) + be(2**31 - 1),
        # one global attribute of type double with 2**30 values and 8 bytes of data
        "attlen": head + be(0, 4) + be(0) + be(12, 4) + be(1) + be(1) + b"a\0\0\0" + be(6, 4)
                  + be(2**30) + bytes(8),
    }
    for name, data in cases.items():
        p = str(tmp_path / f"{name}.nc")
        with open(p, "wb") as f:
            f.write(data + bytes(64))
        with pytest.raises(MpasoError) as e:
            NcFile(p)
        assert e.value.code == 9, name
        assert "truncated or corrupt header" in str(e.value) or "too large" in str(e.value), (name, str(e.value))


@pytest.mark.parametrize("kind,version", [("icosa2", 5), ("hex", 2)])
def test_mpas_mesh_round_trip(tmp_path, kind, version):
    m = mpaso.Mesh.icosa(2) if kind == "icosa2" else mpaso.Mesh.hex(6, 4, 10e3)
    path = str(tmp_path / "mesh.nc")
    write_mesh(m, path, version)
    r = read_mesh(path)
    assert (r.nCells, r.nEdges, r.nVertices, r.on_sphere) == (m.nCells, m.nEdges, m.nVertices, m.on_sphere)
    assert r.radius == m.radius and r.Lx == m.Lx and r.Ly == m.Ly
    for k, v in m.fields.items():
        assert np.array_equal(r.fields[k], v), k
    for k, (off, idx) in m.crs().items():
        assert np.array_equal(r.crs()[k][0], off) and np.array_equal(r.crs()[k][1], idx), k


def test_mpas_mesh_written_elsewhere_with_narrower_columns(tmp_path):
    """A file with maxEdges = 6 / maxEdges2 = 12 (as MPAS tools write for hexagonal
    meshes), written by scipy: read into the path's compiled widths (8 / 16) with
    the same CRS connectivity; a file using more columns than the path holds is
    refused."""
    m = mpaso.Mesh.hex(5, 4, 20e3)
    f = m.fields
    assert not np.any(f["edgesOnCell"][:, 6:]) and not np.any(f["edgesOnEdge"][:, 12:])
    path = str(tmp_path / "narrow.nc")
    width = {"maxEdges": 6, "maxEdges2": 12, "TWO": 2, "vertexDegree": 3}
    second = {"edgesOnCell": "maxEdges", "cellsOnCell": "maxEdges", "verticesOnCell": "maxEdges",
              "cellsOnEdge": "TWO", "verticesOnEdge": "TWO", "edgesOnEdge": "maxEdges2",
              "weightsOnEdge": "maxEdges2", "cellsOnVertex": "vertexDegree", "edgesOnVertex": "vertexDegree",
              "kiteAreasOnVertex": "vertexDegree"}
    ent = {"Cell": "nCells", "Edge": "nEdges", "Vertex": "nVertices", "Triangle": "nVertices"}
    with netcdf_file(path, "w", version=2) as g:
        g.createDimension("nCells", m.nCells), g.createDimension("nEdges", m.nEdges)
        g.createDimension("nVertices", m.nVertices)
        for d, n in width.items():
            g.createDimension(d, n)
        g.on_a_sphere = "NO"
        g.x_period, g.y_period = m.Lx, m.Ly
        for name, a in f.items():
            e = "nEdges" if name in ("nEdgesOnEdge", "cellsOnEdge", "verticesOnEdge", "edgesOnEdge",
                                     "weightsOnEdge") else \
                "nCells" if name in ("nEdgesOnCell", "edgesOnCell", "cellsOnCell", "verticesOnCell") else \
                "nVertices" if name in ("cellsOnVertex", "edgesOnVertex", "kiteAreasOnVertex") else \
                "nCells" if name == "meshDensity" else next(v for s, v in ent.items() if name.endswith(s))
            dims = (e,) + ((second[name],) if a.ndim == 2 else ())
            v = g.createVariable(name, a.dtype, dims)
            v[:] = a[:, :width[second[name]]] if a.ndim == 2 else a
    r = read_mesh(path)
    assert r.fields["edgesOnCell"].shape == (m.nCells, 8) and r.fields["edgesOnEdge"].shape == (m.nEdges, 16)
    for k, (off, idx) in m.crs().items():
        assert np.array_equal(r.crs()[k][0], off) and np.array_equal(r.crs()[k][1], idx), k
    assert np.array_equal(r.fields["weightsOnEdge"], f["weightsOnEdge"])
    assert not r.on_sphere and r.Lx == m.Lx
    # a mesh whose cells need 9 edge slots does not fit maxEdges = 8
    wide = str(tmp_path / "wide.nc")
    with NcFile(wide, "w", 2) as g:
        for d, n in (("nCells", 2), ("nEdges", 2), ("nVertices", 2), ("maxEdges", 9)):
            g.def_dim(d, n)
        g.def_var("edgesOnCell", 4, ["nCells", "maxEdges"])
        g.enddef()
        g.put_var("edgesOnCell", np.ones((2, 9), np.int32))
    with pytest.raises(ValueError):
        read_mesh(wide)

