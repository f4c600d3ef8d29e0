"""Property-based round trips of the netCDF classic reader/writer (host code,
no GPU): random layouts written here and read back, and read by scipy for CDF-1/2."""
import numpy as np
import pytest

from mpaso.mpas_io import NcFile

netcdf_file = pytest.importorskip("scipy.io").netcdf_file

pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

_TYPES = [(1, np.int8), (3, np.int16), (4, np.int32), (5, np.float32), (6, np.float64), (10, np.int64)]


@settings(max_examples=40, deadline=None)
@given(version=st.sampled_from([1, 2, 5]), nrec=st.integers(0, 3),
       dims=st.lists(st.integers(1, 5), min_size=1, max_size=3),
       kinds=st.lists(st.integers(0, len(_TYPES) - 1), min_size=1, max_size=4), seed=st.integers(0, 2**31))
def test_round_trip_any_layout(tmp_path_factory, version, nrec, dims, kinds, seed):
    """Random dimensions, types (int64 only in CDF-5), fixed and record variables
    (including the unpadded lone small-type record variable): written here, read
    back identical; for CDF-1/2 scipy reads the same values."""
    rng = np.random.default_rng(seed)
    path = str(tmp_path_factory.mktemp("nc") / "r.nc")
    names = [f"d{i}" for i in range(len(dims))]
    vars_ = {}
    with NcFile(path, "w", version) as f:
        f.def_dim("rec", 0)
        for n, d in zip(names, dims):
            f.def_dim(n, d)
        for j, kind in enumerate(kinds):
            code, dt = _TYPES[kind]
            if code == 10 and version != 5:
                code, dt = 4, np.int32
            rec = (j % 2 == 1)
            vd = (["rec"] if rec else []) + names[: 1 + j % len(names)]
            shape = ((nrec,) if rec else ()) + tuple(dims[: 1 + j % len(names)])
            a = (rng.standard_normal(shape) * 100).astype(dt) if np.dtype(dt).kind == "f" else \
                rng.integers(np.iinfo(dt).min // 2, np.iinfo(dt).max // 2, size=shape, dtype=np.int64).astype(dt)
            f.def_var(f"v{j}", code, vd)
            vars_[f"v{j}"] = (a, rec)
        f.enddef()
        for n, (a, rec) in vars_.items():
            if rec:
                for r in range(nrec):
                    f.put_rec(n, r, a[r])
            else:
                f.put_var(n, a)
    with NcFile(path) as g:
        assert g.numrecs == (nrec if any(rec for _, rec in vars_.values()) else 0)
        for n, (a, rec) in vars_.items():
            got = g.get_var(n)
            assert got.dtype == a.dtype and np.array_equal(got, a), n
    if version in (1, 2):
        with netcdf_file(path, "r", mmap=False) as s:
            for n, (a, rec) in vars_.items():
                if a.size:
                    assert np.array_equal(s.variables[n][:], a), n
