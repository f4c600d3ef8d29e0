"""The FleCSI wrapper library (mpas-o-flecsi-2.0_gb300/flecsi/) executing tasks
on the GPU.

The reference's own driver logic (apps/sw/run.cc:13-70 and
apps/ocean/run.cc:10-50, as oracle/ref_driver.cc states them) calls the
wrapper task bodies, which hand the accessors' raw storage (`raw(acc)`: one
vltensor / vltracer per entity, contiguous) to libmpaso's per-task entries on
the device; the copy and zero tasks stay on the host.  Every per-task entry
keeps the reference's rounding, so the run must equal the reference's value for
value; a wrong pointer, stride or field order in a wrapper would show as a
difference.

The wrapper library is compiled on this host from the amalgamated translation
units that oracle/build.py writes beside a reference checkout (a git-ignored
build output); where they are absent the tests skip."""
import ctypes
import os
import runpy

import numpy as np
import pytest

import mpaso
from helpers import Golden
from mpaso.initial import ocean_state
from oracle import Oracle

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def wrapped():
    path = runpy.run_path(os.path.join(ROOT, "oracle", "build.py"), run_name="oracle_build")["build_flecsi_wrappers"]()
    if path is None:
        pytest.skip("no wrapper translation units (oracle/build.py makes them where the reference checkout is)")
    lib = ctypes.CDLL(path)
    lib.orc_last_error.restype = ctypes.c_char_p
    yield lib
    lib.flw_destroy_context()


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def centres(mesh):
    return np.ascontiguousarray(np.concatenate([mesh.fields[k] for k in ("xCell", "yCell", "zCell")]), np.float64)


def _make_context(lib, mesh, om, st, fct):
    err = ctypes.create_string_buffer(512)
    xyz = centres(mesh)
    rc = lib.flw_make_context(ctypes.byref(om), ctypes.byref(st), _p(xyz), ctypes.c_int32(int(fct)), err, 512)
    assert rc == 0, err.value.decode()


def _check(lib, rc):
    assert rc == 0, lib.orc_last_error().decode()


@pytest.mark.parametrize("name", ["sw_fct_icosa3_L1T1", "sw_hex16_L1T1"])
def test_sw_driver_through_wrappers_matches_reference(wrapped, name):
    """The sw driver (with FCT + del2 tracers on the sphere) through the
    wrappers on the GPU reproduces the reference's goldens after 1 and 10
    steps, value for value."""
    g = Golden(name)
    S = Oracle("restatement")
    om, st = S.mesh(g.mesh), S.static(g.mesh, g.fct)
    _make_context(wrapped, g.mesh, om, st, g.fct is not None)
    cfg = S.config(g.L, g.T, **g.opts)
    for n in g.steps:
        h, u, tr = (np.ascontiguousarray(g[k], np.float64).copy() for k in ("h0", "u0", "tr0"))
        _check(wrapped, wrapped.orc_sw_run(ctypes.byref(om), ctypes.byref(st), ctypes.byref(cfg),
                                           ctypes.c_double(g.dt), ctypes.c_int32(n), _p(h), _p(u), _p(tr)))
        for got, key in ((h, f"h_{n}"), (u, f"u_{n}"), (tr, f"tr_{n}")):
            assert np.array_equal(got, g[key]), (key, float(np.abs(got - g[key]).max()))
    wrapped.flw_destroy_context()


def test_ocean_driver_through_wrappers_matches_oracle(wrapped):
    """The ocean driver's FCT + del2 tracer sequence through the wrappers on
    the GPU equals the oracle's run of the same driver over 10 steps (one
    level, one tracer: the wrapper library's compiled sizes)."""
    mesh = mpaso.Mesh.icosa(3)
    S = Oracle("restatement")
    fct = S.fct_statics(mesh, 1)
    om, st = S.mesh(mesh), S.static(mesh, fct)
    _make_context(wrapped, mesh, om, st, True)
    h, hE, u, tr = ocean_state(mesh, 1234, 1, 1)
    cfg = S.config(1, 1, fct=True, hmix=True, kappa=1e4)
    want = S.ocean_run(mesh, st, cfg, 600.0, 10, h, hE, u, tr)
    args = [np.ascontiguousarray(a, np.float64) for a in (h, hE, u)]
    got = np.ascontiguousarray(tr, np.float64).copy()
    _check(wrapped, wrapped.orc_ocean_run(ctypes.byref(om), ctypes.byref(st), ctypes.byref(cfg),
                                          ctypes.c_double(600.0), ctypes.c_int32(10), *[_p(a) for a in args],
                                          _p(got)))
    assert not np.array_equal(got, tr)
    assert np.array_equal(got, want), float(np.abs(got - want).max())
    wrapped.flw_destroy_context()

