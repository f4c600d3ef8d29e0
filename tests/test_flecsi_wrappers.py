"""The FleCSI-side wrapper library (mpas-o-flecsi-2.0_gb300/flecsi/): its task
bodies replace the reference's apps/sw/tasks/solve.cc and
apps/ocean/tasks/solve.cc in a build of the reference's own driver logic
through the header shim.  The build links only if every task the driver calls
is defined with the signature the reference declares; the calls then reach
libmpaso (on a host without a GPU they stop at its no-device error).  Needs
the reference checkout, so it runs where the oracle builds; the library's
runs on a GPU are in test_gpu_flecsi_wrappers.py."""
import ctypes
import runpy
import os

import numpy as np
import pytest

import mpaso
from mpaso.initial import sw_state
from oracle import Oracle, ref_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.skipif(not ref_available(1, 1), reason="reference checkout not here")


@pytest.fixture(scope="module")
def wrapped():
    path = runpy.run_path(os.path.join(ROOT, "oracle", "build.py"), run_name="oracle_build")["build_flecsi_wrappers"]()
    lib = ctypes.CDLL(path)
    lib.orc_last_error.restype = ctypes.c_char_p
    return lib


def test_wrappers_define_every_reference_task(wrapped):
    """No task of mpas::sw::task / mpas::ocean::task is left undefined: the
    wrapper bodies matched every declaration the driver's calls resolve to."""
    import subprocess
    path = os.path.join(ROOT, "oracle", "_ref", "libref_gb300_L1_T1.so")
    undefined = subprocess.run(["nm", "-uC", path], capture_output=True, text=True).stdout
    assert "mpas::" not in undefined
    assert "mpaso_sw_compute_tend" in undefined and "mpaso_oc_correct_and_rescale" in undefined


def test_wrappers_reach_libmpaso(wrapped):
    S = Oracle("restatement")
    m = mpaso.Mesh.icosa(2)
    om, st = S.mesh(m), S.static(m)
    err = ctypes.create_string_buffer(512)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    xyz = np.concatenate([m.fields[k] for k in ("xCell", "yCell", "zCell")])
    rc = wrapped.flw_make_context(ctypes.byref(om), ctypes.byref(st), p(xyz), 0, err, 512)
    from mpaso.gpu import device_count
    if device_count() == 0:
        assert rc == 1 and "mpaso_mesh_create" in err.value.decode()
    h, u, tr = sw_state(m, 1, 1, 1)
    if rc != 0:  # the reference driver through the wrappers, without a context
        rc2 = wrapped.orc_sw_run(ctypes.byref(om), ctypes.byref(st), ctypes.byref(S.config(1, 1)),
                                 ctypes.c_double(300.0), 1, p(h), p(u), p(tr))
        assert rc2 == 1 and "make_mesh_context" in wrapped.orc_last_error().decode()


def test_wrappers_refuse_multi_color_runs(wrapped):
    """More than one color (process) is refused before any device work: the
    device mesh context has no halo exchange."""
    S = Oracle("restatement")
    m = mpaso.Mesh.icosa(2)
    om, st = S.mesh(m), S.static(m)
    err = ctypes.create_string_buffer(512)
    xyz = np.concatenate([m.fields[k] for k in ("xCell", "yCell", "zCell")])
    wrapped.flw_set_processes(2)
    try:
        rc = wrapped.flw_make_context(ctypes.byref(om), ctypes.byref(st), xyz.ctypes.data_as(ctypes.c_void_p), 0,
                                      err, 512)
    finally:
        wrapped.flw_set_processes(1)
    assert rc == 1 and "single-color" in err.value.decode()
