"""The C ABI library (CPU): it loads without a GPU, exports every function
include/*.h declares, and its host-only entries work."""
import ctypes
import os
import re

import numpy as np

import mpaso
from mpaso._lib import LIB_PATH, lib

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if f.endswith(".h"):
            src = open(os.path.join(INCLUDE, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(mpaso_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_every_declared_function():
    names = declared_functions()
    assert len(names) > 40
    L = ctypes.CDLL(LIB_PATH)
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_no_device_is_reported_cleanly():
    import mpaso.gpu as G
    if G.device_count() > 0:
        return  # with a device present this test has nothing to check
    n = ctypes.c_int32(7)
    assert lib().mpaso_device_count(ctypes.byref(n)) == 0 and n.value == 0
    out = ctypes.c_void_p()
    rc = lib().mpaso_mesh_create(None, 0, ctypes.byref(out))
    assert rc != 0


def test_host_entries_and_error_codes():
    h = ctypes.c_void_p()
    assert lib().mpaso_genmesh_hex(3, 3, ctypes.c_double(1.0), ctypes.c_double(0.0), ctypes.byref(h)) != 0
    assert b"ny even" in lib().mpaso_last_error()
    m = mpaso.Mesh.hex(8, 8, 1e3)
    assert lib().mpaso_genmesh_field(m._h, b"noSuchField", None, None, None) == 5  # MPASO_ERR_NOTFOUND
    assert set(m.fields) >= {"weightsOnEdge", "kiteAreasOnVertex", "edgesOnEdge"}
    assert np.all(m.fields["nEdgesOnEdge"] == 10)
