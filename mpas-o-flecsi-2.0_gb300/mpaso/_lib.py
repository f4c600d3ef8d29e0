"""ctypes loader for libmpaso.so (built in-tree by build.py)."""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(_HERE)
LIB_PATH = os.path.join(PKG, "lib", "libmpaso.so")

_lib = None


class MpasoError(RuntimeError):
    """Nonzero status from a libmpaso call; `code` is the MPASO_ERR_* value."""

    def __init__(self, code, msg):
        super().__init__(f"[mpaso error {code}] {msg}")
        self.code = code


def lib():
    """Returns the loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MpasoError(-1, f"{LIB_PATH} is missing: run build.py (or __graft_entry__.build())")
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.mpaso_last_error.restype = ctypes.c_char_p
        _lib.mpaso_genmesh_names.restype = ctypes.c_char_p
    return _lib


def check(status):
    if status != 0:
        raise MpasoError(status, lib().mpaso_last_error().decode())
    return status
