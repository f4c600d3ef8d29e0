"""Python binding of libmpaso: the GB300 path of MPAS-O-FleCSI's RK4 tendency tasks.

The product is the C ABI in include/*.h (libmpaso.so); this module is a thin
ctypes layer over it for the test suite, the benchmark and Python callers.
"""
from ._lib import LIB_PATH, MpasoError, check, lib  # noqa: F401
from .mesh import EARTH_RADIUS, OMEGA, Mesh  # noqa: F401
