"""GB300-native NeoPZ linear FEM path: assembly and iterative solve on sm_103a.

The compute lives in ``_build/libgpz.so`` (C ABI: include/gpz.h); the host
mesh builder in ``_build/libgpzhost.so``.  ``neopz_gb300.gpz`` is the ctypes
front end.
"""
from . import gpz  # noqa: F401
