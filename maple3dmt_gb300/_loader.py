"""Loads the in-tree native library (maple3dmt_gb300/_lib/libm3d_gb300.so).

There is no Python or CPU fallback for the solve: if the library is missing,
loading raises, so nothing silently runs another path.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(_HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libm3d_gb300.so")

_lib = None


def load(path: str | None = None) -> ctypes.CDLL:
    """Return the native library, building nothing: call build.build_library() first."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or os.environ.get("M3D_LIB") or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"maple3dmt_gb300 native library not found at {p}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(p, mode=ctypes.RTLD_GLOBAL)
    from . import _abi
    _abi.declare(lib)
    if path is None:
        _lib = lib
    return lib
