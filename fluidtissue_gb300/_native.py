"""ctypes binding of libfts.so (include/fts.h).

The library is built in-tree by ``fluidtissue_gb300.build``; loading fails
loudly when it is missing — there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

_LIB = None


def lib_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = False) -> C.CDLL:
    """Load libfts.so (optionally building it first)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError(
                f"{path} is missing: build it with `python -m fluidtissue_gb300.build` "
                "(the CUDA extension is required; there is no CPU fallback)")
        _build.build()
    lib = C.CDLL(str(path))
    _declare(lib)
    _LIB = lib
    return lib


def _p(t):
    return C.POINTER(t)


def _declare(lib: C.CDLL) -> None:
    try:
        from . import _api
        _api.declare(lib)
    except ImportError:
        pass


def ptr(a: np.ndarray | None, ctype):
    """Pointer to a contiguous numpy array (or NULL)."""
    if a is None:
        return C.POINTER(ctype)()
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(C.POINTER(ctype))
