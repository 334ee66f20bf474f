"""ctypes binding of libfts.so (include/fts.h, include/fts_gen.h).

The library is built in-tree by ``fluidtissue_gb300.build``; loading fails
loudly when it is missing — there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

_LIB = None


class FtsGenShape(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("center", C.c_double * 3),
        ("radius", C.c_double),
        ("axes", C.c_double * 3),
        ("center2", C.c_double * 3),
        ("radius2", C.c_double),
    ]


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
    i32, i64, u64, dbl, f32, u8 = C.c_int32, C.c_int64, C.c_uint64, C.c_double, C.c_float, C.c_uint8
    sig = {
        "fts_gen_kuhn_counts": (C.c_int, [i32, _p(i64), _p(i64)]),
        "fts_gen_kuhn_mesh": (C.c_int, [i32, dbl, u64, _p(f32), _p(C.c_int32), _p(u8)]),
        "fts_gen_shape_phi": (dbl, [_p(FtsGenShape), dbl, dbl, dbl]),
        "fts_gen_surface_points": (C.c_int, [_p(FtsGenShape), i32, u64, _p(dbl)]),
        "fts_gen_fields": (C.c_int, [_p(FtsGenShape), i64, i64, _p(f32), _p(C.c_int32), i32,
                                     _p(dbl), dbl, dbl, _p(dbl), _p(dbl), _p(dbl), _p(dbl)]),
        "fts_gen_viscosity": (C.c_int, [i64, _p(dbl), _p(dbl), i32, dbl, dbl, dbl, _p(dbl)]),
        "fts_gen_uniform": (dbl, [u64, u64, u64]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
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
