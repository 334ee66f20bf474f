"""Python mirror of the level-set update of the reference's ``LevelSet``
(src/fem/LevelSet.cpp:89-151 with resetPhi_, :429-455) over the C ABI
(``fts_ls_*``): Crank-Nicolson advection of phi by the Stokes velocity with
Jacobi-BiCGSTAB, then the distance reset and the 0.75 / 0.25 mixing.

    ls = LevelSet()
    ls.init(Mesh(xyz, tets))
    ls.update(flow, phi, par)     # phi (float64[np]) updated in place
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _api as A
from . import _native as N
from .flow import FtsError, Mesh, _par


def make_ls_params(par: dict, reset: bool = True) -> A.FtsLsParams:
    p = A.FtsLsParams()
    p.dt = _par(par, "Advection dt")
    p.tol = _par(par, "Advection tolerance")
    p.max_iter = int(_par(par, "Max. CG iterations"))
    p.reset = 1 if reset else 0
    return p


class LevelSet:
    """LevelSet::update on the GPU (the mass matrix is assembled at init)."""

    def __init__(self):
        self._lib = N.load()
        self._ctx = C.c_void_p()
        self.last_stats: dict = {}

    def init(self, mesh: Mesh, device: int = 0) -> int:
        self.close()
        m = A.FtsMesh()
        m.np = mesh.xyz.shape[0]
        m.nt = mesh.tets.shape[0]
        m.xyz = N.ptr(mesh.xyz, C.c_float)
        m.tets = N.ptr(mesh.tets, C.c_int32)
        m.boundary = N.ptr(mesh.boundary, C.c_uint8)
        rc = self._lib.fts_ls_create(C.byref(m), device, C.byref(self._ctx))
        if rc != 0:
            self._ctx = C.c_void_p()
        return rc

    def update(self, flow: np.ndarray, phi: np.ndarray, par: dict, reset: bool = True) -> int:
        if not self._ctx:
            raise FtsError(1, "LevelSet.init() has not succeeded")
        flow = np.ascontiguousarray(flow, np.float64)
        assert phi.dtype == np.float64 and phi.flags["C_CONTIGUOUS"]
        p = make_ls_params(par, reset)
        st = A.FtsLsStats()
        rc = self._lib.fts_ls_update(self._ctx, C.byref(p), N.ptr(flow, C.c_double),
                                     N.ptr(phi, C.c_double), C.byref(st))
        self.last_stats = st.as_dict()
        return rc

    def last_error(self) -> str:
        return self._lib.fts_ls_last_error(self._ctx if self._ctx else None).decode()

    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self._lib.fts_ls_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass
