"""Python mirror of the level-set update of the reference's ``LevelSet``
(src/fem/LevelSet.cpp:89-151 with resetPhi_, :429-455) over the C ABI
(``fts_ls_*``): Crank-Nicolson advection of phi by the Stokes velocity with
Jacobi-BiCGSTAB, then the distance reset and the 0.75 / 0.25 mixing.

    ls = LevelSet()
    ls.init(Mesh(xyz, tets))
    ls.update(flow, phi, par)     # phi (float64[np]) updated in place
    f = ls.surface_tension(phi, par)   # Flow::surfaceTension_'s nodal load [3, np]
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
        self._n_nodes = m.np
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

    def reset_values(self) -> np.ndarray:
        """LevelSet::phi_ifn_ (LevelSet.cpp:440): the last update's full
        distance-reset values, before the mixing."""
        out = np.empty(self._np())
        rc = self._lib.fts_ls_reset_values(self._ctx, N.ptr(out, C.c_double))
        if rc != 0:
            raise FtsError(rc, self.last_error())
        return out

    def distance_reset(self, phi: np.ndarray) -> np.ndarray:
        """LevelSet::resetPhi_'s full reset values (phi_ifn_, LevelSet.cpp:440)
        of phi: signed distances to its zero level set's edge crossings.  They
        also become this context's reset values."""
        if not self._ctx:
            raise FtsError(1, "LevelSet.init() has not succeeded")
        phi = np.ascontiguousarray(phi, np.float64)
        out = np.empty(phi.shape[0])
        rc = self._lib.fts_ls_distance_reset(self._ctx, N.ptr(phi, C.c_double),
                                             N.ptr(out, C.c_double))
        if rc != 0:
            raise FtsError(rc, self.last_error())
        return out

    def surface_tension(self, phi: np.ndarray, par: dict,
                        phi_reset: np.ndarray | None = None) -> np.ndarray:
        """Flow::surfaceTension_ (Flow.cpp:307-341) with the LevelSet's
        normals, curvature and interface patches: the nodal load [fx, fy, fz]
        (shape [3, np]) that Flow.solve takes as `force` when "Surface tension"
        > 0.  phi_reset None: the reset values of this context's last update."""
        if not self._ctx:
            raise FtsError(1, "LevelSet.init() has not succeeded")
        phi = np.ascontiguousarray(phi, np.float64)
        pr = None if phi_reset is None else np.ascontiguousarray(phi_reset, np.float64)
        force = np.zeros(3 * phi.shape[0])
        st = A.FtsStStats()
        rc = self._lib.fts_ls_surface_tension(
            self._ctx, N.ptr(phi, C.c_double), None if pr is None else N.ptr(pr, C.c_double),
            float(_par(par, "Surface tension")), int(_par(par, "Node density")),
            N.ptr(force, C.c_double), C.byref(st))
        self.last_st_stats = st.as_dict()
        if rc != 0:
            raise FtsError(rc, self.last_error())
        return force.reshape(3, -1)

    def _np(self) -> int:
        return self._n_nodes

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
