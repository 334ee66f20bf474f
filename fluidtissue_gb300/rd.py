"""Python mirror of the reference's ``RD`` class (src/growth/RD.hpp:16-56)
over the C ABI (``fts_rd_*`` in include/fts.h): activator / inhibitor
patterning and the growth factor by explicit Euler on the interior submesh,
all steps in one persistent GPU launch.

    rd = RD()
    rd.init(Mesh(xyz, tets), phi, par)       # RD::init: activator = x + 1 inside
    rd.solve(phi, source_nodes)              # RD::solve: `RD iterations` steps of `RD dt`
    rd.activator, rd.inhibitor, rd.growth_factor
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _api as A
from . import _native as N
from .flow import FtsError, Mesh, _par

# Parameter keys of the reference's parameter files, in fts_rd_params order.
RD_KEYS = ("RD dt", "Act", "Da", "DegA", "Inh", "Di", "DegI", "GF production",
           "GF diffusion", "GF degradation", "GF inhibition")


def make_rd_params(par: dict) -> A.FtsRdParams:
    p = A.FtsRdParams()
    p.dt = _par(par, "RD dt")
    p.iterations = int(_par(par, "RD iterations"))
    p.act, p.da, p.dega = _par(par, "Act"), _par(par, "Da"), _par(par, "DegA")
    p.inh, p.di, p.degi = _par(par, "Inh"), _par(par, "Di"), _par(par, "DegI")
    p.gf_production = _par(par, "GF production")
    p.gf_diffusion = _par(par, "GF diffusion")
    p.gf_degradation = _par(par, "GF degradation")
    p.gf_inhibition = _par(par, "GF inhibition")
    return p


class RD:
    """RD::init / RD::solve and the getters (RD.hpp:22-26)."""

    def __init__(self):
        self._lib = N.load()
        self._ctx = C.c_void_p()
        self.last_stats: dict = {}

    def init(self, mesh: Mesh, phi: np.ndarray, par: dict, device: int = 0) -> int:
        """RD::init (RD.cpp:7-22): zero fields, activator = x + 1 on the
        interior nodes (phi < 0)."""
        self.close()
        m = A.FtsMesh()
        m.np = mesh.xyz.shape[0]
        m.nt = mesh.tets.shape[0]
        m.xyz = N.ptr(mesh.xyz, C.c_float)
        m.tets = N.ptr(mesh.tets, C.c_int32)
        m.boundary = N.ptr(mesh.boundary, C.c_uint8)
        rc = self._lib.fts_rd_create(C.byref(m), device, C.byref(self._ctx))
        if rc != 0:
            self._ctx = C.c_void_p()
            return rc
        self.par = dict(par)
        npn = m.np
        self.activator = np.zeros(npn)
        self.inhibitor = np.zeros(npn)
        self.growth_factor = np.zeros(npn)
        inside = np.asarray(phi) < 0.0
        self.activator[inside] = mesh.xyz[inside, 0].astype(np.float64) + 1.0
        return 0

    def set_state(self, activator, inhibitor, growth_factor) -> None:
        self.activator = np.ascontiguousarray(activator, np.float64).copy()
        self.inhibitor = np.ascontiguousarray(inhibitor, np.float64).copy()
        self.growth_factor = np.ascontiguousarray(growth_factor, np.float64).copy()

    def solve(self, phi: np.ndarray, source_nodes=(), par: dict | None = None) -> int:
        """RD::solve (RD.cpp:27-108) with the growth-factor sources given as
        global node indices (Knots::getSourceNodes); 0 on success."""
        if not self._ctx:
            raise FtsError(1, "RD.init() has not succeeded")
        p = make_rd_params(par if par is not None else self.par)
        phi = np.ascontiguousarray(phi, np.float64)
        src = np.ascontiguousarray(np.asarray(source_nodes, dtype=np.int32))
        st = A.FtsRdStats()
        rc = self._lib.fts_rd_solve(self._ctx, C.byref(p), N.ptr(phi, C.c_double),
                                    N.ptr(src, C.c_int32) if len(src) else None, len(src),
                                    N.ptr(self.activator, C.c_double),
                                    N.ptr(self.inhibitor, C.c_double),
                                    N.ptr(self.growth_factor, C.c_double), C.byref(st))
        self.last_stats = st.as_dict()
        return rc

    def last_error(self) -> str:
        return self._lib.fts_rd_last_error(self._ctx if self._ctx else None).decode()

    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self._lib.fts_rd_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass
