"""Python mirror of the reference's ``EuclideanDistance`` class
(src/fem/EuclideanDistance.hpp:13-51) over the C ABI (``fts_dist_*``), and the
interface points the reference feeds it (LevelSet::findInterfaceNodes_,
src/fem/LevelSet.cpp:261-300).

    d = EuclideanDistance()
    d.init(xyz)                                 # EuclideanDistance::init (mesh nodes)
    d.resetPhi(ifp, phi_n)                      # phi_n <- +-min_j |ifp_j - p_k|
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _api as A
from . import _native as N
from .flow import FtsError

METHOD = {"pruned": A.DIST_PRUNED, "exhaustive": A.DIST_EXHAUSTIVE}


def mesh_edges(tets: np.ndarray) -> np.ndarray:
    """Unique undirected edges (i < j) of a tetrahedral mesh, sorted."""
    t = np.asarray(tets, np.int64)
    pairs = np.concatenate([t[:, [a, b]] for a in range(4) for b in range(a + 1, 4)])
    pairs.sort(axis=1)
    return np.unique(pairs, axis=0)


def interface_points(xyz: np.ndarray, tets: np.ndarray, phi: np.ndarray):
    """Edge crossings of the zero level set (LevelSet.cpp:278-300): edges whose
    end values differ in sign bit, at t = phi0 / (phi0 - phi1) (0.5 when the
    difference is below FLT_MIN), point (1 - t) p0 + t p1 in double, stored as
    float.  Returns (points float32[n, 3], edges int64[n, 2])."""
    sb = np.signbit(np.asarray(phi))
    t4 = np.asarray(tets, np.int64)
    cross = []
    for a in range(4):
        for b in range(a + 1, 4):
            m = sb[t4[:, a]] != sb[t4[:, b]]
            cross.append(t4[m][:, [a, b]])
    e = np.concatenate(cross)
    e.sort(axis=1)
    e = np.unique(e, axis=0)
    f0, f1 = phi[e[:, 0]], phi[e[:, 1]]
    div = f0 - f1
    t = np.where(np.abs(div) > np.finfo(np.float32).tiny, f0 / np.where(div == 0, 1, div), 0.5)
    p0 = xyz[e[:, 0]].astype(np.float64)
    p1 = xyz[e[:, 1]].astype(np.float64)
    pts = (1.0 - t)[:, None] * p0 + t[:, None] * p1
    return pts.astype(np.float32), e


class EuclideanDistance:
    """EuclideanDistance::init / resetPhi on the GPU."""

    def __init__(self):
        self._lib = N.load()
        self._ctx = C.c_void_p()
        self.last_stats: dict = {}

    def init(self, xyz: np.ndarray, device: int = 0) -> int:
        self.close()
        self._xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
        return self._lib.fts_dist_create(N.ptr(self._xyz, C.c_float), self._xyz.shape[0], device,
                                         C.byref(self._ctx))

    def resetPhi(self, ifp: np.ndarray, phi_n: np.ndarray, method: str = "pruned") -> int:
        """phi_n (float64, in place): +-distance to the nearest interface point."""
        if not self._ctx:
            raise FtsError(1, "EuclideanDistance.init() has not succeeded")
        ifp = np.ascontiguousarray(ifp, np.float32).reshape(-1, 3)
        assert phi_n.dtype == np.float64 and phi_n.flags["C_CONTIGUOUS"]
        st = A.FtsDistStats()
        rc = self._lib.fts_dist_reset(self._ctx, N.ptr(ifp, C.c_float) if len(ifp) else None,
                                      ifp.shape[0], N.ptr(phi_n, C.c_double), METHOD[method],
                                      C.byref(st))
        self.last_stats = st.as_dict()
        return rc

    def last_error(self) -> str:
        return self._lib.fts_dist_last_error(self._ctx if self._ctx else None).decode()

    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self._lib.fts_dist_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass
