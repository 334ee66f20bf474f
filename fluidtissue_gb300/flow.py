"""Host-side mirror of the reference's ``Flow`` class over the C ABI.

``Flow.init(mesh, par)`` and ``Flow.solve(phi, source, flow)`` keep the
reference's names, argument meaning and return convention (0 on success,
non-zero on failure; early exits leave ``flow`` untouched), see
src/growth/Flow.hpp:15-63 and src/growth/Flow.cpp:20-94.  ``par`` uses the
reference's parameter-file keys; a missing key reads as 0.0 with a warning,
as ``Parameters::operator[]`` does (src/common/Parameters.hpp:24-34).

All arithmetic runs in libfts.so on the GPU; this module only marshals
arrays.  It raises if the CUDA library is missing.
"""
from __future__ import annotations

import ctypes as C
import sys
from dataclasses import dataclass

import numpy as np

from . import _api as A
from . import _native as N

PREC = {"fp64": A.PREC_FP64, "mixed": A.PREC_MIXED}
PC = {"auto": A.PC_AUTO, "jacobi": A.PC_JACOBI, "multigrid": A.PC_MULTIGRID,
      "multigrid_diag": A.PC_MULTIGRID_DIAG}
SOLVER = {"minres": A.SOLVER_MINRES, "bicgstab": A.SOLVER_BICGSTAB}
OP = {"auto": A.OP_AUTO, "assembled": A.OP_ASSEMBLED, "matfree": A.OP_MATFREE,
      "stencil": A.OP_STENCIL}


@dataclass
class Mesh:
    """Mesh3D's data (src/fem/TetraMesh.hpp:49-62): float node coordinates,
    tetrahedra, and optionally the Dirichlet (exterior boundary) node flags."""
    xyz: np.ndarray
    tets: np.ndarray
    boundary: np.ndarray | None = None

    def __post_init__(self):
        self.xyz = np.ascontiguousarray(self.xyz, np.float32).reshape(-1, 3)
        self.tets = np.ascontiguousarray(self.tets, np.int32).reshape(-1, 4)
        if self.boundary is not None:
            self.boundary = np.ascontiguousarray(self.boundary, np.uint8)


class FtsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{A.STATUS.get(status, status)}: {msg}")
        self.status = status


def _par(par: dict, key: str) -> float:
    if key not in par:
        print(f"** Warning: Parameter '{key}' not defined. Defaulting to value 0.0.",
              file=sys.stderr)
        return 0.0
    return float(par[key])


def make_params(par: dict, precision="fp64", preconditioner="auto", operator="auto",
                warm_start=True, device=0, inner_tol=0.0, verbose=False,
                time_kernels=False, solver="minres") -> A.FtsParams:
    """fts_params from reference parameter keys plus GB300 options."""
    lib = N.load()
    p = A.FtsParams()
    lib.fts_params_default(C.byref(p))
    p.velocity_degree = int(_par(par, "Stokes velocity degree"))
    p.alpha = _par(par, "alpha")
    p.eps = _par(par, "eps")
    p.tol = _par(par, "Stokes tolerance")
    p.max_iter = int(_par(par, "Max. CG iterations"))
    p.mu_interior = _par(par, "Viscosity interior")
    p.mu_exterior = _par(par, "Viscosity exterior")
    p.mu_profile = int(_par(par, "Viscosity profile"))
    p.gf_growth = _par(par, "GF growth")
    p.level_sink = _par(par, "Level sink")
    p.growth_threshold = _par(par, "Growth threshold")
    p.rd_iterations = _par(par, "RD iterations")
    p.gf_production = par.get("GF production", 1.0) if p.rd_iterations <= 0 else _par(
        par, "GF production")
    p.advection_dt = _par(par, "Advection dt")
    p.surface_tension = _par(par, "Surface tension")
    p.precision = PREC[precision]
    p.solver = SOLVER[solver]
    p.preconditioner = PC[preconditioner]
    p.operator_kind = OP[operator]
    p.warm_start = 1 if warm_start else 0
    p.device = int(device)
    p.inner_tol = float(inner_tol)
    p.verbose = 1 if verbose else 0
    p.time_kernels = 1 if time_kernels else 0
    return p


class Flow:
    """Stokes solver with the interface of the reference's ``Flow``."""

    def __init__(self):
        self._lib = N.load()
        self._ctx = C.c_void_p()
        self.np = 0
        self.nt = 0
        self.last_stats: dict = {}

    # Flow::init (Flow.cpp:20-85)
    def init(self, mesh: Mesh, par: dict, **options) -> int:
        self.close()
        p = make_params(par, **options)
        m = A.FtsMesh()
        m.np = mesh.xyz.shape[0]
        m.nt = mesh.tets.shape[0]
        m.xyz = N.ptr(mesh.xyz, C.c_float)
        m.tets = N.ptr(mesh.tets, C.c_int32)
        m.boundary = N.ptr(mesh.boundary, C.c_uint8)
        self._mesh = mesh
        rc = self._lib.fts_create(C.byref(m), C.byref(p), C.byref(self._ctx))
        if rc != 0:
            self._ctx = C.c_void_p()
            self.error = self._lib.fts_last_error(None).decode()
            return rc
        self.np, self.nt = m.np, m.nt
        return 0

    def _check(self):
        if not self._ctx:
            raise FtsError(1, "Flow.init() has not succeeded")

    # Flow::solve (Flow.cpp:89-94)
    def solve(self, phi, source, flow: np.ndarray, mu=None, force=None) -> int:
        self._check()
        phi = np.ascontiguousarray(phi, np.float64)
        source = np.ascontiguousarray(source, np.float64)
        mu = None if mu is None else np.ascontiguousarray(mu, np.float64)
        force = None if force is None else np.ascontiguousarray(force, np.float64)
        if phi.shape != (self.np,) or source.shape != (self.np,):
            raise FtsError(1, "phi and source must have one value per node")
        if mu is not None and mu.shape != (self.nt,):
            raise FtsError(1, "mu must have one value per tetrahedron")
        if force is not None and force.size != 3 * self.np:
            raise FtsError(1, "force must have 3 * np values")
        if flow.dtype != np.float64 or flow.size != 4 * self.np or not flow.flags["C_CONTIGUOUS"]:
            raise FtsError(1, "flow must be a contiguous float64 array of 4 * np values")
        st = A.FtsStats()
        D = C.c_double
        rc = self._lib.fts_solve(self._ctx, N.ptr(phi, D), N.ptr(source, D), N.ptr(mu, D),
                                 N.ptr(force, D), N.ptr(flow, D), C.byref(st))
        self.last_stats = st.as_dict()
        return rc

    def solve_device(self, phi_ptr: int, source_ptr: int, mu_ptr: int | None, flow_ptr: int,
                     force_ptr: int | None = None) -> int:
        """fts_solve_device on device pointers (e.g. torch ``data_ptr()``)."""
        self._check()
        st = A.FtsStats()
        rc = self._lib.fts_solve_device(self._ctx, phi_ptr, source_ptr, mu_ptr or None,
                                        force_ptr or None, flow_ptr, C.byref(st))
        self.last_stats = st.as_dict()
        return rc

    def set_stream(self, stream_handle: int | None) -> int:
        self._check()
        return self._lib.fts_set_stream(self._ctx, stream_handle or None)

    def update_params(self, par: dict, **options) -> int:
        self._check()
        p = make_params(par, **options)
        return self._lib.fts_update_params(self._ctx, C.byref(p))

    def reset_guess(self) -> int:
        self._check()
        return self._lib.fts_reset_guess(self._ctx)

    def last_error(self) -> str:
        return self._lib.fts_last_error(self._ctx if self._ctx else None).decode()

    def sizes(self):
        self._check()
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        self._lib.fts_get_sizes(self._ctx, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    def system(self):
        """Last assembled block system: (rowptr, cols, vals[nnzb,4,4], rhs[np,4])."""
        npn, nnzb, _ = self.sizes()
        rp = np.empty(npn + 1, np.int32)
        ci = np.empty(nnzb, np.int32)
        vals = np.empty((nnzb, 4, 4))
        rhs = np.empty((npn, 4))
        rc = self._lib.fts_get_system(self._ctx, N.ptr(rp, C.c_int32), N.ptr(ci, C.c_int32),
                                      N.ptr(vals, C.c_double), N.ptr(rhs, C.c_double))
        if rc != 0:
            raise FtsError(rc, self.last_error())
        return rp, ci, vals, rhs

    def apply(self, x: np.ndarray, precision="fp64") -> np.ndarray:
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty_like(x)
        rc = self._lib.fts_apply(self._ctx, PREC[precision], N.ptr(x, C.c_double),
                                 N.ptr(y, C.c_double))
        if rc != 0:
            raise FtsError(rc, self.last_error())
        return y

    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self._lib.fts_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent Stokes solves in one batched call (fts_batch_*): each
    instance is a ``Flow.solve`` of its own mesh, inputs and parameters."""

    def __init__(self, meshes: list[Mesh], pars: list[dict], **options):
        self._lib = N.load()
        self._ctx = C.c_void_p()
        self.count = len(meshes)
        self._meshes = meshes
        ms = (A.FtsMesh * self.count)()
        ps = (A.FtsParams * self.count)()
        for i, (m, par) in enumerate(zip(meshes, pars)):
            ms[i].np = m.xyz.shape[0]
            ms[i].nt = m.tets.shape[0]
            ms[i].xyz = N.ptr(m.xyz, C.c_float)
            ms[i].tets = N.ptr(m.tets, C.c_int32)
            ms[i].boundary = N.ptr(m.boundary, C.c_uint8)
            ps[i] = make_params(par, **options)
        rc = self._lib.fts_batch_create(self.count, ms, ps, C.byref(self._ctx))
        if rc != 0:
            msg = self._lib.fts_batch_last_error(None).decode()
            self._ctx = C.c_void_p()
            raise FtsError(rc, msg)
        self.last_stats: list[dict] = []

    def solve(self, phis, sources, flows, mus=None) -> int:
        D = C.c_double
        arr = lambda xs: (C.POINTER(D) * self.count)(  # noqa: E731
            *[N.ptr(None if x is None else np.ascontiguousarray(x, np.float64), D) for x in xs])
        keep = [np.ascontiguousarray(x, np.float64) for x in phis + sources]
        phis = keep[:self.count]
        sources = keep[self.count:]
        for f in flows:
            assert f.dtype == np.float64 and f.flags["C_CONTIGUOUS"]
        st = (A.FtsStats * self.count)()
        rc = self._lib.fts_batch_solve(self._ctx, arr(phis), arr(sources),
                                       arr(mus) if mus is not None else None, arr(flows), st)
        self.last_stats = [s.as_dict() for s in st]
        return rc

    def solve_device(self, phi_ptrs, source_ptrs, mu_ptrs, flow_ptrs) -> int:
        V = C.c_void_p
        arr = lambda xs: (V * self.count)(*[V(x) if x else V() for x in xs])  # noqa: E731
        st = (A.FtsStats * self.count)()
        rc = self._lib.fts_batch_solve_device(self._ctx, arr(phi_ptrs), arr(source_ptrs),
                                              arr(mu_ptrs) if mu_ptrs is not None else None,
                                              arr(flow_ptrs), st)
        self.last_stats = [s.as_dict() for s in st]
        return rc

    def config(self) -> dict:
        c = A.FtsBatchConfig()
        self._lib.fts_batch_get_config(self._ctx, C.byref(c))
        return c.as_dict()

    def set_stream(self, stream_handle: int | None) -> int:
        return self._lib.fts_batch_set_stream(self._ctx, stream_handle or None)

    def set_barrier_limit(self, seconds: float, absent_block: int = -1) -> int:
        """Longest wait at a grid barrier of the persistent launch; a block
        index >= 0 makes that block leave at its first barrier without
        arriving (failure-detection tests)."""
        return self._lib.fts_batch_set_barrier_limit(self._ctx, float(seconds), int(absent_block))

    def last_error(self) -> str:
        return self._lib.fts_batch_last_error(self._ctx).decode()

    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self._lib.fts_batch_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def status_string(rc: int) -> str:
    return N.load().fts_status_string(rc).decode()
