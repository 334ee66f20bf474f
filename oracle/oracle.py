"""ORACLE — test infrastructure only (Python side of oracle/fts_oracle.cpp).

CPU restatement of fluidtissue's Stokes step (src/growth/Flow.cpp:89-402 with
src/fem/Assembler.hpp:134-229, :430-462), used to check the CUDA path and as
the timed CPU baseline.  Parity unpinned: the reference cannot be built here
(Eigen/CGAL/TBB/GMP absent) and ships no golden vectors; the oracle is pinned
by known-answer identities and a direct sparse solve in tests/.

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference arm import this module.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libfts_oracle.so"
_lib = None

FLT_MIN = float(np.finfo(np.float32).tiny)


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def _p(t):
    return C.POINTER(t)


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        build()
    L = C.CDLL(str(LIB))
    i64, dbl, i32, u8, f32 = C.c_int64, C.c_double, C.c_int32, C.c_uint8, C.c_float
    sig = {
        "ora_ref_tables": (None, [_p(dbl), _p(dbl)]),
        "ora_num_threads": (C.c_int, []),
        "ora_set_threads": (None, [C.c_int]),
        "ora_boundary_nodes": (C.c_int, [i64, i64, _p(i32), _p(u8)]),
        "ora_set_viscosity": (C.c_int, [i64, i64, _p(i32), _p(dbl), _p(dbl), dbl, dbl, C.c_int,
                                        dbl, dbl, _p(dbl), _p(dbl)]),
        "ora_source": (C.c_int, [i64, _p(dbl), _p(dbl), dbl, dbl, dbl, _p(dbl)]),
        "ora_block_pattern_size": (C.c_int, [i64, i64, _p(i32), _p(i64)]),
        "ora_assemble_blocks": (C.c_int, [i64, i64, _p(f32), _p(i32), _p(dbl), _p(dbl), _p(dbl),
                                          dbl, dbl, _p(i64), _p(i32), _p(dbl), _p(dbl)]),
        "ora_reduced_size": (C.c_int, [i64, _p(i64), _p(i32), _p(u8), _p(i64), _p(i64)]),
        "ora_reduce": (C.c_int, [i64, _p(i64), _p(i32), _p(dbl), _p(dbl), _p(u8), _p(i64),
                                 _p(i32), _p(dbl), _p(dbl), _p(i32)]),
        "ora_spmv": (C.c_int, [i64, _p(i64), _p(i32), _p(dbl), _p(dbl), _p(dbl)]),
        "ora_bicgstab": (C.c_int, [i64, _p(i64), _p(i32), _p(dbl), _p(dbl), _p(dbl), dbl, i64,
                                   _p(i64), _p(dbl)]),
        "ora_true_residual": (dbl, [i64, _p(i64), _p(i32), _p(dbl), _p(dbl), _p(dbl)]),
        "ora_scatter": (C.c_int, [i64, i64, _p(i32), _p(dbl), _p(dbl)]),
        "ora_now_ms": (dbl, []),
        "ora_minres_tight": (dbl, [i64, i64, _p(i64), _p(i32), _p(dbl), _p(dbl), _p(dbl),
                                   _p(dbl), dbl, i64, C.c_int, _p(i64)]),
        "ora_minres_blockjacobi": (dbl, [i64, i64, _p(i64), _p(i32), _p(dbl), _p(dbl), _p(dbl),
                                         _p(dbl), dbl, _p(dbl), dbl, i64, _p(i64)]),
        "ora_rd_solve": (C.c_int, [i64, i64, _p(f32), _p(i32), _p(dbl), _p(i32), i32, _p(dbl),
                                   i64, _p(dbl), _p(dbl), _p(dbl)]),
        "ora_dist_reset": (C.c_int, [i64, _p(f32), _p(f32), i32, i64, i64, _p(dbl)]),
        "ora_ls_update": (C.c_int, [i64, i64, _p(f32), _p(i32), _p(dbl), _p(dbl), dbl, dbl, i64,
                                    C.c_int, _p(i64), _p(dbl), _p(i64)]),
        "ora_surface_tension": (C.c_int, [i64, i64, _p(f32), _p(i32), _p(dbl), _p(dbl), dbl,
                                          i32, _p(dbl), _p(i64), _p(dbl)]),
        "ora_p2_build": (C.c_void_p, [i64, i64, _p(f32), _p(i32), _p(u8), _p(dbl), _p(dbl),
                                      _p(dbl), dbl, _p(i64), _p(i64), _p(i64)]),
        "ora_p2_fetch": (None, [C.c_void_p, _p(i64), _p(i32), _p(dbl), _p(dbl), _p(i64)]),
        "ora_p2_free": (None, [C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _ptr(a, t):
    if a is None:
        return C.POINTER(t)()
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(t))


D, I32, I64, U8, F32 = C.c_double, C.c_int32, C.c_int64, C.c_uint8, C.c_float


def ref_tables():
    tab = np.empty(16)
    qw = C.c_double()
    lib().ora_ref_tables(_ptr(tab, D), C.byref(qw))
    return tab.reshape(4, 4), qw.value


def set_threads(n: int) -> None:
    lib().ora_set_threads(int(n))


def num_threads() -> int:
    return int(lib().ora_num_threads())


def boundary_nodes(npn, tets):
    bnd = np.empty(npn, np.uint8)
    t = np.ascontiguousarray(tets, np.int32)
    if lib().ora_boundary_nodes(npn, t.shape[0], _ptr(t, I32), _ptr(bnd, U8)) != 0:
        raise ValueError("tetrahedron index out of range")
    return bnd


def set_viscosity(tets, phi, gf, mu_int, mu_ext, profile, rd_iterations=0.0, gf_production=1.0):
    t = np.ascontiguousarray(tets, np.int32)
    mu = np.empty(t.shape[0])
    mm = np.empty(2)
    lib().ora_set_viscosity(phi.shape[0], t.shape[0], _ptr(t, I32), _ptr(phi, D), _ptr(gf, D),
                            mu_int, mu_ext, int(profile), rd_iterations, gf_production,
                            _ptr(mu, D), _ptr(mm, D))
    return mu, mm


def source(phi, c, gf_growth, level_sink=0.0, threshold=0.0):
    s = np.empty(phi.shape[0])
    lib().ora_source(phi.shape[0], _ptr(phi, D), _ptr(c, D), gf_growth, level_sink, threshold,
                     _ptr(s, D))
    return s


@dataclass
class Blocks:
    rowptr: np.ndarray   # int64 [np+1]
    cols: np.ndarray     # int32 [nnzb]
    vals: np.ndarray     # float64 [nnzb, 4, 4], reference sign convention
    rhs: np.ndarray      # float64 [np, 4]


def assemble_blocks(xyz, tets, mu, s, alpha, eps, fst=None) -> Blocks:
    L = lib()
    x = np.ascontiguousarray(xyz, np.float32)
    t = np.ascontiguousarray(tets, np.int32)
    npn, nt = x.shape[0], t.shape[0]
    nnzb = C.c_int64()
    L.ora_block_pattern_size(npn, nt, _ptr(t, I32), C.byref(nnzb))
    rp = np.empty(npn + 1, np.int64)
    ci = np.empty(nnzb.value, np.int32)
    vals = np.empty((nnzb.value, 4, 4))
    rhs = np.empty((npn, 4))
    f = None if fst is None else np.ascontiguousarray(fst, np.float64)
    rc = L.ora_assemble_blocks(npn, nt, _ptr(x, F32), _ptr(t, I32), _ptr(mu, D), _ptr(s, D),
                               _ptr(f, D), alpha, eps, _ptr(rp, I64), _ptr(ci, I32),
                               _ptr(vals, D), _ptr(rhs, D))
    if rc == 2:
        raise ValueError("degenerate element")
    return Blocks(rp, ci, vals, rhs)


@dataclass
class Reduced:
    rowptr: np.ndarray
    cols: np.ndarray
    vals: np.ndarray
    F: np.ndarray
    sidx: np.ndarray
    np_: int

    @property
    def N(self) -> int:
        return self.F.shape[0]

    def scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.vals, self.cols, self.rowptr), shape=(self.N, self.N))


def reduce(B: Blocks, bnd) -> Reduced:
    L = lib()
    npn = B.rowptr.shape[0] - 1
    N, nnz = C.c_int64(), C.c_int64()
    L.ora_reduced_size(npn, _ptr(B.rowptr, I64), _ptr(B.cols, I32), _ptr(bnd, U8),
                       C.byref(N), C.byref(nnz))
    rrp = np.empty(N.value + 1, np.int64)
    rci = np.empty(nnz.value, np.int32)
    rv = np.empty(nnz.value)
    rF = np.empty(N.value)
    sidx = np.empty(N.value, np.int32)
    L.ora_reduce(npn, _ptr(B.rowptr, I64), _ptr(B.cols, I32), _ptr(B.vals, D), _ptr(B.rhs, D),
                 _ptr(bnd, U8), _ptr(rrp, I64), _ptr(rci, I32), _ptr(rv, D), _ptr(rF, D),
                 _ptr(sidx, I32))
    return Reduced(rrp, rci, rv, rF, sidx, npn)


def spmv(R: Reduced, x):
    y = np.empty(R.N)
    lib().ora_spmv(R.N, _ptr(R.rowptr, I64), _ptr(R.cols, I32), _ptr(R.vals, D), _ptr(x, D),
                   _ptr(y, D))
    return y


def bicgstab(R: Reduced, x0=None, tol=1e-10, maxit=-1):
    """Eigen-style un-preconditioned BiCGSTAB (Flow.hpp:62); returns (x, info, iters, err)."""
    x = np.zeros(R.N) if x0 is None else np.array(x0, np.float64, copy=True)
    it, err = C.c_int64(), C.c_double()
    info = lib().ora_bicgstab(R.N, _ptr(R.rowptr, I64), _ptr(R.cols, I32), _ptr(R.vals, D),
                              _ptr(R.F, D), _ptr(x, D), tol, maxit, C.byref(it), C.byref(err))
    return x, info, it.value, err.value


def true_residual(R: Reduced, x) -> float:
    return float(lib().ora_true_residual(R.N, _ptr(R.rowptr, I64), _ptr(R.cols, I32),
                                         _ptr(R.vals, D), _ptr(R.F, D), _ptr(x, D)))


def scatter(R: Reduced, x):
    flow = np.empty(4 * R.np_)
    lib().ora_scatter(R.np_, R.N, _ptr(R.sidx, I32), _ptr(x, D), _ptr(flow, D))
    return flow


def now_ms() -> float:
    return float(lib().ora_now_ms())


def params_get(par: dict, key: str) -> float:
    """Parameters::operator[] (src/common/Parameters.hpp:24-34): missing -> 0.0."""
    return float(par.get(key, 0.0))


def system(xyz, tets, boundary, phi, c, mu, par, fst=None):
    """Assembled reduced system and RHS exactly as Flow::Stokes_ builds them."""
    g = lambda k: params_get(par, k)  # noqa: E731
    if mu is None:
        mu, _ = set_viscosity(tets, phi, c, g("Viscosity interior"), g("Viscosity exterior"),
                              int(g("Viscosity profile")), g("RD iterations"), g("GF production"))
    s = source(phi, c, g("GF growth"), g("Level sink"), g("Growth threshold"))
    B = assemble_blocks(xyz, tets, mu, s, g("alpha"), g("eps"), fst)
    return reduce(B, boundary), B, s, mu


def direct_solve(R: Reduced):
    """SuperLU solve of the reduced system (a cross-check independent of Krylov)."""
    import scipy.sparse.linalg as spla
    return spla.spsolve(R.scipy().tocsc(), R.F)


def schur_diag_weights(R: Reduced, xyz, tets, mu):
    """Inverse diagonal weights of the SPD block-diagonal preconditioner used by
    the tight solve: |diag| on velocity rows; on pressure rows the diagonal of
    alpha D + eps M plus the lumped 1/mu-weighted mass (a Schur-complement
    estimate)."""
    npn = R.np_
    nI = (R.N - npn) // 3
    A = R.scipy()
    d = A.diagonal()
    P = np.asarray(xyz, np.float64)[np.asarray(tets)]
    Bm = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=2)
    vol = np.abs(np.linalg.det(Bm)) / 6.0
    w = np.zeros(npn)
    np.add.at(w, np.asarray(tets).ravel(), np.repeat(vol / (4.0 * mu), 4))
    return np.concatenate([1.0 / np.abs(d[:3 * nI]), 1.0 / (d[3 * nI:] + w)]), nI


def solve_tight(R: Reduced, xyz, tets, mu, x0=None, tol=1e-13, maxit=2_000_000,
                max_restarts=30):
    """Tightly converged solution of the reduced system (parity target):
    preconditioned MINRES on the symmetric form, restarted on the true residual
    until ||b - A x|| / ||b|| <= tol.  Returns (x, true_rel_residual, iters)."""
    minv, nI = schur_diag_weights(R, xyz, tets, mu)
    x = np.zeros(R.N) if x0 is None else np.array(x0, np.float64, copy=True)
    it = C.c_int64()
    tr = lib().ora_minres_tight(R.N, nI, _ptr(R.rowptr, I64), _ptr(R.cols, I32),
                                _ptr(R.vals, D), _ptr(R.F, D), _ptr(minv, D), _ptr(x, D), tol,
                                maxit, max_restarts, C.byref(it))
    return x, float(tr), it.value


def block_jacobi(R: Reduced, xyz, tets, mu, eps):
    """The GPU Jacobi-mode preconditioner on the reduced system: inverse 3x3
    velocity blocks per interior node, pressure weights 1/(|A_pp| + lumped
    mass/mu), and the rank-one weight 1/(eps * volume)."""
    npn = R.np_
    nI = (R.N - npn) // 3
    A = R.scipy().tocsr()
    idx = np.arange(nI)
    blocks = np.empty((nI, 3, 3))
    for a in range(3):
        for c in range(3):
            blocks[:, a, c] = np.asarray(A[a * nI + idx, c * nI + idx]).ravel()
    blocks = 0.5 * (blocks + blocks.transpose(0, 2, 1))
    inv = np.linalg.inv(blocks)
    vinv6 = np.ascontiguousarray(np.stack([inv[:, 0, 0], inv[:, 0, 1], inv[:, 0, 2],
                                           inv[:, 1, 1], inv[:, 1, 2], inv[:, 2, 2]], axis=1))
    P = np.asarray(xyz, np.float64)[np.asarray(tets)]
    Bm = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=2)
    vol = np.abs(np.linalg.det(Bm)) / 6.0
    w = np.zeros(npn)
    np.add.at(w, np.asarray(tets).ravel(), np.repeat(vol / (4.0 * mu), 4))
    d = A.diagonal()[3 * nI:]
    pinv = 1.0 / (np.abs(d) + w)
    crank = 1.0 / (eps * vol.sum()) if eps > 0 else 0.0
    return vinv6, pinv, crank, nI


def minres_blockjacobi(R: Reduced, pre, x0=None, rtol=1e-10, maxit=1000):
    """MINRES iterations with the block-Jacobi preconditioner (CPU baseline)."""
    vinv6, pinv, crank, nI = pre
    x = np.zeros(R.N) if x0 is None else np.array(x0, np.float64, copy=True)
    it = C.c_int64()
    red = lib().ora_minres_blockjacobi(R.N, nI, _ptr(R.rowptr, I64), _ptr(R.cols, I32),
                                       _ptr(R.vals, D), _ptr(R.F, D), _ptr(vinv6, D),
                                       _ptr(pinv, D), crank, _ptr(x, D), rtol, maxit,
                                       C.byref(it))
    return x, float(red), it.value


def flow_solve(xyz, tets, boundary, phi, c, mu, par, x_warm=None, flow=None):
    """Flow::solve restated (src/growth/Flow.cpp:89-94, :218-302): returns
    (status, flow, x_reduced, info dict).  Early exits leave ``flow`` as given."""
    g = lambda k: params_get(par, k)  # noqa: E731
    npn = xyz.shape[0]
    flow = np.zeros(4 * npn) if flow is None else flow
    info = {"iterations": 0, "error": 0.0, "exit": None}
    if (g("Viscosity interior") - g("Viscosity exterior") > FLT_MIN and g("RD iterations") > 0.0
            and np.max(np.abs(c)) <= FLT_MIN):
        info["exit"] = "zero source with variable viscosity"
        return 0, flow, x_warm, info
    if g("Advection dt") < FLT_MIN:
        info["exit"] = "advection dt zero"
        return 0, flow, x_warm, info
    if g("Surface tension") > 0.0:
        raise NotImplementedError("surface tension is outside the restated path")
    t0 = now_ms()
    R, B, s, mu = system(xyz, tets, boundary, phi, c, mu, par)
    info["ms_assembly"] = now_ms() - t0
    if np.linalg.norm(R.F) <= FLT_MIN:
        info["exit"] = "load zero"
        return 0, flow, x_warm, info
    tol = g("Stokes tolerance")
    maxit = int(g("Max. CG iterations"))
    t0 = now_ms()
    x, st, it, err = bicgstab(R, x_warm, tol=tol if tol > 0 else float(np.finfo(float).eps),
                              maxit=maxit if maxit > 0 else -1)
    info.update(iterations=it, error=err, ms_solve=now_ms() - t0)
    if st != 0:
        return -1, flow, x, info
    flow[:] = scatter(R, x)
    return 0, flow, x, info


# Reaction-diffusion parameter keys (the reference's parameter files), in the
# order ora_rd_solve takes them.
RD_KEYS = ("RD dt", "Act", "Da", "DegA", "Inh", "Di", "DegI", "GF production",
           "GF diffusion", "GF degradation", "GF inhibition")


def rd_solve(xyz, tets, phi, src_nodes, par, act, inh, gf):
    """RD::solve restated (src/growth/RD.cpp:27-108): advances (act, inh, gf)
    in place by ``RD iterations`` explicit Euler steps; returns the status."""
    prm = np.array([params_get(par, k) for k in RD_KEYS], np.float64)
    iters = int(params_get(par, "RD iterations"))
    src = np.ascontiguousarray(src_nodes, np.int32)
    for a in (act, inh, gf):
        assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return lib().ora_rd_solve(xyz.shape[0], tets.shape[0], _ptr(xyz, F32), _ptr(tets, I32),
                              _ptr(np.ascontiguousarray(phi, np.float64), D), _ptr(src, I32),
                              len(src), _ptr(prm, D), iters, _ptr(act, D), _ptr(inh, D),
                              _ptr(gf, D))


def dist_reset(xyz, ifp, phi_n, k0=0, k1=None):
    """EuclideanDistance::resetPhi restated (host path): phi_n updated in place
    for nodes k0 <= k < k1; returns the status."""
    xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    ifp = np.ascontiguousarray(ifp, np.float32).reshape(-1, 3)
    assert phi_n.dtype == np.float64 and phi_n.flags["C_CONTIGUOUS"]
    k1 = xyz.shape[0] if k1 is None else k1
    return lib().ora_dist_reset(xyz.shape[0], _ptr(xyz, F32), _ptr(ifp, F32), ifp.shape[0], k0,
                                k1, _ptr(phi_n, D))


def ls_update(xyz, tets, flow, phi, dt, tol=1e-6, maxit=0, reset=True):
    """LevelSet::update restated (advection + distance reset + mixing): phi
    updated in place; returns (status, iterations, error, interface points)."""
    assert phi.dtype == np.float64 and phi.flags["C_CONTIGUOUS"]
    flow = np.ascontiguousarray(flow, np.float64)
    it, err, nif = C.c_int64(), C.c_double(), C.c_int64()
    st = lib().ora_ls_update(xyz.shape[0], tets.shape[0], _ptr(xyz, F32), _ptr(tets, I32),
                             _ptr(flow, D), _ptr(phi, D), dt, tol, maxit, 1 if reset else 0,
                             C.byref(it), C.byref(err), C.byref(nif))
    return st, it.value, err.value, nif.value


def p2_edges(tets):
    """The P2 edge DOFs in the oracle's numbering: pairs (i < j) of the node
    graph in row order (DOF np + e is the midpoint of edge e)."""
    t = np.asarray(tets, np.int64)
    pairs = np.concatenate([t[:, [a, b]] for a, b in ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3),
                                                      (2, 3))])
    pairs.sort(axis=1)
    return np.unique(pairs, axis=0)


def p2_system(xyz, tets, boundary, phi, c, mu, par, fst=None, full=False):
    """The P2-P1 system of Flow::Stokes_ with velocity degree 2, in the
    reference's form, restricted to sidx: (scipy CSR A, F, sidx, nd); full:
    the unrestricted matrix and load instead."""
    import scipy.sparse as sp
    g = lambda k: params_get(par, k)  # noqa: E731
    xyz = np.ascontiguousarray(xyz, np.float32)
    tets = np.ascontiguousarray(tets, np.int32)
    npn = xyz.shape[0]
    s = source(phi, c, g("GF growth"), g("Level sink"), g("Growth threshold"))
    bnd = np.ascontiguousarray(boundary, np.uint8)
    mu = np.ascontiguousarray(mu, np.float64)
    s_raw = np.ascontiguousarray(s, np.float64)
    f = None if fst is None else np.ascontiguousarray(fst, np.float64)
    ntrip, nd, nred = C.c_int64(), C.c_int64(), C.c_int64()
    L = lib()
    h = L.ora_p2_build(npn, tets.shape[0], _ptr(xyz, F32), _ptr(tets, I32), _ptr(bnd, U8),
                       _ptr(mu, D), _ptr(s_raw, D), _ptr(f, D), g("eps"), C.byref(ntrip),
                       C.byref(nd), C.byref(nred))
    try:
        rows = np.empty(ntrip.value, np.int64)
        cols = np.empty(ntrip.value, np.int32)
        vals = np.empty(ntrip.value)
        F = np.empty(3 * nd.value + npn)
        sidx = np.empty(nred.value, np.int64)
        L.ora_p2_fetch(h, _ptr(rows, I64), _ptr(cols, I32), _ptr(vals, D), _ptr(F, D),
                       _ptr(sidx, I64))
    finally:
        L.ora_p2_free(h)
    n = 3 * nd.value + npn
    A = sp.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsr()
    A.sum_duplicates()
    if full:
        return A, F, sidx, nd.value
    return A[sidx][:, sidx].tocsr(), F[sidx], sidx, nd.value


def p2_flow(xyz, tets, boundary, phi, c, mu, par, fst=None):
    """Direct solve of the P2-P1 reduced system, scattered as Flow.cpp:290-300:
    [ux, uy, uz, p] at the vertices (boundary velocity 0)."""
    import scipy.sparse.linalg as spla
    A, F, sidx, nd = p2_system(xyz, tets, boundary, phi, c, mu, par, fst)
    x = spla.spsolve(A.tocsc(), F)
    npn = xyz.shape[0]
    full = np.zeros(3 * nd + npn)
    full[sidx] = x
    flow = np.concatenate([full[0:npn], full[nd:nd + npn], full[2 * nd:2 * nd + npn],
                           full[3 * nd:3 * nd + npn]])
    return flow, A, F


def surface_tension(xyz, tets, phi, phi_reset, st, rho):
    """Flow::surfaceTension_ with its LevelSet inputs restated: returns
    (force[3, np] as [fx, fy, fz], interface points, total patch area)."""
    xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    tets = np.ascontiguousarray(tets, np.int32)
    phi = np.ascontiguousarray(phi, np.float64)
    phi_reset = np.ascontiguousarray(phi_reset, np.float64)
    npn = xyz.shape[0]
    force = np.zeros(3 * npn)
    nif, area = C.c_int64(), C.c_double()
    st_ = lib().ora_surface_tension(npn, tets.shape[0], _ptr(xyz, F32), _ptr(tets, I32),
                                    _ptr(phi, D), _ptr(phi_reset, D), float(st), int(rho),
                                    _ptr(force, D), C.byref(nif), C.byref(area))
    assert st_ == 0, "element with a crossing count other than 3 or 4"
    return force.reshape(3, npn), nif.value, area.value


__all__ = ["build", "lib", "ref_tables", "boundary_nodes", "set_viscosity", "source",
           "assemble_blocks", "reduce", "spmv", "bicgstab", "true_residual", "scatter",
           "system", "direct_solve", "solve_tight", "flow_solve", "rd_solve", "RD_KEYS",
           "surface_tension", "p2_edges", "p2_system", "p2_flow",
           "dist_reset", "ls_update"]
