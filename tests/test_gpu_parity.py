"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

FP64 path: relative L2 error <= 1e-8 in velocity and in pressure against the
oracle's tightly converged solve of the same system (true relative residual
<= 1e-13).  Mixed path: velocity error <= 1e-7.  Assembly: every block entry
within 1e-12 of the largest entry of its block row.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import oracle_solution, workload

pytestmark = pytest.mark.gpu

VEL_TOL_FP64 = 1e-8
P_TOL_FP64 = 1e-8
VEL_TOL_MIXED = 1e-7


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _errors(flow, ref, npn):
    return _rel(flow[:3 * npn], ref[:3 * npn]), _rel(flow[3 * npn:], ref[3 * npn:])


def _solve(inst, par=None, mu="given", **opts):
    from fluidtissue_gb300.flow import Flow, Mesh
    f = Flow()
    rc = f.init(Mesh(inst.xyz, inst.tets), par or inst.params, **opts)
    assert rc == 0, f.last_error()
    flow = np.zeros(4 * inst.np)
    rc = f.solve(inst.phi, inst.source, flow, mu=inst.mu if mu == "given" else None)
    return f, rc, flow


def _oracle_gpu_form(B, bnd):
    """Oracle blocks (reference signs) -> the GPU's symmetric, Dirichlet-masked form."""
    vals = B.vals.copy()
    vals[:, 3, :] *= -1.0
    rows = np.repeat(np.arange(B.rowptr.shape[0] - 1), np.diff(B.rowptr))
    bi = bnd[rows].astype(bool)
    bj = bnd[B.cols].astype(bool)
    vals[bj, :, :3] = 0.0
    vals[bi, :3, :] = 0.0
    diag = bi & (rows == B.cols)
    for r in range(3):
        vals[diag, r, r] = 1.0
    return vals


@pytest.mark.parametrize("name,n", [("sphere17", 17), ("sphere65", 17)])
def test_assembly_matches_oracle(name, n):
    import oracle as O
    inst = workload(name, n)
    f, rc, _ = _solve(inst)
    assert rc == 0
    rp, ci, vals, rhs = f.system()
    s = O.source(inst.phi, inst.source, inst.params["GF growth"])
    B = O.assemble_blocks(inst.xyz, inst.tets, inst.mu, s, inst.params["alpha"],
                          inst.params["eps"])
    assert np.array_equal(rp, B.rowptr) and np.array_equal(ci, B.cols)
    want = _oracle_gpu_form(B, inst.boundary)
    rows = np.repeat(np.arange(inst.np), np.diff(B.rowptr))
    scale = np.zeros(inst.np)
    np.maximum.at(scale, rows, np.abs(want).reshape(-1, 16).max(axis=1))
    err = np.abs(vals - want).reshape(-1, 16).max(axis=1) / scale[rows]
    assert err.max() <= 1e-12, f"max block error {err.max():.3e}"
    want_rhs = B.rhs.copy()
    want_rhs[:, 3] *= -1
    want_rhs[inst.boundary.astype(bool), :3] = 0.0
    assert _rel(rhs, want_rhs) <= 1e-12
    f.close()


def test_fp64_parity_sphere17():
    inst = workload("sphere17")
    ref, _, _ = oracle_solution("sphere17")
    f, rc, flow = _solve(inst, precision="fp64")
    assert rc == 0, f.last_error()
    ev, ep = _errors(flow, ref, inst.np)
    assert ev <= VEL_TOL_FP64 and ep <= P_TOL_FP64, (ev, ep, f.last_stats)
    assert f.last_stats["rel_residual"] <= inst.params["Stokes tolerance"]
    f.close()


def test_mixed_parity_sphere17():
    inst = workload("sphere17")
    ref, _, _ = oracle_solution("sphere17")
    f, rc, flow = _solve(inst, precision="mixed")
    assert rc == 0, f.last_error()
    st = f.last_stats
    ev, ep = _errors(flow, ref, inst.np)
    assert ev <= VEL_TOL_MIXED, (ev, ep, st)
    assert st["rel_residual"] <= inst.params["Stokes tolerance"]
    assert st["iterations_fp32"] > 0
    f.close()


def test_reported_residual_is_true_residual():
    """The residual in the stats equals ||F - A x|| / ||F|| of the reference's
    reduced system evaluated by the oracle on the returned flow."""
    import oracle as O
    inst = workload("sphere17")
    _, R, _ = oracle_solution("sphere17")
    f, rc, flow = _solve(inst, precision="mixed")
    assert rc == 0
    x = flow[R.sidx]
    tr = O.true_residual(R, x)
    assert tr <= inst.params["Stokes tolerance"] * 1.01
    assert abs(tr - f.last_stats["rel_residual"]) <= 0.05 * tr + 1e-15
    f.close()


def test_profile_viscosity_matches_oracle():
    """mu = NULL: the GPU evaluates setViscosity (ViscosityProfiles.hpp:27-72)."""
    import oracle as O
    inst = workload("sphere17", 13)
    for profile in (0, 1, 2):
        par = dict(inst.params)
        par.update({"Viscosity interior": 20.0, "Viscosity exterior": 1.0,
                    "Viscosity profile": float(profile), "RD iterations": 1.0,
                    "GF production": 2.0})
        f, rc, flow = _solve(inst, par=par, mu=None)
        assert rc == 0, f.last_error()
        R, _, _, mu = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, None,
                               par)
        x, tr, _ = O.solve_tight(R, inst.xyz, inst.tets, mu, tol=1e-13)
        ev, ep = _errors(flow, O.scatter(R, x), inst.np)
        assert ev <= VEL_TOL_FP64 and ep <= P_TOL_FP64, (profile, ev, ep)
        mu_o, mm = O.set_viscosity(inst.tets, inst.phi, inst.source, 20.0, 1.0, profile, 1.0, 2.0)
        assert abs(f.last_stats["mu_min"] - mm[0]) <= 1e-12 * abs(mm[0])
        assert abs(f.last_stats["mu_max"] - mm[1]) <= 1e-12 * abs(mm[1])
        f.close()


@pytest.mark.parametrize("n", [16, 10])
def test_even_n_multigrid_parity(n):
    """Even lattice sizes coarsen to n/2 + 1 (the last coarse layer on the
    Dirichlet boundary layer); FP64 parity and fewer iterations than Jacobi."""
    import oracle as O
    inst = workload("sphere17", n)
    par = dict(inst.params)
    its = {}
    for pc in ("multigrid", "jacobi"):
        f, rc, flow = _solve(inst, par=par, precision="fp64", preconditioner=pc)
        assert rc == 0, f.last_error()
        its[pc] = f.last_stats["iterations"]
        if pc == "multigrid":
            R, _, _, mu = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source,
                                   inst.mu, par)
            x, tr, _ = O.solve_tight(R, inst.xyz, inst.tets, mu, tol=1e-13)
            ev, ep = _errors(flow, O.scatter(R, x), inst.np)
            assert ev <= VEL_TOL_FP64 and ep <= P_TOL_FP64, (ev, ep)
        f.close()
    assert its["multigrid"] < its["jacobi"], its
