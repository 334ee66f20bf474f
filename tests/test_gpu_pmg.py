"""Pressure-block multigrid (FTS_PC_MULTIGRID, the default on Kuhn lattices):
one scalar V-cycle of (alpha D + eps M) + lumped 1/mu mass replaces the
pressure diagonal of the MINRES preconditioner.  The preconditioner changes
the iteration, not the answer: solutions agree with the diagonal variant and
the oracle, and the high-contrast workloads need fewer iterations."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import workload

pytestmark = pytest.mark.gpu


def _solve(inst, par, **opts):
    from fluidtissue_gb300.flow import Flow, Mesh
    f = Flow()
    assert f.init(Mesh(inst.xyz, inst.tets), par, warm_start=False, **opts) == 0, f.last_error()
    flow = np.zeros(4 * inst.np)
    rc = f.solve(inst.phi, inst.source, flow, mu=inst.mu)
    assert rc == 0, f.last_error()
    st = dict(f.last_stats)
    f.close()
    return flow, st


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n", [33, 32])
def test_pressure_multigrid_fewer_iterations_same_answer(precision, n):
    """mu = clip(1/(0.01 + c), 0.01, 100) (four decades): the pressure V-cycle
    cuts the iterations; both preconditioners reach the same solution within
    the tolerance (1e-10 asked, 1e-7 compared)."""
    inst = workload("ellipsoid129", n)
    par = dict(inst.params, **{"Stokes tolerance": 1e-10})
    x_mg, st_mg = _solve(inst, par, precision=precision, preconditioner="multigrid")
    x_dg, st_dg = _solve(inst, par, precision=precision, preconditioner="multigrid_diag")
    assert st_mg["rel_residual"] <= 1e-10 and st_dg["rel_residual"] <= 1e-10
    npn = inst.np
    vel, prs = slice(0, 3 * npn), slice(3 * npn, 4 * npn)
    assert _rel(x_mg[vel], x_dg[vel]) <= 1e-7
    assert _rel(x_mg[prs], x_dg[prs]) <= 1e-7
    assert st_mg["iterations"] < 0.8 * st_dg["iterations"], (st_mg["iterations"],
                                                              st_dg["iterations"])


@pytest.mark.parametrize("n", [17, 16])
def test_pressure_multigrid_matches_oracle(n):
    """FP64 solve with both V-cycles against the oracle's tight solve."""
    import oracle as O
    inst = workload("sphere17", n)
    par = dict(inst.params)
    flow, st = _solve(inst, par, precision="fp64", preconditioner="multigrid")
    R, _, _, mu = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                           par)
    x, tr, _ = O.solve_tight(R, inst.xyz, inst.tets, mu, tol=1e-13)
    ref = O.scatter(R, x)
    npn = inst.np
    assert _rel(flow[:3 * npn], ref[:3 * npn]) <= 1e-8, st
    assert _rel(flow[3 * npn:], ref[3 * npn:]) <= 1e-8, st


def test_pressure_multigrid_matrix_free():
    """Matrix-free operator: the pressure hierarchy's fine level comes from the
    elements; same answer as the assembled stencil path."""
    inst = workload("sphere65", 33)
    par = dict(inst.params, **{"Stokes tolerance": 1e-10})
    x_mf, st_mf = _solve(inst, par, precision="mixed", operator="matfree")
    x_st, st_st = _solve(inst, par, precision="mixed", operator="stencil")
    npn = inst.np
    assert _rel(x_mf[:3 * npn], x_st[:3 * npn]) <= 1e-7
    assert _rel(x_mf[3 * npn:], x_st[3 * npn:]) <= 1e-7
    # same preconditioner up to FP32 rounding of the fine level
    assert abs(st_mf["iterations"] - st_st["iterations"]) <= 0.1 * st_st["iterations"] + 5
