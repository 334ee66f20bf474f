"""P2-P1 (the reference's "Stokes velocity degree" = 2, Taylor-Hood) on the
GPU: vertices and edges as system nodes, FP64 assembly from reference
integrals, MINRES with the P2 -> P1 multigrid V-cycle (or block Jacobi);
against the oracle's direct solve of the reference's own P2-P1 system."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import workload

pytestmark = pytest.mark.gpu


def _solve(inst, par, **opts):
    from fluidtissue_gb300.flow import Flow, Mesh
    f = Flow()
    rc = f.init(Mesh(inst.xyz, inst.tets), par, warm_start=False, **opts)
    assert rc == 0, f.last_error()
    flow = np.zeros(4 * inst.np)
    return f, flow


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n", [9, 8])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_p2_matches_oracle(n, precision):
    import oracle as O
    inst = workload("sphere17", n)
    par = dict(inst.params, **{"Stokes velocity degree": 2.0, "Stokes tolerance": 1e-11})
    f, flow = _solve(inst, par, precision=precision)
    assert f.solve(inst.phi, inst.source, flow, mu=inst.mu) == 0, f.last_error()
    st = f.last_stats
    assert st["rel_residual"] <= 1e-11, st
    ref, _, _ = O.p2_flow(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu, par)
    npn = inst.np
    tol = 1e-8 if precision == "fp64" else 1e-7
    assert _rel(flow[:3 * npn], ref[:3 * npn]) <= tol, (_rel(flow[:3 * npn], ref[:3 * npn]), st)
    assert _rel(flow[3 * npn:], ref[3 * npn:]) <= tol
    # boundary velocity is zero (Flow.cpp:290-300)
    assert np.all(flow[:npn][inst.boundary.astype(bool)] == 0.0)
    # system size: vertices + edges
    npx, nnzb, nred = f.sizes()
    edges = len(O.p2_edges(inst.tets))
    assert npx == npn + edges
    f.close()


def test_p2_body_force_matches_oracle():
    """A uniform body force and no source (the load N f of Flow.cpp:392-395):
    the GPU solve against the oracle's direct solve of the same system, and
    close to the hydrostatic balance u = 0, p = x + const that P2-P1 reaches
    exactly as eps -> 0."""
    import oracle as O
    inst = workload("sphere17", 9)
    par = dict(inst.params, **{"Stokes velocity degree": 2.0, "GF growth": 0.0,
                               "Stokes tolerance": 1e-11})
    f, flow = _solve(inst, par, precision="fp64")
    force = np.zeros(3 * inst.np)
    force[:inst.np] = 1.0
    assert f.solve(inst.phi, inst.source, flow, mu=inst.mu, force=force) == 0, f.last_error()
    ref, _, _ = O.p2_flow(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                          par, fst=force)
    npn = inst.np
    assert _rel(flow[3 * npn:], ref[3 * npn:]) <= 1e-8
    assert np.abs(flow[:3 * npn] - ref[:3 * npn]).max() <= 1e-8 * np.abs(ref[3 * npn:]).max()
    p = flow[3 * npn:]
    x = inst.xyz[:, 0].astype(np.float64)
    assert np.abs((p - p.mean()) - (x - x.mean())).max() <= 0.05
    f.close()


def test_p2_options_refused_and_degree_fixed():
    from fluidtissue_gb300.flow import Flow, Mesh
    inst = workload("sphere17", 9)
    par = dict(inst.params, **{"Stokes velocity degree": 2.0})
    for opts in ({"operator": "stencil"}, {"operator": "matfree", "precision": "mixed"}):
        f = Flow()
        assert f.init(Mesh(inst.xyz, inst.tets), par, **opts) == 6, opts
    f, _ = _solve(inst, par, precision="fp64")
    assert f.update_params(dict(par, **{"Stokes velocity degree": 1.0})) == 1
    f.close()


def test_p2_matches_golden_fixture():
    """The committed P2-P1 fixture (the oracle's direct solve, 7^3 sphere)."""
    from conftest import ROOT
    g = np.load(ROOT / "tests" / "golden" / "p2_sphere17_n7.npz")
    inst = workload(str(g["name"]), int(g["n"]))
    par = dict(inst.params, **{"Stokes velocity degree": 2.0, "Stokes tolerance": 1e-11})
    f, flow = _solve(inst, par, precision="fp64")
    assert f.solve(inst.phi, inst.source, flow, mu=inst.mu) == 0, f.last_error()
    assert _rel(flow, g["flow"]) <= 1e-8
    f.close()


@pytest.mark.parametrize("n", [9, 10])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_p2_multigrid_matches_oracle_and_beats_jacobi(n, precision):
    """The P2 -> P1 V-cycle (P2 level above the vertex lattice's hierarchy):
    the same answer as the oracle's direct solve, in far fewer iterations than
    block Jacobi."""
    import oracle as O
    inst = workload("sphere65", n)
    par = dict(inst.params, **{"Stokes velocity degree": 2.0, "Stokes tolerance": 1e-10})
    ref, _, _ = O.p2_flow(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu, par)
    npn = inst.np
    tol = 1e-8 if precision == "fp64" else 1e-7
    its = {}
    for pc in ("multigrid", "jacobi"):
        f, flow = _solve(inst, par, precision=precision, preconditioner=pc)
        assert f.solve(inst.phi, inst.source, flow, mu=inst.mu) == 0, (pc, f.last_error())
        st = f.last_stats
        its[pc] = st["iterations"]
        assert st["rel_residual"] <= 1e-10, (pc, st)
        assert _rel(flow[:3 * npn], ref[:3 * npn]) <= tol, (pc, _rel(flow[:3 * npn], ref[:3 * npn]))
        assert _rel(flow[3 * npn:], ref[3 * npn:]) <= tol, pc
        f.close()
    assert its["multigrid"] * 3 < its["jacobi"], its
