"""The reference's edge behaviour through the C ABI: early exits that leave the
flow untouched (Flow.cpp:223-228, 248-251), errors instead of undefined
results (degenerate element, NaN input, iteration cap), the warm start, and the
reference's own BiCGSTAB run on the GPU."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import oracle_solution, workload

pytestmark = pytest.mark.gpu

OK, DEGENERATE, NOT_CONVERGED, UNSUPPORTED, NAN = 0, 2, 3, 6, 7


def _flow(inst, par=None, **opts):
    from fluidtissue_gb300.flow import Flow, Mesh
    f = Flow()
    rc = f.init(Mesh(inst.xyz, inst.tets), par or inst.params, **opts)
    return f, rc


def test_zero_advection_dt_leaves_flow_untouched():
    inst = workload("sphere17", 9)
    par = dict(inst.params, **{"Advection dt": 0.0})
    f, rc = _flow(inst, par)
    assert rc == OK
    flow = np.full(4 * inst.np, 7.0)
    assert f.solve(inst.phi, inst.source, flow, mu=inst.mu) == OK
    assert np.all(flow == 7.0) and f.last_stats["solved"] == 0
    f.close()


def test_zero_source_with_rd_leaves_flow_untouched():
    """mu_in > mu_out with RD on and max|source| <= FLT_MIN (Flow.cpp:223-226)."""
    inst = workload("sphere17", 9)
    par = dict(inst.params, **{"Viscosity interior": 10.0, "Viscosity exterior": 1.0,
                               "RD iterations": 1.0})
    f, rc = _flow(inst, par)
    assert rc == OK
    flow = np.full(4 * inst.np, -2.0)
    assert f.solve(inst.phi, np.zeros(inst.np), flow) == OK
    assert np.all(flow == -2.0) and f.last_stats["solved"] == 0
    f.close()


def test_zero_load_exit():
    """Zero right-hand side (source below the growth threshold everywhere):
    ||F|| = 0, nothing to solve (Flow.cpp:248-251)."""
    inst = workload("sphere17", 9)
    par = dict(inst.params, **{"Growth threshold": 1e9})
    f, rc = _flow(inst, par)
    assert rc == OK
    flow = np.full(4 * inst.np, 5.0)
    assert f.solve(inst.phi, inst.source, flow, mu=inst.mu) == OK
    assert np.all(flow == 5.0) and f.last_stats["solved"] == 0
    f.close()


def test_degenerate_element_is_an_error():
    inst = workload("sphere17", 9)
    xyz = inst.xyz.copy()
    t = inst.tets[0]
    xyz[t[3]] = xyz[t[0]]  # collapse one tetrahedron
    from fluidtissue_gb300.flow import Flow, Mesh
    f = Flow()
    assert f.init(Mesh(xyz, inst.tets), inst.params) == DEGENERATE


@pytest.mark.parametrize("what", ["phi", "source", "mu"])
def test_nan_input_is_an_error_and_flow_untouched(what):
    inst = workload("sphere17", 9)
    f, rc = _flow(inst)
    assert rc == OK
    args = {"phi": inst.phi.copy(), "source": inst.source.copy(), "mu": inst.mu.copy()}
    args[what][3] = np.nan
    flow = np.full(4 * inst.np, 1.5)
    assert f.solve(args["phi"], args["source"], flow, mu=args["mu"]) == NAN
    assert np.all(flow == 1.5)
    # the context stays usable
    assert f.solve(inst.phi, inst.source, flow, mu=inst.mu) == OK
    f.close()


def test_iteration_cap_reports_not_converged():
    inst = workload("sphere17", 13)
    par = dict(inst.params, **{"Max. CG iterations": 3.0, "Stokes tolerance": 1e-12})
    f, rc = _flow(inst, par, precision="fp64")
    assert rc == OK
    flow = np.full(4 * inst.np, 4.0)
    assert f.solve(inst.phi, inst.source, flow, mu=inst.mu) == NOT_CONVERGED
    assert np.all(flow == 4.0)
    f.close()


def test_surface_tension_without_its_load_refused():
    """"Surface tension" > 0 needs the nodal load that fts_ls_surface_tension
    computes from the level set; without it the solve is refused and flow
    stays untouched."""
    inst = workload("sphere17", 9)
    par = dict(inst.params, **{"Surface tension": 1.0})
    f, rc = _flow(inst, par)
    assert rc == OK
    flow = np.full(4 * inst.np, 3.0)
    assert f.solve(inst.phi, inst.source, flow, mu=inst.mu) == UNSUPPORTED
    assert np.all(flow == 3.0)
    f.close()


def test_warm_start_converges_immediately_on_the_same_input():
    """The context keeps the previous solution (Flow.cpp:15, up_): solving the
    same system again starts at the answer."""
    inst = workload("sphere17", 13)
    f, rc = _flow(inst, precision="fp64", warm_start=True)
    assert rc == OK
    flow = np.zeros(4 * inst.np)
    assert f.solve(inst.phi, inst.source, flow, mu=inst.mu) == OK
    first = f.last_stats["iterations"]
    flow2 = np.zeros(4 * inst.np)
    assert f.solve(inst.phi, inst.source, flow2, mu=inst.mu) == OK
    assert f.last_stats["iterations"] <= max(1, first // 10), (first, f.last_stats)
    assert np.allclose(flow, flow2, rtol=0, atol=1e-7 * np.abs(flow).max())
    f.reset_guess()
    assert f.solve(inst.phi, inst.source, flow2, mu=inst.mu) == OK
    assert f.last_stats["iterations"] >= first // 2
    f.close()


def test_reference_bicgstab_on_gpu_matches_oracle():
    """solver = BiCGSTAB: the reference's own algorithm (un-preconditioned,
    Eigen's stopping rule) on the GPU reaches the tolerance on sphere17, and its
    answer matches the oracle's tight solve to the accuracy the tolerance
    allows."""
    inst = workload("sphere17")
    ref, _, _ = oracle_solution("sphere17")
    par = dict(inst.params)
    f, rc = _flow(inst, par, precision="fp64", solver="bicgstab", warm_start=False)
    assert rc == OK
    flow = np.zeros(4 * inst.np)
    assert f.solve(inst.phi, inst.source, flow, mu=inst.mu) == OK, f.last_error()
    st = f.last_stats
    assert st["rel_residual"] <= par["Stokes tolerance"] * 1.0001, st
    npn = inst.np
    ev = np.linalg.norm(flow[:3 * npn] - ref[:3 * npn]) / np.linalg.norm(ref[:3 * npn])
    assert ev <= 1e-4, (ev, st)
    f.close()
