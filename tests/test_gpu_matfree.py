"""Matrix-free element operator (operator_kind = FTS_OP_MATFREE): the same
solution as the assembled path and the oracle, within the mixed-precision bar."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import workload

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [17, 33])
def test_matfree_matches_assembled_and_oracle(n):
    import oracle as O
    from fluidtissue_gb300.flow import Flow, Mesh
    inst = workload("spheres257", n)
    par = dict(inst.params)
    par["Stokes tolerance"] = 1e-10
    flows, its = {}, {}
    for op in ("matfree", "assembled"):
        f = Flow()
        assert f.init(Mesh(inst.xyz, inst.tets), par, precision="mixed", operator=op,
                      warm_start=False) == 0, f.last_error()
        flow = np.zeros(4 * inst.np)
        rc = f.solve(inst.phi, inst.source, flow, mu=inst.mu)
        assert rc == 0, f.last_error()
        assert f.last_stats["rel_residual"] <= 1e-10
        flows[op] = flow
        its[op] = f.last_stats["iterations"]
        f.close()
    npn = inst.np
    rel = lambda a, b, s: np.linalg.norm(a[s] - b[s]) / np.linalg.norm(b[s])  # noqa: E731
    vel, prs = slice(0, 3 * npn), slice(3 * npn, 4 * npn)
    assert rel(flows["matfree"], flows["assembled"], vel) <= 1e-7
    # the FP32 inner operators differ only by rounding: the same convergence
    assert its["matfree"] <= 1.1 * its["assembled"] + 5, its
    if n == 17:
        R, _, _, mu = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source,
                               inst.mu, par)
        x, tr, _ = O.solve_tight(R, inst.xyz, inst.tets, mu, tol=1e-13)
        ref = O.scatter(R, x)
        assert rel(flows["matfree"], ref, vel) <= 1e-7
        assert rel(flows["matfree"], ref, prs) <= 1e-7


def test_matfree_refuses_fp64_and_inspection():
    from fluidtissue_gb300.flow import Flow, Mesh
    inst = workload("spheres257", 9)
    f = Flow()
    assert f.init(Mesh(inst.xyz, inst.tets), inst.params, precision="fp64",
                  operator="matfree") == 6
    f = Flow()
    assert f.init(Mesh(inst.xyz, inst.tets), inst.params, precision="mixed",
                  operator="matfree") == 0
    with pytest.raises(Exception):
        f.system()
    f.close()


def test_matfree_element_records_on_reordered_elements():
    """Elements not in the lattice generator's order: the operator falls back
    to per-element FP32 records over the node-element map; same answer."""
    from fluidtissue_gb300.flow import Flow, Mesh
    inst = workload("spheres257", 17)
    par = dict(inst.params)
    par["Stokes tolerance"] = 1e-10
    perm = np.random.default_rng(3).permutation(inst.tets.shape[0])
    flows = {}
    for name, tets, mu in (("lattice", inst.tets, inst.mu),
                           ("records", inst.tets[perm], inst.mu[perm])):
        f = Flow()
        assert f.init(Mesh(inst.xyz, tets), par, precision="mixed", operator="matfree",
                      warm_start=False) == 0, f.last_error()
        flow = np.zeros(4 * inst.np)
        assert f.solve(inst.phi, inst.source, flow, mu=mu) == 0, f.last_error()
        assert f.last_stats["rel_residual"] <= 1e-10
        flows[name] = flow
        f.close()
    npn = inst.np
    a, b = flows["records"][:3 * npn], flows["lattice"][:3 * npn]
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-7
