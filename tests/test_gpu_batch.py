"""Batched solves (fts_batch_*): every instance of a batch equals its own
single solve — and the oracle — within the precision's parity bar."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instances(count=6, nmin=9, nmax=17):
    from fluidtissue_gb300 import workloads as W
    return [W.batch_instance(i, nmin, nmax) for i in range(count)]


def _renumbered(inst, seed=1):
    """The same instance with its nodes renumbered (no longer in lattice order:
    the batch treats it as a general mesh, block Jacobi)."""
    perm = np.random.default_rng(seed).permutation(inst.np).astype(np.int32)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(inst.np, dtype=np.int32)
    return perm, inv


@pytest.mark.parametrize("precision,pc", [("fp64", "auto"), ("mixed", "auto"),
                                          ("mixed", "jacobi")])
def test_batch_matches_oracle(precision, pc):
    import oracle as O
    from fluidtissue_gb300.flow import Batch, Mesh
    insts = _instances()
    pars = []
    for inst in insts:
        par = dict(inst.params)
        par["Stokes tolerance"] = 1e-10
        pars.append(par)
    b = Batch([Mesh(i.xyz, i.tets) for i in insts], pars, precision=precision,
              warm_start=False, preconditioner=pc)
    flows = [np.zeros(4 * i.np) for i in insts]
    rc = b.solve([i.phi for i in insts], [i.source for i in insts], flows,
                 mus=[i.mu for i in insts])
    assert rc == 0, b.last_error()
    cfg = b.config()
    assert cfg["threads"] in (128, 256, 512) and cfg["tpr"] in (4, 8) and cfg["blocks"] > 0
    tol_v = 1e-8 if precision == "fp64" else 1e-7
    for inst, par, flow, st in zip(insts, pars, flows, b.last_stats):
        assert st["status"] == 0 and st["solved"] == 1
        assert st["rel_residual"] <= 1e-10
        R, _, _, mu = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source,
                               inst.mu, par)
        x, tr, _ = O.solve_tight(R, inst.xyz, inst.tets, mu, tol=1e-13)
        ref = O.scatter(R, x)
        npn = inst.np
        ev = np.linalg.norm(flow[:3 * npn] - ref[:3 * npn]) / np.linalg.norm(ref[:3 * npn])
        ep = np.linalg.norm(flow[3 * npn:] - ref[3 * npn:]) / np.linalg.norm(ref[3 * npn:])
        assert ev <= tol_v, (inst.name, ev, ep, st)
        if precision == "fp64":
            assert ep <= 1e-8, (inst.name, ev, ep)
    # a second solve replays the captured graph and gives the same answer
    flows2 = [np.zeros(4 * i.np) for i in insts]
    rc = b.solve([i.phi for i in insts], [i.source for i in insts], flows2,
                 mus=[i.mu for i in insts])
    assert rc == 0
    for f1, f2 in zip(flows, flows2):
        assert np.allclose(f1, f2, rtol=0, atol=1e-12 * np.abs(f1).max())
    b.close()


def test_batch_zero_load_instance_left_untouched():
    from fluidtissue_gb300.flow import Batch, Mesh
    insts = _instances(3)
    b = Batch([Mesh(i.xyz, i.tets) for i in insts], [i.params for i in insts],
              precision="fp64", warm_start=False)
    flows = [np.full(4 * i.np, 3.0) for i in insts]
    sources = [i.source for i in insts]
    sources[1] = np.zeros(insts[1].np)
    rc = b.solve([i.phi for i in insts], sources, flows, mus=[i.mu for i in insts])
    assert rc == 0, b.last_error()
    assert b.last_stats[1]["solved"] == 0 and np.all(flows[1] == 3.0)
    assert b.last_stats[0]["solved"] == 1 and not np.all(flows[0] == 3.0)
    b.close()


def test_batch_multigrid_and_jacobi_instances_together():
    """A batch whose instances mix lattice meshes (multigrid V-cycle inside the
    persistent launch) and a renumbered mesh (block Jacobi): every instance
    equals its own single solve, and multigrid instances need fewer iterations
    than the same instance under Jacobi."""
    from fluidtissue_gb300.flow import Batch, Flow, Mesh
    insts = _instances(5, 9, 16)
    meshes = [Mesh(i.xyz, i.tets) for i in insts]
    perm, inv = _renumbered(insts[2])
    meshes[2] = Mesh(insts[2].xyz[perm], inv[insts[2].tets])
    phis = [i.phi for i in insts]
    srcs = [i.source for i in insts]
    phis[2], srcs[2] = insts[2].phi[perm], insts[2].source[perm]
    pars = [dict(i.params, **{"Stokes tolerance": 1e-10}) for i in insts]
    b = Batch(meshes, pars, precision="mixed", warm_start=False)
    flows = [np.zeros(4 * i.np) for i in insts]
    rc = b.solve(phis, srcs, flows, mus=[i.mu for i in insts])
    assert rc == 0, b.last_error()
    its_batch = [s["iterations"] for s in b.last_stats]
    b.close()
    for k, inst in enumerate(insts):
        single = {}
        for pc in ("auto", "jacobi"):
            f = Flow()
            assert f.init(meshes[k], pars[k], precision="mixed", warm_start=False,
                          preconditioner=pc) == 0, f.last_error()
            fl = np.zeros(4 * inst.np)
            assert f.solve(phis[k], srcs[k], fl, mu=inst.mu) == 0, f.last_error()
            single[pc] = (fl, f.last_stats["iterations"])
            f.close()
        ref = single["auto"][0]
        npn = inst.np
        ev = np.linalg.norm(flows[k][:3 * npn] - ref[:3 * npn]) / np.linalg.norm(ref[:3 * npn])
        assert ev <= 1e-7, (k, ev)
        if k != 2:
            assert its_batch[k] < single["jacobi"][1], (k, its_batch[k], single["jacobi"][1])
