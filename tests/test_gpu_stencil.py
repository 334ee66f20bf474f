"""Lattice half-stencil operator (operator_kind = FTS_OP_STENCIL, the default on
Kuhn lattices): its FP32 product equals the FP64 assembled operator's to FP32
rounding, and mixed-precision solves through it match the sliced-ELL path and
the oracle within the mixed-precision bar."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import workload

pytestmark = pytest.mark.gpu


def _flow(inst, par, **opts):
    from fluidtissue_gb300.flow import Flow, Mesh
    f = Flow()
    assert f.init(Mesh(inst.xyz, inst.tets), par, warm_start=False, **opts) == 0, f.last_error()
    flow = np.zeros(4 * inst.np)
    rc = f.solve(inst.phi, inst.source, flow, mu=inst.mu)
    assert rc == 0, f.last_error()
    return f, flow


@pytest.mark.parametrize("name,n", [("sphere65", 12), ("sphere65", 17), ("ellipsoid129", 33)])
def test_stencil_product_matches_fp64(name, n):
    """S x through the half stencil (own blocks + neighbours' transposed blocks)
    vs the FP64 BSR product, on random x: max error relative to |S| |x| row sums."""
    inst = workload(name, n)
    f, _ = _flow(inst, dict(inst.params), precision="mixed", operator="stencil")
    rp, ci, vals, _ = f.system()
    rng = np.random.default_rng(5)
    x = rng.standard_normal(4 * inst.np)
    y64 = f.apply(x, "fp64")
    y32 = f.apply(x, "mixed")
    rows = np.repeat(np.arange(inst.np), np.diff(rp))
    absrow = np.zeros((inst.np, 4))
    np.add.at(absrow, rows, np.einsum("brc,bc->br", np.abs(vals),
                                      np.abs(x.reshape(-1, 4))[ci]))
    err = np.abs(y32 - y64).reshape(-1, 4) / np.maximum(absrow, 1e-300)
    assert err.max() <= 2e-6, err.max()
    f.close()


@pytest.mark.parametrize("n", [17, 16])
def test_stencil_solve_matches_ell_and_oracle(n):
    import oracle as O
    inst = workload("sphere17", n)
    par = dict(inst.params)
    par["Stokes tolerance"] = 1e-10
    flows, its = {}, {}
    for op in ("stencil", "assembled"):
        f, flow = _flow(inst, par, precision="mixed", operator=op)
        assert f.last_stats["rel_residual"] <= 1e-10
        flows[op], its[op] = flow, f.last_stats["iterations"]
        f.close()
    npn = inst.np
    rel = lambda a, b, s: np.linalg.norm(a[s] - b[s]) / np.linalg.norm(b[s])  # noqa: E731
    vel, prs = slice(0, 3 * npn), slice(3 * npn, 4 * npn)
    R, _, _, mu = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                           par)
    x, tr, _ = O.solve_tight(R, inst.xyz, inst.tets, mu, tol=1e-13)
    ref = O.scatter(R, x)
    for op in flows:
        assert rel(flows[op], ref, vel) <= 1e-7, (op, its)
        assert rel(flows[op], ref, prs) <= 1e-7, (op, its)


def test_stencil_refused_off_lattice():
    from fluidtissue_gb300.flow import Flow, Mesh
    inst = workload("sphere17", 9)
    tets = inst.tets  # same elements, nodes renumbered: no longer lattice order
    perm = np.random.default_rng(1).permutation(inst.np).astype(np.int32)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(inst.np, dtype=np.int32)
    f = Flow()
    rc = f.init(Mesh(inst.xyz[perm], inv[tets]), inst.params, precision="mixed",
                operator="stencil")
    assert rc == 6, rc


@pytest.mark.parametrize("name,n", [("sphere65", 17), ("ellipsoid129", 24)])
def test_lattice_fp64_residual_matches_bsr(name, n):
    """Mixed precision on a lattice assembles only the FP64 / FP32 half
    stencils; the outer residual it reports (from the FP64 half stencil) equals
    ||b - A x|| / ||b|| recomputed on the host from the BSR the context then
    assembles on request, for the returned solution."""
    inst = workload(name, n)
    par = dict(inst.params)
    f, flow = _flow(inst, par, precision="mixed", operator="stencil")
    rp, ci, vals, rhs = f.system()
    npn = inst.np
    x = flow.reshape(4, npn).T.copy()  # (ux, uy, uz, p) per node
    rows = np.repeat(np.arange(npn), np.diff(rp))
    ax = np.zeros((npn, 4))
    np.add.at(ax, rows, np.einsum("brc,bc->br", vals, x[ci]))
    rel = np.linalg.norm(rhs - ax) / np.linalg.norm(rhs)
    st = f.last_stats
    assert st["rel_residual"] <= par["Stokes tolerance"]
    assert abs(rel - st["rel_residual"]) <= 1e-3 * st["rel_residual"] + 1e-14, (rel, st)
    f.close()
