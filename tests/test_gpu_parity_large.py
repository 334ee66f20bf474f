"""Parity at the benchmark sizes, against the oracle's own reduced system.

A tight CPU solve at 129^3 (8.3M unknowns, 474M nonzeros) is out of reach of
the oracle in test time, so at these sizes the GPU's answers are checked with
the quantity the reference itself stops on: the oracle assembles the
reference's reduced system (Flow.cpp:102-206 with the row gather of
Assembler.hpp:134-229, the right-hand side of Flow.cpp:345-399) and evaluates
the true relative residual ||F - A x|| / ||F|| on each GPU flow.  Assembly and
residual are the oracle's; the GPU's own residual estimate plays no part.

  * ellipsoid129 (129^3, mu = clip(1/(0.01+c), 0.01, 100), tol 1e-8): the FP64
    path and the mixed path (FP32 inner solve on the lattice half stencil) each
    reach the tolerance on the oracle's system; an FP64 solve to 1e-12 (checked
    the same way) is the FP64 reference the mixed velocity is compared with
    (<= 1e-7).
  * the two-sphere shape of the 257^3 workload at 129^3 (the largest size whose
    assembled oracle system fits the host comfortably), through the
    matrix-free operator the 257^3 workload uses: the same checks.
  * sphere65 (65^3, jitter +-0.1h, mu = 1): the FP64 path against the
    oracle's tight solve started from zero, <= 1e-8 in velocity and pressure.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VEL_TOL_MIXED = 1e-7
TOL_FP64 = 1e-8


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _gpu_flow(inst, tol, precision, operator="auto"):
    from fluidtissue_gb300.flow import Flow, Mesh
    par = dict(inst.params, **{"Stokes tolerance": tol})
    f = Flow()
    rc = f.init(Mesh(inst.xyz, inst.tets), par, precision=precision, warm_start=False,
                operator=operator)
    assert rc == 0, f.last_error()
    flow = np.zeros(4 * inst.np)
    rc = f.solve(inst.phi, inst.source, flow, mu=inst.mu)
    assert rc == 0, (rc, f.last_error())
    st = dict(f.last_stats)
    f.close()
    return flow, st


def _check_on_oracle_system(inst, mixed_operator):
    import oracle as O
    npn = inst.np
    tol = inst.params["Stokes tolerance"]
    f64, s64 = _gpu_flow(inst, tol, "fp64")
    fmx, smx = _gpu_flow(inst, tol, "mixed", mixed_operator)
    ftight, stight = _gpu_flow(inst, 1e-12, "fp64")
    R, _, _, _ = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                          inst.params)
    tr64 = O.true_residual(R, f64[R.sidx])
    trmx = O.true_residual(R, fmx[R.sidx])
    trt = O.true_residual(R, ftight[R.sidx])
    del R
    # each flow reaches the tolerance on the oracle's reduced system, and the
    # residual the GPU reports is that residual (to the rounding of two FP64
    # sums over 8.3M rows, about 1e-13 of ||F||)
    assert tr64 <= tol * 1.01, (tr64, s64)
    assert trmx <= tol * 1.01, (trmx, smx)
    assert trt <= 1e-12 * 1.01, (trt, stight)
    for tr, st in ((tr64, s64), (trmx, smx), (trt, stight)):
        assert abs(tr - st["rel_residual"]) <= 0.05 * tr + 2e-13, (tr, st["rel_residual"])
    ev = _rel(fmx[:3 * npn], ftight[:3 * npn])
    ep = _rel(fmx[3 * npn:], ftight[3 * npn:])
    ev64 = _rel(f64[:3 * npn], ftight[:3 * npn])
    print(f"\n{inst.name} {inst.n}^3: oracle residual fp64 {tr64:.3e} mixed {trmx:.3e} "
          f"tight {trt:.3e}; error vs the 1e-12 FP64 flow: mixed vel {ev:.3e} p {ep:.3e}, "
          f"fp64 vel {ev64:.3e}; iterations fp64 {s64['iterations']} mixed "
          f"{smx['iterations']} tight {stight['iterations']}")
    assert ev <= VEL_TOL_MIXED, ev
    return ev


def test_ellipsoid129_on_oracle_system():
    from fluidtissue_gb300 import workloads as W
    _check_on_oracle_system(W.ellipsoid129(), "stencil")


def test_two_spheres_129_matrix_free_on_oracle_system():
    from fluidtissue_gb300 import workloads as W
    inst = W.spheres257(129)
    _check_on_oracle_system(inst, "matfree")


def test_sphere65_fp64_cold_oracle_solve():
    """65^3, jitter +-0.1h, mu = 1: the oracle's own tight solve from a zero
    start (about 7,000 preconditioned MINRES iterations on the host) against
    the GPU's FP64 flow."""
    import oracle as O
    from fluidtissue_gb300 import workloads as W
    inst = W.sphere65()
    flow, st = _gpu_flow(inst, inst.params["Stokes tolerance"], "fp64")
    R, _, _, mu = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                           inst.params)
    x, tr, its = O.solve_tight(R, inst.xyz, inst.tets, mu, tol=1e-12)
    assert tr <= 1.01e-12, tr
    ref = O.scatter(R, x)
    npn = inst.np
    ev, ep = _rel(flow[:3 * npn], ref[:3 * npn]), _rel(flow[3 * npn:], ref[3 * npn:])
    print(f"\nsphere65 cold oracle solve: {its} iterations, residual {tr:.2e}; GPU FP64 "
          f"error vel {ev:.3e} p {ep:.3e}")
    assert ev <= TOL_FP64 and ep <= TOL_FP64, (ev, ep, st)
