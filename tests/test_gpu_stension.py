"""Surface tension (fts_ls_surface_tension, the reference's
Flow::surfaceTension_ with LevelSet's normals, curvature and interface
patches) on the GPU against the oracle's restatement, and the Stokes solve
with that load ("Surface tension" > 0) against the oracle's solve of the same
system."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import workload

pytestmark = pytest.mark.gpu

# float arithmetic in the curvature and the patch areas, summed in another
# order: agreement to a few float ulps of the largest nodal load
TOL = 1e-5


def _ls(xyz, tets):
    from fluidtissue_gb300.flow import Mesh
    from fluidtissue_gb300.levelset import LevelSet
    ls = LevelSet()
    assert ls.init(Mesh(xyz, tets)) == 0, ls.last_error()
    return ls


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("n", [17, 33, 32])
def test_sphere_load_matches_oracle(n):
    import oracle as O
    from fluidtissue_gb300 import workloads as W
    xyz, tets, _ = W.kuhn_mesh(n, 0.0, 1)
    c = np.array([0.5, 0.5, 0.5])
    phi = np.linalg.norm(xyz.astype(np.float64) - c, axis=1) - 0.25
    ls = _ls(xyz, tets)
    par = {"Surface tension": 0.7, "Node density": 3.0}
    f = ls.surface_tension(phi, par, phi_reset=phi)
    fo, nif, area = O.surface_tension(xyz, tets, phi, phi, 0.7, 3)
    st = ls.last_st_stats
    assert st["interface_points"] == nif
    assert abs(st["area"] - area) <= 1e-5 * area
    assert _rel(f, fo) <= TOL, _rel(f, fo)
    ls.close()


def test_load_after_update_matches_oracle():
    """Jittered lattice: advect and reset on the GPU, then the load from the
    context's own reset values (phi_reset = NULL) against the oracle given the
    same phi and reset values."""
    import oracle as O
    inst = workload("sphere65", 25)
    ls = _ls(inst.xyz, inst.tets)
    flow = np.zeros(4 * inst.np)
    flow[0:inst.np] = 0.3  # uniform x velocity
    flow[3 * inst.np:] = 1.0
    phi = np.ascontiguousarray(inst.phi, np.float64).copy()
    assert ls.update(flow, phi, {"Advection dt": 0.02, "Advection tolerance": 1e-10,
                                 "Max. CG iterations": 0.0}) == 0, ls.last_error()
    ifn = ls.reset_values()
    par = {"Surface tension": 1.0, "Node density": 1.0}
    f = ls.surface_tension(phi, par)
    fo, nif, _ = O.surface_tension(inst.xyz, inst.tets, phi, ifn, 1.0, 1)
    assert ls.last_st_stats["interface_points"] == nif > 0
    assert _rel(f, fo) <= TOL, _rel(f, fo)
    ls.close()


def test_stokes_with_surface_tension_matches_oracle():
    """The load enters the right-hand side as N fx (Flow.cpp:392-395): the FP64
    GPU solve with "Surface tension" > 0 and the load against the oracle's
    tight solve of the same system."""
    import oracle as O
    from fluidtissue_gb300.flow import Flow, Mesh
    inst = workload("sphere17", 13)
    ls = _ls(inst.xyz, inst.tets)
    par = dict(inst.params, **{"Surface tension": 2.0, "Node density": 1.0})
    phi = np.ascontiguousarray(inst.phi, np.float64)
    force = ls.surface_tension(phi, par, phi_reset=phi)
    assert np.abs(force).max() > 0
    f = Flow()
    assert f.init(Mesh(inst.xyz, inst.tets), par, precision="fp64", warm_start=False) == 0
    flow = np.zeros(4 * inst.np)
    assert f.solve(phi, inst.source, flow, mu=inst.mu, force=force.ravel()) == 0, f.last_error()
    R, _, _, mu = O.system(inst.xyz, inst.tets, inst.boundary, phi, inst.source, inst.mu, par,
                           fst=force)
    x, tr, _ = O.solve_tight(R, inst.xyz, inst.tets, mu, tol=1e-13)
    ref = O.scatter(R, x)
    npn = inst.np
    ev = np.linalg.norm(flow[:3 * npn] - ref[:3 * npn]) / np.linalg.norm(ref[:3 * npn])
    ep = np.linalg.norm(flow[3 * npn:] - ref[3 * npn:]) / np.linalg.norm(ref[3 * npn:])
    assert ev <= 1e-8 and ep <= 1e-8, (ev, ep)
    # the load changes the answer
    flow0 = np.zeros(4 * inst.np)
    f.update_params(dict(par, **{"Surface tension": 0.0}), precision="fp64", warm_start=False)
    assert f.solve(phi, inst.source, flow0, mu=inst.mu) == 0
    assert np.linalg.norm(flow0[:3 * npn] - flow[:3 * npn]) > 1e-3 * np.linalg.norm(flow[:3 * npn])
    f.close()
    ls.close()


def test_reset_values_need_an_update():
    inst = workload("sphere17", 9)
    ls = _ls(inst.xyz, inst.tets)
    from fluidtissue_gb300.flow import FtsError
    with pytest.raises(FtsError):
        ls.reset_values()
    with pytest.raises(FtsError):
        ls.surface_tension(inst.phi, {"Surface tension": 1.0, "Node density": 1.0})
    ls.close()


def test_load_matches_golden_fixture():
    """The committed surface-tension fixture (the oracle's load, 17^3 sphere)."""
    from conftest import ROOT
    from fluidtissue_gb300 import workloads as W
    g = np.load(ROOT / "tests" / "golden" / "st_sphere_n17.npz")
    xyz, tets, _ = W.kuhn_mesh(int(g["n"]), 0.0, 1)
    ls = _ls(xyz, tets)
    f = ls.surface_tension(g["phi"], {"Surface tension": 1.0, "Node density": 1.0},
                           phi_reset=g["phi"])
    assert ls.last_st_stats["interface_points"] == int(g["interface_points"])
    assert _rel(f, g["force"]) <= TOL
    ls.close()
