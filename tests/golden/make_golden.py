"""Regenerates tests/golden/*.npz: the oracle's tightly converged solution of
small seeded workloads, with their inputs, so that the oracle (and through it
the CUDA path) is checked against fixed numbers on any machine.

The reference itself cannot be built here (Eigen/CGAL/TBB/GMP are absent), so
these fixtures come from the oracle's restatement; they pin regressions, not
the reference.  Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def mesh_hash(xyz, tets) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(xyz, np.float32).tobytes())
    h.update(np.ascontiguousarray(tets, np.int32).tobytes())
    return h.hexdigest()


def make(name: str, n: int, out: Path) -> None:
    from fluidtissue_gb300 import workloads as W
    import oracle as O
    inst = W.WORKLOADS[name](n)
    R, B, s, mu = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                           inst.params)
    x, tr, its = O.solve_tight(R, inst.xyz, inst.tets, mu, tol=1e-13)
    assert tr <= 1e-12, tr
    flow = O.scatter(R, x)
    np.savez_compressed(out, n=n, name=name, mesh_sha256=mesh_hash(inst.xyz, inst.tets),
                        boundary=inst.boundary, phi=inst.phi, source=inst.source, mu=inst.mu,
                        flow=flow, rel_residual=tr, F=R.F, params=repr(inst.params))
    print(f"{out.name}: N={R.N} true rel residual {tr:.2e} ({its} MINRES iterations)")


def make_p2(name: str, n: int, out: Path) -> None:
    """The oracle's direct solve of the P2-P1 system (velocity degree 2)."""
    from fluidtissue_gb300 import workloads as W
    import oracle as O
    inst = W.WORKLOADS[name](n)
    par = dict(inst.params, **{"Stokes velocity degree": 2.0})
    flow, A, F = O.p2_flow(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                           par)
    np.savez_compressed(out, n=n, name=name, mesh_sha256=mesh_hash(inst.xyz, inst.tets),
                        flow=flow, F=F, params=repr(par))
    print(f"{out.name}: P2-P1, {A.shape[0]} reduced unknowns")


def make_st(n: int, out: Path) -> None:
    """The oracle's surface-tension load of the sphere of radius 0.25 (phi =
    phi_reset = the exact distance) on the Kuhn lattice of n^3 nodes."""
    from fluidtissue_gb300 import workloads as W
    import oracle as O
    xyz, tets, _ = W.kuhn_mesh(n, 0.0, 1)
    phi = np.linalg.norm(xyz.astype(np.float64) - 0.5, axis=1) - 0.25
    f, nif, area = O.surface_tension(xyz, tets, phi, phi, 1.0, 1)
    np.savez_compressed(out, n=n, mesh_sha256=mesh_hash(xyz, tets), phi=phi, force=f,
                        interface_points=nif, area=area)
    print(f"{out.name}: {nif} interface points, patch area {area:.6f}")


if __name__ == "__main__":
    make("sphere17", 17, HERE / "sphere17.npz")
    make("sphere65", 9, HERE / "sphere65_n9.npz")
    make_p2("sphere17", 7, HERE / "p2_sphere17_n7.npz")
    make_st(17, HERE / "st_sphere_n17.npz")
