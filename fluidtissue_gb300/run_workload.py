"""Run one named workload's Stokes solve a few times and print its stats.

    python -m fluidtissue_gb300.run_workload sphere65 --n 65 --precision mixed --reps 1
    python -m fluidtissue_gb300.run_workload ellipsoid129 --rd-iterations 2000

A small, fixed command line for profilers: it builds the seeded instance,
creates one context and calls ``Flow.solve`` (or ``RD.solve``) ``--reps`` times.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import workloads as W
from .flow import Flow, Mesh


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("workload", choices=sorted(W.WORKLOADS))
    ap.add_argument("--n", type=int, default=None, help="lattice nodes per axis")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--preconditioner", default="auto")
    ap.add_argument("--operator", default="auto")
    ap.add_argument("--reps", type=int, default=1)
    ap.add_argument("--rd-iterations", type=int, default=0,
                    help="run reaction-diffusion (this many Euler steps) on the workload's "
                         "mesh and level set instead of the Stokes solve")
    a = ap.parse_args(argv)
    inst = W.WORKLOADS[a.workload](a.n) if a.n else W.WORKLOADS[a.workload]()
    if a.rd_iterations > 0:
        return _run_rd(inst, a)
    f = Flow()
    rc = f.init(Mesh(inst.xyz, inst.tets), inst.params, precision=a.precision,
                preconditioner=a.preconditioner, operator=a.operator, warm_start=False)
    if rc != 0:
        print(f.last_error())
        return 1
    flow = np.zeros(4 * inst.np)
    for _ in range(a.reps):
        rc = f.solve(inst.phi, inst.source, flow, mu=inst.mu)
        if rc != 0:
            print(f.last_error())
            return 1
    print(json.dumps(f.last_stats))
    f.close()
    return 0


def _run_rd(inst, a) -> int:
    from .rd import RD
    par = {"RD dt": 1.0 / 32.0, "RD iterations": float(a.rd_iterations), "Act": 2.0,
           "Da": 5.0e-6, "DegA": 0.01, "Inh": 1.0, "Di": 7.5e-5, "DegI": 0.02,
           "GF production": 40.0, "GF diffusion": 1.25e-4, "GF degradation": 0.02,
           "GF inhibition": 200.0}
    rd = RD()
    if rd.init(Mesh(inst.xyz, inst.tets), inst.phi, par) != 0:
        print(rd.last_error())
        return 1
    inside = np.where(inst.phi < 0)[0]
    src = inside[np.linspace(0, len(inside) - 1, 16).astype(int)]
    for _ in range(a.reps):
        if rd.solve(inst.phi, src) != 0:
            print(rd.last_error())
            return 1
    print(json.dumps(rd.last_stats))
    rd.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
