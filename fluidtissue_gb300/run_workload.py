"""Run one named workload's Stokes solve a few times and print its stats.

    python -m fluidtissue_gb300.run_workload sphere65 --n 65 --precision mixed --reps 1

A small, fixed command line for profilers: it builds the seeded instance,
creates one context and calls ``Flow.solve`` ``--reps`` times.
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
    a = ap.parse_args(argv)
    inst = W.WORKLOADS[a.workload](a.n) if a.n else W.WORKLOADS[a.workload]()
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


if __name__ == "__main__":
    raise SystemExit(main())
