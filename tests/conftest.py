"""Shared fixtures: the repo root and the oracle directory on sys.path, a
``gpu`` marker for tests that need a CUDA device, and cached workloads."""
from __future__ import annotations

import functools
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@functools.lru_cache(maxsize=None)
def workload(name: str, n: int | None = None):
    from fluidtissue_gb300 import workloads as W
    fn = W.WORKLOADS[name]
    return fn() if n is None else fn(n)


@functools.lru_cache(maxsize=None)
def oracle_solution(name: str, n: int | None = None, tol: float = 1e-13):
    """Tight oracle solution of a workload: (flow, reduced system, mu)."""
    import oracle as O
    inst = workload(name, n)
    R, _, _, mu = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                           inst.params)
    x, tr, _ = O.solve_tight(R, inst.xyz, inst.tets, mu, tol=tol)
    assert tr <= tol * 10, f"oracle tight solve stalled at {tr}"
    return O.scatter(R, x), R, mu


@pytest.fixture(scope="session")
def lib_built():
    import __graft_entry__ as g
    g.build()
    return True
