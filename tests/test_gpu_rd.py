"""Reaction-diffusion (fts_rd_*, the reference's RD::solve) on the GPU against
the oracle's restatement: FP64 fields within 1e-11 relative after hundreds of
explicit Euler steps, and the reference's edge behaviour."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import workload

pytestmark = pytest.mark.gpu

# Fig. 5-6 growth parameters of the reference's parameter summary, fewer steps
RD_PAR = {"RD dt": 1.0 / 32.0, "RD iterations": 300.0, "Act": 2.0, "Da": 5.0e-6, "DegA": 0.01,
          "Inh": 1.0, "Di": 7.5e-5, "DegI": 0.02, "GF production": 40.0,
          "GF diffusion": 1.25e-4, "GF degradation": 0.02, "GF inhibition": 200.0}


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _setup(name, n, par=None):
    from fluidtissue_gb300.flow import Mesh
    from fluidtissue_gb300.rd import RD
    inst = workload(name, n)
    p = dict(RD_PAR, **(par or {}))
    rd = RD()
    assert rd.init(Mesh(inst.xyz, inst.tets), inst.phi, p) == 0, rd.last_error()
    interior = np.where(inst.phi < 0)[0]
    src = interior[np.linspace(0, len(interior) - 1, 5).astype(int)]
    return inst, p, rd, src


@pytest.mark.parametrize("name,n", [("sphere17", 17), ("sphere65", 13)])
def test_rd_matches_oracle(name, n):
    import oracle as O
    inst, par, rd, src = _setup(name, n)
    a, i, g = rd.activator.copy(), rd.inhibitor.copy(), rd.growth_factor.copy()
    for call in range(2):  # the state carries over between calls, as in the reference
        assert rd.solve(inst.phi, src) == 0, rd.last_error()
        assert O.rd_solve(inst.xyz, inst.tets, inst.phi, src, par, a, i, g) == 0
        st = rd.last_stats
        assert st["alive"] == 1 and st["steps"] == 300
        assert st["interior_nodes"] == int((inst.phi < 0).sum())
        for got, want in ((rd.activator, a), (rd.inhibitor, i), (rd.growth_factor, g)):
            assert _rel(got, want) <= 1e-11, (call, _rel(got, want))
    outside = inst.phi >= 0
    assert np.all(rd.activator[outside] == 0) and np.all(rd.growth_factor[outside] == 0)
    assert np.all(rd.growth_factor[src] == par["GF production"])
    rd.close()


def test_rd_dead_patterning_only_diffuses_growth_factor():
    """Activator and inhibitor zero everywhere (RD.cpp:60-62): they stay zero
    and only the growth factor is advanced."""
    import oracle as O
    inst, par, rd, src = _setup("sphere17", 13)
    rd.set_state(np.zeros(inst.np), np.zeros(inst.np), np.zeros(inst.np))
    assert rd.solve(inst.phi, src) == 0
    assert rd.last_stats["alive"] == 0
    assert np.all(rd.activator == 0) and np.all(rd.inhibitor == 0)
    a, i, g = np.zeros(inst.np), np.zeros(inst.np), np.zeros(inst.np)
    assert O.rd_solve(inst.xyz, inst.tets, inst.phi, src, par, a, i, g) == 0
    assert _rel(rd.growth_factor, g) <= 1e-11
    rd.close()


def test_rd_no_steps_leaves_state_untouched():
    inst, par, rd, src = _setup("sphere17", 9, {"RD iterations": 0.0})
    before = rd.activator.copy()
    before[inst.phi >= 0] = 7.0  # would be zeroed by a solve that ran
    rd.set_state(before, np.ones(inst.np), np.ones(inst.np))
    assert rd.solve(inst.phi, src) == 0
    assert np.array_equal(rd.activator, before) and np.all(rd.inhibitor == 1.0)
    rd.close()


def test_rd_source_outside_interior_is_refused():
    inst, par, rd, src = _setup("sphere17", 9)
    outside = np.where(inst.phi >= 0)[0][:1]
    assert rd.solve(inst.phi, np.concatenate([src, outside])) == 1
    rd.close()
