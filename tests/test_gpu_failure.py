"""Failure detection in the batched persistent launch, in forms that fault,
trap or hang no GPU.

  * A block that never arrives at a grid barrier: a host-set test hook makes
    one block leave at its first barrier without arriving; every other
    block's wait runs out after a 1 ms limit, the launch returns, and the solve
    reports FTS_ERR_TIMEOUT.  The same batch then solves normally once the hook
    is cleared (the context stays usable).
  * An iteration cap: instances whose "Max. CG iterations" is too small end
    with FTS_ERR_NOT_CONVERGED and their flow untouched, while the other
    instances of the same launch are solved.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FTS_ERR_NOT_CONVERGED = 3
FTS_ERR_TIMEOUT = 8


def _instances(count=3):
    from fluidtissue_gb300 import workloads as W
    return [W.batch_instance(i, 9, 17) for i in range(count)]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_absent_block_times_out_and_batch_recovers(precision):
    from fluidtissue_gb300.flow import Batch, Mesh
    insts = _instances()
    b = Batch([Mesh(i.xyz, i.tets) for i in insts], [i.params for i in insts],
              precision=precision, warm_start=False)
    args = ([i.phi for i in insts], [i.source for i in insts])
    mus = [i.mu for i in insts]
    ref = [np.zeros(4 * i.np) for i in insts]
    assert b.solve(*args, ref, mus=mus) == 0, b.last_error()  # tunes and captures the graph

    assert b.set_barrier_limit(1e-3, absent_block=0) == 0
    flows = [np.full(4 * i.np, 7.0) for i in insts]
    rc = b.solve(*args, flows, mus=mus)
    assert rc == FTS_ERR_TIMEOUT, (rc, b.last_error())
    assert "barrier" in b.last_error()

    assert b.set_barrier_limit(2.0, absent_block=-1) == 0
    flows = [np.zeros(4 * i.np) for i in insts]
    assert b.solve(*args, flows, mus=mus) == 0, b.last_error()
    for f, r, st in zip(flows, ref, b.last_stats):
        assert st["solved"] == 1
        assert np.abs(f - r).max() <= 1e-12 * np.abs(r).max()
    b.close()


def test_batch_rejects_bad_barrier_limits():
    from fluidtissue_gb300.flow import Batch, Mesh
    insts = _instances(1)
    b = Batch([Mesh(i.xyz, i.tets) for i in insts], [i.params for i in insts],
              precision="fp64", warm_start=False)
    assert b.set_barrier_limit(0.0) == 1
    assert b.set_barrier_limit(1.0, absent_block=-2) == 1
    b.close()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_iteration_cap_per_instance(precision):
    from fluidtissue_gb300.flow import Batch, Mesh
    insts = _instances()
    pars = [dict(i.params) for i in insts]
    pars[1]["Max. CG iterations"] = 3.0
    b = Batch([Mesh(i.xyz, i.tets) for i in insts], pars, precision=precision,
              warm_start=False)
    flows = [np.full(4 * i.np, 5.0) for i in insts]
    rc = b.solve([i.phi for i in insts], [i.source for i in insts], flows,
                 mus=[i.mu for i in insts])
    assert rc == FTS_ERR_NOT_CONVERGED, (rc, b.last_error())
    st = b.last_stats
    assert st[1]["status"] == FTS_ERR_NOT_CONVERGED and st[1]["solved"] == 0
    assert np.all(flows[1] == 5.0)
    for k in (0, 2):
        assert st[k]["status"] == 0 and st[k]["solved"] == 1, st[k]
        assert st[k]["rel_residual"] <= pars[k]["Stokes tolerance"]
        assert not np.all(flows[k] == 5.0)
    b.close()
