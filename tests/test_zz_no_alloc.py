"""fts_bsr_residual_noalloc — the residual entry point for callers that cannot
allocate device memory (they own the GPU's memory through their own arena, or
cannot afford the device synchronisation of cudaMalloc/cudaFree).

The test allocates the inputs and outputs itself (as such a caller would, from
its own pool), calls the entry point twice in a row through the C ABI, and
checks both calls against the existing entry points: the residual fts_solve
reports for the same x, and b - S x formed from fts_apply.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import workload

pytestmark = pytest.mark.gpu

TOL = 1e-12


def test_noalloc_residual_matches_existing_entry_points():
    import torch
    from fluidtissue_gb300 import _api, _native
    from fluidtissue_gb300.flow import Flow, Mesh

    lib = _native.load()
    inst = workload("sphere17")
    f = Flow()
    assert f.init(Mesh(inst.xyz, inst.tets), inst.params, precision="fp64") == 0
    flow = np.zeros(4 * inst.np)
    assert f.solve(inst.phi, inst.source, flow, mu=inst.mu) == 0, f.last_error()
    solve_rel = f.last_stats["rel_residual"]
    rowptr, cols, vals, rhs = f.system()
    npn = inst.np
    assert npn <= _api.NOALLOC_MAX_NODES
    x = np.ascontiguousarray(flow.reshape(4, npn).T)          # node-interleaved
    y = f.apply(x.ravel(), "fp64").reshape(npn, 4)            # S x via fts_apply
    r_ref = rhs - y

    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    d_rowptr, d_cols, d_vals = t(rowptr), t(cols), t(vals.reshape(-1))
    d_x, d_b = t(x.reshape(-1)), t(rhs.reshape(-1))
    stream = torch.cuda.current_stream(dev)
    results = []
    for _ in range(2):
        d_r = torch.full((4 * npn,), float("nan"), dtype=torch.float64, device=dev)
        d_norms = torch.full((2,), float("nan"), dtype=torch.float64, device=dev)
        rc = lib.fts_bsr_residual_noalloc(
            npn, d_rowptr.data_ptr(), d_cols.data_ptr(), d_vals.data_ptr(), d_x.data_ptr(),
            d_b.data_ptr(), d_r.data_ptr(), d_norms.data_ptr(), C.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize(dev)
        results.append((d_r.cpu().numpy().reshape(npn, 4), d_norms.cpu().numpy()))

    for r, norms in results:
        assert np.abs(r - r_ref).max() <= TOL * np.abs(rhs).max()
        rel = np.sqrt(norms[0] / norms[1])
        # the solve reports the residual of its own operator storage (the
        # lattice half stencil on this mesh), summed in another order: at a
        # residual of ~1e-12 the two agree to the rounding of the products
        assert abs(rel - solve_rel) <= 1e-3 * solve_rel + 1e-15
        assert abs(norms[1] - float(np.sum(rhs * rhs))) <= TOL * norms[1]
        assert abs(norms[0] - float(np.sum(r_ref * r_ref))) <= 1e-9 * norms[0]
    # the second call starts from the shared scratch the first call left behind
    assert np.array_equal(results[0][0], results[1][0])
    assert np.array_equal(results[0][1], results[1][1])

    # sizes beyond the static scratch are refused before any launch
    rc = lib.fts_bsr_residual_noalloc(
        _api.NOALLOC_MAX_NODES + 1, d_rowptr.data_ptr(), d_cols.data_ptr(),
        d_vals.data_ptr(), d_x.data_ptr(), d_b.data_ptr(), d_r.data_ptr(),
        d_norms.data_ptr(), C.c_void_p(stream.cuda_stream))
    assert rc == 1
    f.close()
