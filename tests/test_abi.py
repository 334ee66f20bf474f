"""CPU tests of the C ABI library and the host-side logic (no GPU compute).

libfts.so must load and export every function include/fts.h declares; the
numpy input generator and the parameter mapping run on the host.
"""
from __future__ import annotations

import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared(header: str) -> list[str]:
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(fts_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(lib_built):
    from fluidtissue_gb300 import _native
    lib = _native.load()
    for header in ("fts.h",):
        names = _declared(header)
        assert names, header
        for name in names:
            assert hasattr(lib, name), f"{name} declared in {header} but not exported"


def test_abi_signatures_cover_header(lib_built):
    from fluidtissue_gb300 import _api
    assert set(_declared("fts.h")) == set(_api.SIGNATURES)


def test_params_default_and_status_strings(lib_built):
    from fluidtissue_gb300 import _api, _native
    lib = _native.load()
    p = _api.FtsParams()
    lib.fts_params_default(C.byref(p))
    assert p.velocity_degree == 1 and p.alpha == 0.032 and p.eps == 1e-3 and p.tol == 1e-4
    assert p.warm_start == 1 and p.precision == _api.PREC_FP64
    for code, name in _api.STATUS.items():
        assert lib.fts_status_string(code).decode() != "unknown status", name
    assert lib.fts_status_string(99).decode() == "unknown status"


def test_create_rejects_bad_meshes_on_the_host(lib_built):
    """Validation happens before any device work: bad input -> FTS_ERR_BAD_INPUT."""
    from fluidtissue_gb300 import _api, _native
    from fluidtissue_gb300.flow import Mesh, make_params
    lib = _native.load()
    xyz = np.zeros((4, 3), np.float32)
    tets = np.array([[0, 1, 2, 7]], np.int32)  # index out of range
    m = _api.FtsMesh()
    m.np, m.nt = 4, 1
    m.xyz = xyz.ctypes.data_as(C.POINTER(C.c_float))
    m.tets = tets.ctypes.data_as(C.POINTER(C.c_int32))
    ctx = C.c_void_p()
    p = make_params({"Stokes velocity degree": 1, "alpha": 0.1, "eps": 1e-3,
                     "Stokes tolerance": 1e-8, "Advection dt": 1.0, "GF growth": 1.0},
                    precision="fp64")
    assert lib.fts_create(C.byref(m), C.byref(p), C.byref(ctx)) == 1
    assert "out of range" in lib.fts_last_error(None).decode()
    p.velocity_degree = 3  # neither P1-P1 nor P2-P1
    assert lib.fts_create(C.byref(m), C.byref(p), C.byref(ctx)) == 6
    p.velocity_degree = 2  # P2-P1 passes the parameter check; the mesh is still refused
    assert lib.fts_create(C.byref(m), C.byref(p), C.byref(ctx)) == 1
    p.velocity_degree = 1
    # surface tension passes the parameter check (its load comes with the
    # solve); the mesh is still refused
    p.surface_tension = 1.0
    assert lib.fts_create(C.byref(m), C.byref(p), C.byref(ctx)) == 1
    del Mesh


def test_parameters_mapping_uses_reference_keys(lib_built, capsys):
    from fluidtissue_gb300.flow import make_params
    par = {"Stokes velocity degree": 1.0, "alpha": 0.2, "eps": 1e-4, "Stokes tolerance": 1e-9,
           "Max. CG iterations": 500, "Viscosity interior": 100.0, "Viscosity exterior": 1.0,
           "Viscosity profile": 2.0, "GF growth": 0.7, "Level sink": 0.1,
           "Growth threshold": 0.2, "RD iterations": 16000.0, "GF production": 40.0,
           "Advection dt": 0.015625, "Surface tension": 0.0}
    p = make_params(par, precision="mixed", preconditioner="jacobi")
    assert (p.alpha, p.eps, p.tol, p.max_iter) == (0.2, 1e-4, 1e-9, 500)
    assert (p.mu_interior, p.mu_exterior, p.mu_profile) == (100.0, 1.0, 2)
    assert (p.gf_growth, p.level_sink, p.growth_threshold) == (0.7, 0.1, 0.2)
    assert (p.rd_iterations, p.gf_production, p.advection_dt) == (16000.0, 40.0, 0.015625)
    assert p.precision == 1 and p.preconditioner == 1
    # a missing key reads as 0.0 with the reference's warning (Parameters.hpp:24-34)
    par.pop("Advection dt")
    p = make_params(par)
    assert p.advection_dt == 0.0
    assert "Parameter 'Advection dt' not defined" in capsys.readouterr().err


def test_kuhn_generator():
    from fluidtissue_gb300 import workloads as W
    xyz, tets, bnd = W.kuhn_mesh(5, 0.1, 3)
    assert xyz.shape == (125, 3) and tets.shape == (6 * 64, 4)
    P = xyz.astype(np.float64)[tets]
    B = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=2)
    vol = np.abs(np.linalg.det(B)) / 6.0
    assert vol.min() > 0 and abs(vol.sum() - 1.0) < 1e-6
    idx = np.arange(125)
    i, j, k = idx % 5, (idx // 5) % 5, idx // 25
    face = (i == 0) | (i == 4) | (j == 0) | (j == 4) | (k == 0) | (k == 4)
    assert np.array_equal(bnd.astype(bool), face)
    # boundary nodes stay on their faces, interior nodes moved by at most 0.1 h
    h = 0.25
    grid = np.stack([i, j, k], axis=1) * h
    d = np.abs(xyz - grid)
    assert d.max() <= 0.1 * h + 1e-7
    assert np.all(d[i == 0, 0] == 0) and np.all(d[k == 4, 2] == 0)
    # determinism
    xyz2, tets2, _ = W.kuhn_mesh(5, 0.1, 3)
    assert np.array_equal(xyz, xyz2) and np.array_equal(tets, tets2)


def test_workload_shapes():
    from fluidtissue_gb300 import workloads as W
    inst = W.sphere17()
    assert inst.np == 17 ** 3 and inst.nt == 24576
    assert inst.mu.min() >= 0.01 - 1e-15 and inst.mu.max() <= 1.0 + 1e-15
    assert np.all(inst.source >= 0)
    sz = W.system_sizes(129)
    assert sz["nt"] == 12582912 and sz["N_reduced"] == 8291838 and sz["N_block"] == 8586756
    b = W.batch_instance(5)
    assert 17 <= b.n <= 65
    assert b.params["Stokes tolerance"] == 1e-8


@pytest.mark.parametrize("n", [3, 9])
def test_boundary_detection_matches_generator(n):
    import oracle as O
    from fluidtissue_gb300 import workloads as W
    xyz, tets, bnd = W.kuhn_mesh(n, 0.0, 1)
    assert np.array_equal(O.boundary_nodes(n ** 3, tets), bnd)
