"""The C++ drop-in (include/fts_flow.hpp) compiles against stand-ins for the
reference's types, links against libfts.so and, on a GPU, solves."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from conftest import ROOT


def _build(tmp_path):
    from fluidtissue_gb300 import build as B
    exe = tmp_path / "flow_shim"
    cmd = ["g++", "-O2", "-std=c++17", f"-I{ROOT / 'include'}",
           str(ROOT / "tests" / "cpp" / "flow_shim_main.cpp"), "-o", str(exe),
           f"-L{B.BUILD}", "-lfts", f"-Wl,-rpath,{B.BUILD}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_compiles_and_refuses_without_gpu(lib_built, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: covered by the gpu-marked test")
    exe = _build(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 10, (r.returncode, r.stdout, r.stderr)
    assert "FlowGPU::init()" in r.stderr


def _crossings(xyz, tets, phi):
    """Edge crossings of phi's zero level set (LevelSet.cpp:278-300), restated
    here for the checker: edges whose end values differ in sign bit, the point
    at t = phi0 / (phi0 - phi1) in double, stored as float."""
    sb = np.signbit(phi)
    t4 = np.asarray(tets, np.int64)
    e = np.concatenate([t4[sb[t4[:, a]] != sb[t4[:, b]]][:, [a, b]]
                        for a in range(4) for b in range(a + 1, 4)])
    e = np.unique(np.sort(e, axis=1), axis=0)
    f0, f1 = phi[e[:, 0]], phi[e[:, 1]]
    t = f0 / (f0 - f1)
    p = (1.0 - t)[:, None] * xyz[e[:, 0]].astype(np.float64) + \
        t[:, None] * xyz[e[:, 1]].astype(np.float64)
    return p.astype(np.float32)


@pytest.mark.gpu
def test_shim_solves_on_gpu(lib_built, tmp_path):
    """FlowGPU's two solves: without surface tension, and with "Surface
    tension" 1 / "Node density" 2, where FlowGPU builds the load itself from
    getPhi().  The second is checked against the C ABI route (distance reset,
    load, fts_solve with `force`) and its load against the oracle's
    restatement of Flow::surfaceTension_ given the oracle's own distance reset."""
    import oracle as O
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.flow import Flow, Mesh
    from fluidtissue_gb300.levelset import LevelSet
    exe = _build(tmp_path)
    out = tmp_path / "shim.bin"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert "FlowGPU solved" in r.stdout and "with surface tension" in r.stdout
    raw = out.read_bytes()
    npn = int(np.frombuffer(raw[:8], np.int64)[0])
    v = np.frombuffer(raw[8:], np.float64)
    phi, src = v[:npn], v[npn:2 * npn]
    flow_st = v[6 * npn:10 * npn]
    load = v[10 * npn:13 * npn].reshape(3, npn)
    xyz, tets, _ = W.kuhn_mesh(9, 0.0, 1)
    assert xyz.shape[0] == npn

    par = {"Stokes velocity degree": 1.0, "alpha": 0.1, "eps": 1e-3, "Stokes tolerance": 1e-9,
           "Viscosity interior": 10.0, "Viscosity exterior": 1.0, "Viscosity profile": 0.0,
           "GF growth": 0.5, "Advection dt": 1.0, "Surface tension": 1.0, "Node density": 2.0}
    ls = LevelSet()
    assert ls.init(Mesh(xyz, tets)) == 0, ls.last_error()
    reset = ls.distance_reset(phi)
    force = ls.surface_tension(phi, par, phi_reset=reset)
    assert np.abs(force - load).max() <= 1e-12 * np.abs(load).max()
    f = Flow()
    assert f.init(Mesh(xyz, tets), par, precision="fp64") == 0, f.last_error()
    flow = np.zeros(4 * npn)
    assert f.solve(phi, src, flow, force=force.ravel()) == 0, f.last_error()
    assert np.linalg.norm(flow - flow_st) <= 1e-10 * np.linalg.norm(flow)
    f.close()
    ls.close()

    # the oracle: its distance reset of phi's crossings (float distances: equal
    # to a few ulps), then its load from the same reset values (the load goes
    # through float curvature of the reset's second differences, which moves by
    # percents under ulp changes of the reset, so both sides take one reset)
    ref_reset = phi.copy()
    assert O.dist_reset(xyz, _crossings(xyz, tets, phi), ref_reset) == 0
    ulp = np.spacing(np.abs(ref_reset).astype(np.float32)).astype(np.float64)
    assert np.all(np.abs(reset - ref_reset) <= 4 * ulp)
    fo, nif, _ = O.surface_tension(xyz, tets, phi, reset, 1.0, 2)
    assert nif > 0
    assert np.abs(load - fo).max() <= 1e-5 * np.abs(fo).max()
