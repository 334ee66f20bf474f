"""The C++ drop-in (include/fts_flow.hpp) compiles against stand-ins for the
reference's types, links against libfts.so and, on a GPU, solves."""
from __future__ import annotations

import subprocess

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


@pytest.mark.gpu
def test_shim_solves_on_gpu(lib_built, tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert "FlowGPU solved" in r.stdout
