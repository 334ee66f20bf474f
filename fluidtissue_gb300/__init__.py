"""fluidtissue_gb300 — GB300-native variable-viscosity P1-P1 Stokes solve.

A drop-in for the Stokes step of tjhakkin/fluidtissue (``Flow::init`` /
``Flow::solve``, src/growth/Flow.cpp:20-94): the same mesh, level set, growth
factor and viscosity go in; the same nodal velocity and pressure come out.
The compute path is hand-written sm_103a CUDA behind the C ABI in
``include/fts.h`` (``libfts.so``); :mod:`fluidtissue_gb300.flow` mirrors the
reference's ``Flow`` class on top of it.
"""
from __future__ import annotations

__all__ = ["flow", "workloads", "build"]
