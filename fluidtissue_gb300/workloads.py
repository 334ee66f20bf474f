"""Seeded synthetic Stokes-solve workloads (the five benchmark shapes).

Each workload builds, through the C++ generator in libfts.so
(include/fts_gen.h), exactly the arrays the reference's ``Flow::solve``
consumes (src/growth/Flow.cpp:89): a tetrahedral mesh with float coordinates,
a nodal level set ``phi`` (negative inside), a nodal growth factor ``source``
and, because the workloads prescribe viscosity laws instead of the
reference's growth-factor profiles (src/growth/ViscosityProfiles.hpp), a
per-element viscosity ``mu`` evaluated at element centroids.

  * ``sphere17``      17^3 Kuhn lattice, no jitter, sphere r=0.25, 3 centres
                      sigma 0.08 (seed 42), mu 1 inside / 0.01 outside blended
                      over 1.5h, source 0.5 c inside, tol 1e-10.
  * ``sphere65``      65^3, jitter +-0.1h (seed 7), same sphere, 8 centres
                      sigma 0.05, mu = 1, tol 1e-10 (parity case).
  * ``ellipsoid129``  129^3, jitter +-0.1h, ellipsoid (0.3,0.2,0.25), 16
                      centres sigma 0.04, mu = clip(1/(0.01+c), 0.01, 100),
                      tol 1e-8 (the benchmark workload).
  * ``batch96``       96 instances, n ~ U{17..65}, jitter +-0.1h, seed = id,
                      r ~ U[0.15,0.35], mu_in/mu_out log-uniform in [1,1e3],
                      3..12 centres, tol 1e-8.
  * ``spheres257``    257^3, jitter +-0.1h, union of spheres r=0.2 and 0.15 with
                      centres 0.3 apart, 24 centres sigma 0.03,
                      mu = clip(1/(0.01+c), 0.01, 100), tol 1e-8.

The source law g = 0.5 c inside / 0 outside maps onto the reference's
parameters "GF growth" = 0.5, "Level sink" = 0, "Growth threshold" = 0
(src/growth/Flow.cpp:368-372), including its zero-mean shift.  alpha = 0.1
(stabilisation 0.1 h^2), eps = 1e-3 (parameters/summary.txt:5).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N

SPHERE, ELLIPSOID, TWO_SPHERES = 0, 1, 2
MU_BAND, MU_INVERSE, MU_CONSTANT = 0, 1, 2


@dataclass
class Instance:
    name: str
    n: int
    xyz: np.ndarray          # float32 [np, 3]
    tets: np.ndarray         # int32 [nt, 4]
    boundary: np.ndarray     # uint8 [np]
    phi: np.ndarray          # float64 [np]
    source: np.ndarray       # float64 [np]
    mu: np.ndarray           # float64 [nt]
    params: dict = field(default_factory=dict)

    @property
    def np(self) -> int:
        return self.xyz.shape[0]

    @property
    def nt(self) -> int:
        return self.tets.shape[0]


def base_params(tol: float) -> dict:
    """Reference parameter keys (src/growth/Flow.cpp, ViscosityProfiles.hpp)."""
    return {
        "Stokes velocity degree": 1.0,
        "alpha": 0.1,
        "eps": 1e-3,
        "Stokes tolerance": tol,
        "Max. CG iterations": -1.0,
        "GF growth": 0.5,
        "Level sink": 0.0,
        "Growth threshold": 0.0,
        "Surface tension": 0.0,
        "Advection dt": 1.0,
        "RD iterations": 0.0,
        # the explicit per-element mu overrides the profile; these only matter
        # for the early-exit rule of Flow.cpp:223-225
        "Viscosity interior": 1.0,
        "Viscosity exterior": 1.0,
        "Viscosity profile": 0.0,
    }


def kuhn_mesh(n: int, jitter: float, seed: int):
    lib = N.load()
    np_, nt_ = C.c_int64(), C.c_int64()
    if lib.fts_gen_kuhn_counts(n, C.byref(np_), C.byref(nt_)) != 0:
        raise ValueError(f"bad lattice size {n}")
    xyz = np.empty((np_.value, 3), np.float32)
    tets = np.empty((nt_.value, 4), np.int32)
    bnd = np.empty(np_.value, np.uint8)
    rc = lib.fts_gen_kuhn_mesh(n, jitter, seed, N.ptr(xyz, C.c_float), N.ptr(tets, C.c_int32),
                               N.ptr(bnd, C.c_uint8))
    if rc != 0:
        raise RuntimeError("fts_gen_kuhn_mesh failed")
    return xyz, tets, bnd


def shape(kind: int, center=(0.5, 0.5, 0.5), radius=0.25, axes=(0.3, 0.2, 0.25),
          center2=(0.5, 0.5, 0.5), radius2=0.0) -> N.FtsGenShape:
    s = N.FtsGenShape()
    s.kind = kind
    s.center[:] = list(center)
    s.radius = radius
    s.axes[:] = list(axes)
    s.center2[:] = list(center2)
    s.radius2 = radius2
    return s


def surface_points(sh: N.FtsGenShape, m: int, seed: int) -> np.ndarray:
    lib = N.load()
    pts = np.empty((m, 3), np.float64)
    lib.fts_gen_surface_points(C.byref(sh), m, seed, N.ptr(pts, C.c_double))
    return pts


def fields(sh, xyz, tets, centres, sigma, amp=1.0, elem=True):
    lib = N.load()
    npn, nt = xyz.shape[0], tets.shape[0]
    phi = np.empty(npn)
    c = np.empty(npn)
    phe = np.empty(nt) if elem else None
    ce = np.empty(nt) if elem else None
    cen = np.ascontiguousarray(centres, np.float64)
    rc = lib.fts_gen_fields(C.byref(sh), npn, nt, N.ptr(xyz, C.c_float), N.ptr(tets, C.c_int32),
                            cen.shape[0], N.ptr(cen, C.c_double), sigma, amp,
                            N.ptr(phi, C.c_double), N.ptr(c, C.c_double),
                            N.ptr(phe, C.c_double), N.ptr(ce, C.c_double))
    if rc != 0:
        raise RuntimeError("fts_gen_fields failed")
    return phi, c, phe, ce


def viscosity(law, phe, ce, p0, p1=0.0, p2=0.0):
    lib = N.load()
    nt = (phe if phe is not None else ce).shape[0]
    mu = np.empty(nt)
    rc = lib.fts_gen_viscosity(nt, N.ptr(phe, C.c_double), N.ptr(ce, C.c_double), law,
                               p0, p1, p2, N.ptr(mu, C.c_double))
    if rc != 0:
        raise RuntimeError("fts_gen_viscosity failed")
    return mu


def uniform(seed: int, stream: int, index: int) -> float:
    return float(N.load().fts_gen_uniform(seed, stream, index))


def _instance(name, n, jitter, mesh_seed, sh, ncent, cent_seed, sigma, mu_law, tol):
    xyz, tets, bnd = kuhn_mesh(n, jitter, mesh_seed)
    cen = surface_points(sh, ncent, cent_seed)
    phi, c, phe, ce = fields(sh, xyz, tets, cen, sigma)
    h = 1.0 / (n - 1)
    law, p0, p1, p2 = mu_law(h)
    mu = viscosity(law, phe, ce, p0, p1, p2)
    return Instance(name, n, xyz, tets, bnd, phi, c, mu, base_params(tol))


def sphere17(n: int = 17) -> Instance:
    return _instance("sphere17", n, 0.0, 0, shape(SPHERE, radius=0.25), 3, 42, 0.08,
                     lambda h: (MU_BAND, 1.0, 0.01, 1.5 * h), 1e-10)


def sphere65(n: int = 65) -> Instance:
    return _instance("sphere65", n, 0.1, 7, shape(SPHERE, radius=0.25), 8, 7, 0.05,
                     lambda h: (MU_CONSTANT, 1.0, 0.0, 0.0), 1e-10)


def ellipsoid129(n: int = 129) -> Instance:
    return _instance("ellipsoid129", n, 0.1, 129, shape(ELLIPSOID, axes=(0.3, 0.2, 0.25)), 16,
                     129, 0.04, lambda h: (MU_INVERSE, 0.01, 0.01, 100.0), 1e-8)


def spheres257(n: int = 257) -> Instance:
    sh = shape(TWO_SPHERES, center=(0.35, 0.5, 0.5), radius=0.2, center2=(0.65, 0.5, 0.5),
               radius2=0.15)
    return _instance("spheres257", n, 0.1, 257, sh, 24, 257, 0.03,
                     lambda h: (MU_INVERSE, 0.01, 0.01, 100.0), 1e-8)


def batch_instance(i: int, nmin: int = 17, nmax: int = 65) -> Instance:
    """Instance i of the batched workload (all draws seeded by i)."""
    u = lambda k: uniform(i, 900, k)  # noqa: E731
    n = nmin + min(int(u(0) * (nmax - nmin + 1)), nmax - nmin)
    r = 0.15 + 0.2 * u(1)
    ratio = 10.0 ** (3.0 * u(2))
    ncent = 3 + min(int(u(3) * 10), 9)
    mu_in, mu_out = 1.0, 1.0 / ratio
    return _instance(f"batch{i}", n, 0.1, i, shape(SPHERE, radius=r), ncent, i, 0.05,
                     lambda h: (MU_BAND, mu_in, mu_out, 1.5 * h), 1e-8)


def batch96(count: int = 96, nmin: int = 17, nmax: int = 65) -> list[Instance]:
    return [batch_instance(i, nmin, nmax) for i in range(count)]


WORKLOADS = {
    "sphere17": sphere17,
    "sphere65": sphere65,
    "ellipsoid129": ellipsoid129,
    "spheres257": spheres257,
}


def system_sizes(n: int) -> dict:
    npn = n ** 3
    ni = (n - 2) ** 3
    return {"np": npn, "nt": 6 * (n - 1) ** 3, "nI": ni, "N_reduced": 3 * ni + npn,
            "N_block": 4 * npn}


__all__ = ["Instance", "WORKLOADS", "sphere17", "sphere65", "ellipsoid129", "spheres257",
           "batch96", "batch_instance", "kuhn_mesh", "base_params", "system_sizes"]
