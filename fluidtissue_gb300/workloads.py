"""Seeded synthetic Stokes-solve workloads (the five benchmark shapes).

Each workload builds, in plain numpy, exactly the arrays the reference's
``Flow::solve`` consumes (src/growth/Flow.cpp:89): a tetrahedral mesh with float
coordinates, a nodal level set ``phi`` (negative inside), a nodal growth factor
``source`` and, because the workloads prescribe viscosity laws instead of the
reference's growth-factor profiles (src/growth/ViscosityProfiles.hpp), a
per-element viscosity ``mu`` evaluated at element centroids.

The reference builds its mesh by CGAL Delaunay of a node lattice
(src/fem/TetraMesh.cpp:23-165) and gets phi, the growth factor and the
viscosity from its level-set, reaction-diffusion and viscosity-profile
modules; none of those is on the Stokes path, so this generator stands in for
them.  It is numpy only (no compiled code), so the CUDA path, the CPU oracle,
the tests and both benchmark arms read the same arrays and none of them needs
the other's library to make its inputs.  Everything is deterministic for a
given seed: a counter-based hash (splitmix64 finaliser), no global RNG state.

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

import concurrent.futures as cf
import os
from dataclasses import dataclass, field

import numpy as np

SPHERE, ELLIPSOID, TWO_SPHERES = 0, 1, 2
MU_BAND, MU_INVERSE, MU_CONSTANT = 0, 1, 2

_M64 = (1 << 64) - 1
_CHUNK = 1 << 18  # elements or nodes per worker task


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


@dataclass
class Shape:
    """Analytic level set (negative inside): a sphere |x - c| - r, a
    first-order distance estimate to an axis-aligned ellipsoid, or the union
    (minimum) of two sphere distances."""
    kind: int
    center: tuple = (0.5, 0.5, 0.5)
    radius: float = 0.25
    axes: tuple = (0.3, 0.2, 0.25)
    center2: tuple = (0.5, 0.5, 0.5)
    radius2: float = 0.0


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


# ---- counter-based uniform numbers ----------------------------------------

def _mix64(z: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on uint64 arrays (wrapping arithmetic)."""
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform_array(seed: int, stream: int, index: np.ndarray) -> np.ndarray:
    """Uniform doubles in [0, 1) with 53 random bits, one per index."""
    idx = np.asarray(index).astype(np.uint64)
    inner = np.uint64((stream * 0xD1B54A32D192ED03) & _M64) ^ _mix64(idx)
    h = _mix64(np.uint64(seed & _M64) ^ _mix64(inner))
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def uniform(seed: int, stream: int, index: int) -> float:
    return float(uniform_array(seed, stream, np.array([index]))[0])


# ---- mesh -----------------------------------------------------------------

# The 6 Kuhn tetrahedra of a cube: the monotone lattice paths from corner
# (0,0,0) to (1,1,1), one per axis permutation (element 6c + t of cube c).
_PERM = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))


def _pool():
    return cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1))


def kuhn_mesh(n: int, jitter: float, seed: int):
    """Kuhn-split lattice of [0,1]^3 with n nodes per axis.  Node (i,j,k) has
    index i + n j + n^2 k and sits at (i,j,k)/(n-1), moved by a uniform jitter
    in [-jitter h, +jitter h] (h = 1/(n-1)) along every axis in which it is not
    on a cube face, so the faces stay planar.  Returns xyz float32 [np,3],
    tets int32 [nt,4] and boundary uint8 [np] (1 on the cube faces)."""
    if n < 2:
        raise ValueError(f"bad lattice size {n}")
    npn = n ** 3
    h = 1.0 / (n - 1)
    xyz = np.empty((npn, 3), np.float32)
    bnd = np.empty(npn, np.uint8)

    def nodes(lo):
        hi = min(lo + _CHUNK, npn)
        v = np.arange(lo, hi, dtype=np.int64)
        ijk = (v % n, (v // n) % n, v // (n * n))
        onb = np.zeros(hi - lo, bool)
        for a in range(3):
            face = (ijk[a] == 0) | (ijk[a] == n - 1)
            onb |= face
            x = ijk[a].astype(np.float64) * h
            if jitter != 0.0:
                u = uniform_array(seed, 1 + a, v)
                x = np.where(face, x, x + (2.0 * u - 1.0) * jitter * h)
            xyz[lo:hi, a] = x.astype(np.float32)
        bnd[lo:hi] = onb

    m = n - 1
    ncube = m ** 3
    tets = np.empty((ncube, 6, 4), np.int32)
    off = (1, n, n * n)

    def cubes(lo):
        hi = min(lo + _CHUNK, ncube)
        c = np.arange(lo, hi, dtype=np.int64)
        base = (c % m) + n * (((c // m) % m) + n * (c // (m * m)))
        far = base + 1 + n + n * n
        for t, p in enumerate(_PERM):
            tets[lo:hi, t, 0] = base
            tets[lo:hi, t, 1] = base + off[p[0]]
            tets[lo:hi, t, 2] = base + off[p[0]] + off[p[1]]
            tets[lo:hi, t, 3] = far

    with _pool() as ex:
        list(ex.map(nodes, range(0, npn, _CHUNK)))
        list(ex.map(cubes, range(0, ncube, _CHUNK)))
    return xyz, tets.reshape(6 * ncube, 4), bnd


# ---- level sets, growth factor, viscosity ---------------------------------

def shape(kind: int, center=(0.5, 0.5, 0.5), radius=0.25, axes=(0.3, 0.2, 0.25),
          center2=(0.5, 0.5, 0.5), radius2=0.0) -> Shape:
    return Shape(kind, tuple(center), radius, tuple(axes), tuple(center2), radius2)


def _sq(v):
    return v * v


def shape_phi(s: Shape, x, y, z):
    """Level-set value at points (float64 arrays)."""
    if s.kind == SPHERE:
        c = s.center
        return np.sqrt(_sq(x - c[0]) + _sq(y - c[1]) + _sq(z - c[2])) - s.radius
    if s.kind == ELLIPSOID:
        # k0 (k0 - 1) / k1 with k0 = |p/a|, k1 = |p/a^2|: exact sign, first-order
        # distance near the surface
        a, c = s.axes, s.center
        px, py, pz = x - c[0], y - c[1], z - c[2]
        k0 = np.sqrt(_sq(px / a[0]) + _sq(py / a[1]) + _sq(pz / a[2]))
        k1 = np.sqrt(_sq(px / (a[0] * a[0])) + _sq(py / (a[1] * a[1])) +
                     _sq(pz / (a[2] * a[2])))
        with np.errstate(divide="ignore", invalid="ignore"):
            out = k0 * (k0 - 1.0) / k1
        return np.where(k1 == 0.0, -min(a), out)
    if s.kind == TWO_SPHERES:
        c, d = s.center, s.center2
        d1 = np.sqrt(_sq(x - c[0]) + _sq(y - c[1]) + _sq(z - c[2])) - s.radius
        d2 = np.sqrt(_sq(x - d[0]) + _sq(y - d[1]) + _sq(z - d[2])) - s.radius2
        return np.fmin(d1, d2)
    return np.zeros_like(x)


def surface_points(s: Shape, m: int, seed: int) -> np.ndarray:
    """m seeded points on the zero level set: a uniform direction on the unit
    sphere (attempt index k*64 + a), mapped onto the sphere / ellipsoid; for two
    spheres one sphere is picked with probability proportional to r^2 and a
    point buried inside the other sphere is redrawn (up to 63 times)."""
    pts = np.empty((m, 3))
    two_pi = 6.283185307179586476925286766559
    for k in range(m):
        for attempt in range(64):
            idx = np.array([k * 64 + attempt])
            zc = 2.0 * uniform_array(seed, 101, idx)[0] - 1.0
            th = two_pi * uniform_array(seed, 102, idx)[0]
            rr = np.sqrt(max(0.0, 1.0 - zc * zc))
            d = (rr * np.cos(th), rr * np.sin(th), zc)
            if s.kind == SPHERE:
                p = [s.center[a] + s.radius * d[a] for a in range(3)]
            elif s.kind == ELLIPSOID:
                p = [s.center[a] + s.axes[a] * d[a] for a in range(3)]
            else:
                w1, w2 = s.radius * s.radius, s.radius2 * s.radius2
                first = uniform_array(seed, 103, idx)[0] * (w1 + w2) < w1
                c, r = (s.center, s.radius) if first else (s.center2, s.radius2)
                p = [c[a] + r * d[a] for a in range(3)]
                co, ro = (s.center2, s.radius2) if first else (s.center, s.radius)
                dist = np.sqrt(_sq(p[0] - co[0]) + _sq(p[1] - co[1]) + _sq(p[2] - co[2]))
                if dist < ro and attempt < 63:
                    continue  # buried inside the other sphere
            pts[k] = p
            break
    return pts


def _gaussians(x, y, z, centres, inv2s2, amp):
    acc = np.zeros_like(x)
    for cx, cy, cz in centres:
        r2 = _sq(x - cx) + _sq(y - cy) + _sq(z - cz)
        acc += amp * np.exp(-r2 * inv2s2)
    return acc


def fields(sh: Shape, xyz, tets, centres, sigma, amp=1.0, elem=True):
    """Nodal phi and growth factor c = sum of Gaussians, and (elem) the same
    two laws at every element's centroid (coordinates summed in double in
    local order, times 1/4)."""
    npn, nt = xyz.shape[0], tets.shape[0]
    inv2s2 = 1.0 / (2.0 * sigma * sigma)
    cen = [tuple(map(float, c)) for c in np.asarray(centres, np.float64)]
    phi, c = np.empty(npn), np.empty(npn)
    phe = np.empty(nt) if elem else None
    ce = np.empty(nt) if elem else None

    def nodes(lo):
        hi = min(lo + _CHUNK, npn)
        p = xyz[lo:hi].astype(np.float64)
        x, y, z = p[:, 0], p[:, 1], p[:, 2]
        phi[lo:hi] = shape_phi(sh, x, y, z)
        c[lo:hi] = _gaussians(x, y, z, cen, inv2s2, amp)

    def elems(lo):
        hi = min(lo + _CHUNK, nt)
        t = tets[lo:hi]
        g = xyz[t[:, 0]].astype(np.float64)
        for j in range(1, 4):
            g += xyz[t[:, j]].astype(np.float64)
        g *= 0.25
        x, y, z = g[:, 0], g[:, 1], g[:, 2]
        phe[lo:hi] = shape_phi(sh, x, y, z)
        ce[lo:hi] = _gaussians(x, y, z, cen, inv2s2, amp)

    with _pool() as ex:
        list(ex.map(nodes, range(0, npn, _CHUNK)))
        if elem:
            list(ex.map(elems, range(0, nt, _CHUNK)))
    return phi, c, phe, ce


def viscosity(law, phe, ce, p0, p1=0.0, p2=0.0):
    """Per-element viscosity: BAND blends p0 (inside) to p1 (outside) linearly
    in phi over a band of width p2 centred on the interface; INVERSE is
    1/(p0 + c) clipped to [p1, p2]; CONSTANT is p0."""
    if law == MU_BAND:
        t = np.clip(0.5 - phe / p2, 0.0, 1.0)
        return p1 + (p0 - p1) * t
    if law == MU_INVERSE:
        return np.clip(1.0 / (p0 + ce), p1, p2)
    nt = (phe if phe is not None else ce).shape[0]
    return np.full(nt, float(p0))


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


__all__ = ["Instance", "Shape", "WORKLOADS", "sphere17", "sphere65", "ellipsoid129",
           "spheres257", "batch96", "batch_instance", "kuhn_mesh", "base_params",
           "system_sizes", "uniform"]
