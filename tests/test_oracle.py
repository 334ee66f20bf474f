"""CPU tests of the oracle (the checker) — no GPU.

The reference has no tests or golden vectors and cannot be built here, so the
oracle is pinned by known-answer identities of the P1 forms, by a direct
sparse solve of the same system, and by the committed fixtures in
tests/golden (regression pins).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ROOT, workload

import oracle as O  # noqa: E402


def _blocks(inst, alpha=None, eps=None, mu=None, s=None):
    par = inst.params
    s = O.source(inst.phi, inst.source, par["GF growth"]) if s is None else s
    return O.assemble_blocks(inst.xyz, inst.tets, inst.mu if mu is None else mu, s,
                             par["alpha"] if alpha is None else alpha,
                             par["eps"] if eps is None else eps)


def _volumes(inst):
    P = inst.xyz.astype(np.float64)[inst.tets]
    B = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=2)
    return np.abs(np.linalg.det(B)) / 6.0


def test_reference_tables():
    tab, qw = O.ref_tables()
    a = (5 + 3 * np.sqrt(5)) / 20
    b = (5 - np.sqrt(5)) / 20
    # float-rounded P1 values at the 4-point rule (Quadrature.hpp:24-36)
    assert tab[1, 0] == float(np.float32(a)) and tab[1, 1] == float(np.float32(b))
    assert tab[0, 3] == float(np.float32(1.0 - 3 * float(np.float32(b))))
    assert qw == 0.25 / 6.0
    assert np.allclose(tab.sum(axis=0), 1.0, atol=1e-7)


@pytest.mark.parametrize("name,n", [("sphere17", 9), ("sphere65", 9)])
def test_mass_matrix_sums_to_volume(name, n):
    inst = workload(name, n)
    B = _blocks(inst, alpha=0.0, eps=1.0)
    M = B.vals[:, 3, 3]
    # The basis table is float-rounded (Tetrahedron.hpp:17-18), so the mass
    # matrix sums to volume * sum_q w_q (sum_a phi_a(q))^2, not exactly to 1.
    tab, _ = O.ref_tables()
    table_factor = float(np.sum(0.25 * tab.sum(axis=0) ** 2))
    assert abs(table_factor - 1.0) < 1e-7
    assert abs(M.sum() - _volumes(inst).sum() * table_factor) <= 1e-12
    assert abs(_volumes(inst).sum() - 1.0) <= 1e-6


@pytest.mark.parametrize("name,n", [("sphere17", 9), ("sphere65", 9)])
def test_rigid_and_constant_identities(name, n):
    inst = workload(name, n)
    B = _blocks(inst, alpha=1.0, eps=0.0)
    npn = inst.np
    rows = np.repeat(np.arange(npn), np.diff(B.rowptr))
    V = B.vals
    # K applied to a constant velocity field vanishes on every row
    for comp in range(3):
        rs = np.zeros((npn, 3))
        np.add.at(rs, rows, V[:, :3, comp])
        assert np.abs(rs).max() <= 1e-12 * np.abs(V[:, :3, :3]).max()
    # D applied to a constant pressure vanishes (sum_j D_ij = 0)
    ds = np.zeros(npn)
    np.add.at(ds, rows, V[:, 3, 3])
    assert np.abs(ds).max() <= 1e-12 * np.abs(V[:, 3, 3]).max()
    # sum_i B_al(i, k) = int d_al(sum_i phi_i) psi_k = 0 for every pressure column k
    cs = np.zeros((npn, 3))
    np.add.at(cs, B.cols, -V[:, :3, 3])
    assert np.abs(cs).max() <= 1e-12 * np.abs(V[:, :3, 3]).max()


def test_block_symmetry():
    inst = workload("sphere65", 9)
    B = _blocks(inst)
    npn = inst.np
    pos = {}
    rows = np.repeat(np.arange(npn), np.diff(B.rowptr))
    for q, (i, j) in enumerate(zip(rows, B.cols)):
        pos[(i, j)] = q
    for q, (i, j) in enumerate(zip(rows, B.cols)):
        t = B.vals[pos[(j, i)]]
        b = B.vals[q]
        assert np.allclose(b[:3, :3], t[:3, :3].T, rtol=0, atol=1e-15)
        assert np.allclose(b[3, :3], -t[:3, 3], rtol=0, atol=1e-15)  # B^T vs -B
        assert abs(b[3, 3] - t[3, 3]) <= 1e-15


def test_zero_source_gives_zero_rhs():
    inst = workload("sphere17", 9)
    s = np.zeros(inst.np)
    B = _blocks(inst, s=s)
    assert np.abs(B.rhs).max() == 0.0


def test_source_zero_mean_and_interior():
    inst = workload("sphere17", 9)
    s = O.source(inst.phi, inst.source, 0.5, 0.1, 0.2)
    assert abs(s.sum()) <= 1e-12 * max(1.0, np.abs(s).sum())
    raw = np.where((inst.phi < 0) & (inst.source > 0.2), (inst.source - 0.1) * 0.5, 0.0)
    assert np.allclose(s, raw - raw.mean(), atol=1e-15)


def test_boundary_nodes_are_cube_faces():
    inst = workload("sphere65", 9)
    bnd = O.boundary_nodes(inst.np, inst.tets)
    assert np.array_equal(bnd, inst.boundary)


@pytest.mark.parametrize("profile", [0, 1, 2])
def test_viscosity_profile_restatement(profile):
    inst = workload("sphere17", 9)
    mu, mm = O.set_viscosity(inst.tets, inst.phi, inst.source, 30.0, 2.0, profile, 1.0, 1.5)
    inside = np.all(inst.phi[inst.tets] < 0, axis=1)
    c3 = inst.source[inst.tets].max(axis=1)
    if profile == 2:
        c3 = np.minimum(4 * c3, 1.5)
    f = c3 / 1.5
    want = 2.0 * f + 30.0 * (1 - f) if profile == 0 else 30.0 * f + 2.0 * (1 - f)
    ref = np.where(inside, want, 2.0)
    assert np.allclose(mu, ref, rtol=1e-15, atol=0)
    assert mm[0] == ref[inside].min() and mm[1] == ref[inside].max()


def test_tight_solve_matches_direct_solve():
    inst = workload("sphere17", 9)
    R, _, _, mu = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                           inst.params)
    x, tr, _ = O.solve_tight(R, inst.xyz, inst.tets, mu, tol=1e-13)
    xd = O.direct_solve(R)
    assert tr <= 1e-12
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) <= 1e-10


def test_bicgstab_reference_algorithm():
    """Un-preconditioned BiCGSTAB (the reference's solver) reaches its stopping
    rule and agrees with the direct solve to the accuracy its tolerance allows."""
    inst = workload("sphere17", 9)
    R, _, _, _ = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                          inst.params)
    # Eigen's default cap is 2N iterations; near it the outcome depends on
    # rounding (OpenMP reduction order), so only the cap itself is checked.
    x, info, it, err = O.bicgstab(R, None, tol=1e-10)
    assert it <= 2 * R.N and (info == 0) == (err <= 1e-10)
    x, info, it, err = O.bicgstab(R, None, tol=1e-8)
    assert info == 0 and err <= 1e-8
    assert O.true_residual(R, x) <= 2e-8
    xd = O.direct_solve(R)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) <= 1e-4
    # warm start from the solution: converged at iteration 0
    x2, info2, it2, _ = O.bicgstab(R, x, tol=1e-8)
    assert info2 == 0 and it2 == 0


def test_flow_solve_early_exits():
    inst = workload("sphere17", 9)
    par = dict(inst.params)
    par["Advection dt"] = 0.0
    flow = np.full(4 * inst.np, 7.0)
    st, out, _, info = O.flow_solve(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source,
                                    inst.mu, par, flow=flow)
    assert st == 0 and np.all(out == 7.0) and info["exit"] == "advection dt zero"
    par = dict(inst.params)
    st, out, _, info = O.flow_solve(inst.xyz, inst.tets, inst.boundary, inst.phi,
                                    np.zeros(inst.np), inst.mu, par, flow=flow)
    assert st == 0 and np.all(out == 7.0) and info["exit"] == "load zero"


@pytest.mark.parametrize("fixture", ["sphere17.npz", "sphere65_n9.npz"])
def test_golden_fixture(fixture):
    """The oracle reproduces the committed fixture from the stored inputs."""
    import importlib.util
    from fluidtissue_gb300 import workloads as W
    spec = importlib.util.spec_from_file_location("mk", ROOT / "tests/golden/make_golden.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    g = np.load(ROOT / "tests" / "golden" / fixture)
    n = int(g["n"])
    inst = W.WORKLOADS[str(g["name"])](n)
    assert mk.mesh_hash(inst.xyz, inst.tets) == str(g["mesh_sha256"])
    R, _, _, mu = O.system(inst.xyz, inst.tets, g["boundary"], g["phi"], g["source"], g["mu"],
                           inst.params)
    assert np.allclose(R.F, g["F"], rtol=0, atol=1e-13 * np.abs(g["F"]).max())
    x, tr, _ = O.solve_tight(R, inst.xyz, inst.tets, mu, tol=1e-13)
    flow = O.scatter(R, x)
    ref = g["flow"]
    npn = inst.np
    ev = np.linalg.norm(flow[:3 * npn] - ref[:3 * npn]) / np.linalg.norm(ref[:3 * npn])
    ep = np.linalg.norm(flow[3 * npn:] - ref[3 * npn:]) / np.linalg.norm(ref[3 * npn:])
    assert ev <= 1e-10 and ep <= 1e-10


# ---- reaction-diffusion (RD.cpp) restatement --------------------------------

_RD0 = {"RD dt": 0.05, "RD iterations": 40.0, "Act": 0.0, "Da": 0.0, "DegA": 0.0, "Inh": 0.0,
        "Di": 0.0, "DegI": 0.0, "GF production": 0.0, "GF diffusion": 0.0,
        "GF degradation": 0.0, "GF inhibition": 0.0}


def _lumped_mass(inst):
    """Row sums of the P1 mass matrix over the interior elements, per node,
    with the float-rounded basis table (local node a's row sum is
    detB sum_b sum_q qw phi_b(q) phi_a(q), not exactly vol / 4)."""
    tab, qw = O.ref_tables()
    row = np.array([sum(qw * tab[b, q] * tab[a, q] for b in range(4) for q in range(4))
                     for a in range(4)])
    inside = inst.phi < 0
    el = np.all(inside[inst.tets], axis=1)
    m = np.zeros(inst.np)
    detb = 6.0 * _volumes(inst)[el]
    for a in range(4):
        np.add.at(m, inst.tets[el, a], detb * row[a])
    return m, inside


def test_rd_constant_fields_only_decay():
    """L 1 = 0 (K annihilates constants): uniform fields under diffusion keep
    their value; pure degradation gives g_n = g_0 (1 - dt deg)^n exactly in
    the limit of rounding."""
    inst = workload("sphere65", 13)
    par = dict(_RD0, **{"Da": 1e-3, "Di": 1e-3, "GF diffusion": 1e-3, "GF degradation": 0.1})
    inside = inst.phi < 0
    a = np.where(inside, 2.0, 0.0)
    i = np.zeros(inst.np)
    g = np.where(inside, 3.0, 0.0)
    assert O.rd_solve(inst.xyz, inst.tets, inst.phi, [], par, a, i, g) == 0
    m, _ = _lumped_mass(inst)
    live = inside & (m > 0)
    assert np.allclose(a[live], 2.0, rtol=0, atol=1e-12)
    assert np.allclose(g[live], 3.0 * (1 - 0.05 * 0.1) ** 40, rtol=1e-12)
    assert np.all(a[~inside] == 0) and np.all(g[~inside] == 0)


def test_rd_diffusion_conserves_lumped_mass():
    """sum_i m_i (L u)_i = sum_ij K_ij u_j = 0: pure diffusion conserves the
    lumped-mass-weighted total."""
    inst = workload("sphere65", 13)
    par = dict(_RD0, **{"GF diffusion": 2e-3})
    m, inside = _lumped_mass(inst)
    rng = np.random.default_rng(2)
    g = np.where(inside, rng.random(inst.np), 0.0)
    total0 = float((m * g).sum())
    a, i = np.zeros(inst.np), np.zeros(inst.np)
    assert O.rd_solve(inst.xyz, inst.tets, inst.phi, [], par, a, i, g) == 0
    assert abs(float((m * g).sum()) - total0) <= 1e-12 * total0
    assert g[inside].std() < np.where(inside, rng.random(inst.np), 0.0)[inside].std()


def test_rd_reaction_step_by_hand():
    """One Euler step on a node with no interior element around it (L row
    empty): the reaction terms alone, as in RD.cpp:79-84."""
    inst = workload("sphere17", 9)
    par = dict(_RD0, **{"RD iterations": 1.0, "Act": 2.0, "DegA": 0.01, "Inh": 1.0,
                        "DegI": 0.02, "GF inhibition": 200.0, "GF degradation": 0.02})
    m, inside = _lumped_mass(inst)
    iso = np.where(inside & (m == 0))[0]
    node = iso[0] if len(iso) else np.where(inside)[0][0]
    a = np.where(inside, 0.7, 0.0)
    i = np.where(inside, 0.3, 0.0)
    g = np.where(inside, 0.01, 0.0)
    a0, i0, g0 = a[node], i[node], g[node]
    assert O.rd_solve(inst.xyz, inst.tets, inst.phi, [], par, a, i, g) == 0
    if len(iso):
        dt = 0.05
        u2 = a0 * a0
        de = 1.0 + 1.0 * i0 + 200.0 * g0
        assert a[node] == a0 + dt * (-0.0 * 0.0 + 2.0 * (u2 / de) - 0.01 * a0)
        assert i[node] == i0 + dt * (-0.0 * 0.0 + u2 - 0.02 * i0)
        assert g[node] == g0 + dt * (-0.0 * 0.0 - 0.02 * g0)
    # a uniform interior state changes by the reaction terms only (L 1 = 0)
    live = np.where(inside & (m > 0))[0]
    u2 = 0.49
    want = 0.7 + 0.05 * (2.0 * (u2 / (1.0 + 0.3 + 200.0 * 0.01)) - 0.01 * 0.7)
    assert np.allclose(a[live], want, rtol=1e-12)


def test_rd_sources_and_refusal():
    inst = workload("sphere17", 9)
    par = dict(_RD0, **{"GF production": 5.0, "GF diffusion": 1e-3})
    inside = np.where(inst.phi < 0)[0]
    a, i, g = np.zeros(inst.np), np.zeros(inst.np), np.zeros(inst.np)
    assert O.rd_solve(inst.xyz, inst.tets, inst.phi, inside[:2], par, a, i, g) == 0
    assert np.all(g[inside[:2]] == 5.0) and g.max() == 5.0 and (g > 0).sum() > 2
    outside = np.where(inst.phi >= 0)[0][:1]
    assert O.rd_solve(inst.xyz, inst.tets, inst.phi, outside, par, a, i, g) == -1


# ---- distance reset (EuclideanDistance) restatement --------------------------

def test_distance_reset_matches_numpy_float32():
    """The host path in float: min_j sqrt(dx*dx + dy*dy + dz*dz), sign of the
    old value; against the same sums in numpy float32."""
    inst = workload("sphere17", 9)
    rng = np.random.default_rng(4)
    ifp = rng.random((257, 3)).astype(np.float32)
    phi = np.ascontiguousarray(inst.phi, np.float64).copy()
    assert O.dist_reset(inst.xyz, ifp, phi) == 0
    d = ifp[None, :, :] - inst.xyz[:, None, :]
    dd = np.sqrt(d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1] + d[..., 2] * d[..., 2]).min(axis=1)
    want = np.where(inst.phi < 0, -dd.astype(np.float64), dd.astype(np.float64))
    ulp = np.spacing(np.abs(want).astype(np.float32)).astype(np.float64)
    assert np.all(np.abs(phi - want) <= ulp)
    empty = np.ascontiguousarray(inst.phi, np.float64).copy()
    assert O.dist_reset(inst.xyz, np.zeros((0, 3), np.float32), empty) == 0
    assert np.all(np.abs(empty) == np.finfo(np.float32).max)


# ---- level-set update (LevelSet::update) restatement ---------------------------

def test_levelset_zero_velocity_and_constant_phi():
    """With no velocity the advection solve is M phi' = M phi, so phi' = phi;
    a uniform velocity field translates nothing for a constant phi either."""
    inst = workload("sphere65", 11)
    phi = np.ascontiguousarray(inst.phi, np.float64).copy()
    flow = np.zeros(4 * inst.np)
    flow[3 * inst.np:] = 1.0  # pressure only: ||flow|| > 0, velocity 0
    st, it, err, _ = O.ls_update(inst.xyz, inst.tets, flow, phi, 0.1, tol=1e-14, reset=False)
    assert st == 0 and np.allclose(phi, inst.phi, rtol=0, atol=1e-13)
    const = np.full(inst.np, 0.3)
    flow[:3 * inst.np] = 0.2
    st, *_ = O.ls_update(inst.xyz, inst.tets, flow, const, 0.1, tol=1e-14, reset=False)
    assert st == 0 and np.allclose(const, 0.3, rtol=0, atol=1e-12)
    # early return: zero dt
    phi2 = np.ascontiguousarray(inst.phi, np.float64).copy()
    assert O.ls_update(inst.xyz, inst.tets, flow, phi2, 0.0)[0] == 3
    assert np.array_equal(phi2, inst.phi)


def test_levelset_reset_is_distance_away_from_crossings():
    """After the reset, nodes away from crossing edges hold 0.75 phi_ifn +
    0.25 phi_ifn = the signed distance to the nearest interface point."""
    import fluidtissue_gb300.distance as Dm
    inst = workload("sphere65", 13)
    flow = np.zeros(4 * inst.np)
    flow[3 * inst.np:] = 1.0
    phi = np.ascontiguousarray(inst.phi, np.float64).copy()
    st, it, err, nif = O.ls_update(inst.xyz, inst.tets, flow, phi, 0.1, tol=1e-14, reset=True)
    assert st == 0 and nif > 0
    pts, edges = Dm.interface_points(inst.xyz, inst.tets, inst.phi)
    assert len(pts) == nif
    crossing = np.zeros(inst.np, bool)
    crossing[edges.ravel()] = True
    d = np.ascontiguousarray(inst.phi, np.float64).copy()
    O.dist_reset(inst.xyz, pts, d)
    far = ~crossing
    assert np.allclose(phi[far], d[far], rtol=1e-6, atol=1e-7)


def _sphere_lattice(n, r=0.25):
    from fluidtissue_gb300 import workloads as W
    xyz, tets, _ = W.kuhn_mesh(n, 0.0, 1)
    c = np.array([0.5, 0.5, 0.5])
    d = np.linalg.norm(xyz.astype(np.float64) - c, axis=1)
    return xyz, tets, d - r, (xyz.astype(np.float64) - c) / np.maximum(d, 1e-12)[:, None]


def test_surface_tension_sphere_known_answers():
    """phi = phi_reset = exact distance to a sphere of radius r: the patches
    tile the sphere (total area -> 4 pi r^2), the curvature is 2/r, so the
    inward load sums to st rho (2/r) 3 (4 pi r^2) = 24 pi r st rho (each
    triangle's area goes to its 3 points); the net force vanishes by symmetry;
    the load is linear in st * rho."""
    r = 0.25
    xyz, tets, phi, radial = _sphere_lattice(33, r)
    f, nif, area = O.surface_tension(xyz, tets, phi, phi, 1.0, 1)
    assert nif > 1000
    assert abs(area - 4 * np.pi * r * r) <= 0.01 * 4 * np.pi * r * r
    fr = np.sum(f.T * radial)
    assert abs(fr + 24 * np.pi * r) <= 0.01 * 24 * np.pi * r, fr
    assert np.abs(f.sum(axis=1)).max() <= 1e-6 * np.abs(f).sum()
    f6, _, _ = O.surface_tension(xyz, tets, phi, phi, 2.0, 3)
    assert np.allclose(f6, 6.0 * f, rtol=1e-6, atol=1e-9 * np.abs(f).max())


@pytest.mark.parametrize("signs,count,area", [
    ((-1.0, 1.0, 1.0, 1.0), 3, 0.5 * np.sqrt(3.0) / 4.0),     # one triangle
    ((-1.0, -1.0, 1.0, 1.0), 4, 0.5 * np.sqrt(0.5)),          # a quad as two triangles
])
def test_surface_tension_patches_by_hand(signs, count, area):
    """One unit right tetrahedron: the crossing edges' midpoints (|phi| equal)
    form one triangle (one node inside) or a 0.5 x sqrt(0.5) rectangle split
    in two (two inside); a linear phi has zero curvature, so no load."""
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    tets = np.array([[0, 1, 2, 3]], np.int32)
    phi = np.array(signs)
    f, nif, a = O.surface_tension(xyz, tets, phi, phi, 1.0, 1)
    assert nif == count
    assert abs(a - area) <= 1e-6
    assert np.all(f == 0.0)


def _p2_case(n=7):
    inst = workload("sphere17", n)
    par = dict(inst.params)
    return inst, par


def test_p2_rigid_motions_are_in_the_kernel():
    """Rigid rotations and translations have zero symmetric gradient and
    divergence: the full P2-P1 operator maps them (velocity at the vertices
    and edge midpoints, zero pressure) to zero, up to the float rounding of
    the reference's basis tables."""
    inst, par = _p2_case()
    A, F, sidx, nd = O.p2_system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source,
                                 inst.mu, par, full=True)
    E = O.p2_edges(inst.tets)
    assert nd == inst.np + len(E)
    X = inst.xyz.astype(np.float64)
    P = np.concatenate([X, 0.5 * (X[E[:, 0]] + X[E[:, 1]])])
    for u in ((-P[:, 1], P[:, 0], 0 * P[:, 0]), (0 * P[:, 0], -P[:, 2], P[:, 1]),
              (np.ones(nd), np.zeros(nd), np.zeros(nd))):
        x = np.concatenate([u[0], u[1], u[2], np.zeros(inst.np)])
        r = A @ x
        # the basis tables pass through float (Tetrahedron.hpp:17-18): identities
        # hold to float rounding
        assert np.abs(r).max() <= 1e-7 * abs(A).max() * np.abs(x).max(), np.abs(r).max()


def test_p2_load_partition_of_unity_and_hydrostatic_balance():
    """A uniform body force f = (1, 0, 0) with no source: the x load sums to
    the volume (sum_i phi_i = 1); as eps -> 0 the discrete solution is u = 0,
    p = x + const (-B p = N f holds exactly for linear p on P2-P1)."""
    inst, par = _p2_case()
    par = dict(par, **{"GF growth": 0.0, "eps": 1e-10})
    npn = inst.np
    f = np.zeros(3 * npn)
    f[:npn] = 1.0
    A, F, sidx, nd = O.p2_system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source,
                                 inst.mu, par, fst=f, full=True)
    vol = _volumes(inst).sum()
    assert abs(F[:nd].sum() - vol) <= 1e-7 * vol
    assert np.abs(F[nd:]).max() == 0.0
    flow, _, _ = O.p2_flow(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                           par, fst=f)
    assert np.abs(flow[:3 * npn]).max() <= 1e-6
    p = flow[3 * npn:]
    x = inst.xyz[:, 0].astype(np.float64)
    assert np.abs((p - p.mean()) - (x - x.mean())).max() <= 1e-6


def _golden_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("mk", ROOT / "tests/golden/make_golden.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    return mk


def test_golden_p2_fixture():
    """The oracle's P2-P1 solve reproduces the committed fixture."""
    from fluidtissue_gb300 import workloads as W
    mk = _golden_module()
    g = np.load(ROOT / "tests" / "golden" / "p2_sphere17_n7.npz")
    inst = W.WORKLOADS[str(g["name"])](int(g["n"]))
    assert mk.mesh_hash(inst.xyz, inst.tets) == str(g["mesh_sha256"])
    par = dict(inst.params, **{"Stokes velocity degree": 2.0})
    flow, _, F = O.p2_flow(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                           par)
    assert np.allclose(F, g["F"], rtol=0, atol=1e-13 * np.abs(g["F"]).max())
    assert np.linalg.norm(flow - g["flow"]) <= 1e-10 * np.linalg.norm(g["flow"])


def test_golden_surface_tension_fixture():
    """The oracle's surface-tension load reproduces the committed fixture
    (float arithmetic: to 1e-6 of the largest nodal value)."""
    from fluidtissue_gb300 import workloads as W
    mk = _golden_module()
    g = np.load(ROOT / "tests" / "golden" / "st_sphere_n17.npz")
    xyz, tets, _ = W.kuhn_mesh(int(g["n"]), 0.0, 1)
    assert mk.mesh_hash(xyz, tets) == str(g["mesh_sha256"])
    f, nif, area = O.surface_tension(xyz, tets, g["phi"], g["phi"], 1.0, 1)
    assert nif == int(g["interface_points"])
    assert abs(area - float(g["area"])) <= 1e-9 * float(g["area"])
    assert np.abs(f - g["force"]).max() <= 1e-6 * np.abs(g["force"]).max()

