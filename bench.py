"""Benchmark: variable-viscosity P1-P1 Stokes solves/s on one GB300.

Workload (default): ``ellipsoid129`` — 129^3 Kuhn lattice (12.6M tets),
jitter +-0.1h, ellipsoid level set, 16 Gaussian centres, mu = clip(1/(0.01+c),
0.01, 100), relative residual 1e-8.  One step = one complete Stokes solve
(viscosity, source, RHS and matrix assembly, Krylov solve, scatter to flow)
from a zero initial guess, inputs resident in HBM.  Inputs come from the numpy
generator (fluidtissue_gb300/workloads.py).

Reported:
  value     mixed-precision solves/s (device-resident inputs, no per-launch
            instrumentation in the timed region)
  e2e       the same through fts_solve with pinned host buffers (H2D of
            phi/source/mu and D2H of flow inside the timed region)
  fp64      the plain FP64 GPU path on the same workload and operator storage
            (the FP64 lattice half stencil)
  roofline  the Krylov loop's operator kernel (the FP32 lattice half-stencil
            SpMV fused with the MINRES dots), algorithmic bytes / CUDA-event
            time per launch, vs the measured HBM peak
  roofline_iteration  algorithmic bytes of one whole MINRES iteration (operator,
            both V-cycles over every level, updates) / time per iteration
  batch96, spheres257, components  the batched and the 257^3 matrix-free
            configurations, and the solve's neighbours (reaction-diffusion,
            distance reset, level-set update, surface-tension load)
  cpu_baseline  the CPU oracle (restated reference algorithm) on the box's
            host cores, bounded sample, with the measured fraction stated

``--impl reference`` times the reference's CPU path (the oracle port) on the
host cores with the same config dict: the reference's own BiCGSTAB to the end
where it converges, else the restated assembly plus timed chunks of a
converging CPU method (see run_reference); ``--workload dist129 --impl
reference`` times the reference's own CUDA distance kernel.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Stokes solves/s at 129^3 to 1e-8 resid: mixed-prec vs FP64 GPU; SpMV HBM GB/s"
UNIT = "solves/s"


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# the operator kernel of the FP32 inner solve, per operator storage
KERNELS = {
    "stencil": ("k_minres_A_lat", "FP32 lattice half-stencil 4x4-block SpMV + MINRES dots"),
    "assembled": ("k_minres_A_ell", "FP32 sliced-ELL 4x4-block SpMV + MINRES dots"),
    "matfree": ("k_mf_cube+k_mf_gather_minres_A", "FP32 matrix-free lattice operator: element "
                "geometry and rows once per cube, corner sums gathered per node, + MINRES dots"),
}


def _traffic(kernel: str, bytes_per_launch: float | None):
    """DRAM bytes per launch: the ratio of measured DRAM traffic to algorithmic
    bytes from one ncu capture of this kernel (profiles/traffic.json), scaled to
    this launch's algorithmic bytes (traffic grows with the rows processed)."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists() or not bytes_per_launch:
        return None
    d = json.loads(p.read_text()).get(kernel)
    if not d:
        return None
    return round(d["traffic_over_algorithmic"] * bytes_per_launch)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, idx: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(idx), f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _setup_dist(ws, local, backend="nccl"):
    import torch
    import torch.distributed as dist
    if ws > 1 and not dist.is_initialized():
        torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return dist if ws > 1 else None


def _max_over_ranks(v: float, dist) -> float:
    """Max of a per-rank time over all ranks (NCCL on GPUs, gloo on CPU)."""
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_ids(count: int, rank: int, world: int) -> list[int]:
    """Instances a rank solves: independent solves are dealt round-robin over
    the ranks (replicas, no data exchange)."""
    return list(range(rank, count, world))


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def hierarchy_fraction(n: int) -> float:
    """Sum over the multigrid levels below the finest of (level nodes / finest
    nodes): the lattices n -> (n - 1) / 2 + 1 (odd n; even n: n / 2 + 1) down to
    3^3 or 4^3."""
    tot, m = 0.0, n
    while m > 4:
        m = (m - 1) // 2 + 1 if m % 2 else m // 2 + 1
        tot += (m / n) ** 3
    return tot


# Algorithmic bytes per node of one MINRES iteration of the mixed solve (each
# kernel's stencil and vectors read once, outputs written once; FP32 vectors,
# FP16 velocity stencil of 144 B/node, FP32 pressure stencil of 32 B/node):
#   operator (lattice half stencil 512 B + x, r1, q)                         560
#   stage 1 (q, r1, r2 in; r_new out; velocity and pressure b, d_0, D^-1)    124
#   stage 2 vectors (r_new in, y out)                                         32
#   update of w and x (y, w_prev, w_cur, x in; w, x out)                      96
#   finest velocity level, degree-1 smoothing: r = b - K d_0 180, restriction
#     18, prolongation x = d_0 + P e 25.5, post d_0 = D^-1 (b - K x) 204,
#     x + d_0 24                                                             451.5
#   finest pressure level, degree 1: 44, 6, 8.5, 48, 8                       114.5
#   every coarser velocity level node, degree 2: pre-step 228, residual 180,
#     restriction 18, prolongation 25.5, post residual + d_0 216, post-step 240  907.5
#   every coarser pressure level node: 56, 44, 6, 8.5, 52, 60                 226.5
ITERATION_BYTES = {"operator": 560.0, "stage1": 124.0, "stage2": 32.0, "update": 96.0,
                   "velocity_finest": 451.5, "pressure_finest": 114.5,
                   "velocity_level": 907.5, "pressure_level": 226.5}


def iteration_bytes(n: int) -> float:
    """Algorithmic bytes of one mixed-precision MINRES iteration on an n^3
    lattice (velocity and pressure V-cycles over every level)."""
    B = ITERATION_BYTES
    per = (B["operator"] + B["stage1"] + B["stage2"] + B["update"] + B["velocity_finest"] +
           B["pressure_finest"] + hierarchy_fraction(n) * (B["velocity_level"] +
                                                           B["pressure_level"]))
    return per * n ** 3


def measure_flow(args, inst, operator: str, steps: int, warmup: int, want_fp64: bool,
                 steps_fp64: int, local: int, dist, ws: int) -> dict:
    """Times Flow.solve_device (device-resident inputs) and Flow.solve (host
    buffers) for one workload; the operator kernel's CUDA-event timings come
    from extra solves with per-launch events, outside the timed region."""
    import torch
    from fluidtissue_gb300.flow import Flow, Mesh
    dev = torch.device("cuda", local)
    par = dict(inst.params)
    npn = inst.np
    stream = torch.cuda.Stream(device=dev)
    phi_d = torch.from_numpy(inst.phi).to(dev)
    src_d = torch.from_numpy(inst.source).to(dev)
    mu_d = torch.from_numpy(inst.mu).to(dev)
    flow_d = torch.zeros(4 * npn, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()

    def opts(precision, time_kernels):
        return dict(precision=precision, warm_start=False, device=local,
                    preconditioner=args.preconditioner, time_kernels=time_kernels,
                    inner_tol=args.inner_tol, operator=operator)

    def make(precision):
        f = Flow()
        rc = f.init(Mesh(inst.xyz, inst.tets), par, **opts(precision, False))
        if rc != 0:
            raise RuntimeError(f"fts_create failed ({rc}): {f.last_error()}")
        f.set_stream(stream.cuda_stream)
        return f

    def device_steps(f, k):
        stats = []
        for _ in range(k):
            rc = f.solve_device(phi_d.data_ptr(), src_d.data_ptr(), mu_d.data_ptr(),
                                flow_d.data_ptr())
            if rc != 0:
                raise RuntimeError(f"fts_solve_device failed ({rc}): {f.last_error()}")
            stats.append(dict(f.last_stats))
        return stats

    def timed(fn, k, clocks_idx=None):
        _barrier(dist)
        torch.cuda.synchronize()
        clk = Clocks(clocks_idx) if clocks_idx is not None else None
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn(k)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        _barrier(dist)
        clocks = clk.stop() if clk else None
        return out, _max_over_ranks(ms, dist), clocks

    # ---- mixed precision, device-resident inputs (value) --------------------
    fm = make("mixed")
    device_steps(fm, warmup)
    stats_m, ms_m, clocks = timed(lambda k: device_steps(fm, k), steps, local)
    value = ws * steps / (ms_m / 1e3)

    # ---- e2e through fts_solve with pinned host buffers ----------------------
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    phi_h, src_h, mu_h = pin(inst.phi), pin(inst.source), pin(inst.mu)
    flow_h = torch.zeros(4 * npn, dtype=torch.float64).pin_memory().numpy()

    def host_steps(k):
        for _ in range(k):
            rc = fm.solve(phi_h, src_h, flow_h, mu=mu_h)
            if rc != 0:
                raise RuntimeError(f"fts_solve failed ({rc}): {fm.last_error()}")
        return None

    host_steps(1)
    _, ms_e, _ = timed(host_steps, steps)
    e2e = ws * steps / (ms_e / 1e3)
    rel_mixed = float(fm.last_stats["rel_residual"])
    flow_mixed = flow_h.copy()

    # ---- operator kernel timings: the same solve with per-launch events -----
    if fm.update_params(par, **opts("mixed", True)) != 0:
        raise RuntimeError(f"fts_update_params failed: {fm.last_error()}")
    stats_t = device_steps(fm, 2)
    spmv_ms = sum(s["ms_spmv"] for s in stats_t)
    spmv_n = sum(s["spmv_launches"] for s in stats_t)
    per = spmv_ms / max(spmv_n, 1)
    bytes_per = stats_t[0]["spmv_bytes"]
    achieved = bytes_per / (per / 1e3) / 1e9 if spmv_n else None
    fm.close()

    # ---- plain FP64 on the same workload and operator storage ----------------
    stats_d, ms_d, value_fp64, vel_err, p_err, k64, ach64, it_d = (None,) * 8
    if want_fp64:
        f64 = make("fp64")
        device_steps(f64, 1)
        k64 = max(1, steps_fp64)
        stats_d, ms_d, _ = timed(lambda k: device_steps(f64, k), k64)
        value_fp64 = ws * k64 / (ms_d / 1e3)
        flow64 = flow_d.cpu().numpy()
        vel_err = float(np.linalg.norm(flow_mixed[:3 * npn] - flow64[:3 * npn]) /
                        np.linalg.norm(flow64[:3 * npn]))
        p_err = float(np.linalg.norm(flow_mixed[3 * npn:] - flow64[3 * npn:]) /
                      np.linalg.norm(flow64[3 * npn:]))
        it_d = statistics.mean(s["iterations"] for s in stats_d)
        if f64.update_params(par, **opts("fp64", True)) == 0:
            st64 = device_steps(f64, 1)
            n64 = sum(s["spmv_launches"] for s in st64)
            if n64:
                ach64 = st64[0]["spmv_bytes"] / (sum(s["ms_spmv"] for s in st64) / n64 / 1e3) / 1e9
        f64.close()

    it_m = statistics.mean(s["iterations"] for s in stats_m)
    ms_solve = statistics.mean(s["ms_solve"] for s in stats_m)
    return {"value": value, "ms_m": ms_m, "e2e": e2e, "clocks": clocks, "stats_m": stats_m,
            "rel_mixed": rel_mixed, "achieved": achieved, "per": per, "bytes_per": bytes_per,
            "value_fp64": value_fp64, "ms_d": ms_d, "k64": k64, "it_d": it_d, "ach64": ach64,
            "vel_err": vel_err, "p_err": p_err, "it_m": it_m, "ms_solve": ms_solve,
            "h2d": int(phi_h.nbytes + src_h.nbytes + mu_h.nbytes), "d2h": int(flow_h.nbytes),
            "launches": int(sum(s["kernel_launches"] for s in stats_m))}


def spheres257_subresult(args, local, dist, ws) -> dict:
    """The 257^3 two-sphere workload through the matrix-free operator: mixed
    solves/s (device-resident inputs and e2e), iterations, residual, device
    bytes and the operator's CUDA-event GB/s."""
    from fluidtissue_gb300 import workloads as W
    inst = W.spheres257()
    m = measure_flow(args, inst, "matfree", 2, 3, False, 0, local, dist, ws)
    st = m["stats_m"][0]
    peak, _ = _peaks()
    return {"workload": f"spheres257: {inst.np} nodes, {inst.nt} tets, tol "
                        f"{inst.params['Stokes tolerance']}, matrix-free operator",
            "solves_per_s": round(m["value"], 4), "e2e_solves_per_s": round(m["e2e"], 4),
            "ms_per_solve": round(m["ms_m"] / 2, 2), "iterations": m["it_m"],
            "rel_residual": m["rel_mixed"], "device_bytes": int(st["device_bytes"]),
            "operator_gbs": round(m["achieved"], 1) if m["achieved"] else None,
            "operator_frac": round(m["achieved"] / peak, 4) if m["achieved"] else None,
            "operator_ms": round(m["per"], 4), "steps": 2, "warmup": 3, "clocks": m["clocks"]}


def components_subresult(args, local, dist, ws, rank) -> dict:
    """The solve's neighbours on the ellipsoid129 mesh, device figures only
    (their own workloads add the CPU baselines): reaction-diffusion (32000
    Euler steps), distance reset, level-set update and surface-tension load,
    each with 3 warm-up and 3 timed calls."""
    import copy
    a = copy.copy(args)
    a.steps, a.warmup, a.no_cpu_baseline = 3, 3, True
    sub = (local, dist, ws, rank)
    out = {}
    for name, fn in (("rd129", run_rd), ("dist129", run_dist), ("ls129", run_ls),
                     ("st129", run_st)):
        line = fn(a, sub)
        keep = {k: line[k] for k in ("metric", "value", "unit", "ms_per_step", "config", "e2e",
                                     "gpu_launches", "clocks") if k in line}
        for k in ("ms_device_per_call", "device_steps_per_s", "pruned", "iterations",
                  "ms_assembly", "ms_solve", "ms_reset", "interface_points"):
            if k in line:
                keep[k] = line[k]
        out[name] = keep
    return out


def run_ours(args):
    import torch
    from fluidtissue_gb300 import workloads as W

    ws, rank, local = _dist()
    dist = _setup_dist(ws, local)
    torch.cuda.set_device(local)
    inst = W.WORKLOADS[args.workload]()
    npn = inst.np
    operator = args.operator or ("matfree" if args.workload == "spheres257" else "auto")
    if operator == "auto":  # every bench workload is a Kuhn lattice: the half-stencil copy
        operator = "stencil"
    want_fp64 = not args.no_fp64 and operator != "matfree"
    m = measure_flow(args, inst, operator, args.steps, args.warmup, want_fp64, args.steps_fp64,
                     local, dist, ws)
    stats_m = m["stats_m"]
    peak, peak_kind = _peaks()
    achieved, bytes_per, per = m["achieved"], m["bytes_per"], m["per"]
    dofs = 4 * npn
    it_m = m["it_m"]
    res = {
        "metric": METRIC, "value": round(m["value"], 4), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(m["ms_m"] / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 outer",
        "data": "synthetic (seeded Kuhn lattice, analytic level set, Gaussian growth factor)",
        "config": workload_config(args, inst),
        "precision": "mixed", "preconditioner": args.preconditioner,
        "e2e": {"value": round(m["e2e"], 4), "unit": UNIT, "h2d_bytes_per_step": m["h2d"],
                "d2h_bytes_per_step": m["d2h"]},
        "fp64": ({"value": round(m["value_fp64"], 4), "unit": UNIT,
                  "ms_per_step": round(m["ms_d"] / m["k64"], 3), "iterations": m["it_d"],
                  "operator": operator + " (FP64 storage)",
                  "spmv_gbs": round(m["ach64"], 1) if m["ach64"] else None}
                 if m["value_fp64"] else None),
        "mixed_vs_fp64": round(m["value"] / m["value_fp64"], 3) if m["value_fp64"] else None,
        "operator": operator,
        "device_bytes": int(stats_m[0]["device_bytes"]),
        "mixed": {"iterations": it_m, "iterations_fp32": statistics.mean(
            s["iterations_fp32"] for s in stats_m),
                  "outer": statistics.mean(s["outer_iterations"] for s in stats_m),
                  "rel_residual": m["rel_mixed"], "vel_err_vs_fp64": m["vel_err"],
                  "p_err_vs_fp64": m["p_err"]},
        "dof_iterations_per_s": round(m["value"] * it_m * dofs, 1),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1) if achieved else None,
                     "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4) if achieved else None,
                     "traffic": _traffic(KERNELS[operator][0], bytes_per),
                     "kernel": f"{KERNELS[operator][0]} ({KERNELS[operator][1]})",
                     "bytes_per_launch": bytes_per, "ms_per_launch": round(per, 5),
                     "timing": "CUDA events around every launch, in solves outside the "
                               "timed region",
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "gpu_launches": m["launches"],
        "clocks": m["clocks"],
        "ms_assembly": round(statistics.mean(s["ms_assembly"] for s in stats_m), 3),
    }
    if operator == "stencil" and inst.n % 2 == 1:
        t_it = m["ms_solve"] / max(it_m, 1)
        ib = iteration_bytes(inst.n)
        ach_it = ib / (t_it / 1e3) / 1e9
        res["roofline_iteration"] = {
            "bound": "hbm", "achieved": round(ach_it, 1), "peak": peak, "unit": "GB/s",
            "frac": round(ach_it / peak, 4), "bytes_per_iteration": round(ib),
            "ms_per_iteration": round(t_it, 4),
            "what": "one MINRES iteration of the mixed solve: operator, both V-cycles over "
                    "every level, Lanczos and solution updates (algorithmic bytes); time = "
                    "solve time / iterations (outer residuals included)"}
    if args.workload == "ellipsoid129" and not args.no_subresults:
        res["batch96"] = batch_measure(args, 2, 3, local, dist, ws)
        res["spheres257"] = spheres257_subresult(args, local, dist, ws)
        res["components"] = components_subresult(args, local, dist, ws, rank)
    if rank == 0 and not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_baseline(inst, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(res), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def batch_measure(args, steps: int, warmup: int, local: int, dist, ws: int) -> dict:
    """The batched workload: `--batch-count` independent instances (n ~
    U{17..65}, seeded per instance) per step, solved by fts_batch_solve_device
    (one persistent launch per Krylov run, CUDA graph, autotuned); FP64 and
    mixed.  Under N ranks each rank solves its share (replicas)."""
    import torch
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.flow import Batch, Mesh
    _, rank, _ = _dist()
    dev = torch.device("cuda", local)
    count = args.batch_count
    # replicas: rank r solves instances r, r + ws, ... of the batch (no collective)
    ids = replica_ids(count, rank, ws)
    insts = [W.batch_instance(i) for i in ids]
    stream = torch.cuda.Stream(device=dev)
    phis = [torch.from_numpy(i.phi).to(dev) for i in insts]
    srcs = [torch.from_numpy(i.source).to(dev) for i in insts]
    mus = [torch.from_numpy(i.mu).to(dev) for i in insts]
    flows = [torch.zeros(4 * i.np, dtype=torch.float64, device=dev) for i in insts]
    out = {}
    for prec in ("mixed", "fp64"):
        b = Batch([Mesh(i.xyz, i.tets) for i in insts], [i.params for i in insts],
                  precision=prec, warm_start=False, device=local,
                  preconditioner=args.preconditioner)
        b.set_stream(stream.cuda_stream)

        def step():
            rc = b.solve_device([p.data_ptr() for p in phis], [s.data_ptr() for s in srcs],
                                [m.data_ptr() for m in mus], [f.data_ptr() for f in flows])
            if rc != 0:
                raise RuntimeError(f"fts_batch_solve_device failed ({rc}): {b.last_error()}")

        for _ in range(warmup):
            step()
        _barrier(dist)
        torch.cuda.synchronize()
        clk = Clocks(local)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = _max_over_ranks(e0.elapsed_time(e1), dist)
        clocks = clk.stop()
        st = b.last_stats
        its = [s["iterations"] for s in st]
        out[prec] = {"solves_per_s": round(ws * len(insts) * steps / (ms / 1e3), 3),
                     "ms_per_batch": round(ms / steps, 2),
                     "iterations_mean": statistics.mean(its), "iterations_max": max(its),
                     "max_rel_residual": max(s["rel_residual"] for s in st),
                     "dof_iterations_per_s": round(
                         sum(4 * i.np * s["iterations"] for i, s in zip(insts, st)) * ws
                         * steps / (ms / 1e3), 1),
                     "device_bytes": int(sum(s["device_bytes"] for s in st)),
                     "autotuned": b.config(), "clocks": clocks}
        if prec == "mixed":
            out["flows_mixed"] = [f.cpu().numpy() for f in flows]
        b.close()
    fm = out.pop("flows_mixed")
    errs = []
    for f64, fmx, i in zip(flows, fm, insts):
        a = f64.cpu().numpy()
        errs.append(float(np.linalg.norm(fmx[:3 * i.np] - a[:3 * i.np]) /
                          np.linalg.norm(a[:3 * i.np])))
    return {"workload": f"batch{count}: {count} instances, n ~ U{{17..65}}, tol 1e-8, "
                        f"{sum(i.np for i in insts)} nodes",
            "steps": steps, "warmup": warmup, "mixed": out["mixed"], "fp64": out["fp64"],
            "mixed_vs_fp64": round(out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"], 3),
            "max_vel_err_mixed_vs_fp64": max(errs)}


def run_batch(args):
    """The batched workload as its own bench line (see batch_measure)."""
    import torch
    ws, rank, local = _dist()
    dist = _setup_dist(ws, local)
    torch.cuda.set_device(local)
    r = batch_measure(args, args.steps, args.warmup, local, dist, ws)
    if rank == 0:
        res = {"metric": "batched Stokes solves/s (96 instances, n ~ U{17..65}, tol 1e-8)",
               "value": r["mixed"]["solves_per_s"], "unit": UNIT, "n_gpus": ws,
               "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": r["mixed"]["ms_per_batch"], "higher_is_better": True,
               "scaling": "strong" if ws > 1 else "weak", "dtype": "f32 inner / f64 outer",
               "data": "synthetic", "config": {"workload": r["workload"]},
               "mixed": r["mixed"], "fp64": r["fp64"], "mixed_vs_fp64": r["mixed_vs_fp64"],
               "max_vel_err_mixed_vs_fp64": r["max_vel_err_mixed_vs_fp64"]}
        print(json.dumps(res), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# Workloads on which the reference's own algorithm (assembly + Eigen-style
# un-preconditioned BiCGSTAB, Flow.cpp:102-285) reaches the tolerance: the CPU
# baselines run it to the end, fully measured.  On ellipsoid129 it diverges
# (relative residual 4.3e79 after 150,000 iterations), so the baselines there
# time the restated assembly in full and a sample of block-Jacobi + rank-one
# MINRES iterations (the same method as the GPU's Jacobi mode, FP64).
FULL_SOLVE = ("sphere17", "sphere65")

# Iterations of FP64 block-Jacobi + rank-one MINRES to the workload tolerance,
# counted by the same FP64 method (the GPU's Jacobi mode) on the same system:
# the sampled baselines' iteration count.
CPU_BASELINE_ITERATIONS: dict = {"sphere17": 1940, "sphere65": 4204, "ellipsoid129": 42647}


def _oracle():
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    return O


def cpu_full_solve(inst) -> dict:
    """The reference's Stokes step restated on the host (oracle, OpenMP,
    FP64): assembly, un-preconditioned BiCGSTAB to the workload tolerance and
    scatter, one complete solve, every part measured."""
    O = _oracle()
    t0 = time.perf_counter()
    rc, _, _, info = O.flow_solve(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source,
                                  inst.mu, inst.params)
    t = time.perf_counter() - t0
    if rc != 0:
        raise RuntimeError(f"oracle BiCGSTAB did not converge: {info}")
    return {"seconds": t, "iterations": int(info["iterations"]), "error": info["error"],
            "ms_assembly": info.get("ms_assembly")}


class SampledCpuSolve:
    """The restated assembly in full plus chunks of block-Jacobi MINRES
    iterations on the reduced system, continued from the last chunk's iterate;
    solves/s = 1 / (t_assembly + N t_iteration) with N the method's iteration
    count to the tolerance."""

    def __init__(self, inst):
        O = _oracle()
        self.O, self.inst = O, inst
        t0 = time.perf_counter()
        self.R, _, _, mu = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source,
                                    inst.mu, inst.params)
        self.pre = O.block_jacobi(self.R, inst.xyz, inst.tets, mu, inst.params["eps"])
        self.t_asm = time.perf_counter() - t0
        self.x = None
        self.t_it, self.its = 0.0, 0

    def chunk(self, iterations: int) -> float:
        t0 = time.perf_counter()
        self.x, _, done = self.O.minres_blockjacobi(self.R, self.pre, x0=self.x, rtol=1e-30,
                                                    maxit=iterations)
        t = time.perf_counter() - t0
        self.t_it += t
        self.its += max(done, 1)
        return t

    def result(self) -> dict:
        t_it = self.t_it / max(self.its, 1)
        n_it = CPU_BASELINE_ITERATIONS[self.inst.name]
        total = self.t_asm + n_it * t_it
        measured = self.t_asm + self.its * t_it
        threads = self.O.num_threads()
        return {"value": 1.0 / total, "unit": UNIT, "cores": threads, "kind": "port",
                "measured_fraction": round(measured / total, 4),
                "sample": (f"oracle on {self.inst.name} ({threads} threads): the restated "
                           f"assembly and preconditioner set-up in full ({self.t_asm:.2f} s) + "
                           f"{self.its} block-Jacobi MINRES iterations ({t_it * 1e3:.1f} ms "
                           f"each); solves/s = 1/(t_asm + N t_iter) with N = {n_it}, the "
                           f"iterations of the same FP64 method to tol "
                           f"{self.inst.params['Stokes tolerance']}; the reference's "
                           f"un-preconditioned BiCGSTAB diverges on this workload; "
                           f"{100 * measured / total:.1f} % of the time measured"),
                "t_assembly_s": self.t_asm, "t_iteration_s": t_it, "iterations_timed": self.its}


def cpu_baseline(inst, seconds: float) -> dict:
    """The CPU oracle on this host's cores (OpenMP, FP64), about ``seconds``
    of work: the reference's algorithm to the end where it converges
    (FULL_SOLVE), else the sampled solve."""
    O = _oracle()
    threads = O.num_threads()
    if inst.name in FULL_SOLVE:
        r = cpu_full_solve(inst)
        return {"value": 1.0 / r["seconds"], "unit": UNIT, "cores": threads, "kind": "port",
                "measured_fraction": 1.0,
                "sample": (f"oracle on {inst.name} ({threads} threads): the reference's "
                           f"algorithm restated (assembly, un-preconditioned BiCGSTAB, "
                           f"{r['iterations']} iterations to {r['error']:.2e}), one complete "
                           f"solve of {r['seconds']:.2f} s"), "iterations": r["iterations"]}
    S = SampledCpuSolve(inst)
    it = 8
    while S.t_asm + S.t_it < seconds and S.its < 20000:
        S.chunk(it)
        it = min(2 * it, 512)
    return S.result()


def workload_config(args, inst) -> dict:
    """The config dict both arms print (the workload, not the implementation)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return {"workload": f"{inst.name}: {inst.np} nodes, {inst.nt} tets, {4 * inst.np} block "
                        f"DOF, tol {inst.params['Stokes tolerance']}",
            "l2": "inputs larger than L2 (operator > 1 GB streamed every iteration)",
            "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"}


def run_reference(args):
    """The reference's CPU path for this workload on the host cores (the oracle
    port; the reference itself needs Eigen, CGAL, TBB and GMP, absent here).
    Inputs come from the numpy generator, so no library of this package is
    loaded.  Where the reference's BiCGSTAB converges (FULL_SOLVE) each step is
    one complete solve; on ellipsoid129 the warm-up steps are assemblies, then
    the assembly is timed once and each step is a chunk of `--ref-chunk`
    block-Jacobi MINRES iterations continuing the same solve, and the line
    states the measured fraction of the extrapolated time."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    from fluidtissue_gb300 import workloads as W
    if args.workload == "dist129":
        run_reference_dist(args, ws)
        return
    O = _oracle()
    inst = W.WORKLOADS[args.workload]()
    threads = O.num_threads()
    extra = {}
    if inst.name in FULL_SOLVE:
        for _ in range(args.warmup):
            O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                     inst.params)
        runs = [cpu_full_solve(inst) for _ in range(args.steps)]
        secs = sum(r["seconds"] for r in runs)
        v = args.steps / secs
        cb = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "measured_fraction": 1.0,
              "sample": (f"oracle on {inst.name} ({threads} threads): {args.steps} complete "
                         f"solves with the reference's algorithm restated (assembly, "
                         f"un-preconditioned BiCGSTAB to tol {inst.params['Stokes tolerance']}, "
                         f"{runs[-1]['iterations']} iterations)")}
        ms = 1e3 * secs / args.steps
        extra = {"iterations": runs[-1]["iterations"], "error": runs[-1]["error"]}
    else:
        for _ in range(args.warmup):
            O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                     inst.params)
        S = SampledCpuSolve(inst)
        for _ in range(args.steps):
            S.chunk(args.ref_chunk)
        cb = S.result()
        v = cb["value"]
        ms = 1e3 / v
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded Kuhn lattice, analytic level set, Gaussian growth factor)",
           "config": workload_config(args, inst), "cpu_baseline": cb,
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    out.update(extra)
    print(json.dumps(out), flush=True)


def run_reference_dist(args, ws):
    """Reference arm of the distance workload: the reference's own CUDA kernel
    (oracle/_ref) through resetPhi's host sequence, on the ellipsoid129 mesh and
    its interface points."""
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.distance import interface_points
    inst = W.ellipsoid129()
    ifp, _ = interface_points(inst.xyz, inst.tets, inst.phi)
    r = reference_distance_kernel(inst, ifp, args.steps, args.warmup)
    if r is None:
        print(json.dumps({"impl": "reference", "unavailable": "oracle/_ref/EuclideanDistance."
                          "cubin was not built (reference sources absent where the repository "
                          "was built)"}), flush=True)
        return
    r.pop("phi")
    v = r["resets_per_s"]
    print(json.dumps({"impl": "reference", "metric": "level-set distance resets/s (ellipsoid129 "
                      "nodes x its interface points)", "value": v, "unit": "resets/s",
                      "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": r["ms_per_reset"], "higher_is_better": True,
                      "config": {"workload": f"dist129: {inst.np} nodes x {len(ifp)} interface "
                                             f"points"},
                      "reference_kernel": r,
                      "e2e": {"value": v, "unit": "resets/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}), flush=True)


# Fig. 5-6 growth parameters of the reference's parameter summary
# (parameters/summary.txt): 32000 explicit Euler steps of 1/32 per RD call.
RD_PAR = {"RD dt": 1.0 / 32.0, "RD iterations": 32000.0, "Act": 2.0, "Da": 5.0e-6,
          "DegA": 0.01, "Inh": 1.0, "Di": 7.5e-5, "DegI": 0.02, "GF production": 40.0,
          "GF diffusion": 1.25e-4, "GF degradation": 0.02, "GF inhibition": 200.0}


def _rd_sources(inst, count=16):
    """Interior nodes nearest `count` seeded points of the level set's interior
    (stand-ins for the signalling centres' source nodes)."""
    inside = np.where(inst.phi < 0)[0]
    pick = np.linspace(0, len(inside) - 1, count).astype(int)
    return inside[pick].astype(np.int32)


def run_rd(args, sub=None):
    """Reaction-diffusion (RD::solve) on the ellipsoid129 mesh and level set:
    value = RD calls/s, one call = 32000 FP64 explicit Euler steps of the
    activator, inhibitor and growth factor on the interior submesh (all steps
    in one persistent launch).  The state is copied in from and out to host
    memory every call (the reference's RD keeps it on the host)."""
    import torch
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.flow import Mesh
    from fluidtissue_gb300.rd import RD

    if sub is None:
        ws, rank, local = _dist()
        dist = _setup_dist(ws, local)
        torch.cuda.set_device(local)
    else:
        local, dist, ws, rank = sub
    inst = W.ellipsoid129()
    src = _rd_sources(inst)
    rd = RD()
    if rd.init(Mesh(inst.xyz, inst.tets), inst.phi, RD_PAR, device=local) != 0:
        raise RuntimeError(f"fts_rd_create failed: {rd.last_error()}")
    a0, i0, g0 = rd.activator.copy(), rd.inhibitor.copy(), rd.growth_factor.copy()

    def step():
        rd.set_state(a0, i0, g0)
        rc = rd.solve(inst.phi, src)
        if rc != 0:
            raise RuntimeError(f"fts_rd_solve failed ({rc}): {rd.last_error()}")
        return rd.last_stats

    for _ in range(args.warmup):
        step()
    _barrier(dist)
    clk = Clocks(local)
    t0 = time.perf_counter()
    stats = [step() for _ in range(args.steps)]
    wall = (time.perf_counter() - t0) * 1e3
    clocks = clk.stop()
    ms = _max_over_ranks(wall, dist)
    ms_dev = statistics.mean(s["ms_steps"] for s in stats)
    st = stats[-1]
    n_steps = int(RD_PAR["RD iterations"])
    nint = st["interior_nodes"]
    res = {"metric": "RD calls/s (32000 FP64 Euler steps, ellipsoid129 interior)",
           "value": round(ws * args.steps / (ms / 1e3), 4), "unit": "calls/s", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (ellipsoid129 level set; activator ramp x + 1; 16 source nodes)",
           "config": {"workload": f"rd129: {nint} interior nodes, "
                                  f"{st['interior_elements']} interior tets, {n_steps} steps"},
           "e2e": {"value": round(ws * args.steps / (ms / 1e3), 4), "unit": "calls/s",
                   "h2d_bytes_per_step": 4 * 8 * inst.np + 4 * len(src),
                   "d2h_bytes_per_step": 3 * 8 * inst.np},
           "device_steps_per_s": round(n_steps / (ms_dev / 1e3), 1),
           "ms_device_per_call": round(ms_dev, 3), "ms_setup": round(st["ms_setup"], 3),
           "node_steps_per_s": round(nint * n_steps / (ms_dev / 1e3), 1),
           "gpu_launches": int(st["kernel_launches"]), "clocks": clocks}
    if sub is not None:
        rd.close()
        return res
    if rank == 0 and not args.no_cpu_baseline:
        res["cpu_baseline"] = rd_cpu_baseline(inst, src, a0, i0, g0, n_steps)
    if rank == 0:
        print(json.dumps(res), flush=True)
    rd.close()


def rd_cpu_baseline(inst, src, a0, i0, g0, n_steps, sample_steps=200):
    """The oracle's RD restatement (OpenMP, FP64) on this host: the Laplacian
    assembly in full plus `sample_steps` Euler steps, scaled to n_steps."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    par = dict(RD_PAR)
    a, i, g = a0.copy(), i0.copy(), g0.copy()
    par["RD iterations"] = 1.0
    t0 = time.perf_counter()
    O.rd_solve(inst.xyz, inst.tets, inst.phi, src, par, a, i, g)
    t_one = time.perf_counter() - t0
    par["RD iterations"] = float(sample_steps + 1)
    t0 = time.perf_counter()
    O.rd_solve(inst.xyz, inst.tets, inst.phi, src, par, a, i, g)
    t_more = time.perf_counter() - t0
    t_step = max(t_more - t_one, 0.0) / sample_steps
    t_setup = max(t_one - t_step, 0.0)
    total = t_setup + n_steps * t_step
    return {"value": 1.0 / total, "unit": "calls/s", "cores": O.num_threads(), "kind": "port",
            "sample": (f"oracle RD on the same interior ({O.num_threads()} threads): set-up "
                       f"{t_setup:.2f} s + {sample_steps} steps of {t_step * 1e3:.3f} ms, "
                       f"scaled to {n_steps} steps"),
            "t_setup_s": t_setup, "t_step_s": t_step}


def run_dist(args, sub=None):
    """Distance reset (EuclideanDistance::resetPhi) on the ellipsoid129 mesh
    against its own interface points (the zero level set's edge crossings,
    LevelSet.cpp:278-300): value = resets/s of the pruned search, through the
    C ABI with host buffers (H2D, device binning of the points, search, D2H).
    Beside it the reference's algorithm (every node against every point) on the
    same GPU, and the oracle's host restatement on all nodes."""
    import torch
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.distance import EuclideanDistance, interface_points

    if sub is None:
        ws, rank, local = _dist()
        dist = _setup_dist(ws, local)
        torch.cuda.set_device(local)
    else:
        local, dist, ws, rank = sub
    inst = W.ellipsoid129()
    ifp, _ = interface_points(inst.xyz, inst.tets, inst.phi)
    d = EuclideanDistance()
    if d.init(inst.xyz, device=local) != 0:
        raise RuntimeError(f"fts_dist_create failed: {d.last_error()}")
    out = {}
    for method in ("pruned", "exhaustive"):
        def step():
            phi = inst.phi.copy()
            rc = d.resetPhi(ifp, phi, method)
            if rc != 0:
                raise RuntimeError(f"fts_dist_reset failed ({rc}): {d.last_error()}")
            return d.last_stats, phi
        for _ in range(args.warmup):
            step()
        _barrier(dist)
        clk = Clocks(local) if method == "pruned" else None
        t0 = time.perf_counter()
        res = [step() for _ in range(args.steps)]
        wall = _max_over_ranks((time.perf_counter() - t0) * 1e3, dist)
        out[method] = {"resets_per_s": round(ws * args.steps / (wall / 1e3), 3),
                       "ms_per_reset": round(wall / args.steps, 3),
                       "ms_kernel": round(statistics.mean(r[0]["ms_kernel"] for r in res), 3),
                       "points_scanned": int(res[-1][0]["points_scanned"]),
                       "clocks": clk.stop() if clk else None}
        out[method]["phi"] = res[-1][1]
    pr_phi = out["pruned"]["phi"]
    same = bool(np.array_equal(out["pruned"].pop("phi"), out["exhaustive"].pop("phi")))
    pr = out["pruned"]
    line = {"metric": "level-set distance resets/s (ellipsoid129 nodes x its interface points)",
            "value": pr["resets_per_s"], "unit": "resets/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": pr["ms_per_reset"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (distances), f64 (phi)",
            "data": "synthetic (ellipsoid129 mesh and level set; its edge crossings)",
            "config": {"workload": f"dist129: {inst.np} nodes x {len(ifp)} interface points"},
            "e2e": {"value": pr["resets_per_s"], "unit": "resets/s",
                    "h2d_bytes_per_step": 12 * len(ifp) + 8 * inst.np,
                    "d2h_bytes_per_step": 8 * inst.np},
            "pruned": pr, "reference_algorithm_on_gpu": out["exhaustive"],
            "pruned_equals_reference_algorithm": same,
            "kernel_speedup": round(out["exhaustive"]["ms_kernel"] / max(pr["ms_kernel"], 1e-9), 1),
            "gpu_launches": 6, "clocks": pr.pop("clocks")}
    if sub is not None:
        d.close()
        return line
    if rank == 0:
        ref = reference_distance_kernel(inst, ifp, args.steps, args.warmup)
        if ref is not None:
            ref["equals_pruned"] = bool(np.array_equal(ref.pop("phi"), pr_phi))
            ref["kernel_speedup_of_pruned"] = round(ref["ms_kernel"] / max(pr["ms_kernel"], 1e-9),
                                                   1)
        line["reference_kernel"] = ref
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle as O
        k1 = inst.np  # all nodes: about 8 s on 16 host threads
        phi = inst.phi.copy()
        t0 = time.perf_counter()
        O.dist_reset(inst.xyz, ifp, phi, 0, k1)
        t = time.perf_counter() - t0
        line["cpu_baseline"] = {
            "value": 1.0 / (t * inst.np / k1), "unit": "resets/s", "cores": O.num_threads(),
            "kind": "port",
            "sample": (f"oracle host path on {k1} of {inst.np} nodes ({O.num_threads()} threads, "
                       f"{t:.2f} s), scaled to all nodes")}
    if rank == 0:
        print(json.dumps(line), flush=True)
    d.close()


def reference_distance_kernel(inst, ifp, steps: int, warmup: int):
    """The reference's own distance kernel (distanceToInterface_k, built
    unchanged from its source into oracle/_ref) on this GPU with its own launch
    shape: device time per launch (CUDA events, inputs resident) and time per
    reset with its host copies (EuclideanDistance::resetPhi's sequence: points
    and phi up, launch, phi down).  None when the image was not built."""
    import torch
    sys.path.insert(0, str(ROOT / "oracle"))
    import ref_dist
    if not ref_dist.available():
        return None
    K = ref_dist.ReferenceDistanceKernel()
    dev = torch.device("cuda")
    xyz = torch.from_numpy(np.ascontiguousarray(inst.xyz, np.float32).reshape(-1)).to(dev)
    pts = torch.from_numpy(np.ascontiguousarray(ifp, np.float32).reshape(-1)).to(dev)
    phi = torch.from_numpy(np.ascontiguousarray(inst.phi, np.float64)).to(dev)
    phi0 = phi.clone()
    n, m = inst.np, len(ifp)
    for _ in range(warmup):
        phi.copy_(phi0)
        K.launch(xyz.data_ptr(), n, pts.data_ptr(), m, phi.data_ptr())
    torch.cuda.synchronize()
    ms = []
    for _ in range(steps):
        phi.copy_(phi0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        K.launch(xyz.data_ptr(), n, pts.data_ptr(), m, phi.data_ptr())
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    t0 = time.perf_counter()
    for _ in range(steps):
        out = K.reset_phi(inst.xyz, ifp, inst.phi)
    wall = (time.perf_counter() - t0) * 1e3 / steps
    K.close()
    return {"ms_kernel": round(statistics.mean(ms), 3), "ms_per_reset": round(wall, 3),
            "resets_per_s": round(1e3 / wall, 3), "phi": out,
            "what": "distanceToInterface_k compiled unchanged from src/fem/EuclideanDistance.cu, "
                    "512 threads per block, ceil(n/512) blocks (EuclideanDistance.cu:90-118)"}


def run_p2(args):
    """P2-P1 (Taylor-Hood, "Stokes velocity degree" 2) on the jittered 33^3
    sphere workload (mu = 1, 8 Gaussian centres, tol 1e-8): value = mixed-
    precision solves/s with device-resident inputs, e2e through fts_solve with
    host buffers, beside the FP64 GPU path.  CPU baseline: the oracle's P2-P1
    assembly (the reference's element loop) in full plus its reduced system's
    sparse products, two per iteration of the reference's BiCGSTAB, times the
    iterations block-Jacobi MINRES needs in FP64 (a lower bound: the
    reference's un-preconditioned BiCGSTAB needs more)."""
    import torch
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.flow import Flow, Mesh

    ws, rank, local = _dist()
    dist = _setup_dist(ws, local)
    torch.cuda.set_device(local)
    inst = W.sphere65(33)
    par = dict(inst.params, **{"Stokes velocity degree": 2.0, "Stokes tolerance": 1e-8})
    res = {}
    for prec in ("mixed", "fp64"):
        f = Flow()
        if f.init(Mesh(inst.xyz, inst.tets), par, precision=prec, warm_start=False,
                  device=local) != 0:
            raise RuntimeError(f.last_error())
        phi_d = torch.from_numpy(inst.phi).cuda()
        src_d = torch.from_numpy(inst.source).cuda()
        mu_d = torch.from_numpy(inst.mu).cuda()
        flow_d = torch.zeros(4 * inst.np, dtype=torch.float64, device="cuda")
        phi_h = torch.from_numpy(inst.phi).pin_memory()
        src_h = torch.from_numpy(inst.source).pin_memory()
        mu_h = torch.from_numpy(inst.mu).pin_memory()
        flow_h = torch.zeros(4 * inst.np, dtype=torch.float64).pin_memory()

        def dev_step():
            rc = f.solve_device(phi_d.data_ptr(), src_d.data_ptr(), mu_d.data_ptr(),
                                flow_d.data_ptr())
            if rc != 0:
                raise RuntimeError(f"fts_solve_device failed ({rc}): {f.last_error()}")
            return dict(f.last_stats)

        def e2e_step():
            rc = f.solve(phi_h.numpy(), src_h.numpy(), flow_h.numpy(), mu=mu_h.numpy())
            if rc != 0:
                raise RuntimeError(f"fts_solve failed ({rc}): {f.last_error()}")

        for _ in range(args.warmup):
            dev_step()
        _barrier(dist)
        clk = Clocks(local) if prec == "mixed" else None
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        stats = [dev_step() for _ in range(args.steps)]
        torch.cuda.synchronize()
        wall = _max_over_ranks((time.perf_counter() - t0) * 1e3, dist)
        clocks = clk.stop() if clk else None
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        wall_e2e = _max_over_ranks((time.perf_counter() - t0) * 1e3, dist)
        res[prec] = {"ms": wall / args.steps, "ms_e2e": wall_e2e / args.steps, "st": stats[-1],
                     "clocks": clocks, "flow": flow_d.cpu().numpy()}
        npx, nnzb, nred = f.sizes()
        f.close()
    m, d = res["mixed"], res["fp64"]
    npn = inst.np
    vel_err = float(np.linalg.norm(m["flow"][:3 * npn] - d["flow"][:3 * npn]) /
                    np.linalg.norm(d["flow"][:3 * npn]))
    line = {"metric": "P2-P1 Stokes solves/s (33^3 sphere, mu 1, tol 1e-8), mixed vs FP64 GPU",
            "value": round(ws * 1e3 / m["ms"], 4), "unit": "solves/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(m["ms"], 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 inner / f64 outer",
            "data": "synthetic (seeded jittered Kuhn lattice, analytic level set)",
            "config": {"workload": f"p2sphere33: {npn} vertices + {npx - npn} edges, "
                                   f"{nnzb} 4x4 blocks, {nred} reduced unknowns"},
            "e2e": {"value": round(ws * 1e3 / m["ms_e2e"], 4), "unit": "solves/s",
                    "h2d_bytes_per_step": 8 * (2 * npn + inst.nt),
                    "d2h_bytes_per_step": 8 * 4 * npn},
            "fp64": {"value": round(ws * 1e3 / d["ms"], 4), "unit": "solves/s",
                     "iterations": d["st"]["iterations"]},
            "mixed": {"iterations": m["st"]["iterations"], "outer": m["st"]["outer_iterations"],
                      "rel_residual": m["st"]["rel_residual"], "vel_err_vs_fp64": vel_err},
            "ms_assembly": round(m["st"]["ms_assembly"], 3),
            "gpu_launches": int(m["st"]["kernel_launches"]), "clocks": m["clocks"]}
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle as O
        t0 = time.perf_counter()
        A, F, _, _ = O.p2_system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source,
                                 inst.mu, par)
        t_asm = time.perf_counter() - t0
        x = np.ones(A.shape[0])
        reps = 20
        t0 = time.perf_counter()
        for _ in range(reps):
            A @ x
        t_spmv = (time.perf_counter() - t0) / reps
        # the iterations of a Krylov method the CPU has without a multigrid:
        # FP64 MINRES with the block-Jacobi preconditioner (counted on the GPU)
        from fluidtissue_gb300.flow import Flow, Mesh
        fj = Flow()
        if fj.init(Mesh(inst.xyz, inst.tets), par, precision="fp64", warm_start=False,
                   preconditioner="jacobi", device=local) != 0:
            raise RuntimeError(fj.last_error())
        flow_j = np.zeros(4 * inst.np)
        if fj.solve(inst.phi, inst.source, flow_j, mu=inst.mu) != 0:
            raise RuntimeError(fj.last_error())
        its = int(fj.last_stats["iterations"])
        fj.close()
        t_cpu = t_asm + 2 * its * t_spmv
        line["cpu_baseline"] = {
            "value": 1.0 / t_cpu, "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": (f"oracle P2-P1 assembly in full ({t_asm:.2f} s) + 2 x {its} sparse "
                       f"products of the reduced system ({t_spmv * 1e3:.1f} ms each, scipy, "
                       f"1 thread), {its} = the iterations of block-Jacobi MINRES in FP64: "
                       f"a lower bound for the reference's un-preconditioned BiCGSTAB")}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_st(args, sub=None):
    """Surface-tension load (Flow::surfaceTension_ with LevelSet's normals,
    curvature and interface patches) on the ellipsoid129 mesh, phi = the
    workload's level set, phi_reset = its distance reset computed once on the
    GPU; "Surface tension" 1, "Node density" 1: value = loads/s through the C
    ABI with host buffers (phi and phi_reset in, the 3 np load out)."""
    import torch
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.flow import Mesh
    from fluidtissue_gb300.levelset import LevelSet

    if sub is None:
        ws, rank, local = _dist()
        dist = _setup_dist(ws, local)
        torch.cuda.set_device(local)
    else:
        local, dist, ws, rank = sub
    inst = W.ellipsoid129()
    ls = LevelSet()
    if ls.init(Mesh(inst.xyz, inst.tets), device=local) != 0:
        raise RuntimeError(ls.last_error())
    # the reset values: one update with a zero velocity (advection is the identity)
    flow = np.zeros(4 * inst.np)
    flow[3 * inst.np:] = 1.0
    phi = np.ascontiguousarray(inst.phi, np.float64).copy()
    if ls.update(flow, phi, {"Advection dt": 1.0 / 32.0, "Advection tolerance": 1e-10,
                             "Max. CG iterations": 0.0}) != 0:
        raise RuntimeError(ls.last_error())
    ifn = ls.reset_values()
    par = {"Surface tension": 1.0, "Node density": 1.0}

    def step():
        ls.surface_tension(phi, par, phi_reset=ifn)
        return ls.last_st_stats

    for _ in range(args.warmup):
        step()
    _barrier(dist)
    clk = Clocks(local)
    t0 = time.perf_counter()
    stats = [step() for _ in range(args.steps)]
    wall = _max_over_ranks((time.perf_counter() - t0) * 1e3, dist)
    st = stats[-1]
    dev_ms = float(np.mean([s["ms_kernels"] for s in stats]))
    line = {"metric": "surface-tension loads/s (ellipsoid129: normals, curvature, patches)",
            "value": round(ws * 1e3 / dev_ms, 3), "unit": "loads/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(dev_ms, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 / f32",
            "data": "synthetic (ellipsoid129 level set and its distance reset)",
            "config": {"workload": f"st129: {inst.np} nodes, {inst.nt} tets"},
            "e2e": {"value": round(ws * args.steps / (wall / 1e3), 3), "unit": "loads/s",
                    "h2d_bytes_per_step": 2 * 8 * inst.np, "d2h_bytes_per_step": 3 * 8 * inst.np},
            "interface_points": st["interface_points"], "area": st["area"],
            "gpu_launches": int(st["kernel_launches"]), "clocks": clk.stop()}
    if sub is not None:
        ls.close()
        return line
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle as O
        t0 = time.perf_counter()
        O.surface_tension(inst.xyz, inst.tets, phi, ifn, 1.0, 1)
        t_cpu = time.perf_counter() - t0
        line["cpu_baseline"] = {
            "value": 1.0 / t_cpu, "unit": "loads/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"oracle, the same load in full ({O.num_threads()} threads, {t_cpu:.2f} s)"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ls.close()


def run_ls(args, sub=None):
    """Level-set update (LevelSet::update: Crank-Nicolson advection with
    Jacobi-BiCGSTAB, distance reset, mixing) on the ellipsoid129 mesh, advected
    by the velocity of its own mixed-precision Stokes solve (Advection dt 1/32,
    tolerance 1e-6 as in the reference's parameter summary): value =
    updates/s through the C ABI with host buffers."""
    import torch
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.flow import Flow, Mesh
    from fluidtissue_gb300.levelset import LevelSet

    if sub is None:
        ws, rank, local = _dist()
        dist = _setup_dist(ws, local)
        torch.cuda.set_device(local)
    else:
        local, dist, ws, rank = sub
    inst = W.ellipsoid129()
    f = Flow()
    if f.init(Mesh(inst.xyz, inst.tets), inst.params, precision="mixed", device=local) != 0:
        raise RuntimeError(f.last_error())
    flow = np.zeros(4 * inst.np)
    if f.solve(inst.phi, inst.source, flow, mu=inst.mu) != 0:
        raise RuntimeError(f.last_error())
    f.close()
    par = {"Advection dt": 1.0 / 32.0, "Advection tolerance": 1e-6, "Max. CG iterations": 0.0}
    ls = LevelSet()
    if ls.init(Mesh(inst.xyz, inst.tets), device=local) != 0:
        raise RuntimeError(ls.last_error())

    def step():
        phi = np.ascontiguousarray(inst.phi, np.float64).copy()
        rc = ls.update(flow, phi, par)
        if rc != 0:
            raise RuntimeError(f"fts_ls_update failed ({rc}): {ls.last_error()}")
        return ls.last_stats

    for _ in range(args.warmup):
        step()
    _barrier(dist)
    clk = Clocks(local)
    t0 = time.perf_counter()
    stats = [step() for _ in range(args.steps)]
    wall = _max_over_ranks((time.perf_counter() - t0) * 1e3, dist)
    st = stats[-1]
    line = {"metric": "level-set updates/s (ellipsoid129: advection + distance reset)",
            "value": round(ws * args.steps / (wall / 1e3), 3), "unit": "updates/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(wall / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (ellipsoid129; velocity of its own Stokes solve)",
            "config": {"workload": f"ls129: {inst.np} nodes, dt 1/32, tol 1e-6"},
            "e2e": {"value": round(ws * args.steps / (wall / 1e3), 3), "unit": "updates/s",
                    "h2d_bytes_per_step": 5 * 8 * inst.np, "d2h_bytes_per_step": 8 * inst.np},
            "iterations": st["iterations"], "interface_points": st["interface_points"],
            "ms_assembly": round(st["ms_assembly"], 3), "ms_solve": round(st["ms_solve"], 3),
            "ms_reset": round(st["ms_reset"], 3), "gpu_launches": int(st["kernel_launches"]),
            "clocks": clk.stop()}
    if sub is not None:
        ls.close()
        return line
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle as O
        from fluidtissue_gb300.distance import interface_points
        phi = np.ascontiguousarray(inst.phi, np.float64).copy()
        t0 = time.perf_counter()
        O.ls_update(inst.xyz, inst.tets, flow, phi, par["Advection dt"], tol=1e-6, reset=False)
        t_adv = time.perf_counter() - t0
        pts, _ = interface_points(inst.xyz, inst.tets, phi)
        k1 = inst.np  # all nodes: about 8 s on 16 host threads
        d = phi.copy()
        t0 = time.perf_counter()
        O.dist_reset(inst.xyz, pts, d, 0, k1)
        t_dist = (time.perf_counter() - t0) * inst.np / k1
        line["cpu_baseline"] = {
            "value": 1.0 / (t_adv + t_dist), "unit": "updates/s", "cores": O.num_threads(),
            "kind": "port",
            "sample": (f"oracle on the same update ({O.num_threads()} threads): assembly + "
                       f"Jacobi-BiCGSTAB {t_adv:.2f} s in full; distance reset timed on "
                       f"{k1} of {inst.np} nodes and scaled ({t_dist:.2f} s)")}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ls.close()


def _free_port() -> int:
    import socket
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def spawn_ranks(n: int, argv: list[str]) -> int:
    """Runs this script as n local ranks (torch.distributed.run, rendezvous on
    127.0.0.1) with the same arguments; returns the launcher's exit status."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           f"--nproc-per-node={n}", "--master-addr", "127.0.0.1", "--master-port",
           str(_free_port()), str(Path(__file__).resolve()), *argv]
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--steps-fp64", type=int, default=2)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ellipsoid129")
    ap.add_argument("--preconditioner", default="auto",
                    choices=["auto", "jacobi", "multigrid", "multigrid_diag"])
    ap.add_argument("--inner-tol", type=float, default=0.0)
    ap.add_argument("--cpu-seconds", type=float, default=30.0)
    ap.add_argument("--ref-chunk", type=int, default=200,
                    help="MINRES iterations per step of the sampled reference arm")
    ap.add_argument("--batch-count", type=int, default=96)
    ap.add_argument("--operator", default=None, choices=["stencil", "assembled", "matfree"])
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-subresults", action="store_true",
                    help="skip the batch96 and spheres257 sub-results of the default line")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.gpus < 1:
        ap.error("--gpus must be >= 1")
    world = os.environ.get("WORLD_SIZE")
    if world is None and args.gpus > 1:
        # no launcher: start one rank per GPU on this node and wait for them
        sys.exit(spawn_ranks(args.gpus, sys.argv[1:]))
    if world is not None and int(world) != args.gpus:
        ap.error(f"--gpus {args.gpus} does not match WORLD_SIZE={world} of the launcher")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload.startswith("batch"):
        run_batch(args)
    elif args.workload == "rd129":
        run_rd(args)
    elif args.workload == "dist129":
        run_dist(args)
    elif args.workload == "ls129":
        run_ls(args)
    elif args.workload == "st129":
        run_st(args)
    elif args.workload == "p2sphere33":
        run_p2(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
