"""Benchmark: variable-viscosity P1-P1 Stokes solves/s on one GB300.

Workload (default): ``ellipsoid129`` — 129^3 Kuhn lattice (12.6M tets),
jitter +-0.1h, ellipsoid level set, 16 Gaussian centres, mu = clip(1/(0.01+c),
0.01, 100), relative residual 1e-8.  One step = one complete Stokes solve
(viscosity, source, RHS and matrix assembly, Krylov solve, scatter to flow)
from a zero initial guess, inputs resident in HBM.

Reported:
  value     mixed-precision solves/s (device-resident inputs)
  e2e       the same through fts_solve with pinned host buffers (H2D of
            phi/source/mu and D2H of flow inside the timed region)
  fp64      the plain FP64 GPU path on the same workload
  roofline  the Krylov loop's operator kernel (BSR SpMV fused with the MINRES
            dots), algorithmic bytes / CUDA-event time, vs measured HBM peak
  cpu_baseline  the CPU oracle (restated reference algorithm) on the box's
            host cores, bounded sample

``--impl reference`` times the reference's algorithm on the host CPU (the
oracle port): assembly + un-preconditioned BiCGSTAB, bounded sample.
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


def run_ours(args):
    import torch
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.flow import Flow, Mesh

    ws, rank, local = _dist()
    dist = _setup_dist(ws, local)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    inst = W.WORKLOADS[args.workload]()
    par = dict(inst.params)
    npn, nt = inst.np, inst.nt

    stream = torch.cuda.Stream(device=dev)
    phi_d = torch.from_numpy(inst.phi).to(dev)
    src_d = torch.from_numpy(inst.source).to(dev)
    mu_d = torch.from_numpy(inst.mu).to(dev)
    flow_d = torch.zeros(4 * npn, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()

    operator = args.operator or ("matfree" if args.workload == "spheres257" else "auto")
    if operator == "auto":  # every bench workload is a Kuhn lattice: the half-stencil copy
        operator = "stencil"
    with_fp64 = not args.no_fp64 and operator != "matfree"

    def make(precision):
        f = Flow()
        rc = f.init(Mesh(inst.xyz, inst.tets), par, precision=precision, warm_start=False,
                    device=local, preconditioner=args.preconditioner, time_kernels=True,
                    inner_tol=args.inner_tol,
                    operator=operator if precision == "mixed" else "assembled")
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
        t0 = time.perf_counter()
        out = fn(k)
        e1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        ms = e0.elapsed_time(e1)
        _barrier(dist)
        clocks = clk.stop() if clk else None
        return out, _max_over_ranks(ms, dist), wall, clocks

    # ---- mixed precision, device-resident inputs (value) --------------------
    fm = make("mixed")
    device_steps(fm, args.warmup)
    stats_m, ms_m, wall_m, clocks = timed(lambda k: device_steps(fm, k), args.steps, local)
    value = ws * args.steps / (ms_m / 1e3)

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
    _, ms_e, wall_e, _ = timed(host_steps, args.steps)
    e2e = ws * args.steps / (ms_e / 1e3)
    rel_mixed = float(fm.last_stats["rel_residual"])
    flow_mixed = flow_h.copy()

    # ---- plain FP64 on the same workload -------------------------------------
    f64 = None
    stats_d, ms_d, value_fp64, vel_err, p_err, k64 = None, None, None, None, None, 0
    if with_fp64:
        f64 = make("fp64")
        device_steps(f64, 1)
        k64 = max(1, args.steps_fp64)
        stats_d, ms_d, _, _ = timed(lambda k: device_steps(f64, k), k64)
        value_fp64 = ws * k64 / (ms_d / 1e3)
        flow64 = flow_d.cpu().numpy()
        vel_err = float(np.linalg.norm(flow_mixed[:3 * npn] - flow64[:3 * npn]) /
                        np.linalg.norm(flow64[:3 * npn]))
        p_err = float(np.linalg.norm(flow_mixed[3 * npn:] - flow64[3 * npn:]) /
                      np.linalg.norm(flow64[3 * npn:]))

    # ---- roofline of the dominant kernel (live CUDA-event timing) -----------
    spmv_ms = sum(s["ms_spmv"] for s in stats_m)
    spmv_n = sum(s["spmv_launches"] for s in stats_m)
    per = spmv_ms / max(spmv_n, 1)
    bytes_per = stats_m[0]["spmv_bytes"]
    achieved = bytes_per / (per / 1e3) / 1e9 if spmv_n else None
    peak, peak_kind = _peaks()
    ach64, it_d = None, None
    if stats_d:
        spmv64_ms = sum(s["ms_spmv"] for s in stats_d)
        spmv64_n = sum(s["spmv_launches"] for s in stats_d)
        ach64 = (stats_d[0]["spmv_bytes"] / (spmv64_ms / spmv64_n / 1e3) / 1e9) if spmv64_n else None
        it_d = statistics.mean(s["iterations"] for s in stats_d)

    launches = int(sum(s["kernel_launches"] for s in stats_m))
    it_m = statistics.mean(s["iterations"] for s in stats_m)
    dofs = 4 * npn

    res = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_m / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 outer",
        "data": "synthetic (seeded Kuhn lattice, analytic level set, Gaussian growth factor)",
        "config": {"workload": f"{args.workload}: {npn} nodes, {nt} tets, "
                               f"{dofs} block DOF, tol {par['Stokes tolerance']}",
                   "precision": "mixed", "preconditioner": args.preconditioner,
                   "l2": "inputs larger than L2 (operator > 1 GB streamed every iteration)",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
        "e2e": {"value": round(e2e, 4), "unit": UNIT,
                "h2d_bytes_per_step": int(phi_h.nbytes + src_h.nbytes + mu_h.nbytes),
                "d2h_bytes_per_step": int(flow_h.nbytes)},
        "fp64": ({"value": round(value_fp64, 4), "unit": UNIT,
                  "ms_per_step": round(ms_d / k64, 3), "iterations": it_d,
                  "spmv_gbs": round(ach64, 1) if ach64 else None} if value_fp64 else None),
        "mixed_vs_fp64": round(value / value_fp64, 3) if value_fp64 else None,
        "operator": operator,
        "device_bytes": int(stats_m[0]["device_bytes"]),
        "mixed": {"iterations": it_m, "iterations_fp32": statistics.mean(
            s["iterations_fp32"] for s in stats_m),
                  "outer": statistics.mean(s["outer_iterations"] for s in stats_m),
                  "rel_residual": rel_mixed, "vel_err_vs_fp64": vel_err,
                  "p_err_vs_fp64": p_err},
        "dof_iterations_per_s": round(value * it_m * dofs, 1),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1) if achieved else None,
                     "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4) if achieved else None,
                     "traffic": _traffic(KERNELS[operator][0], bytes_per),
                     "kernel": f"{KERNELS[operator][0]} ({KERNELS[operator][1]})",
                     "bytes_per_launch": bytes_per, "ms_per_launch": round(per, 5),
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "gpu_launches": launches,
        "clocks": clocks,
        "ms_assembly": round(statistics.mean(s["ms_assembly"] for s in stats_m), 3),
    }
    if rank == 0 and not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_baseline(inst, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(res), flush=True)
    fm.close()
    if f64 is not None:
        f64.close()
    if dist is not None:
        dist.destroy_process_group()


def run_batch(args):
    """Batched workload: 96 independent instances (n ~ U{17..65}, seeded per
    instance) per step, solved by fts_batch_solve_device (one persistent
    launch per Krylov run, CUDA graph, autotuned); FP64 and mixed."""
    import torch
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.flow import Batch, Mesh

    ws, rank, local = _dist()
    dist = _setup_dist(ws, local)
    torch.cuda.set_device(local)
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

        for _ in range(args.warmup):
            step()
        _barrier(dist)
        torch.cuda.synchronize()
        clk = Clocks(local) if prec == "mixed" else None
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = _max_over_ranks(e0.elapsed_time(e1), dist)
        clocks = clk.stop() if clk else None
        st = b.last_stats
        dofs = sum(4 * i.np for i in insts)
        its = [s["iterations"] for s in st]
        out[prec] = {"solves_per_s": round(ws * len(insts) * args.steps / (ms / 1e3), 3),
                     "ms_per_batch": round(ms / args.steps, 2),
                     "iterations_mean": statistics.mean(its), "iterations_max": max(its),
                     "max_rel_residual": max(s["rel_residual"] for s in st),
                     "dof_iterations_per_s": round(
                         sum(4 * i.np * s["iterations"] for i, s in zip(insts, st)) * ws
                         * args.steps / (ms / 1e3), 1),
                     "autotuned": b.config(), "clocks": clocks}
        b.close()
    if rank == 0:
        res = {"metric": "batched Stokes solves/s (96 instances, n ~ U{17..65}, tol 1e-8)",
               "value": out["mixed"]["solves_per_s"], "unit": UNIT, "n_gpus": ws,
               "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": out["mixed"]["ms_per_batch"], "higher_is_better": True,
               "scaling": "strong" if ws > 1 else "weak", "dtype": "f32 inner / f64 outer",
               "data": "synthetic", "config": {"workload": f"batch{count}",
                                               "instances": count,
                                               "nodes_total": sum(i.np for i in insts)},
               "mixed": out["mixed"], "fp64": out["fp64"],
               "mixed_vs_fp64": round(out["mixed"]["solves_per_s"] /
                                      out["fp64"]["solves_per_s"], 3)}
        print(json.dumps(res), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def cpu_baseline(inst, seconds: float) -> dict:
    """The CPU oracle on this host's cores (OpenMP, FP64), bounded to about
    ``seconds``: the restated reference assembly (row gather, block
    composition, restriction to the reduced system) in full, plus a sample of
    preconditioned MINRES iterations with the block-Jacobi + rank-one
    preconditioner of the GPU's Jacobi mode.  The reference's own
    un-preconditioned BiCGSTAB does not converge on this workload (see
    profiles/cpu_baseline.md), so the CPU baseline uses the oracle's
    preconditioned method; solves/s = 1 / (t_assembly + N t_iteration) with N
    the iterations that method needs to the tolerance (measured with the same
    FP64 method on the GPU, profiles/cpu_baseline.md)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    threads = O.num_threads()
    t0 = time.perf_counter()
    R, _, _, mu = O.system(inst.xyz, inst.tets, inst.boundary, inst.phi, inst.source, inst.mu,
                           inst.params)
    pre = O.block_jacobi(R, inst.xyz, inst.tets, mu, inst.params["eps"])
    t_asm = time.perf_counter() - t0
    it = 8
    while True:
        t1 = time.perf_counter()
        _, _, done = O.minres_blockjacobi(R, pre, rtol=1e-30, maxit=it)
        t_run = time.perf_counter() - t1
        t_it = t_run / max(done, 1)
        if t_asm + t_run > seconds * 0.5 or it >= 8192:
            break
        it *= 2
    n_it = CPU_BASELINE_ITERATIONS.get(inst.name)
    value = 1.0 / (t_asm + n_it * t_it) if n_it else None
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": (f"oracle on {inst.name} ({threads} threads): full assembly + "
                       f"preconditioner set-up ({t_asm:.2f} s) + {done} block-Jacobi MINRES "
                       f"iterations ({t_it * 1e3:.1f} ms each); solves/s = 1/(t_asm + N t_iter) "
                       f"with N = {n_it} iterations of the same FP64 method to tol "
                       f"{inst.params['Stokes tolerance']} (profiles/cpu_baseline.md)"),
            "t_assembly_s": t_asm, "t_iteration_s": t_it}


# Iterations of FP64 block-Jacobi + rank-one MINRES to the workload tolerance
# (profiles/cpu_baseline.md): the CPU baseline's iteration count.
CPU_BASELINE_ITERATIONS: dict = {"sphere17": 1940, "sphere65": 4204, "ellipsoid129": 42647}


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    from fluidtissue_gb300 import workloads as W
    inst = W.WORKLOADS[args.workload]()
    vals = []
    cb = None
    for _ in range(args.warmup + args.steps):
        cb = cpu_baseline(inst, args.cpu_seconds / max(1, args.steps + args.warmup))
        vals.append(cb["value"])
    v = vals[-1]
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
           "config": {"workload": inst.name}, "cpu_baseline": cb,
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


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


def run_rd(args):
    """Reaction-diffusion (RD::solve) on the ellipsoid129 mesh and level set:
    value = RD calls/s, one call = 32000 FP64 explicit Euler steps of the
    activator, inhibitor and growth factor on the interior submesh (all steps
    in one persistent launch).  The state is copied in from and out to host
    memory every call (the reference's RD keeps it on the host)."""
    import torch
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.flow import Mesh
    from fluidtissue_gb300.rd import RD

    ws, rank, local = _dist()
    dist = _setup_dist(ws, local)
    torch.cuda.set_device(local)
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


def run_dist(args):
    """Distance reset (EuclideanDistance::resetPhi) on the ellipsoid129 mesh
    against its own interface points (the zero level set's edge crossings,
    LevelSet.cpp:278-300): value = resets/s of the pruned search, through the
    C ABI with host buffers (H2D, device binning of the points, search, D2H).
    Beside it the reference's algorithm (every node against every point) on the
    same GPU, and the oracle's host restatement on all nodes."""
    import torch
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.distance import EuclideanDistance, interface_points

    ws, rank, local = _dist()
    dist = _setup_dist(ws, local)
    torch.cuda.set_device(local)
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


def run_p2(args):
    """P2-P1 (Taylor-Hood, "Stokes velocity degree" 2) on the jittered 33^3
    sphere workload (mu = 1, 8 Gaussian centres, tol 1e-8): value = mixed-
    precision solves/s with device-resident inputs, e2e through fts_solve with
    host buffers, beside the FP64 GPU path.  CPU baseline: the oracle's P2-P1
    assembly (the reference's element loop) in full plus its reduced system's
    sparse products, two per iteration of the reference's BiCGSTAB, times the
    iterations the GPU's FP64 MINRES needs (a lower bound: the reference's
    un-preconditioned BiCGSTAB needs more)."""
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
        its = d["st"]["iterations"]
        t_cpu = t_asm + 2 * its * t_spmv
        line["cpu_baseline"] = {
            "value": 1.0 / t_cpu, "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": (f"oracle P2-P1 assembly in full ({t_asm:.2f} s) + 2 x {its} sparse "
                       f"products of the reduced system ({t_spmv * 1e3:.1f} ms each, scipy, "
                       f"1 thread): a lower bound for the reference's BiCGSTAB")}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_st(args):
    """Surface-tension load (Flow::surfaceTension_ with LevelSet's normals,
    curvature and interface patches) on the ellipsoid129 mesh, phi = the
    workload's level set, phi_reset = its distance reset computed once on the
    GPU; "Surface tension" 1, "Node density" 1: value = loads/s through the C
    ABI with host buffers (phi and phi_reset in, the 3 np load out)."""
    import torch
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.flow import Mesh
    from fluidtissue_gb300.levelset import LevelSet

    ws, rank, local = _dist()
    dist = _setup_dist(ws, local)
    torch.cuda.set_device(local)
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


def run_ls(args):
    """Level-set update (LevelSet::update: Crank-Nicolson advection with
    Jacobi-BiCGSTAB, distance reset, mixing) on the ellipsoid129 mesh, advected
    by the velocity of its own mixed-precision Stokes solve (Advection dt 1/32,
    tolerance 1e-6 as in the reference's parameter summary): value =
    updates/s through the C ABI with host buffers."""
    import torch
    from fluidtissue_gb300 import workloads as W
    from fluidtissue_gb300.flow import Flow, Mesh
    from fluidtissue_gb300.levelset import LevelSet

    ws, rank, local = _dist()
    dist = _setup_dist(ws, local)
    torch.cuda.set_device(local)
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
    ap.add_argument("--batch-count", type=int, default=96)
    ap.add_argument("--operator", default=None, choices=["stencil", "assembled", "matfree"])
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
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
