#!/usr/bin/env python3
"""Benchmark of the GB300 solve path on the 3D Q2 convection-diffusion workload.

Workload (default): unit cube, 32^3 hexahedra, Q2 (274,625 DOFs), eps = 1e-2,
b = (1, 0.5, 0.25), u = 0 on the boundary, f from u = sin(pi x) sin(pi y) sin(pi z),
Gauss 3x3x3 quadrature, FGMRES(30) preconditioned by a multigrid V(2,2) cycle with
damped Jacobi (0.8) over 4 levels and a direct coarse solve, stopped at a 1e-8
relative FP64 residual. Inputs are synthetic (generated mesh, manufactured data).

One step = one solve request: assembly of all four levels on the device plus the
FGMRES solve. `value` is the mixed-precision form (FP32 multigrid inside FP64
FGMRES) in solves/s with the mesh resident in HBM; `e2e` is the same request
through pm_problem_run_host with the mesh geometry copied in from pinned host
memory and the solution copied back every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 (launched by torchrun): independent replicas, one per GPU, no collective
on the data path; rank 0 prints max-over-ranks timing.
"""
from __future__ import annotations

import argparse
import faulthandler
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "solves/sec, DOFs/s at 1e-8 FP64 residual (mixed vs FP64); SpMV GB/s; p99"

WORKLOADS = {
    "cd3d_q2_32": dict(geometry=1, root_n=1, n_refine=5, n_levels=4, elem=2, eps=1e-2,
                       b=(1.0, 0.5, 0.25), quad=3, restart=30, reduction=1e-8,
                       desc="3D Q2 convection-diffusion, 32^3 hexahedra (274,625 DOFs), "
                            "FGMRES(30) + MG V(2,2) Jacobi(0.8), 4 levels, to 1e-8"),
    "cd2d_q1_128": dict(geometry=0, root_n=1, n_refine=7, n_levels=4, elem=1, eps=0.1,
                        b=(1.0, 0.0, 0.0), quad=3, restart=20, reduction=1e-10,
                        desc="2D Q1 convection-diffusion, 128^2 quadrilaterals (16,641 DOFs), "
                             "FGMRES(20) + MG V(2,2) Jacobi(0.8), 4 levels, to 1e-10"),
    # Stokes P2/P1 on 24^3 cubes x 6 tetrahedra; nodal Vanka (cell Vanka is
    # singular on the cells along the cube edges and converges poorly with a
    # continuous pressure)
    "stokes3d_p2p1_24": dict(kind="stokes", geometry=2, root_n=3, n_refine=3, n_levels=3, elem=12, nu=1.0,
                             restart=30, reduction=1e-8, smoother="nodal_vanka", coarse="nodal_vanka_jacobi",
                             damp=0.8, pre=1, post=1, sample=dict(root_n=3, n_refine=2, n_levels=3),
                             desc="3D Stokes P2/P1, 24^3 cubes x 6 tetrahedra (352,947 velocity + 15,625 "
                                  "pressure DOFs), FGMRES(30) + MG V(1,1) nodal Vanka (colour order, damping "
                                  "0.8), 3 levels, coarse level: additive nodal Vanka, at most 10 sweeps down "
                                  "to a 0.1 residual, to 1e-8"),
    # Navier-Stokes (convective form) at Reynolds number 10 on the same mesh:
    # the reference's example -3 of test/nse3d_solvers_test.c++; one request =
    # assemble_linear_terms + the Picard loop to a 1e-10 nonlinear residual
    "nse3d_p2p1_24": dict(kind="nse", geometry=2, root_n=3, n_refine=3, n_levels=3, elem=12, nu=0.1,
                          restart=30, reduction=1e-8, smoother="nodal_vanka", coarse="nodal_vanka_jacobi",
                          damp=0.8, pre=1, post=1, nl_epsilon=1e-10, nl_maxit=30,
                          sample=dict(root_n=3, n_refine=1, n_levels=1),
                          desc="3D Navier-Stokes P2/P1 (convective form, Picard), Reynolds number 10, "
                               "24^3 cubes x 6 tetrahedra (352,947 velocity + 15,625 pressure DOFs), "
                               "example -3 of the reference's NSE test; each nonlinear step FGMRES(30) + "
                               "MG V(1,1) nodal Vanka (colour order, damping 0.8), 3 levels, to 1e-8 "
                               "relative; nonlinear loop to a 1e-10 residual"),
}


def solver_db(w, precision):
    import mymoonmd_gb300 as m
    db = m.ParameterDatabase.solve_path_database()
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = "fgmres"
    db["preconditioner"] = "multigrid"
    db["residual_tolerance"] = 0.0
    db["residual_reduction"] = w["reduction"]
    db["max_n_iterations"] = 500
    db["gmres_restart"] = w["restart"]
    db["multigrid_n_levels"] = w["n_levels"]
    db["multigrid_smoother"] = w.get("smoother", "jacobi")
    db["multigrid_smoother_coarse"] = w.get("coarse", "direct_solve")
    db["jacobi_damp"] = 0.8
    db["multigrid_vanka_damp_factor"] = w.get("damp", 1.0)
    db["multigrid_n_pre_smooth"] = w.get("pre", 2)
    db["multigrid_n_post_smooth"] = w.get("post", 2)
    db["gpu_precision"] = precision
    if w.get("kind") == "nse":
        db.add("example", -3)
        db.add("problem_type", 5)
        db.add("nonlinloop_epsilon", w["nl_epsilon"])
        db.add("nonlinloop_maxit", w["nl_maxit"])
    return db


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region"""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def large_spmv(ctx, m, np, hbm_peak):
    """SpMV bandwidth on a matrix well above L2: 3D Q2 48^3 (912,673 rows,
    about 54 M nonzeros, 650 MB of FP64 CSR), FP64 and FP32 values"""
    disc = m.Discretization(m.GEO_CUBE_HEXA, 3, 4, 1, m.KIND_CD, 2)
    db = m.ParameterDatabase.solve_path_database()
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = "fgmres"
    db["preconditioner"] = "no_preconditioner"
    prob = m.ConvectionDiffusion(ctx, disc, m.cd_coeffs(1e-2, (1.0, 0.5, 0.25), 0.0, True), db, quad_points=3)
    prob.assemble()
    A = prob.matrix(-1)
    A.make_fp32()
    A.make_sliced64()
    n = A.n_rows
    x, y = m.DeviceVector(ctx, n), m.DeviceVector(ctx, n)
    x32, y32 = m.DeviceVector(ctx, n, np.float32), m.DeviceVector(ctx, n, np.float32)
    A.bench_apply(x, y, 3)
    ms64, b64 = A.bench_apply(x, y, 20)
    A.bench_apply(x32, y32, 3, fp32=True)
    ms32, b32 = A.bench_apply(x32, y32, 20, fp32=True)
    out = {"matrix": "3D Q2 48^3", "rows": n, "nnz": int(A.nnz),
           "fp64_gbs": round(b64 / (ms64 / 1e3) / 1e9, 1), "fp32_gbs": round(b32 / (ms32 / 1e3) / 1e9, 1)}
    out["fp64_frac"] = round(out["fp64_gbs"] / hbm_peak, 3)
    out["fp32_frac"] = round(out["fp32_gbs"] / hbm_peak, 3)
    prob.close()
    return out


def run_ours(args, w, rank, world, local, pg):
    import numpy as np
    import mymoonmd_gb300 as m

    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))

    ctx = m.Context(local)
    nse = w.get("kind") == "nse"
    stokes = w.get("kind") in ("stokes", "nse")
    disc = m.Discretization(w["geometry"], w["root_n"], w["n_refine"], w["n_levels"],
                            m.KIND_STOKES if stokes else m.KIND_CD, w["elem"])
    cf = None if stokes else m.cd_coeffs(w["eps"], w["b"], 0.0, True)
    fin = disc.level_info(w["n_levels"] - 1)
    n_dofs, nnz = fin["n_dofs"], fin["nnz"]
    if stokes:
        n_dofs = 3 * n_dofs + disc.level_info(w["n_levels"] - 1, 1)["n_dofs"]

    def make_problem(precision):
        if stokes:
            return m.StokesProblem(ctx, disc, w["nu"], solver_db(w, precision))
        return m.ConvectionDiffusion(ctx, disc, cf, solver_db(w, precision), quad_points=w["quad"])

    def solve(prob):
        # a Navier-Stokes request runs the nonlinear loop
        if nse:
            return len(prob.solve_nonlinear()) - 1
        prob.solve()
        return 1

    results = {}
    for precision in ("fp64", "mixed"):
        prob = make_problem(precision)
        for _ in range(args.warmup):
            prob.reset_solution()
            prob.assemble()
            solve(prob)
        # phase split of one request (device time)
        prob.reset_solution()
        ctx.time_begin()
        prob.assemble()
        asm_ms = ctx.time_end()
        ctx.time_begin()
        nl_steps = solve(prob)
        solve_ms = ctx.time_end()
        its = []
        step_ms = []
        barrier(pg)
        ctx.synchronize()
        sampler = ClockSampler(local) if precision == "mixed" else None
        if sampler:
            sampler.start()
        launches0 = ctx.kernel_launches()
        t0 = time.perf_counter()
        ctx.time_begin()
        for _ in range(args.steps):
            ctx_t = time.perf_counter()
            prob.reset_solution()
            prob.assemble()
            solve(prob)
            step_ms.append((time.perf_counter() - ctx_t) * 1e3)
            its.append(prob.last_info()[0])
        dev_ms = ctx.time_end()
        wall = time.perf_counter() - t0
        launches = ctx.kernel_launches() - launches0
        clocks = sampler.stop() if sampler else None
        probe = None
        if precision == "mixed":
            # per-launch device times of the finest-level SpMV family: events around
            # every launch, over requests run right after the timed ones (the
            # captured graphs are bypassed while the probe brackets launches)
            # (the dominant kernel only: the FP32 damped Jacobi sweep)
            # (Stokes: the residual + local-solve pair of every colour of the
            # multiplicative nodal Vanka sweeps, the largest share there)
            if stokes:
                ctx.probe(0)
                ctx.set_option("probe_nodal", 1)
            else:
                ctx.set_option("probe_epilogue", PROBE_EPILOGUE)
                ctx.set_option("probe_precision", 4)
                ctx.probe(nnz)
            for _ in range(min(args.steps, 3)):
                prob.reset_solution()
                prob.assemble()
                solve(prob)
            probe = ctx.probe_result()
            ctx.probe(0)
            ctx.set_option("probe_nodal", 0)
            ctx.set_option("probe_epilogue", -1)
            ctx.set_option("probe_precision", 0)
        barrier(pg)
        ms = max_over_ranks(pg, dev_ms)
        results[precision] = dict(ms=ms, wall=wall, its=its, step_ms=step_ms, launches=launches,
                                  clocks=clocks, probe=probe, info=prob.last_info(), solution=prob.solution(),
                                  nl_steps=nl_steps,
                                  split={"assembly_ms": round(asm_ms, 3), "solve_ms": round(solve_ms, 3)})
        if precision == "mixed":
            keep_prob = prob
        else:
            prob.close()

    # end-to-end through the public API: geometry in from pinned host memory,
    # solution back to pinned host memory, every step
    prob = keep_prob
    verts = [disc.cell_vertices(l) for l in range(w["n_levels"])]
    pinned = []
    for v in verts:
        pa = m.PinnedArray(ctx, v.size)
        pa.array[:] = v.ravel()
        pinned.append(pa)
    sol = m.PinnedArray(ctx, n_dofs)
    h2d = sum(v.nbytes for v in verts) + 64
    d2h = n_dofs * 8
    for _ in range(max(1, args.warmup)):
        prob.run_host(cf, [p.array for p in pinned], sol.array)
    barrier(pg)
    ctx.synchronize()
    t0 = time.perf_counter()
    ctx.time_begin()
    for _ in range(args.steps):
        prob.run_host(cf, [p.array for p in pinned], sol.array)
    e2e_ms = max_over_ranks(pg, ctx.time_end())
    del t0

    # stand-alone SpMV bandwidth of the finest FP64 and FP32 matrices
    A = prob.matrix(-1)
    x = m.DeviceVector(ctx, n_dofs)
    y = m.DeviceVector(ctx, n_dofs)
    x32 = m.DeviceVector(ctx, n_dofs, np.float32)
    y32 = m.DeviceVector(ctx, n_dofs, np.float32)
    A.bench_apply(x, y, 5)
    ms64, b64 = A.bench_apply(x, y, 50)
    A.bench_apply(x32, y32, 5, fp32=True)
    ms32, b32 = A.bench_apply(x32, y32, 50, fp32=True)
    # the row-group kernel on the CSR arrays, for comparison with the sliced copy
    ctx.set_option("fp32_sliced_spmv", 0)
    A.bench_apply(x32, y32, 5, fp32=True)
    msr, br = A.bench_apply(x32, y32, 50, fp32=True)
    ctx.set_option("fp32_sliced_spmv", SLICED_DEFAULT)
    big = None if stokes or args.no_large_spmv else large_spmv(ctx, m, np, hbm_peak)

    if rank != 0:
        return None
    mixed, fp64 = results["mixed"], results["fp64"]
    K = args.steps
    solves_s = world * K / (mixed["ms"] / 1e3)
    fp64_solves_s = world * K / (fp64["ms"] / 1e3)
    n_probe, probe_ms, probe_bytes = mixed["probe"]
    achieved = (probe_bytes / n_probe) / (probe_ms / n_probe / 1e3) / 1e9 if n_probe else None
    lat = sorted(mixed["step_ms"])
    line = {
        "metric": METRIC,
        "value": round(solves_s, 3),
        "unit": "solves/s",
        "n_gpus": world,
        "steps": K,
        "warmup": args.warmup,
        "ms_per_step": round(mixed["ms"] / K, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 multigrid inside f64 FGMRES (outer residuals f64)",
        "data": "synthetic: generated unit-cube mesh and manufactured-solution coefficients",
        "config": {"workload": w["desc"], "dofs": n_dofs, "nnz_finest": nnz,
                   "parallelism": f"replicas x{world} (no collective)",
                   "l2": "inputs larger than L2: finest FP64 matrix "
                         f"{(nnz * 12 + n_dofs * 4) / 1e6:.0f} MB > 126 MB L2",
                   "smoother": w.get("smoother", "jacobi"),
                   "step": ("assemble_linear_terms + Picard loop (per step: FGMRES/MG solve to "
                            f"{w['reduction']:g} relative, restriction of the velocity, assembly of the "
                            f"convective term on all levels) to a {w.get('nl_epsilon', 0):g} nonlinear residual"
                            if nse else "assembly of all levels + FGMRES/MG solve to "
                            f"{w['reduction']:g} relative FP64 residual")},
        "dofs_per_s": round(solves_s * n_dofs, 1),
        "fgmres_iterations": mixed["its"][-1],
        "final_relative_residual": mixed["info"][1] / mixed["info"][2],
        "nonlinear_steps": {"mixed": mixed["nl_steps"], "fp64": fp64["nl_steps"]} if nse else None,
        "phase_ms": mixed["split"],
        "fp64": {"value": round(fp64_solves_s, 3), "unit": "solves/s", "ms_per_step": round(fp64["ms"] / K, 3),
                 "fgmres_iterations": fp64["its"][-1], "dofs_per_s": round(fp64_solves_s * n_dofs, 1),
                 "phase_ms": fp64["split"]},
        "mixed_over_fp64": round(solves_s / fp64_solves_s, 3),
        # the mixed form's solution against the FP64 form's, same request
        "error_vs_fp64": float(np.abs(mixed["solution"] - fp64["solution"]).max() /
                               max(np.abs(fp64["solution"]).max(), 1e-300)),
        "latency_ms": {"p50": round(lat[len(lat) // 2], 3),
                       "p99": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3)},
        "spmv": {"fp64_gbs": round(b64 / (ms64 / 1e3) / 1e9, 1), "fp32_gbs": round(b32 / (ms32 / 1e3) / 1e9, 1),
                 "fp64_frac": round(b64 / (ms64 / 1e3) / 1e9 / hbm_peak, 3),
                 "fp32_frac": round(b32 / (ms32 / 1e3) / 1e9 / hbm_peak, 3),
                 "fp32_row_group_gbs": round(br / (msr / 1e3) / 1e9, 1),
                 "note": "fp32: the sliced-ELL kernel (library default); row_group: the CSR kernel"},
        "spmv_4x_l2": big,
        "e2e": {"value": round(world * K / (e2e_ms / 1e3), 3), "unit": "solves/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": mixed["launches"],
        "roofline": {"bound": "hbm",
                     "kernel": ("sell_kernel<float,8,8,PIPE,EPI_DEFECT> on the patch rows + k_nodal_local<float>: "
                                "one colour of the multiplicative nodal Vanka sweep in FP32 (local residuals of the "
                                "colour's patches from their sliced rows, then their Schur-complement local solves "
                                "and the update; all colours of both fine levels)"
                                if stokes else
                                "sell_kernel<4,8,PIPE,EPI_JACOBI>: finest-level damped Jacobi sweep in FP32 "
                                "on the sliced-ELL copy (the largest share of a mixed request's GPU time)"),
                     "achieved": round(achieved, 1) if achieved else None, "peak": hbm_peak,
                     "unit": "GB/s", "frac": round(achieved / hbm_peak, 3) if achieved else None,
                     "traffic": profiled_traffic(args.workload), "algorithmic_bytes_per_launch":
                         round(probe_bytes / n_probe) if n_probe else None,
                     "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)",
                     "launches_probed": n_probe,
                     "probe": (f"CUDA events around each colour's kernel pair over {min(K, 3)} requests run "
                               "right after the timed ones" if stokes else
                               f"CUDA events around each probed finest-level launch over {min(K, 3)} "
                               "requests run right after the timed ones")},
        "clocks": mixed["clocks"],
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, n_dofs)
    return line


PROBE_EPILOGUE = 3  # EPI_JACOBI (include/pmgpu.h, probe_epilogue)
SLICED_DEFAULT = 481  # the library's default fp32_sliced_spmv shape


def profiled_traffic(wname):
    """DRAM bytes (read + write) per launch of the probed kernel, from the ncu
    summary committed for this workload, or None"""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles",
                        f"sell_kernel_jacobi32_{wname}.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return int(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


def _oracle_solve(wname):
    """one oracle (CPU) request: assembly of all levels + FGMRES/MG solve"""
    from oracle import cd as ocd
    w = WORKLOADS[wname]
    if w.get("kind") == "nse":
        # the bounded sample: the nonlinear loop with the direct solver on the
        # 6^3 mesh of the family
        from oracle import nse as onse
        smp = w["sample"]
        o = onse.OracleNSE(smp["root_n"], smp["n_refine"], smp["n_levels"], 1.0 / w["nu"])
        t0 = time.perf_counter()
        hist = o.run(w["nl_epsilon"], w["nl_maxit"])
        return time.perf_counter() - t0, len(hist) - 1, 0, o.levels[-1].n
    if w.get("kind") == "stokes":
        # the bounded sample: the same family on the 12^3 mesh (three levels)
        from oracle import stokes as ost
        smp = w["sample"]
        o = ost.OracleStokes(smp["root_n"], smp["n_refine"], smp["n_levels"], w["nu"])
        t0 = time.perf_counter()
        o.assemble()
        # the oracle's colour-ordered sweep is the library's multiplicative order
        names = {"nodal_vanka": "nodal_color", "nodal_vanka_jacobi": "nodal_jacobi", "direct_solve": "direct_solve"}
        o.build_mg(smoother=names[w["smoother"]], coarse_smoother=names[w.get("coarse", "direct_solve")],
                   vanka_damp=w["damp"], n_pre=w["pre"], n_post=w["post"])
        sol, it, res, hist, st = o.solve(reduction=w["reduction"], max_it=500, restart=w["restart"])
        return time.perf_counter() - t0, it, st, o.finest.n
    o = ocd.OracleCD(w["geometry"], w["root_n"], w["n_refine"], w["n_levels"], w["elem"], w["eps"], w["b"],
                     0.0, w["quad"])
    t0 = time.perf_counter()
    o.assemble()
    o.build_mg(2, 2, 0.8, 1.0, "V")
    sol, it, res, hist, st = o.solve("fgmres", 0.0, w["reduction"], 500, 0, w["restart"])
    dt = time.perf_counter() - t0
    return dt, it, st, o.finest.n_dofs


def cpu_baseline(w, n_dofs):
    wname = [k for k, v in WORKLOADS.items() if v is w][0]
    dt, it, st, n_sample = _oracle_solve(wname)
    if n_sample == n_dofs:
        return {"value": round(1.0 / dt, 5), "unit": "solves/s", "cores": 1, "kind": "port",
                "sample": f"one full request (assembly of all levels + FGMRES/MG solve, {it} iterations) "
                          f"of the same workload by the C restatement in oracle/, single thread, {dt:.1f} s"}
    # a smaller mesh of the same family, scaled by the DOF ratio (work per
    # request grows at least linearly with the DOFs, so this overstates the CPU)
    if w.get("kind") == "nse":
        return {"value": round(n_sample / n_dofs / dt, 6), "unit": "solves/s", "cores": 1, "kind": "port",
                "sample": f"one full nonlinear request on the 6^3 mesh of the same family ({n_sample} DOFs, "
                          f"{it} Picard steps with a sparse direct solve each, {dt:.1f} s, oracle/nse.py "
                          f"on scipy), scaled by {n_sample}/{n_dofs} DOFs"}
    return {"value": round(n_sample / n_dofs / dt, 6), "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": f"one full request on the 12^3 mesh of the same family ({n_sample} DOFs, {it} "
                      f"iterations, {dt:.1f} s single thread, C restatement in oracle/), scaled by "
                      f"{n_sample}/{n_dofs} DOFs"}


def run_reference(args, w, rank, world):
    """the reference path's CPU implementation (the oracle port: the reference does not
    build here) on all host cores: one independent request per core per step"""
    import multiprocessing as mp
    wname = [k for k, v in WORKLOADS.items() if v is w][0]
    cores = os.cpu_count() or 1
    steps = max(1, min(args.steps, 2))
    warm = min(args.warmup, 1)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        for _ in range(warm):
            pool.map(_oracle_solve, [wname] * cores)
        t0 = time.perf_counter()
        its, n_sample = [], 0
        for _ in range(steps):
            rs = pool.map(_oracle_solve, [wname] * cores)
            its += [r[1] for r in rs]
            n_sample = rs[0][3]
        dt = time.perf_counter() - t0
    value = steps * cores / dt
    scale_note = ""
    if w.get("kind") in ("stokes", "nse"):
        # the CPU runs a smaller mesh of the family; scaled to the 24^3 workload by DOFs
        import mymoonmd_gb300 as m
        d = m.Discretization(w["geometry"], w["root_n"], w["n_refine"], w["n_levels"], m.KIND_STOKES, w["elem"])
        n_full = 3 * d.level_info(w["n_levels"] - 1)["n_dofs"] + d.level_info(w["n_levels"] - 1, 1)["n_dofs"]
        value *= n_sample / n_full
        scale_note = (f"; requests on the {'6' if w.get('kind') == 'nse' else '12'}^3 mesh ({n_sample} DOFs) "
                      f"scaled by {n_sample}/{n_full} DOFs")
    last = its[-1] if its else 0
    if w.get("kind") == "nse":
        what = (f"nonlinear requests ({last} Picard steps with a sparse direct solve each, the restatement "
                "oracle/nse.py on scipy)")
    else:
        what = (f"requests (assembly + FGMRES/MG, {last} iterations), C restatement in oracle/ (the "
                "reference is compiled from its sources where they are present, which is not this "
                "machine; its own solve of the 3D Q2 32^3 request takes about the restatement's time on "
                "one core, 19.4 s on a 2.7 GHz x86 core)")
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 5), "unit": "solves/s", "n_gpus": world,
        "steps": steps, "warmup": warm, "ms_per_step": round(dt / steps * 1e3, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: generated unit-cube mesh and manufactured-solution coefficients",
        "config": {"workload": w["desc"], "parallelism": f"{cores} independent CPU requests per step"},
        "cpu_baseline": {"value": round(value, 5), "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": f"{steps} step(s) (of {args.steps} requested) of {cores} concurrent full "
                                   + what + ", one per host core" + scale_note},
        "e2e": {"value": round(value, 5), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def stream_db(precision, max_it=100, batch_slots=8):
    import mymoonmd_gb300 as m
    db = m.ParameterDatabase.solve_path_database()
    # requests of one set-up solved together by the executor's batch lanes
    db.add("gpu_batch_slots", batch_slots)
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = "fgmres"
    db["preconditioner"] = "multigrid"
    db["residual_tolerance"] = 0.0
    db["residual_reduction"] = 1e-8
    db["max_n_iterations"] = max_it
    db["gmres_restart"] = 30
    db["multigrid_smoother"] = "jacobi"
    db["multigrid_smoother_coarse"] = "direct_solve"
    db["jacobi_damp"] = 0.8
    db["multigrid_n_pre_smooth"] = 2
    db["multigrid_n_post_smooth"] = 2
    db["gpu_precision"] = precision
    return db


def stokes_db(precision, max_it=100):
    db = stream_db(precision, max_it)
    db["multigrid_smoother"] = "nodal_vanka"
    db["multigrid_smoother_coarse"] = "nodal_vanka_jacobi"
    db["multigrid_vanka_damp_factor"] = 0.8
    db["multigrid_n_pre_smooth"] = 1
    db["multigrid_n_post_smooth"] = 1
    return db


def _submit(server, rq, tag, out):
    import mymoonmd_gb300 as m
    cf = m.cd_coeffs(rq["eps"], rq["b"], 0.0, True) if rq["kind"] == m.KIND_CD else None
    server.submit(rq["kind"], rq["geometry"], rq["root_n"], rq["n_refine"], rq["n_levels"], rq["elem"], cf,
                  rq["nu"], out, tag)


def run_stream(args, rank, world, local, pg):
    """the batched stream: 512 independent convection-diffusion requests (seed
    0) through the request executor; every solution is copied back to host
    memory. One untimed pass fills the workers' problem caches, then `steps`
    timed passes (host wall clock from the first submit to the last
    completion, device work included)."""
    import numpy as np
    import mymoonmd_gb300 as m
    from mymoonmd_gb300 import workloads as wl
    reqs = wl.stream_requests(args.requests, 0)
    outs = [np.empty(wl.dofs_of(r)) for r in reqs]
    total_dofs = sum(wl.dofs_of(r) for r in reqs)
    res = {}
    passes = max(1, min(args.steps, 3))
    sols = {}
    for precision in ("fp64", "mixed"):
        srv = m.Server(local, args.workers, stream_db(precision, batch_slots=args.batch_slots), None, int(150e9))
        t0 = time.perf_counter()
        for i, rq in enumerate(reqs):
            _submit(srv, rq, i, outs[i])
        srv.drain()
        cold = time.perf_counter() - t0
        srv.poll(1024)
        clocks = None
        sampler = ClockSampler(local) if precision == "mixed" else None
        if sampler:
            sampler.start()
        barrier(pg)
        t0 = time.perf_counter()
        results = []
        for _ in range(passes):
            for i, rq in enumerate(reqs):
                _submit(srv, rq, i, outs[i])
            srv.drain()
            results += srv.poll(1024)
        dt = max_over_ranks(pg, time.perf_counter() - t0)
        if sampler:
            clocks = sampler.stop()
        st = srv.stats()
        srv.close()
        status = {}
        for r in results[-len(reqs):]:
            status[r["status"]] = status.get(r["status"], 0) + 1
        lat = sorted(r["latency_ms"] for r in results)
        res[precision] = dict(dt=dt, cold=cold, status=status, lat=lat, stats=st, clocks=clocks,
                              its=[r["iterations"] for r in results[-len(reqs):]],
                              converged=sum(1 for r in results if r["status"] == 0),
                              ok={r["tag"] for r in results[-len(reqs):] if r["status"] == 0})
        sols[precision] = [o.copy() for o in outs]
    if rank != 0:
        return None
    mx, fp = res["mixed"], res["fp64"]
    # solves/s counts the requests that reached the 1e-8 residual reduction
    solves = world * mx["converged"] / mx["dt"]
    all_solves = world * passes * len(reqs) / mx["dt"]
    both = sorted(mx["ok"] & fp["ok"])
    errs = [float(np.abs(sols["mixed"][i] - sols["fp64"][i]).max() / max(np.abs(sols["fp64"][i]).max(), 1e-300))
            for i in both]
    names = {0: "converged", 5: "not_converged_at_max_it", 2: "over_hbm_cap"}
    return {
        "metric": METRIC, "value": round(solves, 3), "unit": "solves/s", "n_gpus": world, "steps": passes,
        "warmup": 1, "ms_per_step": round(mx["dt"] / passes * 1e3, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 multigrid inside f64 FGMRES (outer residuals f64)",
        "data": "synthetic: 512 requests drawn from numpy default_rng(0) (mymoonmd_gb300/workloads.py)",
        "config": {"workload": "batched stream of 512 independent 2D/3D convection-diffusion solves (Q1/Q2, "
                               "32-256 cells per side in 2D, 8-32 in 3D, eps log-uniform in [1e-3,1]), "
                               "FGMRES(30) + MG V(2,2) Jacobi(0.8), to 1e-8, at most 100 iterations",
                   "requests": len(reqs), "dofs_total": total_dofs, "workers": args.workers,
                   "parallelism": f"replicas x{world}; one batch lane (stream) per set-up, "
                                  f"{args.batch_slots} slots",
                   "step": "one pass of the 512 requests; caches warm; solutions copied to host",
                   "timing": "host wall clock around submit..drain (several streams)"},
        "dofs_per_s": round(world * passes * total_dofs / mx["dt"], 1),
        "requests_per_s_all_statuses": round(all_solves, 3),
        "status_counts": {names.get(k, str(k)): v for k, v in mx["status"].items()},
        "error_vs_fp64": {"max": max(errs) if errs else None, "median": float(np.median(errs)) if errs else None,
                          "requests": len(errs),
                          "note": "requests converged in both forms: max |u_mixed - u_fp64| / max |u_fp64|"},
        "fgmres_iterations_median": int(np.median(mx["its"])),
        "latency_ms": {"p50": round(mx["lat"][len(mx["lat"]) // 2], 2),
                       "p99": round(mx["lat"][int(0.99 * (len(mx["lat"]) - 1))], 2)},
        "cold_pass_s": round(mx["cold"], 2),
        "fp64": {"value": round(world * fp["converged"] / fp["dt"], 3), "unit": "solves/s",
                 "dofs_per_s": round(world * passes * total_dofs / fp["dt"], 1),
                 "status_counts": {names.get(k, str(k)): v for k, v in fp["status"].items()}},
        "e2e": {"value": round(solves, 3), "unit": "solves/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": int(8 * total_dofs)},
        "server": mx["stats"], "clocks": mx["clocks"],
    }


def run_serve(args, rank, world, local, pg):
    """the serving loop: Poisson arrivals (70% 3D Q2 convection-diffusion, 30%
    Stokes P2/P1) at each swept rate for `--duration` seconds; latency =
    submit -> solution in host memory, measured by the executor"""
    import numpy as np
    import mymoonmd_gb300 as m
    from mymoonmd_gb300 import workloads as wl
    rates = [float(r) for r in args.rates.split(",")]
    sweep = {}
    for precision in ("fp64", "mixed"):
        srv = m.Server(local, args.workers, stream_db(precision, batch_slots=args.batch_slots), stokes_db(precision),
                       int(150e9))
        # warm every set-up of the mix on the workers
        warm = wl.serving_requests(200.0, 2.0, seed=123)
        for i, rq in enumerate(warm):
            _submit(srv, rq, i, None)
        srv.drain()
        srv.poll(4096)
        per_rate = {}
        for rate in rates:
            reqs = wl.serving_requests(rate, args.duration, seed=1)
            t0 = time.perf_counter()
            for i, rq in enumerate(reqs):
                delay = t0 + rq["t"] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                _submit(srv, rq, i, None)
            srv.drain()
            t_end = time.perf_counter()
            rs = srv.poll(len(reqs) + 16)
            lat = sorted(r["latency_ms"] for r in rs)
            ok = sum(1 for r in rs if r["status"] == 0)
            per_rate[str(int(rate))] = {
                "offered_per_s": rate, "requests": len(reqs), "converged": ok,
                "solves_per_s": round(len(rs) / (t_end - t0), 2), "wall_s": round(t_end - t0, 3),
                "p50_ms": round(lat[len(lat) // 2], 2) if lat else None,
                "p99_ms": round(lat[int(0.99 * (len(lat) - 1))], 2) if lat else None}
        sweep[precision] = per_rate
        srv.close()
    if rank != 0:
        return None
    # the value is the throughput at saturation: the highest rate of converged
    # solves over the sweep, with the latencies measured at that rate
    key = max(sweep["mixed"], key=lambda k: sweep["mixed"][k]["converged"] / (sweep["mixed"][k]["wall_s"] or 1))
    top = sweep["mixed"][key]
    return {
        "metric": METRIC, "value": round(top["converged"] / top["wall_s"], 2), "unit": "solves/s", "n_gpus": world,
        "steps": len(rates), "saturation_rate_per_s": top["offered_per_s"],
        "warmup": 1, "ms_per_step": round(args.duration * 1e3, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 multigrid inside f64 FGMRES (outer residuals f64)",
        "data": "synthetic: Poisson arrivals from numpy default_rng(1) (mymoonmd_gb300/workloads.py)",
        "config": {"workload": "serving: Poisson arrivals, 70% 3D Q2 convection-diffusion (8-32 cells per "
                               "side), 30% Stokes P2/P1 (8-24 cubes per side); the mix is read as 70% "
                               "config-2-type CD and 30% config-3-type Stokes",
                   "rates_per_s": rates, "duration_s": args.duration, "workers": args.workers,
                   "hbm_cap_gb": 150},
        "latency_ms": {"p50": top["p50_ms"], "p99": top["p99_ms"]},
        "sweep": sweep,
    }


def main():
    faulthandler.enable()
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=list(WORKLOADS) + ["stream512", "serve"], default="cd3d_q2_32")
    ap.add_argument("--workers", type=int, default=4, help="executor worker streams (stream512, serve)")
    ap.add_argument("--batch-slots", type=int, default=8,
                    help="requests of one set-up solved together (stream512, serve); 0 = one at a time")
    ap.add_argument("--requests", type=int, default=512, help="stream512: requests per pass")
    ap.add_argument("--rates", default="50,100,200,400", help="serve: offered request rates per second")
    ap.add_argument("--duration", type=float, default=10.0, help="serve: seconds of arrivals per rate")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-large-spmv", action="store_true", help="skip the SpMV on the 4x-L2 matrix")
    ap.add_argument("--smoother", default=None, help="override the workload's multigrid smoother")
    ap.add_argument("--damp", type=float, default=None, help="override the Vanka damping factor")
    args = ap.parse_args()
    if args.workload in ("stream512", "serve"):
        rank, world, local, pg = dist_setup(args.gpus)
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the batched stream and the serving "
                                  "loop have no reference implementation (forms added by this library)"}))
            return 0
        fn = run_stream if args.workload == "stream512" else run_serve
        line = fn(args, rank, world, local, pg)
        if rank == 0 and line is not None:
            print(json.dumps(line), flush=True)
        return 0
    w = dict(WORKLOADS[args.workload])
    if args.smoother:
        w["smoother"] = args.smoother
    if args.damp is not None:
        w["damp"] = args.damp
    WORKLOADS[args.workload] = w
    rank, world, local, pg = dist_setup(args.gpus)
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args, w, rank, world)), flush=True)
        return 0
    if args.warmup < 3:
        args.warmup = 3
    line = run_ours(args, w, rank, world, local, pg)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
