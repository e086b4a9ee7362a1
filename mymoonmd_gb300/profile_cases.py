"""Small, fixed workloads for kernel profiling (ncu) of the solve path.

    python -m mymoonmd_gb300.profile_cases request [--precision mixed|fp64]
        one warm-up request, then one request (assembly + solve) of the 3D Q2
        32^3 convection-diffusion workload (274,625 DOFs, 4 levels)
    python -m mymoonmd_gb300.profile_cases spmv
        the finest 32^3 Q2 matrix: two FP64 and two FP32 SpMV launches
    python -m mymoonmd_gb300.profile_cases stokes [--precision ...] [--smoother ...] [--coarse ...]
        one warm-up request, then one request of the 3D Stokes P2/P1 workload
        (24^3 cubes x 6 tetrahedra, 368,572 DOFs, 3 levels, V(1,1) Vanka);
        --cubes 12 runs the 12^3 mesh of the same family
    python -m mymoonmd_gb300.profile_cases nse [--precision ...]
        one warm-up request, then one request of the 3D Navier-Stokes workload
        (24^3 cubes x 6 tetrahedra, Reynolds number 10, example -3): assembly
        and the Picard loop to a 1e-10 nonlinear residual
    python -m mymoonmd_gb300.profile_cases tcd [--precision mixed|fp64] [--scheme ...]
        time-dependent convection-diffusion on the 3D Q2 32^3 mesh (4 levels,
        the request's solver): initial assembly, then 6 time steps of 0.01
        (the first is a warm-up), each assembly + time-discrete rhs + system
        matrices + solve + reset, timed with CUDA events

Each case prints what it ran; device memory stays below 2 GB.
"""
from __future__ import annotations

import argparse

import numpy as np

from . import core as m
from .parameter_database import ParameterDatabase


def _db(precision: str) -> ParameterDatabase:
    db = ParameterDatabase.solve_path_database()
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = "fgmres"
    db["preconditioner"] = "multigrid"
    db["residual_tolerance"] = 0.0
    db["residual_reduction"] = 1e-8
    db["max_n_iterations"] = 500
    db["gmres_restart"] = 30
    db["multigrid_n_levels"] = 4
    db["multigrid_smoother"] = "jacobi"
    db["multigrid_smoother_coarse"] = "direct_solve"
    db["jacobi_damp"] = 0.8
    db["multigrid_n_pre_smooth"] = 2
    db["multigrid_n_post_smooth"] = 2
    db["gpu_precision"] = precision
    return db


def problem(ctx, precision="mixed", n_levels=4):
    disc = m.Discretization(m.GEO_CUBE_HEXA, 1, 5, n_levels, m.KIND_CD, 2)
    cf = m.cd_coeffs(1e-2, (1.0, 0.5, 0.25), 0.0, True)
    return disc, m.ConvectionDiffusion(ctx, disc, cf, _db(precision), quad_points=3)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["request", "spmv", "stokes", "nse", "tcd"])
    ap.add_argument("--scheme", default="crank_nicolson", choices=["backward_euler", "crank_nicolson", "bdf_two"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--smoother", default="nodal_vanka")
    ap.add_argument("--coarse", default="nodal_vanka_jacobi")
    ap.add_argument("--cubes", type=int, default=24, choices=[12, 24])
    args = ap.parse_args()
    ctx = m.Context(0)
    if args.case == "tcd":
        db = _db(args.precision)
        db.merge(ParameterDatabase.default_time_database())
        db["time_discretization"] = args.scheme
        db["time_step_length"] = 0.01
        db["time_end"] = 0.06
        disc = m.Discretization(m.GEO_CUBE_HEXA, 1, 5, 4, m.KIND_CD, 2)
        cf = m.cd_coeffs(1e-2, (1.0, 0.5, 0.25), 0.0, True)
        tcd = m.TimeConvectionDiffusion(ctx, disc, cf, db, quad_points=3)
        tcd.assemble_initial_time()
        times, its = [], []
        while tcd.current_time < 0.06 - 1e-10:
            ctx.time_begin()
            tcd.next_time_step()
            tcd.assemble()
            tcd.solve()
            times.append(ctx.time_end())
            its.append(tcd.last_info()[0])
        steady = times[1:]
        print(f"tcd {args.scheme} {args.precision}: {np.mean(steady):.2f} ms per time step "
              f"(min {min(steady):.2f}, {len(steady)} steps after a warm-up), FGMRES iterations {its}")
        tcd.close()
        ctx.close()
        return
    if args.case == "nse":
        db = _db(args.precision)
        db["multigrid_n_levels"] = 3
        db["multigrid_smoother"] = "nodal_vanka"
        db["multigrid_smoother_coarse"] = "nodal_vanka_jacobi"
        db["multigrid_vanka_damp_factor"] = 0.8
        db["multigrid_n_pre_smooth"] = 1
        db["multigrid_n_post_smooth"] = 1
        db.add("example", -3)
        db.add("problem_type", 5)
        db.add("nonlinloop_epsilon", 1e-10)
        db.add("nonlinloop_maxit", 30)
        disc = m.Discretization(m.GEO_CUBE_TETRA, 3, 3, 3, m.KIND_STOKES, 12)
        prob = m.StokesProblem(ctx, disc, 0.1, db)
        for _ in range(2):
            prob.reset_solution()
            prob.assemble()
            hist = prob.solve_nonlinear()
        print("nse", args.precision, "nonlinear steps", len(hist) - 1, "residual", hist[-1][2])
        prob.close()
        ctx.close()
        return
    if args.case == "stokes":
        db = _db(args.precision)
        db["multigrid_n_levels"] = 3
        db["multigrid_smoother"] = args.smoother
        db["multigrid_smoother_coarse"] = args.coarse
        db["multigrid_vanka_damp_factor"] = 0.8
        db["multigrid_n_pre_smooth"] = 1
        db["multigrid_n_post_smooth"] = 1
        disc = m.Discretization(m.GEO_CUBE_TETRA, 3, 3 if args.cubes == 24 else 2, 3, m.KIND_STOKES, 12)
        prob = m.StokesProblem(ctx, disc, 1.0, db)
        for _ in range(2):
            prob.reset_solution()
            prob.assemble()
            prob.solve()
        print("stokes", args.precision, args.smoother, args.coarse, "iterations", prob.last_info()[0])
        prob.close()
        ctx.close()
        return
    disc, prob = problem(ctx, args.precision)
    if args.case == "request":
        for _ in range(2):
            prob.reset_solution()
            prob.assemble()
            prob.solve()
        print("request", args.precision, "iterations", prob.last_info()[0])
    else:
        prob.assemble()
        A = prob.matrix(-1)
        A.make_fp32()
        A.make_sliced64()
        n = A.n_rows
        x = m.DeviceVector.from_numpy(ctx, np.random.default_rng(0).standard_normal(n))
        y = m.DeviceVector(ctx, n)
        x32 = m.DeviceVector.from_numpy(ctx, np.random.default_rng(0).standard_normal(n).astype(np.float32))
        y32 = m.DeviceVector(ctx, n, np.float32)
        ms, b = A.bench_apply(x, y, 2)
        ms32, b32 = A.bench_apply(x32, y32, 2, fp32=True)
        print(f"spmv fp64 {b / ms / 1e6:.0f} GB/s, fp32 {b32 / ms32 / 1e6:.0f} GB/s (2 launches each)")
    prob.close()
    ctx.close()


if __name__ == "__main__":
    main()
