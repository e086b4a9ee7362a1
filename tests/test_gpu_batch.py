"""Batched solves (pm_problem_solve_batched): problems of one set-up solved
together, every kernel of an Arnoldi step and of the V-cycle launched once for
all slots.

  * each problem's solution and iteration count are bit for bit those of its
    lone solve (pm_problem_solve), in the FP64 and in the mixed form, with
    more problems than slots (problems join as slots free up at restart-cycle
    boundaries);
  * a problem's result is the same alone (a batch of one) and in a mix of
    problems with other coefficients;
  * the batched solutions match the oracle within 1e-10.
"""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from oracle import cd as ocd

pytestmark = pytest.mark.gpu

COEFFS = [(0.1, (1.0, 0.5, 0.25)), (0.02, (0.3, -1.0, 0.5)), (1.0, (0.0, 0.0, 0.0)), (0.05, (-0.7, 0.2, 0.9)),
          (0.3, (0.5, 0.5, -0.5)), (0.01, (0.0, 1.0, 0.0)), (0.2, (1.0, 0.0, 0.0))]


def db(precision, restart=10):
    d = m.ParameterDatabase.solve_path_database()
    d["solver_type"] = "iterative"
    d["iterative_solver_type"] = "fgmres"
    d["preconditioner"] = "multigrid"
    d["residual_tolerance"] = 0.0
    d["residual_reduction"] = 1e-10
    d["max_n_iterations"] = 200
    d["gmres_restart"] = restart
    d["multigrid_n_levels"] = 3
    d["multigrid_smoother"] = "jacobi"
    d["multigrid_smoother_coarse"] = "direct_solve"
    d["jacobi_damp"] = 0.8
    d["multigrid_n_pre_smooth"] = 2
    d["multigrid_n_post_smooth"] = 2
    d["gpu_precision"] = precision
    d.add("gpu_gram_schmidt", "cgs2", ("mgs", "cgs2", "cgs2_cond"))
    d["gpu_mixed_fallback"] = 0
    return d


def problems(ctx, disc, precision, coeffs):
    out = []
    for eps, b in coeffs:
        p = m.ConvectionDiffusion(ctx, disc, m.cd_coeffs(eps, b, 0.0, True), db(precision), quad_points=3)
        p.assemble()
        out.append(p)
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_solves_equal_lone_solves_bit_for_bit(ctx, precision):
    disc = m.Discretization(m.GEO_CUBE_HEXA, 1, 3, 3, m.KIND_CD, 2)  # 8^3 Q2, 3 levels
    try:
        lone = []
        for p in problems(ctx, disc, precision, COEFFS):
            p.solve()
            lone.append((p.solution(), p.last_info()))
            p.close()
        batch = problems(ctx, disc, precision, COEFFS)
        status = m.solve_batched(batch, slots=3)  # 7 problems through 3 slots
        # convection-dominated ones may stop at the iteration cap, alone as in the batch
        expect = [0 if info[1] <= 1e-10 * info[2] else 5 for _, info in lone]
        assert status == expect
        assert expect.count(0) >= 4
        for (sol, info), p in zip(lone, batch):
            got = p.solution()
            assert p.last_info() == info
            assert np.array_equal(got, sol)
            p.close()
    finally:
        disc.close()


def test_result_alone_and_in_the_mix(ctx):
    disc = m.Discretization(m.GEO_SQUARE_QUAD, 1, 5, 3, m.KIND_CD, 1)  # 2D Q1 32^2
    try:
        coeffs2d = [(eps, b[:2]) for eps, b in COEFFS]
        alone = problems(ctx, disc, "mixed", coeffs2d[3:4])
        assert m.solve_batched(alone, slots=1) == [0]
        ref = alone[0].solution()
        mix = problems(ctx, disc, "mixed", coeffs2d)
        status = m.solve_batched(mix, slots=8)
        assert status[3] == 0
        assert np.array_equal(mix[3].solution(), ref)
        # and against the oracle's FP64 solve of the same problem
        eps, b = coeffs2d[3]
        ora = ocd.OracleCD(m.GEO_SQUARE_QUAD, 1, 5, 3, 1, eps, b, 0.0, 3)
        ora.assemble()
        ora.build_mg(2, 2, 0.8, 1.0, "V")
        sol, its, res, hist, st = ora.solve("fgmres", 0.0, 1e-10, 200, 0, 10)
        assert st == 0
        assert float(np.abs(ref - sol).max() / np.abs(sol).max()) <= 1e-8
        for p in alone + mix:
            p.close()
    finally:
        disc.close()


def test_batched_fp64_solutions_match_the_oracle(ctx):
    disc = m.Discretization(m.GEO_CUBE_HEXA, 1, 3, 3, m.KIND_CD, 1)  # 8^3 Q1
    try:
        picked = [COEFFS[k] for k in (0, 2, 3, 4)]
        batch = problems(ctx, disc, "fp64", picked)
        assert m.solve_batched(batch, slots=4) == [0] * 4
        for (eps, b), p in zip(picked, batch):
            ora = ocd.OracleCD(m.GEO_CUBE_HEXA, 1, 3, 3, 1, eps, b, 0.0, 3)
            ora.assemble()
            ora.build_mg(2, 2, 0.8, 1.0, "V")
            sol, its, res, hist, st = ora.solve("fgmres", 0.0, 1e-10, 200, 0, 10)
            assert st == 0 and abs(its - p.last_info()[0]) <= 1
            assert float(np.abs(p.solution() - sol).max() / np.abs(sol).max()) <= 1e-10
            p.close()
    finally:
        disc.close()
