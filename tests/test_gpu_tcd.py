"""Time-dependent convection-diffusion on the GPU (pm_tcd: TimeConvectionDiffusion
with backward Euler, Crank-Nicolson, BDF2) against the known answers of
test/tcd3d_solvers_test.c++ and against the oracle's time stepping
(oracle/tcd.py) step by step.

Tolerances: the known-answer examples stay exact within the reference's 1e-12
(multigrid) and 1e-13 (direct) at every step; on a problem without an exact
discrete solution the GPU and oracle iterates agree within 1e-9 per step
(FGMRES to a 1e-10 reduction in both), iteration counts within one."""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from oracle import tcd as otcd

from test_oracle_tcd import EXAMPLES, MG

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def tcd_db(solver, scheme, tau=0.1, t_end=1.0, precision="fp64", smoother="sor", cycle="W", pre=3, post=3,
           damp=0.8, tol=1e-15, reduction=0.0, n_levels=2):
    db = m.ParameterDatabase.solve_path_database()
    db.merge(m.ParameterDatabase.default_time_database())
    db["time_discretization"] = scheme
    db["time_step_length"] = tau
    db["time_end"] = t_end
    if solver == "direct":
        db["solver_type"] = "direct"
        return db
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = "fgmres"
    db["preconditioner"] = "multigrid"
    db["multigrid_n_levels"] = n_levels
    db["max_n_iterations"] = 100
    db["residual_tolerance"] = tol
    db["residual_reduction"] = reduction
    db["multigrid_cycle_type"] = cycle
    db["multigrid_smoother"] = smoother
    db["multigrid_smoother_coarse"] = "direct_solve"
    db["multigrid_correction_damp_factor"] = damp if smoother == "sor" else 1.0
    db["jacobi_damp"] = damp
    db["multigrid_n_pre_smooth"] = pre
    db["multigrid_n_post_smooth"] = post
    db["gpu_precision"] = precision
    return db


def gpu_example(ctx, example, db):
    elem, eps, b, c, p0, pt = EXAMPLES[example]
    disc = m.Discretization(m.GEO_CUBE_HEXA, 1, 2, 2, m.KIND_CD, elem)
    cf = m.cd_coeffs(eps, b, c, True, poly=p0)
    return m.TimeConvectionDiffusion(ctx, disc, cf, db, quad_points=3, poly_time=pt)


CASES = [("linear_space_time", "backward_euler"), ("linear_space_time", "crank_nicolson"),
         ("linear_space_time", "bdf_two"), ("quadratic_space_time", "crank_nicolson")]


@pytest.mark.parametrize("example,scheme", CASES)
@pytest.mark.parametrize("solver,tol", [("multigrid", 1e-12), ("direct", 1e-13)])
def test_tcd3d_solvers_examples_stay_exact(ctx, example, scheme, solver, tol):
    tcd = gpu_example(ctx, example, tcd_db(solver, scheme))
    elem, eps, b, c, p0, pt = EXAMPLES[example]
    o = otcd.OracleTCD(1, 1, 2, 2, elem, eps, b, c, 3, poly=p0, poly_time=pt, scheme=scheme, tau=0.1)
    nodes = o.cd.finest.node_coords
    tcd.assemble_initial_time()
    errs = []
    while tcd.current_time < tcd.end_time - 1e-10:
        tcd.next_time_step()
        tcd.assemble()
        tcd.solve()
        exact = np.array([o.exact(tcd.current_time, x) for x in nodes])
        errs.append(np.abs(tcd.solution() - exact).max())
    assert tcd.current_step == 10
    assert max(errs) <= tol, errs
    tcd.close()


def test_mixed_precision_time_stepping_stays_exact(ctx):
    """FP32 multigrid inside FP64 FGMRES on the quadratic example with
    Crank-Nicolson: FGMRES works on the FP64 residual, so the steps stay
    exact to the same 1e-12"""
    tcd = gpu_example(ctx, "quadratic_space_time", tcd_db("multigrid", "crank_nicolson", precision="mixed"))
    elem, eps, b, c, p0, pt = EXAMPLES["quadratic_space_time"]
    o = otcd.OracleTCD(1, 1, 2, 2, elem, eps, b, c, 3, poly=p0, poly_time=pt, scheme="crank_nicolson", tau=0.1)
    tcd.assemble_initial_time()
    while tcd.current_time < tcd.end_time - 1e-10:
        tcd.next_time_step()
        tcd.assemble()
        tcd.solve()
        exact = np.array([o.exact(tcd.current_time, x) for x in o.cd.finest.node_coords])
        assert np.abs(tcd.solution() - exact).max() <= 1e-12
    tcd.close()


@pytest.mark.parametrize("scheme", ["backward_euler", "crank_nicolson", "bdf_two"])
def test_time_steps_match_oracle(ctx, scheme):
    """the sine right-hand side (time independent, zero initial and boundary
    values) on 3D Q2 8^3 with three levels: four steps of size 0.02, FGMRES +
    V(2,2) damped Jacobi to a 1e-10 reduction"""
    db = tcd_db("multigrid", scheme, tau=0.02, t_end=0.08, smoother="jacobi", cycle="V", pre=2, post=2,
                damp=0.8, tol=0.0, reduction=1e-10, n_levels=3)
    disc = m.Discretization(m.GEO_CUBE_HEXA, 1, 3, 3, m.KIND_CD, 2)
    cf = m.cd_coeffs(0.1, (1.0, 0.5, 0.25), 0.0, True)
    tcd = m.TimeConvectionDiffusion(ctx, disc, cf, db, quad_points=3)
    o = otcd.OracleTCD(1, 1, 3, 3, 2, 0.1, (1.0, 0.5, 0.25), 0.0, 3, scheme=scheme, tau=0.02, t_end=0.08)
    tcd.assemble_initial_time()
    o.assemble_initial_time()
    mg = dict(n_pre=2, n_post=2, jacobi_damp=0.8, correction_damp=1.0, cycle="V")
    for _ in range(4):
        tcd.next_time_step()
        tcd.assemble()
        tcd.solve()
        o.next_step()
        o.assemble()
        o.solve("multigrid", mg, tol=0.0, reduction=1e-10, max_it=100, restart=20)
        it = tcd.last_info()[0]
        assert abs(it - o.last_it) <= 1, (it, o.last_it)
        assert rel(tcd.solution(), o.sol) <= 1e-9
    assert abs(tcd.current_time - 0.08) < 1e-12
    # the matrices are back to the stiffness matrices after the solve
    for l in range(3):
        assert rel(tcd.matrix(l).values(), o.cd.vals[l]) <= 1e-12
    tcd.close()
