"""The known-answer examples of test/cd3d_solvers_test.c++ on the GPU:
examples -1, -2, -3 (src/Examples/Example_CD3D.C:164-193; exact solutions 1,
1+2x+3y+4z, x^2+yz in Q1 / Q1 / Q2, Dirichlet values from the exact solution)
on the hexahedral unit cube and, with P1 / P1 / P2, on the tetrahedral one
(Default_UnitCube_Tetra), two refinements. The reference requires zero
error within 1e-12 for FGMRES + multigrid (W-cycle, 2 levels, SOR 3+3,
correction damping 0.8, coarse direct, residual_tolerance 1e-15) and within
1e-13 for the direct solver (:113-149, :209-231). The error is taken at the
nodes (an exact discrete solution has zero nodal, L2 and H1 error alike).

Also the assembly of these examples against the oracle (entries and
right-hand side within 1e-13, Dirichlet rows included)."""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from oracle import cd as ocd

from test_oracle_examples import EXAMPLES

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def solver_db(name, precision="fp64"):
    db = m.ParameterDatabase.solve_path_database()
    if name == "direct":
        db["solver_type"] = "direct"
        return db
    if name == "jacobi":
        # set_solver_globals("jacobi"), test/cd3d_solvers_test.c++:75-84
        db["solver_type"] = "iterative"
        db["iterative_solver_type"] = "richardson"
        db["preconditioner"] = "jacobi"
        db["residual_tolerance"] = 1e-10
        db["residual_reduction"] = 0.0
        db["max_n_iterations"] = 1000
        db["min_n_iterations"] = 5
        return db
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = "fgmres"
    db["preconditioner"] = "multigrid"
    db["multigrid_n_levels"] = 2
    db["max_n_iterations"] = 100
    db["residual_tolerance"] = 1e-15
    db["residual_reduction"] = 0.0
    db["multigrid_cycle_type"] = "W"
    db["multigrid_smoother"] = "sor"
    db["multigrid_smoother_coarse"] = "direct_solve"
    db["multigrid_correction_damp_factor"] = 0.8
    db["multigrid_n_pre_smooth"] = 3
    db["multigrid_n_post_smooth"] = 3
    db["gpu_precision"] = precision
    return db


def gpu_example(ctx, example, db, tetra=False):
    """hexahedra (Q1 / Q2, Gauss3) or the tetrahedral unit cube (P1 / P2 on the
    reference's default rules: the library's default quadrature)"""
    elem, eps, b, c, poly = EXAMPLES[example]
    geo, el, qn = (m.GEO_CUBE_TETRA, 10 + elem, 11 if elem == 1 else 15) if tetra else (m.GEO_CUBE_HEXA, elem, 3)
    disc = m.Discretization(geo, 1, 2, 2, m.KIND_CD, el)
    cf = m.cd_coeffs(eps, b, c, True, poly=poly)
    prob = m.ConvectionDiffusion(ctx, disc, cf, db, quad_points=0 if tetra else 3)
    prob.assemble()
    ora = ocd.OracleCD(geo, 1, 2, 2, el, eps=eps, b=b, c=c, quad_points=qn, poly=poly)
    ora.assemble()
    return disc, cf, prob, ora


@pytest.mark.parametrize("tetra", [False, True])
@pytest.mark.parametrize("example", [-1, -2, -3])
def test_polynomial_example_assembly_matches_oracle(ctx, example, tetra):
    disc, cf, prob, ora = gpu_example(ctx, example, solver_db("direct"), tetra)
    for l in range(2):
        assert rel(prob.matrix(l).values(), ora.vals[l]) <= 1e-13
    assert rel(prob.rhs(), ora.rhs[-1]) <= 1e-13
    lv = ora.finest
    assert np.abs(prob.rhs()[lv.n_active:]).max() > 0.5  # the Dirichlet values are in place
    prob.close()


@pytest.mark.parametrize("tetra", [False, True])
@pytest.mark.parametrize("solver,tol", [("multigrid", 1e-12), ("direct", 1e-13), ("jacobi", 1e-8)])
@pytest.mark.parametrize("example", [-1, -2, -3])
def test_cd3d_solvers_polynomial_examples_solved_exactly(ctx, example, solver, tol, tetra):
    """both halves of the test: hexahedra (Q1, Q1, Q2) and tetrahedra (P1, P1,
    P2 on Default_UnitCube_Tetra)"""
    disc, cf, prob, ora = gpu_example(ctx, example, solver_db(solver), tetra)
    prob.solve()
    exact = np.array([ora.exact(x) for x in ora.finest.node_coords])
    assert np.abs(prob.solution() - exact).max() <= tol
    prob.close()


def test_polynomial_example_in_mixed_precision(ctx):
    """the mixed form (FP32 multigrid inside FP64 FGMRES) reaches the exact
    solution too: FGMRES works on the FP64 residual"""
    disc, cf, prob, ora = gpu_example(ctx, -3, solver_db("multigrid", "mixed"))
    prob.solve()
    exact = np.array([ora.exact(x) for x in ora.finest.node_coords])
    assert np.abs(prob.solution() - exact).max() <= 1e-12
    prob.close()

