"""The golden errors of the reference's test/cd2d_test.c++ on the GPU path.

cd2d_test solves the SineLaplace example (include/Examples/CD_2D/SineLaplace.h:
u = sin(pi x) sin(pi y), eps = 1, Neumann boundary on x = 1, Dirichlet on the
other sides) on UnitSquare after 2 refinements with Q1 and Q2, by three
solvers, and checks the L2, H1-semi, SD and L_inf errors of
ConvectionDiffusion::output against golden values (:91-98) with tolerance
1e-11 (:42). Here the same runs go through the library: the Neumann side's
numbering and boundary integral, the device assembly, the GPU solvers and the
device error functional (pm_problem_errors).
"""
import numpy as np
import pytest

import mymoonmd_gb300 as m

pytestmark = pytest.mark.gpu

# test/cd2d_test.c++:91-98
GOLDEN = {1: (0.030136750989447, 0.50136473756928, 0.50136473756928, 0.086620472046938),
          2: (0.0019271846609828, 0.050971302154831, 0.050971302154831, 0.0033739148851507)}
SIDE_X1 = 2  # boundary component 1 of UnitSquare (x = 1) is SineLaplace's Neumann side


def solver_db(kind: str) -> m.ParameterDatabase:
    """the three solver set-ups of cd2d_test.c++:218-262 over the reference's
    defaults (Solver.C:59-101, Multigrid.C:497)"""
    db = m.ParameterDatabase.solve_path_database()
    db["residual_tolerance"] = 1.0e-13
    db["residual_reduction"] = 0.0
    db["gmres_restart"] = 20
    db["sor_omega"] = 1.5
    if kind == "direct":
        db["solver_type"] = "direct"
        return db
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = "fgmres"
    db["max_n_iterations"] = 1000
    if kind == "ssor":
        db["preconditioner"] = "ssor"
        return db
    db["preconditioner"] = "multigrid"
    db["multigrid_n_levels"] = 2
    db["multigrid_cycle_type"] = "W"
    db["multigrid_smoother"] = "jacobi"
    db["multigrid_smoother_coarse"] = "direct_solve"
    db["multigrid_correction_damp_factor"] = 1.0
    db["multigrid_n_pre_smooth"] = 2
    db["multigrid_n_post_smooth"] = 2
    db["jacobi_damp"] = 1.0
    return db


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("kind", ["direct", "ssor", "multigrid"])
def test_sine_laplace_golden_errors(ctx, kind, order):
    n_levels = 2 if kind == "multigrid" else 1
    disc = m.Discretization(m.GEO_SQUARE_QUAD, 1, 2, n_levels, m.KIND_CD, order, neumann_sides=SIDE_X1)
    # SineLaplace: eps = 1 / PE_NR = 1, b = 0, c = 0, f = -Laplace u
    prob = m.ConvectionDiffusion(ctx, disc, m.cd_coeffs(1.0, (0.0, 0.0), 0.0, True), solver_db(kind))
    try:
        prob.assemble()
        prob.solve()
        if kind != "direct":
            its, res, init = prob.last_info()
            assert res <= 1e-13, (kind, its, res)
        err = np.array(prob.errors())
        diff = np.abs(err - np.array(GOLDEN[order]))
        print(f"Q{order} {kind}: errors {err}, largest difference to the golden values {diff.max():.2e}")
        assert diff.max() <= 1e-11, (kind, order, err)
    finally:
        prob.close()
        disc.close()


def test_errors_without_neumann_sides_match_the_oracle(ctx):
    """the functional on a 3D Q2 problem with convection (SD term with the SUPG
    delta) against the oracle's restatement"""
    from oracle import cd as ocd
    cf = m.cd_coeffs(0.05, (1.0, 0.5, 0.25), 0.0, True)
    disc = m.Discretization(m.GEO_CUBE_HEXA, 1, 3, 2, m.KIND_CD, 2)
    db = solver_db("multigrid")
    db["multigrid_cycle_type"] = "V"
    db["residual_tolerance"] = 1e-12
    db["jacobi_damp"] = 0.8
    prob = m.ConvectionDiffusion(ctx, disc, cf, db)
    try:
        prob.assemble()
        prob.solve()
        sol = prob.solution()
        got = np.array(prob.errors())
    finally:
        prob.close()
        disc.close()
    ora = ocd.OracleCD(1, 1, 3, 2, 2, 0.05, (1.0, 0.5, 0.25), 0.0, 4)
    want = ora.errors(sol)
    ora.close()
    assert np.allclose(got, want, rtol=1e-12, atol=0), (got, want)
