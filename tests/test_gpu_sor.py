"""SOR and SSOR on the GPU (multigrid_smoother sor / ssor, preconditioner
sor / ssor, iterative_solver_type sor / ssor) against the oracle's sequential
sweep over the same multicolour row order (TMatrix::sor_sweep,
src/Matrix/Matrix.C:943-1031).

Tolerances: a sweep sums each row in a different order than the oracle's
(lanes of 4 or 8 entries), so single applications agree to 1e-11 relative and
converged solutions to 1e-10 with FGMRES iteration counts within one."""
import numpy as np
import pytest

import mymoonmd_gb300 as m

from test_gpu_parity import make_pair, mg_db, rel
from test_oracle_golden import csr_from_dense, iterative_solver_system

pytestmark = pytest.mark.gpu


def sor_mg_db(n_levels, smoother, omega, **kw):
    db = mg_db(n_levels, **kw)
    db["multigrid_smoother"] = smoother
    db["sor_omega"] = omega
    return db


@pytest.mark.parametrize("omega", [1.0, 1.5])
@pytest.mark.parametrize("smoother", ["sor", "ssor"])
@pytest.mark.parametrize("case", ["q1_2d", "q2_3d"])
def test_sor_multigrid_cycle_matches_oracle(ctx, case, smoother, omega):
    """one V(2,2) cycle with (S)SOR sweeps in colour order on every level but
    the coarsest (direct solve)"""
    disc, prob, ora = make_pair(ctx, case, sor_mg_db(3, smoother, omega))
    prob.solve()  # builds the hierarchy and the colourings
    ora.build_mg(2, 2, 0.8, 1.0, "V", smoother=smoother, sor_omega=omega)
    z = np.random.default_rng(21).standard_normal(ora.finest.n_dofs)
    r = m.DeviceVector(ctx, z.size)
    prob.solver().apply_preconditioner(m.DeviceVector.from_numpy(ctx, z), r)
    assert rel(r.numpy(), ora.mg_apply(z)) <= 1e-11


@pytest.mark.parametrize("cycle", ["W", "F"])
def test_sor_smoother_coarse_loop_and_cycles_match_oracle(ctx, cycle):
    """SOR also on the coarsest level (at most 10 sweeps, stop at 0.1, checked
    on the device) inside W and F cycles"""
    db = sor_mg_db(3, "sor", 1.2, cycle=cycle, pre=1, post=1)
    db["multigrid_smoother_coarse"] = "sor"
    db["multigrid_coarse_max_n_iterations"] = 10
    db["multigrid_coarse_residual"] = 0.1
    disc, prob, ora = make_pair(ctx, "q2_2d", db)
    prob.solve()
    ora.build_mg(1, 1, 0.8, 1.0, cycle, coarse_direct=False, coarse_max_it=10, coarse_residual=0.1,
                 smoother="sor", coarse_smoother="sor", sor_omega=1.2)
    z = np.random.default_rng(22).standard_normal(ora.finest.n_dofs)
    r = m.DeviceVector(ctx, z.size)
    prob.solver().apply_preconditioner(m.DeviceVector.from_numpy(ctx, z), r)
    assert rel(r.numpy(), ora.mg_apply(z)) <= 1e-11


@pytest.mark.parametrize("smoother", ["sor", "ssor"])
def test_fgmres_with_sor_multigrid_matches_oracle(ctx, smoother):
    db = sor_mg_db(3, smoother, 1.5, restart=20, reduction=1e-10)
    disc, prob, ora = make_pair(ctx, "q2_3d", db)
    prob.solve()
    it, res, init = prob.last_info()
    ora.build_mg(2, 2, 0.8, 1.0, "V", smoother=smoother, sor_omega=1.5)
    sol, oit, ores, hist, st = ora.solve("fgmres", 0.0, 1e-10, 200, 0, 20)
    assert st == 0 and abs(it - oit) <= 1, (it, oit)
    assert res <= 1e-10 * init
    assert rel(prob.solution(), sol) <= 1e-10


def test_mixed_precision_with_sor_smoother_reaches_fp64_target(ctx):
    """FP32 SOR sweeps inside the FP32 multigrid, FP64 FGMRES outside"""
    db = sor_mg_db(3, "sor", 1.5, restart=30, reduction=1e-8, precision="mixed")
    disc, prob, ora = make_pair(ctx, "q2_3d", db)
    prob.solve()
    it, res, init = prob.last_info()
    assert res <= 1e-8 * init and it < 100
    ora.build_mg(2, 2, 0.8, 1.0, "V", smoother="sor", sor_omega=1.5)
    sol, *_ = ora.solve("fgmres", 0.0, 1e-10, 200, 0, 30)
    assert rel(prob.solution(), sol) <= 1e-7


def krylov_db(method, prec, omega=1.5, reduction=1e-10, max_it=500, restart=20):
    db = m.ParameterDatabase.solve_path_database()
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = method
    db["preconditioner"] = prec
    db["sor_omega"] = omega
    db["residual_tolerance"] = 0.0
    db["residual_reduction"] = reduction
    db["max_n_iterations"] = max_it
    db["gmres_restart"] = restart
    db["multigrid_n_levels"] = 3
    return db


@pytest.mark.parametrize("prec", ["sor", "ssor"])
@pytest.mark.parametrize("method", ["fgmres", "bi_cgstab"])
def test_sor_preconditioned_krylov_matches_oracle(ctx, method, prec):
    """Iteration_sor::apply as the preconditioner (r = 0, one sweep with rhs z)"""
    disc, prob, ora = make_pair(ctx, "q1_2d", krylov_db(method, prec))
    prob.solve()
    it, res, init = prob.last_info()
    sol, oit, ores, hist, st = ora.solve(method, 0.0, 1e-10, 500, 0, 20, sor=prec, sor_omega=1.5)
    assert st == 0 and oit < 500
    assert abs(it - oit) <= 1, (it, oit)
    assert res <= 1e-10 * init
    assert rel(prob.solution(), sol) <= 1e-9


@pytest.mark.parametrize("method", ["sor", "ssor"])
def test_sor_iteration_matches_oracle(ctx, method):
    """iterative_solver_type sor / ssor (Iteration_sor::iterate): 40 sweeps,
    residual history and iterate"""
    disc, prob, ora = make_pair(ctx, "q1_2d", krylov_db(method, "no_preconditioner", 1.5, 1e-14, 40))
    prob.solve()
    it, res, init = prob.last_info()
    hist = prob.solver().residual_history()
    sol, oit, ores, ohist = ora.sor_iterate(method, 0.0, 1e-14, 40, 1.5)
    assert it == oit == 40
    assert rel(hist, ohist) <= 1e-10
    assert rel(prob.solution(), sol) <= 1e-10


@pytest.mark.parametrize("method", ["fgmres", "right_gmres", "cg", "bi_cgstab", "jacobi", "sor", "ssor",
                                    "richardson", "cgs", "left_gmres"])
def test_reference_test_system_with_ssor_preconditioner(ctx, method):
    """test/iterative_solver_test.c++:104-160: the 7x7 block system with
    preconditioner ssor and sor_omega 1.25; error <= 100 * residual_tolerance"""
    M = iterative_solver_system()
    rp, ci, v = csr_from_dense(M)
    mat = m.FEMatrix.from_csr(ctx, rp, ci, v)
    exact = np.arange(7.0)
    rhs = M @ exact
    db = m.ParameterDatabase.solve_path_database()
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = method
    db["residual_tolerance"] = 1e-11
    db["max_n_iterations"] = 1000
    db["preconditioner"] = "ssor"
    db["sor_omega"] = 1.25
    s = m.Solver(ctx, db)
    s.update_matrix(mat)
    sol = np.zeros(7)
    s.solve(rhs, sol)
    assert np.linalg.norm(sol - exact) <= 100 * 1e-11


def test_sor_on_a_zero_diagonal_is_refused(ctx):
    """TMatrix::sor_sweep throws on a zero diagonal entry (Matrix.C:956-961)"""
    M = iterative_solver_system()
    M[2, 2] = 0.0
    M[2, 0] = 1.0
    rp, ci, v = csr_from_dense(M)
    mat = m.FEMatrix.from_csr(ctx, rp, ci, v)
    db = krylov_db("fgmres", "sor")
    s = m.Solver(ctx, db)
    with pytest.raises(Exception, match="zero on the diagonal"):
        s.update_matrix(mat)


@pytest.mark.parametrize("prec", ["jacobi", "ssor"])
@pytest.mark.parametrize("method", ["cgs", "left_gmres"])
def test_cgs_and_left_gmres_solutions_match_oracle(ctx, method, prec):
    """iterative_solver_type cgs (Iteration_cgs::iterate) and left_gmres
    (Iteration_gmres::left_gmres, preconditioned residual) on the 2D Q1 case
    to a 1e-10 reduction: the solution agrees with the oracle's FGMRES
    solution to a 1e-12 reduction within 1e-8"""
    disc, prob, ora = make_pair(ctx, "q1_2d", krylov_db(method, prec, 1.2, 1e-10, 500))
    prob.solve()
    it, res, init = prob.last_info()
    assert res <= 1e-10 * init and it < 500
    sol, oit, ores, hist, st = ora.solve("fgmres", 0.0, 1e-12, 2000, 0, 50, use_mg=False)
    assert rel(prob.solution(), sol) <= 1e-8
