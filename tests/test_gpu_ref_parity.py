"""GPU parity against the reference itself, at the workloads' full sizes.

The fixtures (tests/golden/ref_*.npz) hold what ParMooN's own classes compute
(compiled from the reference sources; tests/golden/make_ref_fixtures.py): per
level the assembled entries and right-hand side, and the FGMRES + multigrid
solve (iterations, initial residual, solution). Here the same problems are
assembled and solved on the GPU through the C ABI:

  assembled entries, right-hand sides   within 1e-13 of the largest entry
  FP64 solve                            iterations within one of the reference's,
                                        initial residual within 1e-12 relative,
                                        solution within 1e-10 (max norm, relative)
  mixed form (FP32 multigrid inside     reaches the FP64 residual reduction; its
  FP64 FGMRES)                          error against the reference's solution is
                                        stated and held to 1e-7
Cases include the 2D Q1 128^2 workload (16,641 DOFs) and the 3D Q2 32^3
workload (274,625 DOFs, 15.8 M nonzeros, 82 iterations in the reference), and
the reference's SineLaplace example with its Neumann side (sine_*: Neumann
boundary integral in the right-hand side, and the L2 / H1-semi / SD / L_inf
errors of ConvectionDiffusion::output within 1e-10 / h of the reference's).
"""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from ref_fixtures import RefCase, StokesRefCase, names, stokes_names

pytestmark = pytest.mark.gpu


def db_for(rc: RefCase, precision: str) -> m.ParameterDatabase:
    db = m.ParameterDatabase.solve_path_database()
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = "fgmres"
    db["preconditioner"] = "multigrid"
    db["residual_tolerance"] = 0.0
    db["residual_reduction"] = rc.reduction
    db["max_n_iterations"] = 1000
    db["gmres_restart"] = rc.restart
    db["multigrid_n_levels"] = rc.n_levels
    db["multigrid_cycle_type"] = "V"
    db["multigrid_smoother"] = "jacobi"
    db["multigrid_smoother_coarse"] = "direct_solve"
    db["jacobi_damp"] = 0.8
    db["multigrid_n_pre_smooth"] = 2
    db["multigrid_n_post_smooth"] = 2
    db["multigrid_correction_damp_factor"] = 1.0
    db["gpu_precision"] = precision
    return db


def make(ctx, rc: RefCase, precision: str):
    disc = m.Discretization(rc.geometry, 1, rc.n_refine, rc.n_levels, m.KIND_CD, rc.elem,
                            neumann_sides=rc.neumann_sides)
    cf = m.cd_coeffs(rc.eps, rc.b[:rc.dim], 0.0, True)
    return disc, m.ConvectionDiffusion(ctx, disc, cf, db_for(rc, precision), quad_points=rc.quad_points)


@pytest.mark.parametrize("name", names())
def test_gpu_assembly_and_fp64_solve_match_the_reference(ctx, name):
    rc = RefCase(name)
    disc, prob = make(ctx, rc, "fp64")
    try:
        prob.assemble()
        for l in range(rc.n_levels):
            assert rc.compare("vals", prob.matrix(l).values(), l) <= 1e-13, (name, l)
        assert rc.compare("rhs", prob.rhs(), rc.n_levels - 1) <= 1e-13
        prob.solve()
        its, res, init = prob.last_info()
        assert abs(its - rc.iterations) <= 1, (name, its, rc.iterations)
        assert abs(init - rc.initial_residual) <= 1e-12 * rc.initial_residual, (init, rc.initial_residual)
        assert rc.compare("solution", prob.solution()) <= 1e-10
        if rc.errors is not None:
            # ConvectionDiffusion::output's errors of the SineLaplace cases: the
            # solutions agree to 1e-10, so the errors agree to that over h
            tol = 1e-10 * float(rc.z["solution_max"]) * 2 ** rc.n_refine
            assert np.abs(np.array(prob.errors()) - rc.errors).max() <= tol, (prob.errors(), rc.errors)
    finally:
        prob.close()
        disc.close()


@pytest.mark.parametrize("name", ["cd2d_q1_128", "cd3d_q2_32", "cd3d_q2_8"])
def test_gpu_mixed_form_error_against_the_reference(ctx, name):
    rc = RefCase(name)
    disc, prob = make(ctx, rc, "mixed")
    try:
        prob.assemble()
        prob.solve()
        its, res, init = prob.last_info()
        assert res <= rc.reduction * init
        err = rc.compare("solution", prob.solution())
        print(f"{name}: mixed form {its} iterations (reference FP64 {rc.iterations}), "
              f"error against the reference's solution {err:.2e}")
        assert err <= 1e-7
    finally:
        prob.close()
        disc.close()


@pytest.mark.parametrize("name", ["cd2d_q1_128", "cd3d_q2_32"])
def test_gpu_mixed_form_with_the_fp64_coarse_solve(ctx, name):
    """gpu_mixed_coarse = fp64: the mixed cycle's coarse direct solve uses the
    FP64 inverse (FP32 vectors, FP64 products and sums). It takes the
    iterations of the FP32-inverse cycle (within one) and stays within the
    mixed form's 1e-7 of the reference's solution."""
    rc = RefCase(name)
    its = {}
    for coarse in ("fp32", "fp64"):
        disc = m.Discretization(rc.geometry, 1, rc.n_refine, rc.n_levels, m.KIND_CD, rc.elem)
        db = db_for(rc, "mixed")
        db["gpu_mixed_coarse"] = coarse
        prob = m.ConvectionDiffusion(ctx, disc, m.cd_coeffs(rc.eps, rc.b[:rc.dim], 0.0, True), db,
                                     quad_points=rc.quad_points)
        try:
            prob.assemble()
            prob.solve()
            it, res, init = prob.last_info()
            assert res <= rc.reduction * init
            assert rc.compare("solution", prob.solution()) <= 1e-7
            its[coarse] = it
        finally:
            prob.close()
            disc.close()
    assert abs(its["fp64"] - its["fp32"]) <= 1, its


def projected(rp, ci, vals, p0):
    """the system matrix with its first pressure row replaced by the unit row
    (get_combined_submatrix's pressure projection)"""
    lens = np.diff(rp).astype(np.int64)
    keep = np.ones(ci.size, dtype=bool)
    keep[rp[p0]:rp[p0 + 1]] = False
    lens[p0] = 1
    rp2 = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    ci2 = np.insert(ci[keep], rp[p0], p0)
    v2 = np.insert(vals[keep], rp[p0], 1.0)
    return rp2, ci2, v2


@pytest.mark.parametrize("name", stokes_names())
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_stokes_assembly_and_solve_match_the_reference(ctx, name, precision):
    """the reference's NavierStokes<3> as a Stokes problem (P2/P1 on
    Default_UnitCube_Tetra, u = (y^2, xz, -y^2), p = x + y + z - 3/2): every
    level's projected matrix within 1e-13 of the reference's combined matrix,
    the right-hand side within 1e-13, and FGMRES + nodal Vanka multigrid
    against the reference's direct solution (velocity 1e-10, mean-free
    pressure 1e-9)"""
    from test_gpu_stokes_example import example_db
    rc = StokesRefCase(name)
    disc = m.Discretization(m.GEO_CUBE_TETRA, 1, rc.n_refine, rc.n_levels, m.KIND_STOKES, 12)
    db = example_db(precision)
    db["multigrid_n_levels"] = rc.n_levels
    prob = m.StokesProblem(ctx, disc, 1.0, db)
    try:
        prob.assemble()
        for l in range(rc.n_levels):
            rp, ci = disc.structure(l)
            nu = disc.level_info(l, 0)["n_dofs"]
            rp2, ci2, v2 = projected(rp, ci, prob.matrix(l).values(), 3 * nu)
            assert rc.compare_matrix(l, rp2, ci2, v2) <= 1e-13, (name, l)
        fin = rc.level(rc.n_levels - 1)
        assert np.abs(prob.rhs() - fin["rhs"]).max() <= 1e-13 * float(fin["rhs_max"])
        if rc.has("solution"):
            prob.solve()
            x, ref = prob.solution(), rc.z["solution"]
            nu3 = 3 * fin["nu"]
            assert np.abs(x[:nu3] - ref[:nu3]).max() <= 1e-10 * np.abs(ref[:nu3]).max()
            p, pr = x[nu3:], ref[nu3:]
            assert np.abs((p - p.mean()) - (pr - pr.mean())).max() <= 1e-9
    finally:
        prob.close()
        disc.close()
