"""Navier-Stokes P2/P1 (problem_type 5, convective form, the reference's example
-3) through the GPU library against the compiled reference's fixtures and the
oracle (oracle/nse.py):

  * one assemble_nonlinear_term from a fixed finest velocity: every level's
    projected matrix within 1e-13 of the reference's (the convective or the
    skew-symmetric term and the restriction of the velocity to the coarser
    levels);
  * the nonlinear loop of test/nse3d_solvers_test.c++ with FGMRES + nodal
    Vanka multigrid in FP64 and in the mixed form: the same number of
    nonlinear steps as the reference, the residual of every step within 1e-4
    (relative) while it is above the linear solver's tolerance, the solution
    the reference's (velocity 1e-10, pressure 1e-9) and so the known answer of
    the test (the exact solution of example -3 lies in P2 / P1);
  * the pressure of the solution lies in L2_0 and the residual functional is
    the oracle's for the same iterate."""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from oracle import nse
from ref_fixtures import NseRefCase, nse_names
from test_gpu_ref_parity import projected
from test_gpu_stokes import stokes_db

pytestmark = pytest.mark.gpu


def nse_db(n_levels, epsilon=1e-10, maxit=10, precision="fp64", form="convective"):
    db = stokes_db(n_levels, "nodal_vanka", 1.0, max_it=100, reduction=0.0, restart=20, precision=precision)
    db["residual_tolerance"] = 1e-12
    db.add("example", -3)
    db.add("problem_type", 5)
    db.add("nonlinloop_epsilon", epsilon)
    db.add("nonlinloop_maxit", maxit)
    db.add("nse_nonlinear_form", form)
    return db


def make(ctx, nref, nlev, reynolds, db):
    disc = m.Discretization(m.GEO_CUBE_TETRA, 1, nref, nlev, m.KIND_STOKES, 12)
    prob = m.StokesProblem(ctx, disc, 1.0 / reynolds, db)
    return disc, prob


@pytest.mark.parametrize("name", nse_names("none"))
def test_gpu_nonlinear_assembly_matches_the_reference(ctx, name):
    rc = NseRefCase(name)
    disc, prob = make(ctx, rc.n_refine, rc.n_levels, rc.reynolds, nse_db(rc.n_levels, form=rc.form))
    try:
        prob.assemble_linear_terms()
        nu, _, _ = prob.blocks()
        n = prob.size()[0]
        prob.set_solution(rc.fixed_velocity(nu, n))
        prob.assemble_nonlinear_term()
        for l in range(rc.n_levels):
            rp, ci = disc.structure(l)
            lnu = disc.level_info(l, 0)["n_dofs"]
            rp2, ci2, v2 = projected(rp, ci, prob.matrix(l).values(), 3 * lnu)
            assert rc.compare_matrix(l, rp2, ci2, v2) <= 1e-13, l
    finally:
        prob.close()
        disc.close()


def test_gpu_nonlinear_assembly_matches_the_oracle_after_a_solve(ctx):
    """the rhs on the P5Tetra rule and the matrices of every level after a
    solve (a velocity that is not a P2 function of the coarse spaces)"""
    nref, nlev, re = 3, 3, 10.0
    disc, prob = make(ctx, nref, nlev, re, nse_db(nlev))
    o = nse.OracleNSE(1, nref, nlev, re)
    try:
        prob.assemble()
        o.assemble_linear_terms()
        assert np.abs(prob.rhs() - o.rhs[-1]).max() <= 1e-13 * np.abs(o.rhs[-1]).max()
        prob.solve()
        x = prob.solution()
        o.x = x.copy()
        prob.assemble_nonlinear_term()
        o.assemble_nonlinear_term()
        for l in range(nlev):
            v, ref = prob.matrix(l).values(), o.vals[l]
            assert np.abs(v - ref).max() <= 1e-13 * np.abs(ref).max(), l
        g, r = prob.residuals(), o.residuals()
        # the mass residual after a solve is at rounding level (about 1e-13)
        assert abs(g[0] - r[0]) <= 1e-10 * r[0] + 1e-13
        assert abs(g[1] - r[1]) <= 1e-10 * r[1] + 1e-13
    finally:
        prob.close()
        disc.close()


@pytest.mark.parametrize("name", nse_names("direct") + nse_names("mg"))
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_picard_loop_matches_the_reference(ctx, name, precision):
    rc = NseRefCase(name)
    # the direct-solver cases run on two levels of the same mesh
    nlev = max(rc.n_levels, 2)
    disc, prob = make(ctx, rc.n_refine, nlev, rc.reynolds, nse_db(nlev, rc.epsilon, rc.maxit, precision, rc.form))
    try:
        prob.assemble()
        hist = prob.solve_nonlinear()
        ref = rc.z["residuals"]
        assert hist.shape == ref.shape, (hist[:, 2], ref[:, 2])
        assert abs(hist[0, 2] - ref[0, 2]) <= 1e-12 * ref[0, 2]
        big = ref[:, 2] > 1e-8
        assert np.all(np.abs(hist[big, 2] - ref[big, 2]) <= 1e-4 * ref[big, 2]), np.c_[hist[:, 2], ref[:, 2]]
        x = prob.solution()
        idx, sol = rc.full_solution(x.size)
        nu3 = 3 * prob.blocks()[0]
        xv, sv = x[idx], sol
        vel = idx < nu3
        assert np.abs(xv[vel] - sv[vel]).max() <= 1e-10
        assert np.abs(xv[~vel] - sv[~vel]).max() <= 1e-9
        # the pressure lies in L2_0 (NavierStokes::solve's projection)
        o = nse.OracleNSE(1, rc.n_refine, 1, rc.reynolds)
        w = o.pw[-1]
        assert abs(float(w @ x[nu3:])) <= 1e-13
    finally:
        prob.close()
        disc.close()


def test_gpu_unsupported_nonlinear_forms_are_refused(ctx):
    """rotational, divergence and emac couple the velocity components (the
    off-diagonal velocity blocks this set-up does not hold): PM_E_UNSUPPORTED"""
    disc = m.Discretization(m.GEO_CUBE_TETRA, 1, 1, 1, m.KIND_STOKES, 12)
    try:
        for form in ("rotational", "divergence", "emac"):
            with pytest.raises(m.PmError) as e:
                m.StokesProblem(ctx, disc, 1.0, nse_db(1, form=form))
            assert e.value.code == 8, form
    finally:
        disc.close()


def test_gpu_nonlinear_loop_options(ctx):
    """nonlinloop_minit forces steps past convergence; nonlinloop_maxit caps
    them; a damping factor below 1 slows the reduction but converges to the
    same solution"""
    nref, nlev, re = 2, 2, 10.0
    db = nse_db(nlev, 1e-10, 3)
    disc, prob = make(ctx, nref, nlev, re, db)
    try:
        prob.assemble()
        h = prob.solve_nonlinear()
        assert len(h) == 4  # maxit 3: steps 0..3
    finally:
        prob.close()
    db = nse_db(nlev, 1e-3, 20)
    db.add("nonlinloop_minit", 5)
    disc2, prob = make(ctx, nref, nlev, re, db)
    try:
        prob.assemble()
        h = prob.solve_nonlinear()
        assert len(h) == 6  # converged at step 1 or 2, held until minit 5
    finally:
        prob.close()
        disc2.close()
    db = nse_db(nlev, 1e-10, 60)
    db.add("nonlinloop_damping_factor", 0.7)
    disc3, prob = make(ctx, nref, nlev, re, db)
    o = nse.OracleNSE(1, nref, 1, re)
    try:
        prob.assemble()
        h = prob.solve_nonlinear()
        assert h[-1, 2] <= 1e-10 and len(h) > 6
        hist = o.run(1e-10, 60)
        x = prob.solution()
        assert np.abs(x - o.x).max() <= 1e-9
        assert hist[-1, 2] <= 1e-10
    finally:
        prob.close()
        disc3.close()
    disc.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_nse_known_answer_at_the_workload_size(ctx, precision):
    """the Navier-Stokes workload (24^3 cubes x 6 tetrahedra, Reynolds number
    10, the bench's solver): the Picard loop reaches the 1e-10 nonlinear
    residual and the exact solution of example -3: velocity within 1e-8 and
    the pressure, which the loop keeps in L2_0, within 1e-6 of the exact one
    shifted to mean zero (maximum norms; the reference's nse3d_solvers_test
    holds its multigrid runs to 1e-8 in the L2 norms; the 1e-10 nonlinear
    residual leaves velocity errors of about 2e-9 here)"""
    import bench
    from test_gpu_stokes_example import exact_on, level_nodes
    w = bench.WORKLOADS["nse3d_p2p1_24"]
    disc = m.Discretization(m.GEO_CUBE_TETRA, w["root_n"], w["n_refine"], w["n_levels"], m.KIND_STOKES, 12)
    prob = m.StokesProblem(ctx, disc, w["nu"], bench.solver_db(w, precision))
    try:
        prob.assemble()
        hist = prob.solve_nonlinear()
        assert hist[-1, 2] <= 1e-10 and len(hist) <= w["nl_maxit"] + 1
        uc, pc, wp, meas = level_nodes(disc, w["n_levels"] - 1)
        u, pe = exact_on(uc, pc)
        x = prob.solution()
        nu3 = 3 * uc.shape[0]
        assert np.abs(x[:nu3] - u).max() <= 1e-8
        # the loop keeps the pressure in L2_0 (P1 integral weights): the exact
        # pressure's projection
        p = x[nu3:]
        assert np.abs(p - (pe - float(wp @ pe) / meas)).max() <= 1e-6
    finally:
        prob.close()
        disc.close()
