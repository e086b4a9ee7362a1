"""Stokes P2/P1 (Taylor-Hood on tetrahedra) through the GPU library against the
oracle: the combined system from assembly, the multigrid preconditioner with
Vanka smoothers, and FGMRES iterates.

The pressure of the all-Dirichlet Stokes system is determined up to a
constant; solutions are compared after removing the pressure mean."""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from oracle import stokes as ost

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def stokes_db(n_levels, smoother, damp, coarse="direct_solve", pre=1, post=1, max_it=30, reduction=1e-10,
              precision="fp64", restart=30):
    db = m.ParameterDatabase.solve_path_database()
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = "fgmres"
    db["preconditioner"] = "multigrid"
    db["residual_tolerance"] = 0.0
    db["residual_reduction"] = reduction
    db["max_n_iterations"] = max_it
    db["gmres_restart"] = restart
    db["multigrid_n_levels"] = n_levels
    db["multigrid_smoother"] = smoother
    db["multigrid_smoother_coarse"] = coarse
    db["multigrid_vanka_damp_factor"] = damp
    db["multigrid_n_pre_smooth"] = pre
    db["multigrid_n_post_smooth"] = post
    db["gpu_precision"] = precision
    return db


def make_pair(ctx, root, nref, nlev, db, nu=1.0):
    disc = m.Discretization(m.GEO_CUBE_TETRA, root, nref, nlev, m.KIND_STOKES, 12)
    prob = m.StokesProblem(ctx, disc, nu, db)
    prob.assemble()
    ora = ost.OracleStokes(root, nref, nlev, nu)
    ora.assemble()
    return disc, prob, ora


def split(x, lv):
    """velocity and mean-free pressure of a combined vector"""
    p = x[3 * lv.nu:]
    return x[: 3 * lv.nu], p - p.mean()


@pytest.mark.parametrize("nu", [1.0, 0.01])
@pytest.mark.parametrize("root,nref", [(1, 2), (2, 1)])
def test_stokes_assembly_matches_oracle(ctx, root, nref, nu):
    nlev = nref + 1
    disc, prob, ora = make_pair(ctx, root, nref, nlev, stokes_db(nlev, "cell_vanka_jacobi", 0.8), nu)
    for l in range(nlev):
        assert rel(prob.matrix(l).values(), ora.vals[l]) <= 1e-13, l
    assert rel(prob.rhs(), ora.rhs[-1]) <= 1e-13


VANKA = [
    # library smoother, oracle sweep, damping
    ("cell_vanka_jacobi", "cell_jacobi", 0.8),
    ("cell_vanka", "cell_color", 1.0),
]
NODAL = [
    ("nodal_vanka_jacobi", "nodal_jacobi", 0.8),
    ("nodal_vanka", "nodal_color", 1.0),
]


@pytest.mark.parametrize("smoother,okind,damp", VANKA + NODAL)
def test_stokes_multigrid_cycle_matches_oracle(ctx, smoother, okind, damp):
    """one V(1,1) cycle on three levels (coarse direct solve on the projected
    matrix); includes the cells whose pressures are frozen"""
    db = stokes_db(3, smoother, damp)
    disc, prob, ora = make_pair(ctx, 1, 3, 3, db)
    prob.solve()  # builds the hierarchy
    ora.build_mg(smoother=okind, vanka_damp=damp, n_pre=1, n_post=1)
    if okind.startswith("cell"):
        assert ora.finest.n_freeze.max() == 4  # the singular cells are part of the case
    z = np.random.default_rng(7).standard_normal(ora.finest.n)
    zd = m.DeviceVector.from_numpy(ctx, z)
    rd = m.DeviceVector(ctx, z.size)
    prob.solver().apply_preconditioner(zd, rd)
    ref = ora.mg_apply(z)
    assert rel(rd.numpy(), ref) <= 1e-10


@pytest.mark.parametrize("smoother,okind,damp", VANKA)
def test_stokes_fgmres_iterates_match_oracle(ctx, smoother, okind, damp):
    """eight FGMRES iterations: residual history and iterate (cell Vanka on a
    continuous pressure converges slowly; the iterates are compared, not a
    converged solution)"""
    db = stokes_db(2, smoother, damp, max_it=8)
    disc, prob, ora = make_pair(ctx, 1, 2, 2, db)
    prob.solve()
    hist = prob.solver().residual_history()
    ora.build_mg(smoother=okind, vanka_damp=damp, n_pre=1, n_post=1)
    sol, oit, ores, ohist, st = ora.solve(reduction=1e-10, max_it=8, restart=30)
    assert prob.last_info()[0] == oit == 8
    n = min(hist.size, ohist.size)
    assert n >= 8 and rel(hist[:n], ohist[:n]) <= 1e-9
    u, p = split(prob.solution(), ora.finest)
    ou, op = split(sol, ora.finest)
    assert rel(u, ou) <= 1e-9 and rel(p, op) <= 1e-9


@pytest.mark.parametrize("smoother,okind,damp", NODAL)
def test_stokes_nodal_vanka_solution_matches_oracle(ctx, smoother, okind, damp):
    """FGMRES with nodal-Vanka V(1,1) multigrid on three levels to 1e-10:
    iteration counts within one; both solutions meet the 1e-10 residual, so they
    agree to about that level: velocity within 1e-9, the (mean-free) pressure,
    the less well conditioned unknown, within 1e-8"""
    # restart 60: no restart inside the run (a restart amplifies rounding differences)
    db = stokes_db(3, smoother, damp, max_it=100, reduction=1e-10, restart=60)
    disc, prob, ora = make_pair(ctx, 1, 3, 3, db)
    prob.solve()
    it, res, init = prob.last_info()
    ora.build_mg(smoother=okind, vanka_damp=damp, n_pre=1, n_post=1)
    sol, oit, ores, ohist, st = ora.solve(reduction=1e-10, max_it=100, restart=60)
    assert st == 0 and oit < 100
    assert abs(it - oit) <= 1, (it, oit)
    assert res <= 1e-10 * init
    u, p = split(prob.solution(), ora.finest)
    ou, op = split(sol, ora.finest)
    assert rel(u, ou) <= 1e-9 and rel(p, op) <= 1e-8


def test_stokes_mixed_precision_reaches_fp64_target(ctx):
    """FP32 nodal-Vanka multigrid inside FP64 FGMRES: the FP64 residual reaches
    1e-8 and the solution agrees with the FP64 oracle"""
    db = stokes_db(3, "nodal_vanka_jacobi", 0.8, max_it=100, reduction=1e-8, precision="mixed")
    disc, prob, ora = make_pair(ctx, 1, 3, 3, db)
    prob.solve()
    it, res, init = prob.last_info()
    assert res <= 1e-8 * init and it < 100
    ora.build_mg(smoother="nodal_jacobi", vanka_damp=0.8, n_pre=1, n_post=1)
    sol, oit, ores, ohist, st = ora.solve(reduction=1e-10, max_it=100, restart=30)
    u, p = split(prob.solution(), ora.finest)
    ou, op = split(sol, ora.finest)
    assert rel(u, ou) <= 1e-6 and rel(p, op) <= 1e-5


def test_stokes_discrete_solution_converges_to_manufactured_solution(ctx):
    """the discrete velocity approaches u = curl(psi (1,1,1)) under refinement
    (nodal values; P2 gives at least second order on these meshes)"""
    errs = []
    for nref in (2, 3):
        # coarsest level 8 x 6 tetrahedra (the single-cube level has a singular
        # projected coarse matrix)
        db = stokes_db(nref, "nodal_vanka", 1.0, max_it=100, reduction=1e-10)
        disc = m.Discretization(m.GEO_CUBE_TETRA, 1, nref, nref, m.KIND_STOKES, 12)
        prob = m.StokesProblem(ctx, disc, 1.0, db)
        prob.assemble()
        prob.solve()
        lv = ost.stokes_levels(1, nref, 1)[0]
        X = lv.ucoords / lv.ucoords.max()
        x, y, z = X[:, 0], X[:, 1], X[:, 2]
        S = lambda t: np.sin(np.pi * t) ** 2
        D = lambda t: np.pi * np.sin(2 * np.pi * t)
        px, py, pz = D(x) * S(y) * S(z), S(x) * D(y) * S(z), S(x) * S(y) * D(z)
        exact = np.concatenate([py - pz, pz - px, px - py])
        errs.append(np.abs(prob.solution()[: 3 * lv.nu] - exact).max())
    assert errs[1] < errs[0] / 3.5, errs


@pytest.mark.parametrize("coarse_residual", [0.0, 0.1])
def test_stokes_iterative_coarse_level_matches_oracle(ctx, coarse_residual):
    """nodal Vanka also on the coarsest level: at most 10 colour-ordered sweeps,
    stopping at multigrid_coarse_residual (checked on the device)"""
    db = stokes_db(3, "nodal_vanka", 1.0, coarse="nodal_vanka")
    db["multigrid_coarse_max_n_iterations"] = 10
    db["multigrid_coarse_residual"] = coarse_residual
    disc, prob, ora = make_pair(ctx, 1, 3, 3, db)
    prob.solve()
    ora.build_mg(smoother="nodal_color", coarse_smoother="nodal_color", vanka_damp=1.0, n_pre=1, n_post=1,
                 coarse_max_it=10, coarse_residual=coarse_residual)
    z = np.random.default_rng(11).standard_normal(ora.finest.n)
    zd = m.DeviceVector.from_numpy(ctx, z)
    rd = m.DeviceVector(ctx, z.size)
    prob.solver().apply_preconditioner(zd, rd)
    assert rel(rd.numpy(), ora.mg_apply(z)) <= 1e-10


def test_stokes_workload_multigrid_matches_oracle(ctx):
    """the 3D Stokes workload's multigrid: colour-ordered nodal Vanka on the fine
    levels, additive nodal Vanka on the coarsest (at most 10 sweeps, stop at 0.1),
    damping 0.8, one V(1,1) cycle"""
    db = stokes_db(3, "nodal_vanka", 0.8, coarse="nodal_vanka_jacobi")
    db["multigrid_coarse_max_n_iterations"] = 10
    db["multigrid_coarse_residual"] = 0.1
    disc, prob, ora = make_pair(ctx, 3, 2, 3, db)
    prob.solve()
    ora.build_mg(smoother="nodal_color", coarse_smoother="nodal_jacobi", vanka_damp=0.8, n_pre=1, n_post=1,
                 coarse_max_it=10, coarse_residual=0.1)
    z = np.random.default_rng(13).standard_normal(ora.finest.n)
    zd = m.DeviceVector.from_numpy(ctx, z)
    rd = m.DeviceVector(ctx, z.size)
    prob.solver().apply_preconditioner(zd, rd)
    assert rel(rd.numpy(), ora.mg_apply(z)) <= 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nodal_sweep_sliced_rows_match_the_patch_rows(ctx, precision):
    """the colour's local residuals from the sliced copy of the patch rows
    (nodal_sliced 4, the default, or 8 lanes per row) and from the CSR rows,
    one block per patch (nodal_sliced 0): one multigrid cycle within rounding
    (1e-12 FP64, 1e-5 FP32) and the same FGMRES iterations"""
    db = stokes_db(3, "nodal_vanka", 0.8, coarse="nodal_vanka_jacobi", max_it=100, reduction=1e-8,
                   precision=precision)
    db["multigrid_coarse_max_n_iterations"] = 10
    db["multigrid_coarse_residual"] = 0.1
    out = {}
    try:
        for sliced in (4, 8, 0):
            ctx.set_option("nodal_sliced", sliced)
            disc = m.Discretization(m.GEO_CUBE_TETRA, 2, 3, 3, m.KIND_STOKES, 12)
            prob = m.StokesProblem(ctx, disc, 1.0, db)
            prob.assemble()
            prob.solve()
            z = np.random.default_rng(5).standard_normal(prob.size()[0])
            zd = m.DeviceVector.from_numpy(ctx, z)
            rd = m.DeviceVector(ctx, z.size)
            prob.solver().apply_preconditioner(zd, rd)
            out[sliced] = (prob.last_info()[0], prob.solution(), rd.numpy())
            prob.close()
            disc.close()
    finally:
        ctx.set_option("nodal_sliced", 8)
    tol = 1e-12 if precision == "fp64" else 1e-5
    for lanes in (4, 8):
        assert rel(out[lanes][2], out[0][2]) <= tol
        assert abs(out[lanes][0] - out[0][0]) <= (0 if precision == "fp64" else 1)
        assert rel(out[lanes][1], out[0][1]) <= 1e-7
