"""GPU parity of the solve path against the CPU oracle (all through the C ABI).

Tolerances (FP64 unless stated):
  SpMV                 1e-13 relative to sum_j |a_ij x_j|   (summation order differs)
  assembled entries    1e-13 relative to max |entry|
  multigrid cycle      1e-11 relative (max norm)
  final solutions      1e-10 relative, Krylov iteration counts within one
  mixed precision      FP64 residual reduction 1e-8 reached; error against the
                       FP64 oracle solution stated in the assertion (<= 1e-7)
"""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from oracle import cd as ocd

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def mg_db(n_levels, restart=20, reduction=1e-10, precision="fp64", smoother_damp=0.8, pre=2, post=2,
          cycle="V"):
    db = m.ParameterDatabase.solve_path_database()
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = "fgmres"
    db["preconditioner"] = "multigrid"
    db["residual_tolerance"] = 0.0
    db["residual_reduction"] = reduction
    db["max_n_iterations"] = 200
    db["gmres_restart"] = restart
    db["multigrid_n_levels"] = n_levels
    db["multigrid_smoother"] = "jacobi"
    db["multigrid_smoother_coarse"] = "direct_solve"
    db["jacobi_damp"] = smoother_damp
    db["multigrid_n_pre_smooth"] = pre
    db["multigrid_n_post_smooth"] = post
    db["multigrid_cycle_type"] = cycle
    db["gpu_precision"] = precision
    return db


CASES = {
    # name: geometry, root_n, n_refine, n_levels, elem, eps, b, quad
    "q1_2d": (m.GEO_SQUARE_QUAD, 1, 5, 3, 1, 0.1, (1.0, 0.0, 0.0), 3),
    "q2_2d": (m.GEO_SQUARE_QUAD, 1, 4, 3, 2, 0.05, (0.6, 0.8, 0.0), 3),
    "q1_3d": (m.GEO_CUBE_HEXA, 1, 3, 3, 1, 0.1, (1.0, 0.5, 0.25), 3),
    "q2_3d": (m.GEO_CUBE_HEXA, 1, 3, 3, 2, 0.1, (1.0, 0.5, 0.25), 3),
    "q2_3d_root3": (m.GEO_CUBE_HEXA, 3, 1, 2, 2, 0.1, (1.0, 0.5, 0.25), 3),
}


def make_pair(ctx, case, db):
    geo, root, nref, nlev, elem, eps, b, qn = CASES[case]
    disc = m.Discretization(geo, root, nref, nlev, m.KIND_CD, elem)
    cf = m.cd_coeffs(eps, b, 0.0, True)
    prob = m.ConvectionDiffusion(ctx, disc, cf, db, quad_points=qn)
    prob.assemble()
    ora = ocd.OracleCD(geo, root, nref, nlev, elem, eps, b, 0.0, qn)
    ora.assemble()
    return disc, prob, ora


@pytest.mark.parametrize("qloop", [0, 1])
@pytest.mark.parametrize("case", list(CASES))
def test_assembly_matches_oracle(ctx, case, qloop):
    """reference-tensor contraction (default) and per-quadrature-point loop"""
    ctx.set_option("assembly_quadrature_loop", qloop)
    try:
        disc, prob, ora = make_pair(ctx, case, mg_db(CASES[case][3]))
        for l in range(disc.n_levels):
            vals = prob.matrix(l).values()
            assert rel(vals, ora.vals[l]) <= 1e-13, (case, l)
        assert rel(prob.rhs(), ora.rhs[-1]) <= 1e-13
    finally:
        ctx.set_option("assembly_quadrature_loop", 0)


def test_spmv_known_answer(ctx):
    """test/matrix_test.c++:143-147 through the GPU: y = -0.5*CB*x"""
    B = np.zeros((3, 4))
    B[0, 0], B[0, 3], B[1, 2], B[2, 1], B[2, 3] = 4, 1, 5, 6, 1
    C = np.zeros((4, 3))
    C[0, 0], C[0, 2], C[1, 0], C[1, 1], C[2, 1], C[2, 2], C[3, 0], C[3, 2] = 7, 8, 9, 10, 11, 12, 13, 14
    CB = C @ B
    rp = [0]
    ci, v = [], []
    for row in CB:
        for j, a in enumerate(row):
            if a != 0:
                ci.append(j)
                v.append(a)
        rp.append(len(ci))
    A = m.FEMatrix.from_csr(ctx, rp, ci, v)
    x = m.DeviceVector.from_numpy(ctx, np.array([1.0, -2.5, 11.34, -0.004]))
    y = m.DeviceVector(ctx, 4)
    A.apply_scaled_add(x, y, -0.5)
    assert np.allclose(y.numpy(), [46.03, -301.482, -221.826, 79.054], rtol=0, atol=1e-10)


@pytest.mark.parametrize("shape", [None, (0, 0), (8, 2), (32, 4)])
@pytest.mark.parametrize("case", ["q1_2d", "q2_3d"])
def test_spmv_apply_scaled_add_matches_oracle(ctx, case, shape):
    """default launch shape, the row-block streaming kernel (0, 0) and other group shapes"""
    disc, prob, ora = make_pair(ctx, case, mg_db(CASES[case][3]))
    lv = ora.finest
    rng = np.random.default_rng(3)
    x = rng.standard_normal(lv.n_dofs)
    y0 = rng.standard_normal(lv.n_dofs)
    A = prob.matrix(-1)
    if shape is not None:
        A.set_kernel(*shape)
    xd, yd = m.DeviceVector.from_numpy(ctx, x), m.DeviceVector.from_numpy(ctx, y0)
    A.apply_scaled_add(xd, yd, -0.7)
    ref = ocd.apply_scaled_add(lv.row_ptr, lv.cols, ora.vals[-1], ora.active(), x, y0, -0.7)
    scale = ocd.apply_scaled_add(lv.row_ptr, lv.cols, np.abs(ora.vals[-1]), ora.active(), np.abs(x),
                                 np.abs(y0), 0.7)
    assert np.all(np.abs(yd.numpy() - ref) <= 1e-13 * scale)


def test_spmv_fp32_matches_fp64_within_fp32_rounding(ctx):
    disc, prob, ora = make_pair(ctx, "q2_3d", mg_db(3))
    A = prob.matrix(-1)
    A.make_fp32()
    lv = ora.finest
    x = np.random.default_rng(4).standard_normal(lv.n_dofs)
    y = m.DeviceVector(ctx, lv.n_dofs, np.float32)
    A.apply_f32(m.DeviceVector.from_numpy(ctx, x.astype(np.float32)), y)
    ref = ocd.apply_scaled_add(lv.row_ptr, lv.cols, ora.vals[-1], ora.active(), x, np.zeros(lv.n_dofs), 1.0)
    scale = ocd.apply_scaled_add(lv.row_ptr, lv.cols, np.abs(ora.vals[-1]), ora.active(), np.abs(x),
                                 np.zeros(lv.n_dofs), 1.0)
    assert np.all(np.abs(y.numpy() - ref) <= 2e-6 * scale + 1e-30)


@pytest.mark.parametrize("case", ["q1_2d", "q2_3d", "q2_3d_root3"])
def test_multigrid_cycle_matches_oracle(ctx, case):
    nl = CASES[case][3]
    disc, prob, ora = make_pair(ctx, case, mg_db(nl))
    prob.solve()  # builds the hierarchy (update_matrix)
    ora.build_mg(2, 2, 0.8, 1.0, "V")
    rng = np.random.default_rng(5)
    z = rng.standard_normal(ora.finest.n_dofs)
    zd = m.DeviceVector.from_numpy(ctx, z)
    rd = m.DeviceVector(ctx, z.size)
    prob.solver().apply_preconditioner(zd, rd)
    assert rel(rd.numpy(), ora.mg_apply(z)) <= 1e-11


@pytest.mark.parametrize("case", list(CASES))
def test_fgmres_multigrid_solution_matches_oracle(ctx, case):
    nl = CASES[case][3]
    disc, prob, ora = make_pair(ctx, case, mg_db(nl))
    prob.solve()
    it, res, init = prob.last_info()
    ora.build_mg(2, 2, 0.8, 1.0, "V")
    sol, oit, ores, hist, st = ora.solve("fgmres", 0.0, 1e-10, 200, 0, 20)
    assert st == 0
    assert abs(it - oit) <= 1, (it, oit)
    assert rel(prob.solution(), sol) <= 1e-10
    assert res < 1e-10 * init


@pytest.mark.parametrize("gs", ["cgs2", "cgs2_cond"])
def test_cgs2_orthogonalisation_matches_mgs_oracle(ctx, gs):
    """FP64 FGMRES with batched classical Gram-Schmidt (two passes, or the
    second pass only when the DGKS test asks for it) against the oracle's
    modified Gram-Schmidt: same solution within 1e-10, iterations within one"""
    db = mg_db(3)
    db.add("gpu_gram_schmidt", gs)
    disc, prob, ora = make_pair(ctx, "q2_3d", db)
    prob.solve()
    it, res, init = prob.last_info()
    ora.build_mg(2, 2, 0.8, 1.0, "V")
    sol, oit, ores, hist, st = ora.solve("fgmres", 0.0, 1e-10, 200, 0, 20)
    assert abs(it - oit) <= 1, (it, oit)
    assert rel(prob.solution(), sol) <= 1e-10


def test_w_cycle_and_restart_match_oracle(ctx):
    db = mg_db(3, restart=3, cycle="W")
    disc, prob, ora = make_pair(ctx, "q1_2d", db)
    prob.solve()
    it, res, init = prob.last_info()
    ora.build_mg(2, 2, 0.8, 1.0, "W")
    sol, oit, ores, hist, st = ora.solve("fgmres", 0.0, 1e-10, 200, 0, 3)
    assert abs(it - oit) <= 1
    assert rel(prob.solution(), sol) <= 1e-10


def test_mixed_precision_reaches_fp64_target(ctx):
    db = mg_db(3, restart=30, reduction=1e-8, precision="mixed")
    disc, prob, ora = make_pair(ctx, "q2_3d", db)
    prob.solve()
    x = prob.solution()
    lv = ora.finest
    b = ora.rhs[-1]
    x0 = np.zeros_like(b)
    x0[lv.n_active:] = b[lv.n_active:]
    r0 = ocd.apply_scaled_add(lv.row_ptr, lv.cols, ora.vals[-1], ora.active(), x0, b, -1.0)
    r = ocd.apply_scaled_add(lv.row_ptr, lv.cols, ora.vals[-1], ora.active(), x, b, -1.0)
    assert np.linalg.norm(r) <= 1.05e-8 * np.linalg.norm(r0)
    ora.build_mg(2, 2, 0.8, 1.0, "V")
    sol, *_ = ora.solve("fgmres", 0.0, 1e-8, 200, 0, 30)
    err = rel(x, sol)
    assert err <= 1e-7, f"mixed vs FP64 oracle relative error {err:.3e}"


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reassembled_problem_solves_like_a_fresh_one(ctx, precision):
    """a cached problem re-assembled with new coefficients (the request
    executor's reuse) gives the bits of a problem created with them: every
    matrix copy the multigrid reads (FP64, FP32, sliced) follows the new values"""
    geo, root, nref, nlev, elem, eps, b, qn = CASES["q2_3d"]
    disc = m.Discretization(geo, root, nref, nlev, m.KIND_CD, elem)
    first = m.cd_coeffs(eps, b, 0.0, True)
    second = m.cd_coeffs(2e-3, (0.2, -0.9, 0.4), 0.0, True)
    db = mg_db(nlev, restart=30, reduction=1e-8, precision=precision)
    n = disc.level_info(nlev - 1)["n_dofs"]
    reused = m.ConvectionDiffusion(ctx, disc, first, db, quad_points=qn)
    x1 = np.empty(n)
    reused.run_host(first, None, x1)
    x2 = np.empty(n)
    reused.run_host(second, None, x2)
    info_reused = reused.last_info()
    fresh = m.ConvectionDiffusion(ctx, disc, second, db, quad_points=qn)
    x3 = np.empty(n)
    fresh.run_host(second, None, x3)
    assert info_reused == fresh.last_info()
    assert np.array_equal(x2, x3)
    reused.close()
    fresh.close()


@pytest.mark.parametrize("case", ["q1_2d", "q2_2d", "q2_3d", "q2_3d_root3"])
def test_mixed_cycle_with_fp32_coarse_inverse_matches_oracle_cycle(ctx, case):
    """the mixed form's cycle (FP32 smoothing, transfer and coarse solve with the
    FP32 inverse from the one-cluster Gauss-Jordan) against the FP64 oracle
    cycle: agreement to FP32 accuracy (1e-4 relative in the max norm)"""
    nl = CASES[case][3]
    disc, prob, ora = make_pair(ctx, case, mg_db(nl, precision="mixed"))
    prob.solve()
    ora.build_mg(2, 2, 0.8, 1.0, "V")
    z = np.random.default_rng(17).standard_normal(ora.finest.n_dofs)
    rd = m.DeviceVector(ctx, z.size)
    prob.solver().apply_preconditioner(m.DeviceVector.from_numpy(ctx, z), rd)
    assert rel(rd.numpy(), ora.mg_apply(z)) <= 1e-4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("cycle", ["V", "W"])
def test_jacobi_zero_start_gives_the_full_sweeps_bits(ctx, precision, cycle):
    """the first Jacobi sweep from an exactly zero iterate, done as a diagonal
    scaling, leaves every FGMRES iterate and the solution bit for bit unchanged
    (W cycles revisit levels whose iterate is no longer zero)"""
    out = {}
    try:
        for flag in (1, 0):
            ctx.set_option("jacobi_zero_start", flag)
            db = mg_db(3, restart=20, reduction=1e-10, precision=precision, cycle=cycle)
            disc, prob, ora = make_pair(ctx, "q2_3d", db)
            prob.solve()
            out[flag] = (prob.solution(), prob.last_info(), prob.solver().residual_history())
            prob.close()
    finally:
        ctx.set_option("jacobi_zero_start", 1)
    assert out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])
    assert np.array_equal(out[0][0], out[1][0])


@pytest.mark.parametrize("method", ["fgmres", "cg", "bi_cgstab"])
def test_krylov_on_reference_test_system(ctx, method):
    """the 7x7 block system of test/iterative_solver_test.c++ solved on the GPU"""
    A = np.diag([5.5, 7.53, 10.0, 15.0])
    B = np.zeros((3, 4))
    B[0, 0], B[0, 3], B[1, 2], B[2, 1], B[2, 3] = 4, 1, 5, 6, 1
    D = np.array([[50, 0, 0], [0, 19, 0.1], [0, 0.1, 85.6]])
    M = np.block([[A, B.T], [B, D]])
    rp, ci, v = [0], [], []
    for row in M:
        for j, a in enumerate(row):
            if a != 0:
                ci.append(j)
                v.append(a)
        rp.append(len(ci))
    mat = m.FEMatrix.from_csr(ctx, rp, ci, v)
    exact = np.arange(7.0)
    rhs = M @ exact
    db = m.ParameterDatabase.solve_path_database()
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = method
    db["residual_tolerance"] = 1e-11
    db["max_n_iterations"] = 1000
    db["preconditioner"] = "jacobi"
    s = m.Solver(ctx, db)
    s.update_matrix(mat)
    sol = np.zeros(7)
    s.solve(rhs, sol)
    assert np.linalg.norm(sol - exact) <= 100 * 1e-11


def test_solves_are_deterministic(ctx):
    db = mg_db(3, restart=30, reduction=1e-8)
    disc, prob, ora = make_pair(ctx, "q2_3d", db)
    prob.solve()
    a = prob.solution()
    prob.assemble()
    prob.run_host(None, None, np.empty_like(a))
    b = prob.solution()
    assert np.array_equal(a, b)


def test_direct_solver(ctx):
    disc, prob, ora = make_pair(ctx, "q1_2d", mg_db(3))
    lv = ora.finest
    A = m.FEMatrix.from_csr(ctx, lv.row_ptr, lv.cols, ora.vals[-1], n_active=lv.n_active)
    db = m.ParameterDatabase.solve_path_database()
    s = m.Solver(ctx, db)
    s.update_matrix(A)
    b = ora.rhs[-1]
    x = np.zeros_like(b)
    s.solve(b, x)
    r = ocd.apply_scaled_add(lv.row_ptr, lv.cols, ora.vals[-1], ora.active(), x, b, -1.0)
    assert np.linalg.norm(r) <= 1e-12 * np.linalg.norm(b)


def test_config_2d_q1_128_full_size_against_oracle(ctx):
    """2D Q1 128^2, FGMRES(20) + V(2,2) Jacobi(0.8), 4 levels, to 1e-10"""
    disc = m.Discretization(m.GEO_SQUARE_QUAD, 1, 7, 4, m.KIND_CD, 1)
    cf = m.cd_coeffs(0.1, (1.0, 0.0), 0.0, True)
    prob = m.ConvectionDiffusion(ctx, disc, cf, mg_db(4, restart=20, reduction=1e-10), quad_points=3)
    prob.assemble()
    prob.solve()
    it, res, init = prob.last_info()
    ora = ocd.OracleCD(0, 1, 7, 4, 1, 0.1, (1.0, 0.0), 0.0, 3)
    ora.assemble()
    ora.build_mg(2, 2, 0.8, 1.0, "V")
    sol, oit, ores, hist, st = ora.solve("fgmres", 0.0, 1e-10, 200, 0, 20)
    assert abs(it - oit) <= 1
    assert rel(prob.solution(), sol) <= 1e-10
    assert rel(prob.matrix(-1).values(), ora.vals[-1]) <= 1e-13


@pytest.mark.parametrize("coarse_residual", [0.0, 1.0])
def test_multigrid_iterative_coarse_level_matches_oracle(ctx, coarse_residual):
    """Jacobi on the coarsest level: at most 10 sweeps, stopping once the coarse
    defect norm is <= multigrid_coarse_residual (Multigrid.C cycle_step); 1.0
    stops the loop early on this case, 0.0 runs all 10 sweeps"""
    db = mg_db(3)
    db["multigrid_smoother_coarse"] = "jacobi"
    db["multigrid_coarse_max_n_iterations"] = 10
    db["multigrid_coarse_residual"] = coarse_residual
    disc, prob, ora = make_pair(ctx, "q1_2d", db)
    prob.solve()
    ora.build_mg(2, 2, 0.8, 1.0, "V", coarse_direct=False, coarse_max_it=10, coarse_residual=coarse_residual)
    z = np.random.default_rng(5).standard_normal(ora.finest.n_dofs)
    zd = m.DeviceVector.from_numpy(ctx, z)
    rd = m.DeviceVector(ctx, z.size)
    prob.solver().apply_preconditioner(zd, rd)
    assert rel(rd.numpy(), ora.mg_apply(z)) <= 1e-11


def _cd_case(dim, cells, elem, eps, b):
    from mymoonmd_gb300 import workloads as wl
    rq = wl.cd_request(dim, cells, elem, eps, b)
    disc = m.Discretization(rq["geometry"], rq["root_n"], rq["n_refine"], rq["n_levels"], m.KIND_CD, elem)
    return rq, disc, m.cd_coeffs(eps, rq["b"], 0.0, True)


def _solve(ctx, disc, cf, n_levels, precision, fallback=1):
    db = mg_db(n_levels, restart=30, reduction=1e-8, precision=precision)
    db["max_n_iterations"] = 100
    db["gpu_mixed_fallback"] = fallback
    prob = m.ConvectionDiffusion(ctx, disc, cf, db)
    prob.assemble()
    prob.solve()
    out = (prob.solution(), *prob.last_info(), prob.solver().residual_history())
    prob.close()
    return out


def test_mixed_form_switches_to_fp64_when_the_residual_stalls(ctx):
    """a slowly converging request of the batched stream (3D Q1 16^3, eps 5.2e-3):
    its residual is not halved within 10 iterations, so the mixed form switches
    the multigrid to FP64 (gpu_mixed_fallback) and goes on from the current
    Krylov basis; it reaches the 1e-8 FP64 residual like the FP64 form, and its
    residual history leaves the one without the switch"""
    rq, disc, cf = _cd_case(3, 16, 1, 5.21e-3, (-0.06, -0.13, 0.21))
    sol64, it64, res64, init64, _ = _solve(ctx, disc, cf, rq["n_levels"], "fp64")
    solm, itm, resm, initm, histm = _solve(ctx, disc, cf, rq["n_levels"], "mixed")
    soln, itn, resn, initn, histn = _solve(ctx, disc, cf, rq["n_levels"], "mixed", fallback=0)
    assert res64 <= 1e-8 * init64 and resm <= 1e-8 * initm
    assert abs(itm - it64) <= 2, (itm, it64)
    k = min(histm.size, histn.size)
    assert histm.size != histn.size or not np.array_equal(histm[:k], histn[:k])
    assert rel(solm, sol64) <= 1e-6


def test_mixed_form_restarts_in_fp64_after_an_fp32_overflow(ctx):
    """diffusion 1e40 (2D Q1 32^2): the FP64 system is fine, its FP32 copy
    overflows, so the first FP32 cycle gives a non-finite residual; the mixed
    form discards that Krylov cycle and restarts from the same iterate with the
    FP64 multigrid (the FP64 coarse inverse is made then): the FP64 form's
    iterates, one iteration later"""
    rq, disc, cf = _cd_case(2, 32, 1, 1e40, (1.0, 0.0))
    sol64, it64, res64, init64, _ = _solve(ctx, disc, cf, rq["n_levels"], "fp64")
    solm, itm, resm, initm, _ = _solve(ctx, disc, cf, rq["n_levels"], "mixed")
    assert res64 <= 1e-8 * init64 and resm <= 1e-8 * initm
    assert itm == it64 + 1
    assert rel(solm, sol64) <= 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_multigrid_on_fewer_levels_than_the_discretisation_keeps(ctx, precision):
    """multigrid_n_levels = 2 on a discretisation of 3 levels: the cycle runs on
    the two finest levels, and the coarse direct solve factorises the middle
    level once that level is assembled (not the unused coarsest one)"""
    disc, prob, ora = make_pair(ctx, "q1_2d", mg_db(2, precision=precision))
    prob.solve()
    it, res, init = prob.last_info()
    ora.build_mg(2, 2, 0.8, 1.0, "V", n_mg_levels=2)
    sol, oit, ores, hist, st = ora.solve("fgmres", 0.0, 1e-10, 200, 0, 20)
    assert st == 0 and res < 1e-10 * init
    if precision == "fp64":
        assert abs(it - oit) <= 1, (it, oit)
    assert rel(prob.solution(), sol) <= (1e-10 if precision == "fp64" else 1e-7)
    prob.close()
    disc.close()
