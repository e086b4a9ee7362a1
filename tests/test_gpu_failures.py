"""Failure paths of the solver and the request executor, through the C ABI.

The reference reports these by ErrThrow -> std::runtime_error
(include/General/MooNMD_Io.h:210); the C ABI returns a status code and a
message instead and never throws. Every failure here is made on the host (a
non-finite right-hand side, a divergent iteration, a singular Krylov step, a
malformed request); no GPU fault is involved. After each failure the same
handles must still work.
"""
import ctypes as C

import numpy as np
import pytest

import mymoonmd_gb300 as m
from mymoonmd_gb300 import _lib

pytestmark = pytest.mark.gpu

PM_E_INVALID, PM_E_DIVERGED, PM_E_BREAKDOWN = 1, 3, 4


@pytest.fixture(scope="module")
def ctx():
    c = m.Context(0)
    yield c
    c.close()


def solver_status(ctx, db_text, rp, ci, vals, rhs):
    """raw pm_solver_* calls: returns (status, message, solution)"""
    A = m.FEMatrix.from_csr(ctx, np.asarray(rp, np.int32), np.asarray(ci, np.int32),
                            np.asarray(vals, np.float64))
    s = C.c_void_p()
    assert _lib.lib.pm_solver_create(ctx.handle, db_text.encode(), C.byref(s)) == 0
    try:
        assert _lib.lib.pm_solver_update_matrix(s, A.handle) == 0
        b = np.ascontiguousarray(rhs, np.float64)
        x = np.zeros_like(b)
        rc = _lib.lib.pm_solver_solve_host(s, b.ctypes.data_as(C.c_void_p), x.ctypes.data_as(C.c_void_p),
                                           b.size)
        msg = _lib.lib.pm_last_error(ctx.handle)
        return rc, (msg.decode() if isinstance(msg, bytes) else str(msg)), x
    finally:
        _lib.lib.pm_solver_destroy(s)
        A.close()


def laplace_1d(n):
    """the 1D finite-difference Laplacian (SPD, eigenvalues in (0, 4))"""
    rp, ci, v = [0], [], []
    for i in range(n):
        for j, a in ((i - 1, -1.0), (i, 2.0), (i + 1, -1.0)):
            if 0 <= j < n:
                ci.append(j)
                v.append(a)
        rp.append(len(ci))
    return rp, ci, v


# without restarts FGMRES solves an n x n system (n <= 40) in at most n iterations
FGMRES = ("solver_type: iterative\niterative_solver_type: fgmres\npreconditioner: no_preconditioner\n"
          "residual_tolerance: 0\nresidual_reduction: 1e-12\nmax_n_iterations: 200\ngmres_restart: 40\n")


def test_non_finite_right_hand_side_is_reported_not_thrown(ctx):
    rp, ci, v = laplace_1d(32)
    rhs = np.ones(32)
    rhs[17] = np.nan
    rc, msg, _ = solver_status(ctx, FGMRES, rp, ci, v, rhs)
    assert rc == PM_E_DIVERGED and "not finite" in msg
    # the context is still usable: the same system with a finite rhs solves
    rc, _, x = solver_status(ctx, FGMRES, rp, ci, v, np.ones(32))
    A = np.zeros((32, 32))
    for i in range(32):
        for k in range(rp[i], rp[i + 1]):
            A[i, ci[k]] = v[k]
    assert rc == 0 and np.abs(A @ x - 1.0).max() < 1e-8


def test_divergence_factor_stops_a_divergent_iteration(ctx):
    """IterativeMethod::converged (include/Solver/IterativeMethod.h:105-131):
    a residual above divergence_factor times the initial one throws. Richardson
    with damping 10 on a matrix with eigenvalues up to 4 grows the residual by
    about 39 per step."""
    rp, ci, v = laplace_1d(32)
    db = ("solver_type: iterative\niterative_solver_type: richardson\npreconditioner: no_preconditioner\n"
          "damping_factor: 10\ndivergence_factor: 1e6\nresidual_tolerance: 0\nresidual_reduction: 1e-10\n"
          "max_n_iterations: 100\n")
    rng = np.random.default_rng(3)
    rc, msg, _ = solver_status(ctx, db, rp, ci, v, rng.standard_normal(32))
    assert rc == PM_E_DIVERGED and "divergence" in msg


def test_fgmres_breakdown_is_reported(ctx):
    """Iteration_gmres::flexible_gmres (src/Solver/Iteration_gmres.C:468-477):
    H(i+1, i) == 0 throws "Unhappy breakdown". A = [[0, 0], [0, 1]], b = e_0:
    A v_0 = 0, so the first Arnoldi vector has norm zero."""
    rc, msg, _ = solver_status(ctx, FGMRES, [0, 1, 2], [0, 1], [0.0, 1.0], [1.0, 0.0])
    assert rc == PM_E_BREAKDOWN and "breakdown" in msg


def test_bicgstab_omega_zero_is_reported(ctx):
    """Iteration_bicgstab::iterate (src/Solver/Iteration_bicgstab.C): omega == 0
    throws. A = [[-2, -2], [-2, 0]], b = e_0: s = (0, -1), t = A s = (2, 0),
    so omega = (t, s) / (t, t) = 0 in the first iteration (exact arithmetic)."""
    db = ("solver_type: iterative\niterative_solver_type: bi_cgstab\npreconditioner: no_preconditioner\n"
          "residual_tolerance: 0\nresidual_reduction: 1e-10\nmax_n_iterations: 20\n")
    rc, msg, _ = solver_status(ctx, db, [0, 2, 3], [0, 1, 0], [-2.0, -2.0, -2.0], [1.0, 0.0])
    assert rc == PM_E_BREAKDOWN and "Bi-CGStab" in msg


def test_malformed_requests_are_refused_and_the_server_keeps_serving():
    db = m.ParameterDatabase.solve_path_database()
    db["solver_type"] = "iterative"
    db["iterative_solver_type"] = "fgmres"
    db["preconditioner"] = "multigrid"
    db["residual_tolerance"] = 0.0
    db["residual_reduction"] = 1e-8
    db["multigrid_smoother"] = "jacobi"
    db["jacobi_damp"] = 0.8
    srv = m.Server(0, n_workers=2, db_cd=db, db_stokes=db)
    try:
        # kind 7 does not exist: submit refuses it
        rq = srv._Request()
        rq.kind = 7
        assert _lib.lib.pm_server_submit(srv.handle, C.byref(rq)) == PM_E_INVALID
        # geometry 9 does not exist: accepted, then failed by its set-up
        srv.submit(m.KIND_CD, 9, 1, 2, 2, 1, m.cd_coeffs(0.1, (1.0, 0.0, 0.0), 0.0, True), tag=11)
        # a good request after the bad ones
        srv.submit(m.KIND_CD, m.GEO_SQUARE_QUAD, 1, 4, 3, 1, m.cd_coeffs(0.1, (1.0, 0.0, 0.0), 0.0, True),
                   tag=12)
        srv.drain()
        res = {r["tag"]: r for r in srv.poll()}
        assert res[11]["status"] == PM_E_INVALID
        assert res[12]["status"] == 0 and res[12]["iterations"] > 0
    finally:
        srv.close()
