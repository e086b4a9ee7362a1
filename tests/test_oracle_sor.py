"""The oracle's SOR / SSOR (TMatrix::sor_sweep, src/Matrix/Matrix.C:943-1031;
Iteration_sor, src/Solver/Iteration_sor.C) on the CPU: the known-answer system
of test/iterative_solver_test.c++ with the SSOR preconditioner and omega 1.25,
the sweep against a plain restatement of the reference loop, and the
multicolour order the GPU sweeps use (a proper colouring, and the sequential
sweep over that order equals the colour-by-colour update). No GPU needed."""
import numpy as np
import pytest

from oracle import cd as ocd
from oracle import sor as osor
from test_oracle_golden import csr_from_dense, iterative_solver_system


def reference_loop(rp, ci, v, b, x, omega, flag):
    """TMatrix::sor_sweep as written: natural row order, b_row - sum a x,
    divided by the stored diagonal"""
    x = x.copy()
    n = rp.size - 1
    diag = np.zeros(n)
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            if ci[k] == i:
                diag[i] = v[k]
    passes = {0: [False], 1: [True], 2: [False, True]}[flag]
    for backward in passes:
        for r in range(n):
            row = n - 1 - r if backward else r
            s = b[row]
            for k in range(rp[row], rp[row + 1]):
                s -= v[k] * x[ci[k]]
            x[row] = x[row] + omega * s / diag[row]
    return x


@pytest.mark.parametrize("flag", [0, 1, 2])
def test_sweep_equals_reference_loop_bit_for_bit(flag):
    M = iterative_solver_system()
    rp, ci, v = csr_from_dense(M)
    rng = np.random.default_rng(1)
    b, x = rng.standard_normal(7), rng.standard_normal(7)
    got = ocd.sor_sweep(rp, ci, v, b, x, 1.25, np.arange(7, dtype=np.int32), flag)
    assert np.array_equal(got, reference_loop(rp, ci, v, b, x, 1.25, flag))


def test_zero_on_the_diagonal_is_refused():
    M = iterative_solver_system()
    M[2, 2] = 0.0
    M[2, 0] = 1.0  # keep the row non-empty
    rp, ci, v = csr_from_dense(M)
    with pytest.raises(ValueError, match="zero on the diagonal"):
        ocd.sor_sweep(rp, ci, v, np.ones(7), np.zeros(7), 1.5, np.arange(7, dtype=np.int32), 0)


@pytest.mark.parametrize("method", ["fgmres", "cg", "bi_cgstab"])
def test_iterative_solver_test_system_with_ssor_preconditioner(method):
    """test/iterative_solver_test.c++:104-160: preconditioner ssor, sor_omega
    1.25, exact solution x_i = i, error <= 100 * residual_tolerance"""
    M = iterative_solver_system()
    rp, ci, v = csr_from_dense(M)
    exact = np.arange(7.0)
    rhs = M @ exact
    sol = np.zeros(7)
    act = np.ones(7, np.uint8)
    order = np.arange(7, dtype=np.int32)
    it, res, nh = ocd.C.c_int(), ocd.C.c_double(), ocd.C.c_int()
    hist = np.zeros(2000)
    st = ocd.lib().orc_krylov_solve_sor({"fgmres": 0, "cg": 1, "bi_cgstab": 2}[method], 7, ocd._p(act),
                                        ocd._p(rp), ocd._p(ci), ocd._p(v), None, 2, ocd._p(order), 1.25, 1e-11,
                                        0.0, 1000, 0, 20, ocd._p(rhs), ocd._p(sol), ocd.C.byref(it),
                                        ocd.C.byref(res), ocd._p(hist), hist.size, ocd.C.byref(nh))
    assert st == 0
    assert np.linalg.norm(sol - exact) <= 100 * 1e-11


@pytest.mark.parametrize("flag", [0, 2])
def test_iterative_solver_test_system_sor_iteration(flag):
    """the same system solved by iterative_solver_type sor / ssor"""
    M = iterative_solver_system()
    rp, ci, v = csr_from_dense(M)
    exact = np.arange(7.0)
    rhs = M @ exact
    sol, it, res, hist = ocd.sor_iterate(rp, ci, v, np.ones(7, np.uint8), rhs, np.zeros(7), 1.25,
                                         np.arange(7, dtype=np.int32), flag, 1e-11, 0.0, 1000)
    assert it < 1000 and res < 1e-11
    assert np.linalg.norm(sol - exact) <= 100 * 1e-11


def _levels():
    o = ocd.OracleCD(0, 1, 3, 2, 2, eps=0.05, b=(0.6, 0.8), quad_points=3)
    o.assemble()
    return o


def test_greedy_colouring_is_proper():
    o = _levels()
    lv = o.finest
    colour = osor.greedy_colouring(lv.row_ptr, lv.cols)
    rows = np.repeat(np.arange(lv.n_dofs), np.diff(lv.row_ptr))
    off = rows != lv.cols
    assert np.all(colour[rows[off]] != colour[lv.cols[off]])
    # each row takes the smallest colour its earlier neighbours leave free
    assert colour[0] == 0 and colour.max() < 64


def test_colour_ordered_sweep_equals_colour_by_colour_update():
    """rows of one colour do not couple: updating a whole colour at once from
    the iterate before it gives the sequential sweep over the colour order
    (up to the summation order of each row, 1e-14)"""
    o = _levels()
    lv = o.finest
    rp, ci, v = lv.row_ptr, lv.cols, o.vals[-1]
    colour = osor.greedy_colouring(rp, ci)
    order = osor.colour_order(colour)
    rng = np.random.default_rng(2)
    b, x0 = rng.standard_normal(lv.n_dofs), rng.standard_normal(lv.n_dofs)
    seq = ocd.sor_sweep(rp, ci, v, b, x0, 1.5, order, 0)
    rows = np.repeat(np.arange(lv.n_dofs), np.diff(rp))
    diag = v[rows == ci][np.argsort(rows[rows == ci])]
    x = x0.copy()
    for k in range(colour.max() + 1):
        s = np.zeros(lv.n_dofs)
        np.add.at(s, rows, v * x[ci])
        sel = colour == k
        x[sel] = x[sel] + 1.5 * (b[sel] - s[sel]) / diag[sel]
    assert np.abs(x - seq).max() <= 1e-14 * max(1.0, np.abs(seq).max())
    # a different order gives a different sweep: the order matters
    nat = ocd.sor_sweep(rp, ci, v, b, x0, 1.5, np.arange(lv.n_dofs, dtype=np.int32), 0)
    assert np.abs(nat - seq).max() > 1e-6
