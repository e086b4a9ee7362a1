"""The oracle's Navier-Stokes restatement (oracle/nse.py) against the
compiled reference's fixtures: one assemble_nonlinear_term from a fixed
finest velocity (every level's combined matrix and restricted velocity:
the convective or skew-symmetric term and GridTransfer::RestrictFunction),
and the nonlinear loop of test/nse3d_solvers_test.c++ with the direct solver
at Reynolds numbers 1 and 100 in both forms (the residuals of every step, the
number of steps, the solution and the known answer: the exact solution of
example -3 lies in P2 / P1)."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import nse
from ref_fixtures import NseRefCase, nse_names


@pytest.mark.parametrize("name", nse_names("none"))
def test_nonlinear_assembly_matches_the_reference(name):
    rc = NseRefCase(name)
    o = nse.OracleNSE(1, rc.n_refine, rc.n_levels, rc.reynolds, rc.form)
    o.assemble_linear_terms()
    fin = o.levels[-1]
    o.x = rc.fixed_velocity(fin.nu, fin.n)
    o.assemble_nonlinear_term()
    for l, lv in enumerate(o.levels):
        d = rc.level(l)
        assert (d["cells"], d["nu"], d["nu_active"], d["np"]) == (lv.n_cells, lv.nu, lv.nu_active, lv.np_)
        u = o.velocity(l)
        assert np.abs(u - d["velocity"]).max() <= 1e-14 * np.abs(d["velocity"]).max() * 10
        pv = lv.project(o.vals[l])
        assert rc.compare_matrix(l, lv.vrow_ptr, lv.vcols, pv) <= 1e-14 * 10


@pytest.mark.parametrize("name", nse_names("direct"))
def test_picard_loop_matches_the_reference(name):
    rc = NseRefCase(name)
    o = nse.OracleNSE(1, rc.n_refine, rc.n_levels, rc.reynolds, rc.form)
    hist = o.run(rc.epsilon, rc.maxit)
    ref = rc.z["residuals"]
    assert hist.shape == ref.shape
    # the residuals of the steps agree while they are well above rounding
    big = ref[:, 2] > 1e-8 * ref[0, 2]
    assert np.all(np.abs(hist[big, 2] - ref[big, 2]) <= 1e-6 * ref[big, 2])
    # the mass residual: the reference's before the first solve, rounding after
    assert abs(hist[0, 1] - ref[0, 1]) <= 1e-12 * ref[0, 1]
    assert np.all(hist[1:, 1] <= 1e-13)
    idx, sol = rc.full_solution(o.x.size)
    nu3 = 3 * o.levels[-1].nu
    assert np.abs(o.x[:nu3] - sol[:nu3]).max() <= 1e-10
    p, pr = o.x[nu3:], sol[nu3:]
    assert np.abs(p - pr).max() <= 1e-9
    # the known answer: the reference's errors are at rounding level
    assert np.all(rc.z["errors"][:5] <= 1e-8)


def test_residual_is_zero_for_the_exact_solution_and_block_norms_sum():
    """with the interpolant of the exact solution the nonlinear residual is at
    rounding level; the impuls residual sums the three blocks' 2-norms"""
    o = nse.OracleNSE(1, 2, 1, 1.0)
    o.assemble_linear_terms()
    lv = o.levels[-1]
    X = lv.ucoords / lv.ucoords.max()
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    P = lv.pcoords / lv.pcoords.max()
    o.x = np.concatenate([y * y, x * z, -y * y, P.sum(axis=1) - 1.5])
    o.assemble_nonlinear_term()
    r = o.residuals()
    assert r[2] <= 1e-12
    d = o.rhs[-1] - sp.csr_matrix((o.vals[-1], lv.cols, lv.row_ptr)) @ np.zeros(lv.n)
    imp = sum(np.linalg.norm(d[b * lv.nu:(b + 1) * lv.nu]) for b in range(3))
    o.x[:] = 0
    assert abs(o.residuals()[0] - imp) <= 1e-12 * imp


def test_restriction_reproduces_coarse_p2_functions():
    """RestrictFunction is a projection: a function of the coarse P2 space,
    prolongated, restricts to itself"""
    o = nse.OracleNSE(1, 2, 2, 1.0)
    cl, fl = o.levels
    X = cl.ucoords / cl.ucoords.max()
    Xf = fl.ucoords / fl.ucoords.max()
    f = lambda X: 1 + X[:, 0] - 2 * X[:, 1] * X[:, 2] + 3 * X[:, 0] ** 2
    uc = np.concatenate([f(X), 2 * f(X), -f(X)])
    uf = np.concatenate([f(Xf), 2 * f(Xf), -f(Xf)])
    assert np.abs(o.restrict(0, uf) - uc).max() <= 1e-13
