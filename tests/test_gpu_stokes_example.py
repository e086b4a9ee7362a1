"""The Stokes P2/P1 path on the reference's polynomial example -3
(include/Examples/NSE_3D/test_u_2_p_1.h, used by test/nse3d_solvers_test.c++):
u = (y^2, xz, -y^2), p = x + y + z - 3/2 lie in P2 / P1, so the discrete
solution is the exact one. Assembly (with the Dirichlet velocity values)
against the oracle within 1e-13; the solution by FGMRES + nodal Vanka
multigrid (3 levels, V(1,1), coarse direct solve of the projected matrix, in
FP64 and in the mixed form) reproduces the exact velocity within 1e-10 and the
mean-free pressure within 1e-9."""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from oracle import stokes as ost

from test_gpu_stokes import rel, stokes_db

pytestmark = pytest.mark.gpu


def example_db(precision):
    db = stokes_db(3, "nodal_vanka", 1.0, max_it=100, reduction=0.0, restart=60, precision=precision)
    db["residual_tolerance"] = 1e-13
    db.add("example", -3)
    return db


def exact(lv):
    X = lv.ucoords / lv.ucoords.max()
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    u = np.concatenate([y * y, x * z, -y * y])
    P = lv.pcoords / lv.pcoords.max()
    return u, P.sum(axis=1) - 1.5


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_stokes_polynomial_example_solved_exactly(ctx, precision):
    nlev = 3
    disc = m.Discretization(m.GEO_CUBE_TETRA, 1, 3, nlev, m.KIND_STOKES, 12)
    prob = m.StokesProblem(ctx, disc, 1.0, example_db(precision))
    prob.assemble()
    ora = ost.OracleStokes(1, 3, nlev, 1.0, example=-3)
    ora.assemble()
    assert rel(prob.rhs(), ora.rhs[-1]) <= 1e-13
    assert rel(prob.matrix(-1).values(), ora.vals[-1]) <= 1e-13
    prob.solve()
    lv = ora.finest
    u, pe = exact(lv)
    x = prob.solution()
    assert np.abs(x[: 3 * lv.nu] - u).max() <= 1e-10
    p = x[3 * lv.nu:]
    assert np.abs((p - p.mean()) - (pe - pe.mean())).max() <= 1e-9
    prob.close()
