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


# local P2 DOFs of a tetrahedron as pairs of its vertices (C_T_P2_3D order)
_P2_PAIRS = [(0, 0), (0, 1), (1, 1), (0, 2), (1, 2), (2, 2), (0, 3), (1, 3), (2, 3), (3, 3)]


def level_nodes(disc, level):
    """velocity (P2) and pressure (P1) node coordinates of a Stokes level in
    the library's numbering, and the P1 integral weights (sum of |K| / 4 over
    the cells of each pressure DOF), from its dofmaps and cell vertices"""
    v = disc.cell_vertices(level).reshape(-1, 4, 3)
    udm = disc.dofmap(level, 0).reshape(-1, 10)
    pdm = disc.dofmap(level, 1).reshape(-1, 4)
    nu, npr = disc.level_info(level, 0)["n_dofs"], disc.level_info(level, 1)["n_dofs"]
    uc = np.zeros((nu, 3))
    for k, (a, b) in enumerate(_P2_PAIRS):
        uc[udm[:, k]] = 0.5 * (v[:, a] + v[:, b])
    pc = np.zeros((npr, 3))
    for k in range(4):
        pc[pdm[:, k]] = v[:, k]
    J = np.stack([v[:, a + 1] - v[:, 0] for a in range(3)], axis=2)
    vol = np.abs(np.linalg.det(J)) / 6.0
    w = np.zeros(npr)
    np.add.at(w, pdm.ravel(), np.repeat(vol / 4.0, 4))
    return uc, pc, w, float(vol.sum())


def exact_on(uc, pc):
    x, y, z = uc[:, 0], uc[:, 1], uc[:, 2]
    return np.concatenate([y * y, x * z, -y * y]), pc.sum(axis=1) - 1.5


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


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_stokes_polynomial_example_at_the_workload_size(ctx, precision):
    """config 3's mesh (24^3 cubes x 6 tetrahedra, 368,572 unknowns) and
    smoother (nodal Vanka V(1,1) in colour order, damping 0.8, additive nodal
    Vanka on the 6^3 coarse level): the polynomial example is solved exactly,
    velocity within 1e-9 and the pressure within 2e-7 of the exact solution
    (at a 1e-12 residual the pressure of this 368,572-unknown system is
    determined to about 1e-7), the pressure in L2_0 after the solve"""
    import bench
    w = bench.WORKLOADS["stokes3d_p2p1_24"]
    db = bench.solver_db(w, precision)
    db["residual_tolerance"] = 1e-12
    db["residual_reduction"] = 0.0
    db.add("example", -3)
    disc = m.Discretization(m.GEO_CUBE_TETRA, w["root_n"], w["n_refine"], w["n_levels"], m.KIND_STOKES, 12)
    prob = m.StokesProblem(ctx, disc, w["nu"], db)
    try:
        prob.assemble()
        prob.solve()
        it, res, init = prob.last_info()
        assert res <= 1e-12 and it < 500
        uc, pc, wp, meas = level_nodes(disc, w["n_levels"] - 1)
        u, pe = exact_on(uc, pc)
        x = prob.solution()
        nu3 = 3 * uc.shape[0]
        assert np.abs(x[:nu3] - u).max() <= 1e-9
        p = x[nu3:]
        assert abs(float(wp @ p)) <= 1e-12  # NavierStokes::solve moved p into L2_0
        assert np.abs(p - (pe - float(wp @ pe) / meas)).max() <= 2e-7
    finally:
        prob.close()
        disc.close()
