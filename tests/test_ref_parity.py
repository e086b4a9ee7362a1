"""Parity against the reference itself (CPU; no GPU needed).

The fixtures come from ParMooN's own classes, compiled from the reference
sources by oracle/ref/build_ref.py and run by tests/golden/make_ref_fixtures.py
(TDomain refinement, TFESpace2D/3D::ConstructSpace, TStructure,
ConvectionDiffusion<d>::assemble and ::solve with FGMRES + multigrid).

  * the library's host set-up (pm_disc_create: cell order, GlobalNumbers, CSR
    structure, cell vertices) is bit-identical to the reference's on every
    level, at the full sizes of the 2D Q1 128^2 and 3D Q2 32^3 workloads;
  * the oracle's element loop reproduces the reference's assembled entries and
    right-hand sides within 1e-13 (relative to the largest entry), and its
    FGMRES + multigrid solve takes the reference's iteration count with a
    solution within 1e-10;
  * Stokes P2/P1 (the reference's NavierStokes<3> as a Stokes problem on
    Default_UnitCube_Tetra, example -3): the library's velocity and pressure
    numbering and cell vertices are bit-identical on every level; the oracle's
    projected matrices equal the reference's combined matrices within 1e-13 and
    its direct solution the reference's (velocity 1e-12, mean-free pressure);
  * on the reference's SineLaplace example (Neumann boundary on x = 1) the
    oracle's error functional gives the reference's L2 / H1-semi / SD / L_inf
    errors of the same solution, and the oracle's own solutions reproduce the
    golden errors of test/cd2d_test.c++:91-98 within its 1e-11.
"""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from oracle import cd as ocd
from oracle import stokes as ost
from ref_fixtures import RefCase, StokesRefCase, digest, names, stokes_names


@pytest.mark.parametrize("name", names())
def test_setup_is_bit_identical_to_the_reference(name):
    rc = RefCase(name)
    disc = m.Discretization(rc.geometry, 1, rc.n_refine, rc.n_levels, m.KIND_CD, rc.elem,
                            neumann_sides=rc.neumann_sides)
    try:
        for l in range(rc.n_levels):
            ref = rc.level(l)
            info = disc.level_info(l)
            assert (info["n_cells"], info["nloc"], info["n_dofs"], info["n_active"], info["nnz"]) == \
                (ref["cells"], ref["nloc"], ref["n_dofs"], ref["active"], ref["nnz"]), (name, l)
            rp, ci = disc.structure(l)
            got = [digest(disc.dofmap(l), np.int32), digest(rp, np.int32), digest(ci, np.int32),
                   digest(disc.cell_vertices(l), np.float64)]
            assert got == [str(s) for s in ref["digests"]], (name, l)
    finally:
        disc.close()


@pytest.mark.parametrize("name", [n for n in names() if n != "cd3d_q2_32"])
def test_oracle_reproduces_the_reference_assembly_and_solve(name):
    rc = RefCase(name)
    ora = ocd.OracleCD(rc.geometry, 1, rc.n_refine, rc.n_levels, rc.elem, rc.eps, rc.b[:rc.dim], 0.0,
                       rc.quad_points, neumann_sides=rc.neumann_sides)
    ora.assemble()
    for l in range(rc.n_levels):
        assert rc.compare("vals", ora.vals[l], l) <= 1e-13, (name, l)
        assert rc.compare("rhs", ora.rhs[l], l) <= 1e-13, (name, l)
    ora.build_mg(2, 2, 0.8, 1.0, "V")
    sol, its, res, hist, st = ora.solve("fgmres", 0.0, rc.reduction, 1000, 0, rc.restart)
    assert st == 0
    assert abs(its - rc.iterations) <= 1, (its, rc.iterations)
    # the initial residual |b - A x0| of the reference's LoopInfo
    assert abs(hist[0] - rc.initial_residual) <= 1e-12 * rc.initial_residual
    assert rc.compare("solution", sol) <= 1e-10
    if rc.errors is not None:
        if rc.has("solution") and not rc.has("solution_idx"):
            # the functional alone, on the reference's own solution
            assert np.allclose(ora.errors(rc.z["solution"]), rc.errors, rtol=1e-13, atol=0), name
        assert np.allclose(ora.errors(sol), rc.errors, rtol=1e-9, atol=0), (ora.errors(sol), rc.errors)
    ora.close()


# test/cd2d_test.c++:91-98: SineLaplace on UnitSquare after 2 refinements,
# errors L2, H1-semi, SD, L_inf; the test's tolerance is 1e-11 (:42)
CD2D_GOLDEN = {1: (0.030136750989447, 0.50136473756928, 0.50136473756928, 0.086620472046938),
               2: (0.0019271846609828, 0.050971302154831, 0.050971302154831, 0.0033739148851507)}


@pytest.mark.parametrize("order", [1, 2])
def test_oracle_reproduces_the_cd2d_test_golden_errors(order):
    """the W-cycle multigrid run of cd2d_test (2 levels, 2+2 Jacobi with the
    default damping 1, direct coarse solve, residual_tolerance 1e-13) on the
    oracle"""
    ora = ocd.OracleCD(0, 1, 2, 2, order, 1.0, (0.0, 0.0), 0.0, 3 if order == 1 else 4, neumann_sides=2)
    ora.assemble()
    ora.build_mg(2, 2, 1.0, 1.0, "W")
    sol, its, res, hist, st = ora.solve("fgmres", 1e-13, 0.0, 1000, 0, 20)
    assert st == 0 and res <= 1e-13
    err = ora.errors(sol)
    assert np.abs(err - np.array(CD2D_GOLDEN[order])).max() <= 1e-11, err
    ora.close()



@pytest.mark.parametrize("name", stokes_names())
def test_stokes_setup_is_bit_identical_to_the_reference(name):
    rc = StokesRefCase(name)
    disc = m.Discretization(m.GEO_CUBE_TETRA, 1, rc.n_refine, rc.n_levels, m.KIND_STOKES, 12)
    try:
        for l in range(rc.n_levels):
            ref = rc.level(l)
            iu, ip = disc.level_info(l, 0), disc.level_info(l, 1)
            assert (iu["n_cells"], iu["n_dofs"], iu["n_active"], ip["n_dofs"], ip["n_active"]) == \
                (ref["cells"], ref["nu"], ref["nu_active"], ref["np"], ref["np_active"]), (name, l)
            got = [digest(disc.dofmap(l, 0), np.int32), digest(disc.dofmap(l, 1), np.int32),
                   digest(disc.cell_vertices(l), np.float64)]
            assert got == [str(s) for s in ref["digests"]], (name, l)
    finally:
        disc.close()


@pytest.mark.parametrize("name", stokes_names())
def test_oracle_stokes_assembly_matches_the_reference(name):
    rc = StokesRefCase(name)
    ora = ost.OracleStokes(1, rc.n_refine, rc.n_levels, 1.0, example=-3)
    ora.assemble()
    for l, lv in enumerate(ora.levels):
        assert rc.compare_matrix(l, lv.vrow_ptr, lv.vcols, ora.pvals[l]) <= 1e-13, (name, l)
        ref_rhs = rc.level(l)["rhs"]
        assert np.abs(ora.rhs[l] - ref_rhs).max() <= 1e-13 * float(rc.level(l)["rhs_max"]), (name, l)
    if rc.has("solution"):
        import scipy.sparse as sp
        import scipy.sparse.linalg as spla
        lv = ora.finest
        A = sp.csr_matrix((ora.pvals[-1], lv.vcols, lv.vrow_ptr), shape=(lv.n, lv.n))
        x = spla.spsolve(A.tocsc(), ora.rhs[-1])
        ref = rc.z["solution"]
        nu3 = 3 * lv.nu
        assert np.abs(x[:nu3] - ref[:nu3]).max() <= 1e-12 * np.abs(ref[:nu3]).max()
        p, pr = x[nu3:], ref[nu3:]
        assert np.abs((p - p.mean()) - (pr - pr.mean())).max() <= 1e-10
    ora.close()
