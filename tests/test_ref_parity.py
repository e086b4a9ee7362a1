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
    solution within 1e-10.
"""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from oracle import cd as ocd
from ref_fixtures import RefCase, digest, names


@pytest.mark.parametrize("name", names())
def test_setup_is_bit_identical_to_the_reference(name):
    rc = RefCase(name)
    disc = m.Discretization(rc.geometry, 1, rc.n_refine, rc.n_levels, m.KIND_CD, rc.order)
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
    ora = ocd.OracleCD(rc.geometry, 1, rc.n_refine, rc.n_levels, rc.order, rc.eps, rc.b[:rc.dim], 0.0,
                       rc.quad_points)
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
    ora.close()
