"""The allocation-free assembly entry point (pm_assemble_cd_noalloc) against the
allocating one (pm_assemble_cd), through the C ABI.

pm_assemble_cd_noalloc is for callers that cannot call cudaMalloc when they
assemble - for instance a serving worker that must not stall requests already
running on the GPU with an allocation, or a host that reserved all device memory
up front. It keeps its scratch in a static device array of 32 MiB, so it must
give the same matrix and right-hand side as the allocating path (the same
element kernels: the same bits), call after call, agree with the oracle's
element loop, and refuse levels whose scratch would not fit.

This file is collected last so that a failure here comes after every other test
has run; it creates its own context and passes alone in a fresh process too.
"""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from oracle import cd as ocd

pytestmark = pytest.mark.gpu

# the same bound the other assembly parity tests use
TOL = 1e-13


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("quadrature_loop", [0, 1])
def test_noalloc_assembly_matches_allocating_assembly_twice(quadrature_loop):
    ctx = m.Context(0)
    try:
        # both entry points run the element kernel this option selects
        ctx.set_option("assembly_quadrature_loop", quadrature_loop)
        disc = m.Discretization(m.GEO_CUBE_HEXA, 1, 3, 3, m.KIND_CD, 2)  # 8^3 Q2, 3 levels
        cf = m.cd_coeffs(0.05, (1.0, 0.5, 0.25), 0.3, True)
        prob = m.ConvectionDiffusion(ctx, disc, cf, "solver_type: direct\n", quad_points=3)
        ora = ocd.OracleCD(m.GEO_CUBE_HEXA, 1, 3, 3, 2, 0.05, (1.0, 0.5, 0.25), 0.3, 3)
        ora.assemble()
        for level in range(disc.n_levels):
            info = disc.level_info(level)
            rp, ci = disc.structure(level)
            A = m.FEMatrix.from_csr(ctx, rp, ci, None, n_active=info["n_active"])
            rhs = m.DeviceVector(ctx, info["n_dofs"])
            m.assemble_cd(ctx, disc, level, cf, 3, A, rhs)  # existing entry point (allocates scratch)
            ref_vals, ref_rhs = A.values(), rhs.numpy()
            for _ in range(2):  # two calls in a row share the static scratch
                vals = m.DeviceVector(ctx, info["nnz"])
                r = m.DeviceVector(ctx, info["n_dofs"])
                prob.assemble_level_noalloc(level, vals, r, cf)
                got_vals, got_rhs = vals.numpy(), r.numpy()
                assert np.array_equal(got_vals, ref_vals)
                assert np.array_equal(got_rhs, ref_rhs)
                # and the oracle's element loop, within the assembly tolerance
                assert rel(got_vals, ora.vals[level]) <= TOL
                assert rel(got_rhs, ora.rhs[level]) <= TOL
        prob.close()
    finally:
        ctx.close()


def test_noalloc_assembly_refuses_stokes_problems():
    ctx = m.Context(0)
    try:
        disc = m.Discretization(m.GEO_CUBE_TETRA, 1, 1, 2, m.KIND_STOKES, 12)
        prob = m.StokesProblem(ctx, disc, 1.0, "solver_type: direct\n")
        info = disc.level_info(1)
        vals = m.DeviceVector(ctx, info["nnz"])
        r = m.DeviceVector(ctx, info["n_dofs"])
        with pytest.raises(m.PmError, match="convection-diffusion problems only"):
            prob.assemble_level_noalloc(1, vals, r)
        prob.close()
    finally:
        ctx.close()


def test_noalloc_assembly_rejects_levels_beyond_its_scratch():
    ctx = m.Context(0)
    try:
        # 24^3 Q2 hexahedra need 13824 * 27 * 28 doubles > 4 Mi
        disc = m.Discretization(m.GEO_CUBE_HEXA, 3, 3, 2, m.KIND_CD, 2)
        cf = m.cd_coeffs(0.1, (1.0, 0.0, 0.0), 0.0, True)
        prob = m.ConvectionDiffusion(ctx, disc, cf, "solver_type: direct\n", quad_points=3)
        info = disc.level_info(1)
        vals = m.DeviceVector(ctx, info["nnz"])
        r = m.DeviceVector(ctx, info["n_dofs"])
        with pytest.raises(m.PmError, match="scratch"):
            prob.assemble_level_noalloc(1, vals, r)
        prob.assemble_level_noalloc(0, m.DeviceVector(ctx, disc.level_info(0)["nnz"]),
                                    m.DeviceVector(ctx, disc.level_info(0)["n_dofs"]))
        prob.close()
    finally:
        ctx.close()


def test_noalloc_assembly_writes_the_dirichlet_values():
    """the quadratic exact-solution example (x^2 + yz, example -3 of
    test/cd3d_solvers_test.c++): the Dirichlet rows of the right-hand side get
    the exact solution's values, as in the allocating assembly"""
    ctx = m.Context(0)
    try:
        disc = m.Discretization(m.GEO_CUBE_HEXA, 1, 2, 2, m.KIND_CD, 2)
        cf = m.cd_coeffs(1.0, (4.0, 3.0, 2.0), 1.0, True, poly=[0, 0, 0, 0, 1.0, 0, 0, 0, 0, 1.0])
        prob = m.ConvectionDiffusion(ctx, disc, cf, "solver_type: direct\n", quad_points=3)
        info = disc.level_info(1)
        rp, ci = disc.structure(1)
        A = m.FEMatrix.from_csr(ctx, rp, ci, None, n_active=info["n_active"])
        rhs = m.DeviceVector(ctx, info["n_dofs"])
        m.assemble_cd(ctx, disc, 1, cf, 3, A, rhs)
        vals = m.DeviceVector(ctx, info["nnz"])
        r = m.DeviceVector(ctx, info["n_dofs"])
        prob.assemble_level_noalloc(1, vals, r, cf)
        assert rel(vals.numpy(), A.values()) <= TOL
        assert rel(r.numpy(), rhs.numpy()) <= TOL
        assert np.abs(r.numpy()[info["n_active"]:]).max() > 0.5
        prob.close()
    finally:
        ctx.close()
