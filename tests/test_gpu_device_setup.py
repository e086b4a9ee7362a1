"""The set-up on the GPU (pm_disc_create_device): the mesh hierarchy by
regular refinement on the device, the first-touch DOF numbering by two
radix sorts, and the CSR structure and the assembly gather plans of every
convection-diffusion level by one stable radix sort of the element entries,
instead of the host construction. The discretisation must be the same array
for array: cell vertices, numbering, structure, prolongations, and - through
the gather plans and the Dirichlet node coordinates - the assembled matrices
and right-hand sides, bit for bit."""
import numpy as np
import pytest

import mymoonmd_gb300 as m

pytestmark = pytest.mark.gpu

CASES = [
    (m.GEO_SQUARE_QUAD, 2, 5, 3, 1, 0),   # 2D Q1 64^2 on a 2x2 root mesh
    (m.GEO_SQUARE_QUAD, 1, 4, 3, 2, 2),   # 2D Q2 16^2, Neumann side x = 1
    (m.GEO_SQUARE_QUAD, 1, 3, 2, 1, 10),  # 2D Q1 8^2, Neumann sides x = 1 and x = 0
    (m.GEO_CUBE_HEXA, 1, 3, 3, 1, 0),     # 3D Q1 8^3
    (m.GEO_CUBE_HEXA, 1, 4, 3, 2, 0),     # 3D Q2 16^3
    (m.GEO_CUBE_HEXA, 2, 2, 2, 2, 0),     # 3D Q2 8^3 on a 2x2x2 root mesh
    (m.GEO_CUBE_TETRA, 1, 3, 3, 11, 0),   # P1 on 8^3 cubes x 6 tetrahedra
    (m.GEO_CUBE_TETRA, 2, 2, 2, 12, 0),   # P2 on 8^3 cubes x 6 tetrahedra (2x2x2 root)
]


def db():
    d = m.ParameterDatabase.solve_path_database()
    d["solver_type"] = "iterative"
    d["iterative_solver_type"] = "fgmres"
    d["preconditioner"] = "multigrid"
    d["residual_tolerance"] = 0.0
    d["residual_reduction"] = 1e-10
    d["multigrid_smoother"] = "jacobi"
    d["jacobi_damp"] = 0.8
    return d


@pytest.mark.parametrize("case", CASES)
def test_device_setup_equals_the_host_setup(ctx, case):
    geo, root, nref, nlev, elem, neumann = case
    host = m.Discretization(geo, root, nref, nlev, m.KIND_CD, elem, neumann_sides=neumann)
    dev = m.Discretization(geo, root, nref, nlev, m.KIND_CD, elem, neumann_sides=neumann, ctx=ctx)
    probs = []
    try:
        for l in range(nlev):
            assert host.level_info(l) == dev.level_info(l)
            assert np.array_equal(host.cell_vertices(l), dev.cell_vertices(l)), l
            for a, b in zip(host.structure(l), dev.structure(l)):
                assert np.array_equal(a, b), l
            assert np.array_equal(host.dofmap(l), dev.dofmap(l))
            if l + 1 < nlev:
                for a, b in zip(host.prolongation(l)[:3], dev.prolongation(l)[:3]):
                    assert np.array_equal(a, b)
        dim_b = (1.0, 0.5, 0.25) if geo != m.GEO_SQUARE_QUAD else (1.0, 0.5)
        # a quadratic exact solution: its Dirichlet values come from the
        # coordinates of the boundary nodes of each numbering
        cf = m.cd_coeffs(0.05, dim_b, 0.0, poly=(0.3, 1.0, -0.5, 0.25, 0.7, -0.2, 0.4, 0.9, -0.6, 0.1))
        for d in (host, dev):
            p = m.ConvectionDiffusion(ctx, d, cf, db())
            p.assemble()
            probs.append(p)
        for l in range(nlev):
            assert np.array_equal(probs[0].matrix(l).values(), probs[1].matrix(l).values()), l
        assert np.array_equal(probs[0].rhs(), probs[1].rhs())
        for p in probs:
            p.solve()
        assert np.array_equal(probs[0].solution(), probs[1].solution())
    finally:
        for p in probs:
            p.close()
        host.close()
        dev.close()


def test_device_setup_time_of_the_32cube_q2_hierarchy(ctx):
    """the set-up of the 3D Q2 32^3 workload (4 levels): host construction
    against the GPU one (timings printed; the GPU one must be faster)"""
    import time
    t0 = time.perf_counter()
    host = m.Discretization(m.GEO_CUBE_HEXA, 1, 5, 4, m.KIND_CD, 2)
    t1 = time.perf_counter()
    dev = m.Discretization(m.GEO_CUBE_HEXA, 1, 5, 4, m.KIND_CD, 2, ctx=ctx)  # warm-up of the sort kernels
    dev.close()
    t2 = time.perf_counter()
    dev = m.Discretization(m.GEO_CUBE_HEXA, 1, 5, 4, m.KIND_CD, 2, ctx=ctx)
    t3 = time.perf_counter()
    try:
        for a, b in zip(host.structure(3), dev.structure(3)):
            assert np.array_equal(a, b)
        print(f"32^3 Q2 set-up: host {t1 - t0:.3f} s, GPU {t3 - t2:.3f} s")
        assert t3 - t2 < t1 - t0
    finally:
        host.close()
        dev.close()


def test_device_numbering_of_the_stokes_spaces(ctx):
    """the P2 velocity (Dirichlet) and P1 pressure (Neumann, all active)
    numberings and the combined structure of a Stokes set-up from the GPU:
    the same GlobalNumbers, level sizes and structure as the host set-up, and
    through the gather plans and the Dirichlet node coordinates the same
    assembled matrix and right-hand side of the polynomial example, bit for
    bit"""
    host = m.Discretization(m.GEO_CUBE_TETRA, 2, 2, 2, m.KIND_STOKES, 12)
    dev = m.Discretization(m.GEO_CUBE_TETRA, 2, 2, 2, m.KIND_STOKES, 12, ctx=ctx)
    probs = []
    try:
        for l in range(2):
            for space in (0, 1):
                assert host.level_info(l, space) == dev.level_info(l, space)
                assert np.array_equal(host.dofmap(l, space), dev.dofmap(l, space))
            assert np.array_equal(host.cell_vertices(l), dev.cell_vertices(l))
            for a, b in zip(host.structure(l), dev.structure(l)):
                assert np.array_equal(a, b)
        for d in (host, dev):
            sdb = db()
            sdb["multigrid_smoother"] = "nodal_vanka"
            sdb.add("example", -3)
            p = m.StokesProblem(ctx, d, 1.0, sdb)
            p.assemble()
            probs.append(p)
        assert np.array_equal(probs[0].rhs(), probs[1].rhs())
        assert np.array_equal(probs[0].matrix(-1).values(), probs[1].matrix(-1).values())
    finally:
        for p in probs:
            p.close()
        host.close()
        dev.close()


def test_device_setup_of_the_stokes_workload_mesh(ctx):
    """the Stokes workload's hierarchy (24^3 cubes x 6 tetrahedra, 3 levels)
    from the GPU set-up (refinement, both numberings, the combined structure
    and its gather plans): the same arrays as the host set-up (timings
    printed)"""
    import time
    t0 = time.perf_counter()
    host = m.Discretization(m.GEO_CUBE_TETRA, 3, 3, 3, m.KIND_STOKES, 12)
    t1 = time.perf_counter()
    dev = m.Discretization(m.GEO_CUBE_TETRA, 3, 3, 3, m.KIND_STOKES, 12, ctx=ctx)
    t2 = time.perf_counter()
    try:
        for l in range(3):
            for space in (0, 1):
                assert host.level_info(l, space) == dev.level_info(l, space)
                assert np.array_equal(host.dofmap(l, space), dev.dofmap(l, space))
            for a, b in zip(host.structure(l), dev.structure(l)):
                assert np.array_equal(a, b), l
            if l < 2:
                for a, b in zip(host.prolongation(l)[:3], dev.prolongation(l)[:3]):
                    assert np.array_equal(a, b)
        print(f"24^3 Stokes set-up: host {t1 - t0:.3f} s, GPU {t2 - t1:.3f} s")
    finally:
        host.close()
        dev.close()
