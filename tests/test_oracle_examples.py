"""The oracle on the known-answer examples of test/cd3d_solvers_test.c++
(examples -1, -2, -3 of src/Examples/Example_CD3D.C:164-193: exact solutions
1, 1+2x+3y+4z and x^2+yz, which lie in Q1 / Q1 / Q2): on the hexahedral unit
cube with two refinements the discrete solution is the exact one, to 1e-12
with FGMRES + multigrid (W-cycle, two levels, SOR 3+3, correction damping 0.8,
coarse direct solve; :88-106). No GPU needed.

The reference's test measures the L2 and H1 errors; here the error is taken at
the nodes. A discrete solution that equals the exact solution in the space
has zero nodal error and zero L2 / H1 error alike."""
import numpy as np
import pytest

from oracle import cd as ocd

# example: element, eps, b, c, coefficients of u (1, x, y, z, x^2, y^2, z^2, xy, xz, yz)
EXAMPLES = {
    -1: (1, 1.0, (1.0, 1.0, 1.0), 1.0, [1.0]),
    -2: (1, 1.0, (1.0, 2.0, 3.0), 0.0, [1.0, 2.0, 3.0, 4.0]),
    -3: (2, 1.0, (4.0, 3.0, 2.0), 1.0, [0, 0, 0, 0, 1.0, 0, 0, 0, 0, 1.0]),
}


def reference_rhs(example, x, y, z):
    """f as written in the examples' BilinearCoeffs (test_p0.h, test_p1.h,
    test_p2.h)"""
    if example == -1:
        return 1.0
    if example == -2:
        return 1 * 2 + 2 * 3 + 3 * 4
    return -1.0 * 2 + 4 * 2 * x + 3 * z + 2 * y + 1 * (x * x + y * z)


def oracle_example(example, n_levels=2, tetra=False):
    """hexahedra (Q1 / Q2, Gauss3) or, with tetra, the tetrahedral unit cube
    Default_UnitCube_Tetra (P1 / P2 on the reference's default rules P4Tetra /
    P5Tetra), two refinements"""
    elem, eps, b, c, poly = EXAMPLES[example]
    if tetra:
        o = ocd.OracleCD(2, 1, 2, n_levels, 10 + elem, eps=eps, b=b, c=c, quad_points=11 if elem == 1 else 15,
                         poly=poly)
    else:
        o = ocd.OracleCD(1, 1, 2, n_levels, elem, eps=eps, b=b, c=c, quad_points=3, poly=poly)
    o.assemble()
    return o


@pytest.mark.parametrize("example", [-1, -2, -3])
def test_polynomial_rhs_equals_the_examples_formula(example):
    """the oracle's generic f = -eps Lap u + b.grad u + c u of the quadratic
    family (orc_poly_rhs, which the assembly evaluates at the quadrature
    points) is the examples' f, at random points"""
    elem, eps, b, c, poly = EXAMPLES[example]
    p = np.array(poly + [0.0] * (10 - len(poly)))
    bb = np.array(b)
    rng = np.random.default_rng(example + 10)
    for x in rng.random((20, 3)):
        x = np.ascontiguousarray(x)
        f = ocd.lib().orc_poly_rhs(3, ocd._p(x), eps, ocd._p(bb), c, ocd._p(p), None)
        assert abs(f - reference_rhs(example, *x)) <= 1e-14 * max(1.0, abs(f))


@pytest.mark.parametrize("tetra", [False, True])
@pytest.mark.parametrize("example", [-1, -2, -3])
def test_cd3d_solvers_polynomial_examples_are_solved_exactly(example, tetra):
    """both halves of test/cd3d_solvers_test.c++: hexahedra (Q1, Q1, Q2) and
    tetrahedra (P1, P1, P2)"""
    o = oracle_example(example, tetra=tetra)
    lv = o.finest
    o.build_mg(3, 3, 0.8, 0.8, "W", smoother="sor", sor_omega=1.5)
    sol, it, res, hist, st = o.solve("fgmres", 1e-15, 0.0, 100, 0, 20)
    exact = np.array([o.exact(x) for x in lv.node_coords])
    assert np.abs(sol - exact).max() <= 1e-12
    # the Dirichlet rows carry the exact values
    assert np.array_equal(o.rhs[-1][lv.n_active:], exact[lv.n_active:])
