"""The oracle's time-dependent convection-diffusion (oracle/tcd.py) on the
known-answer examples of test/tcd3d_solvers_test.c++ (examples -2 and -1 of
src/Examples/Example_TimeCD3D.C:27-48): u = 1 + 2x + 3ty + 4tz (Q1, linear in
time) and u = t^2 (x^2 + yz) (Q2, quadratic in time) on the hexahedral unit
cube with two refinements, time step 0.1 up to time 1. A scheme that is exact
for the time dependence reproduces the exact solution at every step: backward
Euler and BDF2 (its first step by backward Euler) for the linear one,
Crank-Nicolson for both. The reference requires zero errors within 1e-12
(multigrid, :111-133) and 1e-13 (direct). No GPU needed."""
import numpy as np
import pytest

from oracle import tcd as otcd

# name: element, eps, b, c, P0, (P1, P2)
EXAMPLES = {
    "linear_space_time": (1, 1.0, (1.0, 2.0, 3.0), 0.0, [1.0, 2.0], ([0.0, 0.0, 3.0, 4.0], [0.0])),
    "quadratic_space_time": (2, 1.0, (4.0, 3.0, 2.0), 1.0, [0.0], ([0.0], [0, 0, 0, 0, 1.0, 0, 0, 0, 0, 1.0])),
}

MG = dict(n_pre=3, n_post=3, jacobi_damp=0.8, correction_damp=0.8, cycle="W", smoother="sor", sor_omega=1.5)


def run(example, scheme, solver):
    elem, eps, b, c, p0, pt = EXAMPLES[example]
    o = otcd.OracleTCD(1, 1, 2, 2, elem, eps, b, c, 3, poly=p0, poly_time=pt, scheme=scheme, tau=0.1, t_end=1.0)
    o.assemble_initial_time()
    errs = []
    while o.t < o.t_end - 1e-10:
        o.next_step()
        o.assemble()
        o.solve(solver, MG)
        exact = np.array([o.exact(o.t, x) for x in o.cd.finest.node_coords])
        errs.append(np.abs(o.sol - exact).max())
    return o, errs


@pytest.mark.parametrize("example,scheme", [("linear_space_time", "backward_euler"),
                                            ("linear_space_time", "crank_nicolson"),
                                            ("linear_space_time", "bdf_two"),
                                            ("quadratic_space_time", "crank_nicolson")])
@pytest.mark.parametrize("solver,tol", [("multigrid", 1e-12), ("direct", 1e-13)])
def test_exact_in_time_examples_stay_exact(example, scheme, solver, tol):
    o, errs = run(example, scheme, solver)
    assert o.step == 10
    assert max(errs) <= tol, errs


def test_backward_euler_is_not_exact_for_quadratic_time_dependence():
    """the check has teeth: backward Euler on the quadratic-in-time example
    leaves a first-order time error"""
    o, errs = run("quadratic_space_time", "backward_euler", "direct")
    assert max(errs) > 1e-3
