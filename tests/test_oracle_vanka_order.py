"""How the colour-ordered multiplicative Vanka sweep of the GPU compares with
the reference's sequential sweep (src/Multigrid/VankaSmoother.C:138-271
visits the patches one after another; the GPU visits them colour by colour,
all patches of a colour from the same iterate). Both are multiplicative
Vanka smoothers over the same patches; only the order differs, so their
iterates differ and the solutions agree to the solver tolerance.

Measured with the oracle (FGMRES(30) to a 1e-10 residual reduction, V(1,1)
nodal Vanka on three levels, direct coarse solve, P2/P1 on 2^3 x 6 and 3^3 x 6
root tetrahedra refined twice; the 27 colours of the periodic lattice
colouring the library uses):
  damping 1.0: 20 (sequential) vs 18 (colours) iterations on the 2^3 root,
               23 vs 25 on the 3^3 root;
  damping 0.8: 14 vs 13 on both;
  velocities agree within 4e-10, mean-free pressures within 1.4e-6.
"""
import numpy as np
import pytest

from oracle import stokes as ost


def solve(root, kind, damp):
    o = ost.OracleStokes(root, 2, 3)
    o.assemble()
    o.build_mg(smoother=kind, coarse_smoother="direct_solve", n_pre=1, n_post=1, vanka_damp=damp)
    sol, it, res, hist, st = o.solve(0.0, 1e-10, 200, 30)
    nv = 3 * o.finest.nu
    o.close()
    assert st == 0 and res <= 1e-10 * hist[0]
    return sol, it, nv


@pytest.mark.parametrize("root,damp,its", [(2, 1.0, (20, 18)), (2, 0.8, (14, 13)), (3, 0.8, (14, 13))])
def test_colour_ordered_nodal_vanka_against_the_sequential_sweep(root, damp, its):
    seq, it_seq, nv = solve(root, "nodal", damp)
    col, it_col, _ = solve(root, "nodal_color", damp)
    assert (it_seq, it_col) == its
    assert np.abs(seq[:nv] - col[:nv]).max() <= 5e-10 * np.abs(seq[:nv]).max()
    ps, pc = seq[nv:] - seq[nv:].mean(), col[nv:] - col[nv:].mean()
    assert np.abs(ps - pc).max() <= 2e-6 * np.abs(ps).max()
