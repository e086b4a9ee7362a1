"""The CPU oracle against the known-answer tests of the reference's own test
suite (test/matrix_test.c++, test/iterative_solver_test.c++,
test/block_fe_matrix_test.c++) and against properties of the multigrid cycle
control (src/Multigrid/CycleControl.C). No GPU needed."""
import numpy as np
import pytest

from oracle import cd as ocd


def csr_from_dense(M):
    rp, ci, v = [0], [], []
    for row in M:
        for j, a in enumerate(row):
            if a != 0:
                ci.append(j)
                v.append(a)
        rp.append(len(ci))
    return np.array(rp, np.int32), np.array(ci, np.int32), np.array(v, np.float64)


def matrix_test_CB():
    # matrices B (3x4) and C (4x3) of test/matrix_test.c++:40-73
    B = np.zeros((3, 4))
    B[0, 0], B[0, 3], B[1, 2], B[2, 1], B[2, 3] = 4, 1, 5, 6, 1
    C = np.zeros((4, 3))
    C[0, 0], C[0, 2], C[1, 0], C[1, 1], C[2, 1], C[2, 2], C[3, 0], C[3, 2] = 7, 8, 9, 10, 11, 12, 13, 14
    return C @ B


def test_matrix_test_multiply_known_answer():
    """test/matrix_test.c++:143-147: y = -0.5*CB*x"""
    rp, ci, v = csr_from_dense(matrix_test_CB())
    x = np.array([1.0, -2.5, 11.34, -0.004])
    y = np.zeros(4)
    lib = ocd.lib()
    lib.orc_multiply(4, ocd._p(rp), ocd._p(ci), ocd._p(v), ocd._p(x), ocd._p(y), -0.5)
    assert np.allclose(y, [46.03, -301.482, -221.826, 79.054], rtol=0, atol=1e-10)


def test_non_active_rows_act_as_identity():
    """test/block_fe_matrix_test.c++:236-252: a block matrix whose active blocks
    are zero, applied to ones, returns the non-active part of the vector (norm 4
    with 16 non-active DOFs)"""
    n, na = 40, 24
    rp = np.zeros(n + 1, np.int32)
    ci = np.zeros(0, np.int32)
    v = np.zeros(0)
    active = np.zeros(n, np.uint8)
    active[:na] = 1
    y = ocd.apply_scaled_add(rp, ci, v, active, np.ones(n), np.zeros(n), 1.0)
    assert np.linalg.norm(y) == 4.0


def iterative_solver_system():
    """the 7x7 block system [A C; B D] of test/iterative_solver_test.c++:13-100"""
    A = np.diag([5.5, 7.53, 10.0, 15.0])
    B = np.zeros((3, 4))
    B[0, 0], B[0, 3], B[1, 2], B[2, 1], B[2, 3] = 4, 1, 5, 6, 1
    D = np.array([[50, 0, 0], [0, 19, 0.1], [0, 0.1, 85.6]])
    M = np.block([[A, B.T], [B, D]])
    return M


@pytest.mark.parametrize("method", ["fgmres", "cg", "bi_cgstab"])
def test_iterative_solver_test_system(method):
    """exact solution x_i = i, rhs = M x; error <= 100 * residual_tolerance
    (test/iterative_solver_test.c++:104-160)"""
    M = iterative_solver_system()
    rp, ci, v = csr_from_dense(M)
    n = 7
    exact = np.arange(n, dtype=np.float64)
    rhs = M @ exact
    sol = np.zeros(n)
    act = np.ones(n, np.uint8)
    it, res, nh = ocd.C.c_int(), ocd.C.c_double(), ocd.C.c_int()
    hist = np.zeros(2000)
    st = ocd.lib().orc_krylov_solve({"fgmres": 0, "cg": 1, "bi_cgstab": 2}[method], n, ocd._p(act),
                                    ocd._p(rp), ocd._p(ci), ocd._p(v), None, 1e-11, 0.0, 1000, 0, 20,
                                    ocd._p(rhs), ocd._p(sol), ocd.C.byref(it), ocd.C.byref(res),
                                    ocd._p(hist), hist.size, ocd.C.byref(nh))
    assert st == 0
    assert np.linalg.norm(sol - exact) <= 100 * 1e-11


def test_cycle_control_sequences():
    """V/W cycle direction sequences of CycleControl::fill_recursively"""
    from mymoonmd_gb300 import _lib  # noqa: F401  (library loads without a GPU)
    # literal restatement in Python of CycleControl for 3 levels
    def seq(kind, n):
        rec = [1 if kind == "V" else 2] * n
        rec[n - 1] = 1
        out = ["Dummy"]

        def fill(level):
            if level == 0:
                out.append("Up")
                return
            for _ in range(rec[level]):
                out.append("Down")
                fill(level - 1)
            if kind == "F":
                rec[level] = 1
            out.append("End" if level == n - 1 else "Up")
        fill(n - 1)
        return out
    assert seq("V", 3) == ["Dummy", "Down", "Down", "Up", "Up", "End"]
    assert seq("W", 3) == ["Dummy", "Down", "Down", "Up", "Down", "Up", "Up", "End"]


def test_oracle_mg_fgmres_converges_2d():
    o = ocd.OracleCD(0, 1, 4, 3, 1, eps=0.1, b=(1.0, 0.0), quad_points=3)
    o.assemble()
    o.build_mg(2, 2, 0.8, 1.0, "V")
    sol, it, res, hist, st = o.solve("fgmres", 0.0, 1e-10, 100, 0, 20)
    assert st == 0 and res < 1e-10 * hist[0] and it < 20
    # discretisation error of Q1 on 16x16 against the manufactured solution
    lv = o.finest
    u = np.sin(np.pi * lv.node_coords[:, 0]) * np.sin(np.pi * lv.node_coords[:, 1])
    assert np.abs(sol - u).max() < 1e-2


def test_oracle_transfer_is_interpolation():
    """prolongation of a coarse Q2 function reproduces it at the fine nodes"""
    from oracle import refsetup
    lv = refsetup.cd_levels(1, 1, 2, 2, 2)
    c, f = lv
    rng = np.random.default_rng(0)
    # a trilinear function is in Q2: its prolongation is its interpolation
    g = lambda x: 1 + 2 * x[:, 0] - x[:, 1] + 0.5 * x[:, 2] + x[:, 0] * x[:, 1] * x[:, 2]
    pc = ocd.transfer(3, 2, c, f, g(c.node_coords), True)
    assert np.allclose(pc, g(f.node_coords), atol=1e-14)
    del rng


def _stokes_exact(X):
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    S = lambda t: np.sin(np.pi * t) ** 2
    D = lambda t: np.pi * np.sin(2 * np.pi * t)
    px, py, pz = D(x) * S(y) * S(z), S(x) * D(y) * S(z), S(x) * S(y) * D(z)
    return np.concatenate([py - pz, pz - px, px - py])


def test_oracle_stokes_converges_to_manufactured_solution():
    """P2/P1 restatement pinned by the manufactured solution u = curl(psi (1,1,1)):
    the nodal velocity error falls at least 3.5x per refinement (nodal-Vanka
    multigrid FGMRES to 1e-10)"""
    from oracle import stokes as ost
    errs = []
    for nref in (2, 3):
        o = ost.OracleStokes(1, nref, nref, 1.0)
        o.assemble()
        o.build_mg(smoother="nodal", vanka_damp=1.0, n_pre=1, n_post=1)
        sol, it, res, hist, st = o.solve(reduction=1e-10, max_it=100)
        assert st == 0 and it < 40
        lv = o.finest
        errs.append(np.abs(sol[: 3 * lv.nu] - _stokes_exact(lv.ucoords / lv.ucoords.max())).max())
    assert errs[0] < 0.2 and errs[1] < errs[0] / 3.5, errs


def test_cell_vanka_patches_on_cube_edges_are_singular_and_frozen():
    """cells with a rank-deficient velocity-pressure coupling have singular
    34x34 local matrices; with their pressures frozen every local matrix is
    regular"""
    import scipy.sparse as sp
    from oracle import stokes as ost
    o = ost.OracleStokes(1, 2, 1, 1.0)
    o.assemble()
    lv = o.finest
    V = sp.csr_matrix((o.pvals[-1], lv.vcols, lv.vrow_ptr), shape=(lv.n, lv.n)).tocsr()
    frozen = lv.n_freeze > 0
    assert 0 < frozen.sum() < lv.n_cells
    for c in np.nonzero(frozen)[0][:6]:
        d = lv.patch[c]
        M = V[d][:, d].toarray()
        assert np.linalg.cond(M) > 1e14
        M[30:, :] = 0
        M[:, 30:] = 0
        M[30:, 30:] = np.eye(4)
        assert np.linalg.cond(M) < 1e8
    for c in np.nonzero(~frozen)[0][:20]:
        d = lv.patch[c]
        assert np.linalg.cond(V[d][:, d].toarray()) < 1e8


def test_stokes_polynomial_example_is_reproduced_exactly():
    """include/Examples/NSE_3D/test_u_2_p_1.h (example -3 of the reference's
    nse3d_solvers_test): u = (y^2, xz, -y^2), p = x + y + z - 3/2 lie in P2 / P1,
    so the Galerkin solution of the Stokes system is the exact one. Direct
    solve of the projected system (first pressure row fixed), pressure
    compared after removing the nodal mean."""
    from oracle import stokes as ost
    o = ost.OracleStokes(1, 2, 2, 1.0, example=-3)
    o.assemble()
    lv = o.finest
    n = lv.n
    S = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(lv.vrow_ptr))
    S[rows, lv.vcols] = o.pvals[-1]
    x = np.linalg.solve(S, o.rhs[-1])
    X = lv.ucoords / lv.ucoords.max()
    xx, yy, zz = X[:, 0], X[:, 1], X[:, 2]
    u = np.concatenate([yy * yy, xx * zz, -yy * yy])
    assert np.abs(x[: 3 * lv.nu] - u).max() <= 1e-12
    P = lv.pcoords / lv.pcoords.max()
    pe = P.sum(axis=1) - 1.5
    p = x[3 * lv.nu:]
    assert np.abs((p - p.mean()) - (pe - pe.mean())).max() <= 1e-11
