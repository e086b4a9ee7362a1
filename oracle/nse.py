"""Oracle Navier-Stokes P2/P1 driver (test infrastructure only).

Restates with numpy the nonlinear (Picard) loop of NavierStokes<3> for
problem_type 5 in the convective form (NSTYPE 4, LAPLACETYPE 0, Galerkin) on
the Stokes set-up of oracle.stokes, as the reference's
test/nse3d_solvers_test.c++ drives it:

  assemble_linear_terms  : src/System/NavierStokes.C:407-570 - the Stokes
                           blocks, the example's body force (which holds the
                           convective term) on the P5Tetra rule (degree 3 x 2
                           for nonlinear problems, src/FE/FEDatabase3D.C:
                           1153-1219) and the convective term of the current
                           velocity (zero at the start)
  convective term        : NSNonlinearTerm_convective
                           (src/AssembleRoutinesSaddle/
                           NSE_local_assembling_routines.C): (u . grad phi_j,
                           phi_i) added to A11, A22 and A33; or its
                           skew-symmetric form (NSNonlinearTerm_skew_symmetric)
  assemble_nonlinear_term: NavierStokes.C:573-750 - the finest velocity
                           restricted to every coarser level
                           (GridTransfer::RestrictFunction,
                           src/Multigrid/GridTransfer.C:1218-1501, with the
                           restriction matrices G^{-1} R of
                           TFEDatabase3D::GetRestrictionMatrix3D,
                           src/FE/FEDatabase3D.C:1771-1890), then the velocity
                           blocks reassembled
  compute_residuals      : NavierStokes.C:820-870, the pressure defect moved
                           into L2_0 (TFEFunction3D::project_into_L20,
                           src/FE/FEFunction3D.C:1678); the impuls residual
                           is the sum of the three velocity blocks' 2-norms
                           (BlockVector::norm, src/Matrix/BlockVector.C:293)
  stop_it                : NavierStokes.C:753-816
  solve                  : NavierStokes.C:878-913 with the direct solver on the
                           projected combined matrix, then the pressure moved
                           into L2_0

The Stokes blocks come from the C restatement behind oracle.stokes (P4Tetra:
their integrands are of degree 2, so both rules give them exactly).
"""
from __future__ import annotations

from collections import deque

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import refsetup
from .cd import _pk_values, _tet_rule
from .stokes import OracleStokes, StokesLevel


def _jacobians(lv: StokesLevel):
    """J (cells, 3, 3) with columns v1 - v0, v2 - v0, v3 - v0, and |det J|"""
    v = lv.verts.reshape(lv.n_cells, 4, 3)
    J = np.stack([v[:, a + 1, :] - v[:, 0, :] for a in range(3)], axis=2)
    return J, np.abs(np.linalg.det(J))


def convection_tensor(qn: int = 15, form: str = "convective") -> np.ndarray:
    """C[a, i, j, k] = sum_q w phi_i dhat_a phi_j phi_k on the reference cell;
    for the skew-symmetric form (NSNonlinearTerm_skew_symmetric: (1/2)
    [((u.grad) phi_j, phi_i) - ((u.grad) phi_i, phi_j)]) its antisymmetric
    part in (i, j)"""
    x, y, z, w = _tet_rule(qn)
    phi, dphi = _pk_values(12, x, y, z)
    C = np.einsum("q,qi,aqj,qk->aijk", w, phi, dphi, phi)
    if form == "skew_symmetric":
        return 0.5 * (C - np.transpose(C, (0, 2, 1, 3)))
    if form != "convective":
        raise ValueError("nonlinear forms: convective, skew_symmetric")
    return C


def restriction_matrices() -> np.ndarray:
    """Q_j = G^{-1} R_j (8, 10, 10) of P2 for the 8 children of the regular
    tetrahedral refinement, from the root cell of Default_UnitCube_Tetra and
    its children (GetRestrictionMatrix3D)"""
    meshes, _, scale = refsetup.hierarchy(refsetup.GEO_CUBE_TETRA, 1, 1)
    par = meshes[0][0].astype(np.float64) / scale
    kids = meshes[1][:8].astype(np.float64) / scale
    J = np.stack([par[a + 1] - par[0] for a in range(3)], axis=1)
    Ji = np.linalg.inv(J)
    x, y, z, w = _tet_rule(11)
    phi, _ = _pk_values(12, x, y, z)
    G = np.einsum("q,qi,qj->ij", w, phi, phi)
    Q = np.zeros((8, 10, 10))
    for j in range(8):
        xi = (Ji @ (kids[j] - par[0]).T).T          # child vertices in the parent's reference cell
        Jc = np.stack([xi[a + 1] - xi[0] for a in range(3)], axis=1)
        pts = xi[0][None, :] + np.stack([x, y, z], axis=1) @ Jc.T
        php, _ = _pk_values(12, pts[:, 0], pts[:, 1], pts[:, 2])
        R = np.einsum("q,qk,ql->kl", w * abs(np.linalg.det(Jc)), php, phi)
        Q[j] = np.linalg.solve(G, R)
    return Q


def nse_force(nu: float, x, y, z):
    """body force of example -3 (test_u_2_p_1) with the convective term:
    -nu Lap u + (u . grad) u + grad p for u = (y^2, xz, -y^2), p = x+y+z-3/2"""
    c0 = 2 * x * y * z
    c1 = y * y * z - x * y * y
    return np.stack([-2 * nu + c0 + 1, c1 + 1, 2 * nu - c0 + 1], axis=-1)


class OracleNSE:
    """NavierStokes<3> (problem_type 5, convective form, example -3) on the
    CPU with the direct solver."""

    def __init__(self, root_n: int, n_refine: int, n_levels: int, reynolds: float = 1.0,
                 form: str = "convective"):
        self.nu = 1.0 / reynolds
        self.stokes = OracleStokes(root_n, n_refine, n_levels, self.nu, example=-3)
        self.levels = self.stokes.levels
        self.C = convection_tensor(15, form)
        self.Q = restriction_matrices() if len(self.levels) > 1 else None
        self.x = np.zeros(self.levels[-1].n)
        self.u = [np.zeros(3 * lv.nu) for lv in self.levels]   # coarse velocities
        self.geo = [_jacobians(lv) for lv in self.levels]
        self.pw, self.measure = [], []
        for lv, (J, adet) in zip(self.levels, self.geo):
            w = np.zeros(lv.np_)
            np.add.at(w, lv.pdofmap.ravel(), np.repeat(adet / 24.0, 4))
            self.pw.append(w)
            self.measure.append(float(adet.sum() / 6.0))
        self.base, self.vals, self.rhs = [], [], []

    # -------------------------------------------------------------- pieces --
    def velocity(self, l: int) -> np.ndarray:
        return self.x[: 3 * self.levels[l].nu] if l == len(self.levels) - 1 else self.u[l]

    def convective_entries(self, l: int, u: np.ndarray):
        """(positions in the level's CSR, values) of the convective term"""
        lv = self.levels[l]
        J, adet = self.geo[l]
        G = np.transpose(np.linalg.inv(J), (0, 2, 1))    # J^{-T}: d_k = sum_a G[k, a] dhat_a
        uc = np.stack([u[d * lv.nu + lv.udofmap] for d in range(3)], axis=1)   # (cells, 3, 10)
        V = adet[:, None, None] * np.einsum("cda,cdk->cak", G, uc)
        N = np.einsum("cak,aijk->cij", V, self.C)
        rows, cols, vals = [], [], []
        for comp in range(3):
            d = lv.cdof[:, comp * 10: comp * 10 + 10].astype(np.int64)
            rows.append(np.repeat(d[:, :, None], 10, axis=2).ravel())
            cols.append(np.repeat(d[:, None, :], 10, axis=1).ravel())
            vals.append(N.ravel())
        r, c, v = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
        keep = lv.active[r] == 1
        r, c, v = r[keep], c[keep], v[keep]
        keys = np.repeat(np.arange(lv.n, dtype=np.int64), np.diff(lv.row_ptr)) * lv.n + lv.cols
        pos = np.searchsorted(keys, r * lv.n + c)
        assert np.all(keys[pos] == r * lv.n + c)
        return pos, v

    def _rhs(self, l: int) -> np.ndarray:
        lv = self.levels[l]
        J, adet = self.geo[l]
        x, y, z, w = _tet_rule(15)
        phi, _ = _pk_values(12, x, y, z)
        v0 = lv.verts.reshape(lv.n_cells, 4, 3)[:, 0, :]
        pts = v0[:, None, :] + np.einsum("cda,qa->cqd", J, np.stack([x, y, z], axis=1))
        f = nse_force(self.nu, pts[..., 0], pts[..., 1], pts[..., 2])          # (cells, q, 3)
        F = np.einsum("q,c,cqd,qi->cdi", w, adet, f, phi)                      # (cells, 3, 10)
        rhs = np.zeros(lv.n)
        idx = lv.cdof[:, :30].astype(np.int64).ravel()
        keep = lv.active[idx] == 1
        np.add.at(rhs, idx[keep], F.reshape(lv.n_cells, 30).ravel()[keep])
        rhs[lv.active == 0] = self.stokes.rhs[l][lv.active == 0]   # Dirichlet values u(node)
        return rhs

    def restrict(self, l: int, uf: np.ndarray) -> np.ndarray:
        """RestrictFunction from level l + 1 to level l (three components)"""
        cl, fl = self.levels[l], self.levels[l + 1]
        out = np.zeros(3 * cl.nu)
        cnt = np.bincount(cl.udofmap.ravel(), minlength=cl.nu).astype(np.float64)
        fd = fl.udofmap.reshape(cl.n_cells, 8, 10)
        for comp in range(3):
            vals = uf[comp * fl.nu + fd]                                     # (cells, 8, 10)
            cellval = np.einsum("jkl,cjl->ck", self.Q, vals)
            acc = np.zeros(cl.nu)
            np.add.at(acc, cl.udofmap.ravel(), cellval.ravel())
            out[comp * cl.nu: (comp + 1) * cl.nu] = acc / cnt
        return out

    def project_l20(self, l: int, p: np.ndarray) -> None:
        p -= float(self.pw[l] @ p) / self.measure[l]

    def matrix(self, l: int) -> sp.csr_matrix:
        lv = self.levels[l]
        return sp.csr_matrix((self.vals[l], lv.cols, lv.row_ptr), shape=(lv.n, lv.n))

    # ----------------------------------------------------------- interface --
    def assemble_linear_terms(self) -> None:
        self.stokes.assemble()
        self.base = [v.copy() for v in self.stokes.vals]
        self.rhs = [self._rhs(l) for l in range(len(self.levels))]
        self.vals = []
        for l in range(len(self.levels)):
            v = self.base[l].copy()
            pos, nv = self.convective_entries(l, self.velocity(l))
            np.add.at(v, pos, nv)
            self.vals.append(v)
        fin = self.levels[-1]
        self.x[fin.active == 0] = self.rhs[-1][fin.active == 0]

    def assemble_nonlinear_term(self) -> None:
        nl = len(self.levels)
        for l in range(nl - 2, -1, -1):
            self.u[l] = self.restrict(l, self.velocity(l + 1))
        for l in range(nl):
            v = self.base[l].copy()
            pos, nv = self.convective_entries(l, self.velocity(l))
            np.add.at(v, pos, nv)
            self.vals[l] = v

    def residuals(self):
        lv = self.levels[-1]
        d = self.rhs[-1] - self.matrix(len(self.levels) - 1) @ self.x
        p = d[3 * lv.nu:]
        self.project_l20(len(self.levels) - 1, p)
        # BlockVector::norm(blocks) (src/Matrix/BlockVector.C:293) sums the
        # 2-norms of the blocks: the impuls residual is |d_1| + |d_2| + |d_3|
        imp = sum(float(np.linalg.norm(d[b * lv.nu: (b + 1) * lv.nu])) for b in range(3))
        mass = float(np.linalg.norm(p))
        return imp, mass, np.sqrt(imp * imp + mass * mass)

    def solve(self) -> None:
        lv = self.levels[-1]
        pv = lv.project(self.vals[-1])
        A = sp.csr_matrix((pv, lv.vcols, lv.vrow_ptr), shape=(lv.n, lv.n)).tocsc()
        self.x = spla.spsolve(A, self.rhs[-1])
        self.project_l20(len(self.levels) - 1, self.x[3 * lv.nu:])

    def run(self, epsilon: float = 1e-10, max_it: int = 100, min_it: int = 1, slowfactor: float = 1e10):
        """the loop of test/nse3d_solvers_test.c++; returns the residuals of
        steps 0..n as an (n + 1, 3) array"""
        old = deque([1e10] * 10)
        hist = []

        def stop_it(k: int) -> bool:
            r = self.residuals()
            hist.append(r)
            old.append(r[2])
            old.popleft()
            if k < min_it:
                return False
            return r[2] <= epsilon or k == max_it or r[2] >= slowfactor * old[0]

        self.assemble_linear_terms()
        stop_it(0)
        k = 1
        while True:
            self.solve()
            self.assemble_nonlinear_term()
            if stop_it(k):
                break
            k += 1
        return np.array(hist)

    def close(self):
        self.stokes.close()
