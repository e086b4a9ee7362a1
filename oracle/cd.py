"""Oracle drivers (test infrastructure only): convection-diffusion assembly,
multigrid and Krylov solves of the C restatement in oracle.c, on the set-up of
refsetup.py.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build as _build
from . import refsetup
from . import sor as _sor

# smoother codes of orc_mg (oracle.c)
SMOOTHERS = {"jacobi": 0, "direct_solve": 1, "sor": 5, "ssor": 6}

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        vp, i32, f64 = C.c_void_p, C.c_int, C.c_double
        L.orc_apply_scaled_add.argtypes = [i32, vp, vp, vp, vp, vp, vp, f64]
        L.orc_multiply.argtypes = [i32, vp, vp, vp, vp, vp, f64]
        L.orc_dot.argtypes = [i32, vp, vp]
        L.orc_dot.restype = f64
        L.orc_assemble_cd.argtypes = [i32, i32, i32, i32, vp, i32, vp, i32, i32, vp, vp, f64, vp, f64, i32,
                                      f64, vp, vp]
        L.orc_mg_create.argtypes = [i32, i32, i32, f64, f64, i32, i32, i32, f64]
        L.orc_mg_create.restype = vp
        L.orc_mg_set_level.argtypes = [vp, i32, i32, vp, vp, vp, vp]
        L.orc_mg_set_transfer.argtypes = [vp, i32, i32, i32, i32, i32, vp, vp, vp, vp, vp, i32, i32]
        L.orc_mg_finalize.argtypes = [vp]
        L.orc_mg_finalize.restype = i32
        L.orc_mg_destroy.argtypes = [vp]
        L.orc_mg_apply.argtypes = [vp, vp, vp]
        L.orc_krylov_solve.argtypes = [i32, i32, vp, vp, vp, vp, vp, f64, f64, i32, i32, i32, vp, vp,
                                       C.POINTER(i32), C.POINTER(f64), vp, i32, C.POINTER(i32)]
        L.orc_prolongate_flat.argtypes = [i32, i32, i32, i32, vp, vp, vp, vp, vp, i32, i32, vp, vp]
        L.orc_restrict_flat.argtypes = [i32, i32, i32, i32, vp, vp, vp, vp, vp, i32, i32, vp, vp]
        L.orc_assemble_cd_poly.argtypes = [i32, i32, i32, i32, vp, i32, vp, i32, i32, vp, vp, f64, vp, f64,
                                           i32, f64, vp, vp, vp]
        L.orc_poly_u.argtypes = [vp, vp]
        L.orc_poly_u.restype = f64
        L.orc_poly_rhs.argtypes = [i32, vp, f64, vp, f64, vp, vp]
        L.orc_poly_rhs.restype = f64
        L.orc_sor_sweep.argtypes = [i32, vp, vp, vp, vp, vp, f64, vp, i32]
        L.orc_sor_sweep.restype = i32
        L.orc_mg_set_sor.argtypes = [vp, i32, vp, f64]
        L.orc_mg_set_smoothers.argtypes = [vp, i32, i32, f64]
        L.orc_krylov_solve_sor.argtypes = [i32, i32, vp, vp, vp, vp, vp, i32, vp, f64, f64, f64, i32, i32, i32, vp,
                                           vp, C.POINTER(i32), C.POINTER(f64), vp, i32, C.POINTER(i32)]
        L.orc_lu_factor.argtypes = [i32, vp, vp]
        L.orc_lu_solve.argtypes = [i32, vp, vp, vp]
        _lib = L
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def apply_scaled_add(rp, ci, v, active, x, y, a):
    """BlockFEMatrix::apply_scaled_add on the CPU; returns the new y"""
    y = np.array(y, dtype=np.float64, copy=True)
    act = np.ascontiguousarray(active, dtype=np.uint8)
    rp = np.ascontiguousarray(rp, dtype=np.int32)
    ci = np.ascontiguousarray(ci, dtype=np.int32)
    v = np.ascontiguousarray(v, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    lib().orc_apply_scaled_add(rp.size - 1, _p(act), _p(rp), _p(ci), _p(v), _p(x), _p(y), a)
    return y


def sor_sweep(rp, ci, v, b, x, omega, order, flag):
    """TMatrix::sor_sweep (src/Matrix/Matrix.C:943-1031) over the rows in
    `order` (flag 0 forward, 1 backward, 2 forward then backward); returns the
    new x"""
    x = np.array(x, dtype=np.float64, copy=True)
    rp = np.ascontiguousarray(rp, dtype=np.int32)
    ci = np.ascontiguousarray(ci, dtype=np.int32)
    v = np.ascontiguousarray(v, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    order = np.ascontiguousarray(order, dtype=np.int32)
    if lib().orc_sor_sweep(rp.size - 1, _p(rp), _p(ci), _p(v), _p(b), _p(x), omega, _p(order), flag) != 0:
        raise ValueError("There is a zero on the diagonal. You can not use `sor` in this case")
    return x


def sor_iterate(rp, ci, v, active, rhs, sol, omega, order, flag, tol, reduction, max_it, min_it=0,
                divergence=1e10, stagnation=1e10):
    """Iteration_sor::iterate (src/Solver/Iteration_sor.C:24-60) with the
    stopping test of IterativeMethod::converged (include/Solver/IterativeMethod.h:81-135);
    returns (solution, iterations, residual, history)"""
    x = np.array(sol, dtype=np.float64, copy=True)
    r = apply_scaled_add(rp, ci, v, active, x, rhs, -1.0)
    normb = float(np.linalg.norm(rhs)) or 1.0
    hist = []

    def converged(res, it):
        hist.append(res)
        init, prev = hist[0], hist[-2] if len(hist) > 1 else hist[0]
        if res > divergence * init:
            raise RuntimeError("solver divergence")
        conv = (res < tol or res < reduction * init or res > stagnation * prev) and (it > min_it or min_it == 0)
        return conv or it == max_it

    res = float(np.linalg.norm(r)) / normb
    if converged(res, 0):
        return x, 0, res, np.array(hist)
    for i in range(1, max_it + 1):
        x = sor_sweep(rp, ci, v, rhs, x, omega, order, flag)
        r = apply_scaled_add(rp, ci, v, active, x, rhs, -1.0)
        res = float(np.linalg.norm(r)) / normb
        if converged(res, i):
            return x, i, res, np.array(hist)
    return x, max_it, res, np.array(hist)


def transfer(dim: int, k: int, coarse_level, fine_level, vec: np.ndarray, prolongate: bool) -> np.ndarray:
    """GridTransfer::Prolongate (prolongate=True, vec on the coarse level) or
    DefectRestriction (vec on the fine level) on the CPU"""
    fd = np.ascontiguousarray(fine_level.dofmap, dtype=np.int32)
    cd = np.ascontiguousarray(coarse_level.dofmap, dtype=np.int32)
    fv = np.ascontiguousarray(fine_level.verts, dtype=np.float64)
    cv = np.ascontiguousarray(coarse_level.verts, dtype=np.float64)
    par = np.ascontiguousarray(fine_level.parent, dtype=np.int32)
    vec = np.ascontiguousarray(vec, dtype=np.float64)
    args = (dim, k, fine_level.n_cells, fine_level.nloc, _p(fd), _p(cd), _p(par), _p(fv), _p(cv),
            fine_level.n_dofs, coarse_level.n_dofs)
    if prolongate:
        out = np.zeros(fine_level.n_dofs)
        lib().orc_prolongate_flat(*args, _p(vec), _p(out))
    else:
        out = np.zeros(coarse_level.n_dofs)
        lib().orc_restrict_flat(*args, _p(out), _p(vec))
    return out


def _gauss(n: int):
    """Gauss-Legendre points and weights on [-1, 1]"""
    return np.polynomial.legendre.leggauss(n)


def _lag1d(k: int, x: np.ndarray):
    """Lagrange basis of degree k on the nodes -1, (0,) 1 and its derivative"""
    if k == 1:
        return [0.5 * (1 - x), 0.5 * (1 + x)], [np.full_like(x, -0.5), np.full_like(x, 0.5)]
    return ([0.5 * x * (x - 1), 1 - x * x, 0.5 * x * (x + 1)], [x - 0.5, -2 * x, x + 0.5])


def _qk_values(k: int, d: int, xi: np.ndarray):
    """values (points, nb) and reference derivatives (d, points, nb) of the
    lexicographic Qk basis at reference points xi (points, d)"""
    L = [_lag1d(k, xi[:, a]) for a in range(d)]
    vals, ders = [], [[] for _ in range(d)]
    idx = [(a, b, 0) for b in range(k + 1) for a in range(k + 1)] if d == 2 else \
        [(a, b, c) for c in range(k + 1) for b in range(k + 1) for a in range(k + 1)]
    for t in idx:
        v = np.ones(xi.shape[0])
        for a in range(d):
            v = v * L[a][0][t[a]]
        vals.append(v)
        for da in range(d):
            g = np.ones(xi.shape[0])
            for a in range(d):
                g = g * (L[a][1][t[a]] if a == da else L[a][0][t[a]])
            ders[da].append(g)
    return np.stack(vals, axis=1), np.stack([np.stack(dd, axis=1) for dd in ders])


# the reference's tetrahedral rules (src/QuadFormulas/QuadFormulaTetra.C,
# P4Exact / P5Exact), points in its order, weights summing to 1/6
def _tet_rule(n: int):
    """(x, y, z, w) of the P4Tetra (11 points) or P5Tetra (15 points) rule"""
    if n == 11:
        a, b = 0.399403576166799204996102147462, 0.100596423833200795003897852538
        t1, t2 = 0.0714285714285714285714285714286, 0.785714285714285714285714285714
        x = [.25, t1, t2, t1, t1, a, a, b, b, b, a]
        y = [.25, t1, t1, t2, t1, a, b, a, b, a, b]
        z = [.25, t1, t1, t1, t2, b, a, a, a, b, b]
        w = [-.0131555555555555555555555555556] + [.00762222222222222222222222222222] * 4 + \
            [.0248888888888888888888888888889] * 6
    elif n == 15:
        a, b = 0.066550153573664298239880464226303, 0.43344984642633570176011953577370
        e, g = 1 / 11, 8 / 11
        x = [1 / 3, 1 / 3, 0, 1 / 3, .25, e, e, g, e, a, b, b, a, a, b]
        y = [1 / 3, 0, 1 / 3, 1 / 3, .25, e, g, e, e, b, a, b, a, b, a]
        z = [0, 1 / 3, 1 / 3, 1 / 3, .25, g, e, e, e, b, b, a, b, a, a]
        w = [0.0060267857142857142857142857142857] * 4 + [0.030283678097089175806376972557730] + \
            [0.011645249086028969410893609144338] * 4 + [0.010949141561386459345643019112407] * 6
    else:
        raise ValueError("tetrahedral rules with 11 or 15 points")
    return np.array(x), np.array(y), np.array(z), np.array(w)


def _pk_values(elem: int, x, y, z):
    """P1 (11) / P2 (12) basis values (nq, nb) and reference derivatives
    (3, nq, nb) in local DOF order (C_T_P1_3D, C_T_P2_3D)"""
    one, zero = np.ones_like(x), np.zeros_like(x)
    if elem == 11:
        v = [1 - x - y - z, x, y, z]
        dx = [-one, one, zero, zero]
        dy = [-one, zero, one, zero]
        dz = [-one, zero, zero, one]
    else:
        g0 = -3 + 4 * x + 4 * y + 4 * z
        v = [1 - 3 * x - 3 * y - 3 * z + 2 * x * x + 4 * x * y + 4 * x * z + 2 * y * y + 4 * y * z + 2 * z * z,
             4 * x - 4 * x * x - 4 * x * y - 4 * x * z, -x + 2 * x * x, 4 * y - 4 * x * y - 4 * y * y - 4 * y * z,
             4 * x * y, -y + 2 * y * y, 4 * z - 4 * x * z - 4 * y * z - 4 * z * z, 4 * x * z, 4 * y * z,
             -z + 2 * z * z]
        dx = [g0, 4 - 8 * x - 4 * y - 4 * z, -1 + 4 * x, -4 * y, 4 * y, zero, -4 * z, 4 * z, zero, zero]
        dy = [g0, -4 * x, zero, 4 - 4 * x - 8 * y - 4 * z, 4 * x, -1 + 4 * y, -4 * z, zero, 4 * z, zero]
        dz = [g0, -4 * x, zero, -4 * y, zero, zero, 4 - 4 * x - 4 * y - 8 * z, 4 * x, 4 * y, -1 + 4 * z]
    return np.stack(v, axis=1), np.stack([np.stack(dx, axis=1), np.stack(dy, axis=1), np.stack(dz, axis=1)])


class OracleCD:
    """ConvectionDiffusion<d> restated on the CPU over a multigrid hierarchy."""

    def __init__(self, geometry: int, root_n: int, n_refine: int, n_levels: int, elem: int,
                 eps: float, b=(0.0, 0.0, 0.0), c: float = 0.0, quad_points: int = 3,
                 manufactured: bool = True, f_const: float = 0.0, poly=None, poly_src=None,
                 neumann_sides: int = 0):
        """poly: ten coefficients (1, x, y, z, x^2, y^2, z^2, xy, xz, yz) of a
        quadratic exact solution; f and the Dirichlet values then come from it;
        poly_src (same monomials) is added to f. neumann_sides: bit mask of the
        unit square's sides (0 y=0, 1 x=1, 2 y=1, 3 x=0) with Neumann data
        eps grad u . n of the exact solution"""
        self.geometry = geometry
        self.dim = 2 if geometry == refsetup.GEO_SQUARE_QUAD else 3
        self.elem = elem
        self.neumann_sides = neumann_sides
        self.levels = refsetup.cd_levels(geometry, root_n, n_refine, n_levels, elem, neumann_sides)
        self.eps, self.c = eps, c
        self.b = np.array(list(b) + [0.0] * (3 - len(b)), dtype=np.float64)
        self.qn = quad_points
        self.manufactured, self.f_const = manufactured, f_const
        self.poly = None
        if poly is not None:
            src = [] if poly_src is None else list(poly_src)
            self.poly = np.array(list(poly) + [0.0] * (10 - len(poly)) + src + [0.0] * (10 - len(src)),
                                 dtype=np.float64)
        self.vals = []
        self.rhs = []
        self._mg = None
        self._keep = []

    def exact(self, x) -> float:
        """the quadratic exact solution at one point"""
        X = np.zeros(3)
        X[: len(x)] = x
        return lib().orc_poly_u(_p(self.poly), _p(X))

    @property
    def finest(self):
        return self.levels[-1]

    def _assemble_tetra(self, lv):
        """ConvectionDiffusion's Galerkin element loop on tetrahedra (P1 / P2 on
        the P4Tetra / P5Tetra rule, src/AssembleRoutines/Assemble3D.C:228-470 with
        BilinearAssembleGalerkin, src/AssembleRoutines/ConvDiff.C:1794-1856, on
        TetraAffin): per cell K_ij += w |det J| (eps grad phi_i . grad phi_j
        + (b . grad phi_j) phi_i + c phi_j phi_i), F_i += w |det J| f phi_i,
        added to the active rows; non-active rows keep their unit diagonal and
        the Dirichlet value"""
        X, Y, Z, W = _tet_rule(self.qn)
        phi, dphi = _pk_values(self.elem, X, Y, Z)            # (nq, nb), (3, nq, nb)
        v = lv.verts                                           # (cells, 4, 3)
        J = np.stack([v[:, 1] - v[:, 0], v[:, 2] - v[:, 0], v[:, 3] - v[:, 0]], axis=2)
        det = np.linalg.det(J)
        G = np.linalg.inv(J).transpose(0, 2, 1)
        grad = np.einsum("cda,aqi->cqid", G, dphi)             # (cells, nq, nb, 3)
        w = W[None, :] * np.abs(det)[:, None]                  # (cells, nq)
        b = self.b
        conv = grad @ b                                        # (cells, nq, nb)
        K = (self.eps * np.einsum("cq,cqid,cqjd->cij", w, grad, grad)
             + np.einsum("cq,qi,cqj->cij", w, phi, conv)
             + self.c * np.einsum("cq,qi,qj->cij", w, phi, phi))
        xq = v[:, 0][:, None, :] + np.einsum("cda,qa->cqd", J, np.stack([X, Y, Z], axis=1))
        ex = self.exact_grad(xq.reshape(-1, 3))
        if self.poly is not None:
            pp, ps = np.ascontiguousarray(self.poly[:10]), np.ascontiguousarray(self.poly[10:])
            f = np.array([lib().orc_poly_rhs(3, _p(np.ascontiguousarray(x)), self.eps, _p(self.b), self.c,
                                             _p(pp), _p(ps))
                          for x in xq.reshape(-1, 3)])
        elif self.manufactured:
            s_ = np.sin(np.pi * xq.reshape(-1, 3))
            lap = -3 * np.pi ** 2 * np.prod(s_, axis=1)
            f = -self.eps * lap + ex[:, 1:] @ b + self.c * ex[:, 0]
        else:
            f = np.full(xq.shape[0] * xq.shape[1], self.f_const)
        F = np.einsum("cq,cq,qi->ci", w, f.reshape(xq.shape[0], -1), phi)
        vals = np.zeros(lv.cols.size)
        rhs = np.zeros(lv.n_dofs)
        dm = lv.dofmap
        rows = np.repeat(dm, dm.shape[1], axis=1).ravel()
        cols = np.tile(dm, (1, dm.shape[1])).ravel()
        act = rows < lv.n_active
        key_pat = np.repeat(np.arange(lv.n_dofs, dtype=np.int64), np.diff(lv.row_ptr)) * lv.n_dofs + lv.cols
        pos = np.searchsorted(key_pat, rows[act].astype(np.int64) * lv.n_dofs + cols[act])
        np.add.at(vals, pos, K.ravel()[act])
        ra = dm.ravel() < lv.n_active
        np.add.at(rhs, dm.ravel()[ra], F.ravel()[ra])
        for i in range(lv.n_active, lv.n_dofs):
            vals[lv.row_ptr[i]] = 1.0
        return vals, rhs

    def assemble(self) -> None:
        L = lib()
        self.vals, self.rhs = [], []
        for lv in self.levels:
            if self.geometry == refsetup.GEO_CUBE_TETRA:
                vals, rhs = self._assemble_tetra(lv)
                if self.poly is not None:
                    for i in range(lv.n_active, lv.n_dofs):
                        rhs[i] = self.exact(lv.node_coords[i])
                self.vals.append(vals)
                self.rhs.append(rhs)
                continue
            vals = np.zeros(lv.cols.size, dtype=np.float64)
            rhs = np.zeros(lv.n_dofs, dtype=np.float64)
            verts = np.ascontiguousarray(lv.verts, dtype=np.float64)
            dm = np.ascontiguousarray(lv.dofmap, dtype=np.int32)
            manuf = 2 if self.poly is not None else int(self.manufactured)
            rc = L.orc_assemble_cd_poly(self.dim, self.elem, self.qn, lv.n_cells, _p(verts), lv.nloc, _p(dm),
                                        lv.n_dofs, lv.n_active, _p(lv.row_ptr), _p(lv.cols), self.eps,
                                        _p(self.b), self.c, manuf, self.f_const,
                                        None if self.poly is None else _p(self.poly), _p(vals), _p(rhs))
            if rc != 0:
                raise RuntimeError(f"oracle assembly failed ({rc})")
            if self.poly is not None:
                # Dirichlet values: point values of the exact solution at the
                # nodes of the non-active DOFs (Assemble3D.C:640-665)
                for i in range(lv.n_active, lv.n_dofs):
                    rhs[i] = self.exact(lv.node_coords[i])
            if self.neumann_sides and (self.manufactured or self.poly is not None):
                self._neumann_rhs(lv, rhs)
            self.vals.append(vals)
            self.rhs.append(rhs)

    def exact_grad(self, x: np.ndarray) -> np.ndarray:
        """(u, u_x, u_y[, u_z]) of the exact solution at points x (n, dim);
        zero for a constant right-hand side"""
        n, d = x.shape
        out = np.zeros((n, 1 + d))
        if self.poly is not None:
            X = np.zeros((n, 3))
            X[:, :d] = x
            p = self.poly
            out[:, 0] = (p[0] + p[1] * X[:, 0] + p[2] * X[:, 1] + p[3] * X[:, 2] + p[4] * X[:, 0] ** 2 +
                         p[5] * X[:, 1] ** 2 + p[6] * X[:, 2] ** 2 + p[7] * X[:, 0] * X[:, 1] +
                         p[8] * X[:, 0] * X[:, 2] + p[9] * X[:, 1] * X[:, 2])
            g = [p[1] + 2 * p[4] * X[:, 0] + p[7] * X[:, 1] + p[8] * X[:, 2],
                 p[2] + 2 * p[5] * X[:, 1] + p[7] * X[:, 0] + p[9] * X[:, 2],
                 p[3] + 2 * p[6] * X[:, 2] + p[8] * X[:, 0] + p[9] * X[:, 1]]
            for a in range(d):
                out[:, 1 + a] = g[a]
        elif self.manufactured:
            s, c = np.sin(np.pi * x), np.cos(np.pi * x)
            out[:, 0] = np.prod(s, axis=1)
            for a in range(d):
                t = np.pi * c[:, a]
                for b in range(d):
                    if b != a:
                        t = t * s[:, b]
                out[:, 1 + a] = t
        return out

    def _neumann_rhs(self, lv, rhs: np.ndarray) -> None:
        """boundary integral of Assemble2D (src/AssembleRoutines/Assemble2D.C:716-757):
        for each edge m (vertex m to m+1) of a cell on a Neumann side and each
        line Gauss point zeta_l (degree 2k: k+1 points),
        rhs_i += g(x_l) hE w_l phi_i(xi_l) for active DOFs i, hE = |edge| / 2,
        xi_l on edge m of [-1,1]^2 (src/FE/BaseFunct2D.C:87-118),
        g = eps grad u . n (SineLaplace's BoundValue on x = 1)"""
        k = self.elem
        z, w = np.polynomial.legendre.leggauss(k + 1)
        ref = np.array([[-1.0, -1.0], [1.0, -1.0], [1.0, 1.0], [-1.0, 1.0]])
        normal = {0: (0.0, -1.0), 1: (1.0, 0.0), 2: (0.0, 1.0), 3: (-1.0, 0.0)}
        S = lv.scale
        for c in range(lv.n_cells):
            vl = lv.verts_lattice[c]
            for m in range(4):
                m1 = (m + 1) % 4
                ss = refsetup.square_sides(vl[[m, m1]], S)
                common = int(ss[0] & ss[1])
                for side in range(4):
                    if not (common >> side) & (self.neumann_sides >> side) & 1:
                        continue
                    a, b = lv.verts[c, m], lv.verts[c, m1]
                    hE = np.sqrt(((b - a) ** 2).sum()) / 2
                    f = 0.5 * (z + 1.0)
                    xi = ref[m][None, :] + f[:, None] * (ref[m1] - ref[m])[None, :]
                    x = a[None, :] + f[:, None] * (b - a)[None, :]
                    g = self.eps * (self.exact_grad(x)[:, 1:] @ np.array(normal[side]))
                    phi = _qk_values(k, 2, xi)[0]          # (points, nloc)
                    contrib = (g * hE * w)[:, None] * phi
                    for loc in range(lv.nloc):
                        dof = lv.dofmap[c, loc]
                        if dof < lv.n_active:
                            rhs[dof] += contrib[:, loc].sum()

    def errors(self, sol: np.ndarray) -> np.ndarray:
        """(L2, H1-semi, SD, L_inf) of ConvectionDiffusion<d>::output
        (src/System/ConvectionDiffusion.C:213-283): TFEFunction{2,3}D::GetErrors
        (src/FE/FEFunction2D.C:318-575, FEFunction3D.C:80-245) on the rule
        that GetOrig picks (src/FE/FEDatabase2D.C:1718-1790: degree N_terms x
        k, the assembly's rule) with
        conv_diff_l2_h1_linf_error (src/AssembleRoutines/ConvDiff.C:2134-2185)
        and the SUPG delta of Compute_SDFEM_delta (ConvDiff.C:273-360) at
        SDFEM_TYPE 2, DELTA0 1, polynomial degree 1, hK = cell diameter"""
        lv = self.finest
        d, k = self.dim, self.elem
        qn = self.qn
        x1, w1 = _gauss(qn)
        if d == 2:
            xi = np.array([[x1[a], x1[b]] for b in range(qn) for a in range(qn)])
            wq = np.array([w1[a] * w1[b] for b in range(qn) for a in range(qn)])
        else:
            xi = np.array([[x1[a], x1[b], x1[c]] for c in range(qn) for b in range(qn) for a in range(qn)])
            wq = np.array([w1[a] * w1[b] * w1[c] for c in range(qn) for b in range(qn) for a in range(qn)])
        phi, dphi = _qk_values(k, d, xi)                  # (nq, nb), (d, nq, nb)
        v = lv.verts                                       # (n_cells, nv, d)
        if d == 2:
            x0 = (v[:, 1] + v[:, 3]) / 2
            J = np.stack([(v[:, 1] - v[:, 0]) / 2, (v[:, 3] - v[:, 0]) / 2], axis=2)
        else:
            x0 = (v[:, 1] + v[:, 3] + v[:, 4] - v[:, 0]) / 2
            J = np.stack([(v[:, 1] - v[:, 0]) / 2, (v[:, 3] - v[:, 0]) / 2, (v[:, 4] - v[:, 0]) / 2], axis=2)
        det = np.linalg.det(J)
        G = np.linalg.inv(J).transpose(0, 2, 1)          # J^{-T}
        uc = sol[lv.dofmap]                                # (n_cells, nb)
        val = uc @ phi.T                                   # (n_cells, nq)
        dref = np.stack([uc @ dphi[a].T for a in range(d)], axis=2)   # (n_cells, nq, d)
        grad = np.einsum("cda,cqa->cqd", G, dref)
        x = x0[:, None, :] + np.einsum("cda,qa->cqd", J, xi)
        ex = self.exact_grad(x.reshape(-1, d)).reshape(lv.n_cells, -1, 1 + d)
        w = wq[None, :] * np.abs(det)[:, None]
        e0 = val - ex[:, :, 0]
        eg = grad - ex[:, :, 1:]
        diam = np.sqrt(((v[:, :, None, :] - v[:, None, :, :]) ** 2).sum(axis=3)).max(axis=(1, 2))
        b = self.b[:d]
        nb_ = np.sqrt((b ** 2).sum())
        eps = self.eps if abs(self.eps) >= 1e-20 else 1e-20
        if nb_ > 0:
            alpha = nb_ * diam / (2 * eps)
            delta = diam * (1 / np.tanh(alpha) - 1 / alpha) / (2 * nb_)
        else:
            delta = np.zeros(lv.n_cells)
        e4 = eg @ b
        l2 = (w * e0 ** 2).sum()
        h1 = (w * (eg ** 2).sum(axis=2)).sum()
        sd = (w * (self.eps * (eg ** 2).sum(axis=2) + self.c * e0 ** 2 + delta[:, None] * e4 ** 2)).sum()
        return np.array([np.sqrt(l2), np.sqrt(h1), np.sqrt(sd), np.abs(e0).max()])

    def active(self, l: int = -1) -> np.ndarray:
        lv = self.levels[l]
        a = np.zeros(lv.n_dofs, dtype=np.uint8)
        a[: lv.n_active] = 1
        return a

    def sor_order(self, l: int = -1) -> np.ndarray:
        """the row order of the multicolour SOR sweep of level l"""
        lv = self.levels[l]
        return _sor.colour_order(_sor.greedy_colouring(lv.row_ptr, lv.cols))

    def build_mg(self, n_pre=2, n_post=2, jacobi_damp=0.8, correction_damp=1.0, cycle="V",
                 coarse_direct=True, coarse_max_it=10, coarse_residual=0.1, n_mg_levels=None,
                 smoother="jacobi", coarse_smoother=None, sor_omega=1.5):
        L = lib()
        if self._mg:
            L.orc_mg_destroy(self._mg)
        nl = len(self.levels) if n_mg_levels is None else n_mg_levels
        off = len(self.levels) - nl
        mg = L.orc_mg_create(nl, n_pre, n_post, jacobi_damp, correction_damp, {"V": 0, "W": 1, "F": 2}[cycle],
                             int(coarse_direct), coarse_max_it, coarse_residual)
        keep = []
        for l in range(nl):
            lv = self.levels[off + l]
            act = self.active(off + l)
            keep.append(act)
            rc = L.orc_mg_set_level(mg, l, lv.n_dofs, _p(act), _p(lv.row_ptr), _p(lv.cols), _p(self.vals[off + l]))
            if rc != 0:
                raise RuntimeError("oracle coarse factorisation failed")
        for l in range(nl - 1):
            cl, fl = self.levels[off + l], self.levels[off + l + 1]
            fd = np.ascontiguousarray(fl.dofmap, dtype=np.int32)
            cd = np.ascontiguousarray(cl.dofmap, dtype=np.int32)
            fv = np.ascontiguousarray(fl.verts, dtype=np.float64)
            cv = np.ascontiguousarray(cl.verts, dtype=np.float64)
            par = np.ascontiguousarray(fl.parent, dtype=np.int32)
            keep += [fd, cd, fv, cv, par]
            L.orc_mg_set_transfer(mg, l, self.dim, self.elem, fl.n_cells, fl.nloc, _p(fd), _p(cd), _p(par),
                                  _p(fv), _p(cv), fl.n_dofs, cl.n_dofs)
        coarse = coarse_smoother or ("direct_solve" if coarse_direct else smoother)
        if smoother != "jacobi" or coarse not in ("direct_solve", "jacobi"):
            L.orc_mg_set_smoothers(mg, SMOOTHERS[smoother], SMOOTHERS[coarse], 1.0)
        for l in range(nl):
            code = coarse if l == 0 else smoother
            if code in ("sor", "ssor"):
                order = self.sor_order(off + l)
                keep.append(order)
                L.orc_mg_set_sor(mg, l, _p(order), sor_omega)
        if L.orc_mg_finalize(mg) != 0:
            raise RuntimeError("oracle coarse factorisation failed")
        self._mg = mg
        self._keep = keep
        return mg

    def mg_apply(self, z: np.ndarray) -> np.ndarray:
        z = np.ascontiguousarray(z, dtype=np.float64)
        r = np.zeros_like(z)
        lib().orc_mg_apply(self._mg, _p(z), _p(r))
        return r

    def solve(self, method: str = "fgmres", tol: float = 0.0, reduction: float = 1e-8, max_it: int = 100,
              min_it: int = 0, restart: int = 20, use_mg: bool = True, sol0=None, sor: str | None = None,
              sor_omega: float = 1.5):
        """returns (solution, iterations, residual, history, status); sor = "sor" or
        "ssor" preconditions with one (S)SOR sweep in colour order instead of the
        multigrid"""
        if sor is not None:
            return self._solve_sor(method, tol, reduction, max_it, min_it, restart, sol0, sor, sor_omega)
        lv = self.finest
        act = self.active()
        rhs = self.rhs[-1]
        sol = np.zeros(lv.n_dofs) if sol0 is None else np.array(sol0, dtype=np.float64)
        # copy_nonactive(rhs -> solution)
        sol[lv.n_active:] = rhs[lv.n_active:]
        it, res, nh = C.c_int(), C.c_double(), C.c_int()
        hist = np.zeros(100000)
        st = lib().orc_krylov_solve({"fgmres": 0, "cg": 1, "bi_cgstab": 2}[method], lv.n_dofs, _p(act),
                                    _p(lv.row_ptr), _p(lv.cols), _p(self.vals[-1]),
                                    self._mg if use_mg else None, tol, reduction, max_it, min_it, restart,
                                    _p(rhs), _p(sol), C.byref(it), C.byref(res), _p(hist), hist.size,
                                    C.byref(nh))
        return sol, it.value, res.value, hist[: nh.value].copy(), st

    def sor_iterate(self, sor="sor", tol=0.0, reduction=1e-8, max_it=100, sor_omega=1.5):
        """iterative_solver_type sor / ssor on the finest level in colour order;
        the start has the rhs's non-active entries"""
        lv = self.finest
        rhs = self.rhs[-1]
        sol = np.zeros(lv.n_dofs)
        sol[lv.n_active:] = rhs[lv.n_active:]
        return sor_iterate(lv.row_ptr, lv.cols, self.vals[-1], self.active(), rhs, sol, sor_omega,
                           self.sor_order(-1), {"sor": 0, "ssor": 2}[sor], tol, reduction, max_it)

    def _solve_sor(self, method, tol, reduction, max_it, min_it, restart, sol0, sor, sor_omega):
        lv = self.finest
        act = self.active()
        rhs = self.rhs[-1]
        sol = np.zeros(lv.n_dofs) if sol0 is None else np.array(sol0, dtype=np.float64)
        sol[lv.n_active:] = rhs[lv.n_active:]
        order = self.sor_order(-1)
        it, res, nh = C.c_int(), C.c_double(), C.c_int()
        hist = np.zeros(100000)
        st = lib().orc_krylov_solve_sor({"fgmres": 0, "cg": 1, "bi_cgstab": 2}[method], lv.n_dofs, _p(act),
                                        _p(lv.row_ptr), _p(lv.cols), _p(self.vals[-1]), None,
                                        {"sor": 0, "ssor": 2}[sor], _p(order), sor_omega, tol, reduction, max_it,
                                        min_it, restart, _p(rhs), _p(sol), C.byref(it), C.byref(res), _p(hist),
                                        hist.size, C.byref(nh))
        return sol, it.value, res.value, hist[: nh.value].copy(), st

    def close(self):
        if self._mg:
            lib().orc_mg_destroy(self._mg)
            self._mg = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
