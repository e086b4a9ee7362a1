"""Oracle restatement of the time-dependent convection-diffusion path (test
infrastructure only).

TimeConvectionDiffusion<d> (src/System/TimeConvectionDiffusion.C:252-386) with
TimeDiscretization (src/TimeDiscRoutines/TimeDiscretizations.C:106-232,
341-380): backward Euler, Crank-Nicolson and BDF2 (first step by backward
Euler). Matrices and right-hand sides come from the oracle's convection-
diffusion assembly (oracle.c, orc_assemble_cd_poly); the linear solves use the
oracle's FGMRES + multigrid or a dense direct solve. Element-wise operations
follow FEMatrix::scaleActive / addActive (src/Matrix/FEMatrix.C:139-184) and
BlockVector::scaleActive / addScaledActive; products with the mass and
stiffness matrices follow FEMatrix::multiplyActive (:186-199).
"""
from __future__ import annotations

import numpy as np

from . import cd as ocd

BDF = (4.0 / 3.0, -1.0 / 3.0, 2.0 / 3.0)


class OracleTCD:
    """u = P0 + t P1 + t^2 P2 (poly, poly_time = (P1, P2)) with the examples'
    constant coefficients, or the sine / constant right-hand side of OracleCD
    (time independent) when poly is None."""

    def __init__(self, geometry, root_n, n_refine, n_levels, elem, eps, b, c, quad_points=3, poly=None,
                 poly_time=None, manufactured=True, scheme="backward_euler", tau=0.05, t_start=0.0, t_end=1.0):
        self.p0 = None if poly is None else np.array(list(poly) + [0.0] * (10 - len(poly)))
        pt = poly_time or ([0.0] * 10, [0.0] * 10)
        self.p1 = np.array(list(pt[0]) + [0.0] * (10 - len(pt[0])))
        self.p2 = np.array(list(pt[1]) + [0.0] * (10 - len(pt[1])))
        kw = dict(quad_points=quad_points)
        if poly is not None:
            self.cd = ocd.OracleCD(geometry, root_n, n_refine, n_levels, elem, eps, b, c, poly=self.p0,
                                   poly_src=np.zeros(10), **kw)
        else:
            self.cd = ocd.OracleCD(geometry, root_n, n_refine, n_levels, elem, eps, b, c,
                                   manufactured=manufactured, **kw)
        # the mass matrices: the c u v term (eps = 0, b = 0, c = 1, f = 0)
        self.massp = ocd.OracleCD(geometry, root_n, n_refine, n_levels, elem, 0.0, (0.0, 0.0, 0.0), 1.0,
                                  manufactured=False, f_const=0.0, **kw)
        self.scheme, self.tau, self.t_start, self.t_end = scheme, tau, t_start, t_end
        self.t, self.step = t_start, 0
        self.pre_stage_bdf = scheme == "bdf_two"
        self.factor = None

    # the exact solution's polynomial at time t and its time derivative
    def polys(self, t):
        q = self.p0 + t * self.p1 + (t * t) * self.p2
        r = self.p1 + (2.0 * t) * self.p2
        return q, r

    def exact(self, t, x) -> float:
        q, _ = self.polys(t)
        X = np.zeros(3)
        X[: len(x)] = x
        return ocd.lib().orc_poly_u(ocd._p(np.ascontiguousarray(q)), ocd._p(X))

    def _assemble_stiffness(self, t):
        if self.p0 is not None:
            q, r = self.polys(t)
            self.cd.poly[:10] = q
            self.cd.poly[10:] = r
        self.cd.assemble()

    def _active_entries(self, l):
        lv = self.cd.levels[l]
        return lv.row_ptr[lv.n_active]

    def assemble_initial_time(self):
        self.t, self.step = self.t_start, 0
        self.pre_stage_bdf = self.scheme == "bdf_two"
        self._assemble_stiffness(self.t)
        self.massp.assemble()
        self.mass = [v.copy() for v in self.massp.vals]
        lv = self.cd.finest
        if self.p0 is not None:
            self.sol = np.array([self.exact(self.t, x) for x in lv.node_coords])
        else:
            self.sol = np.zeros(lv.n_dofs)
        self.old_rhs = self.cd.rhs[-1].copy()
        self.sol_m1 = self.sol.copy()
        self.sol_m2 = self.sol_m1.copy()

    def next_step(self):
        self.step += 1
        if self.scheme == "bdf_two" and self.step >= 2:
            self.pre_stage_bdf = False
        self.t += self.tau

    def _mult_active(self, vals, x, y, a):
        """y[i] += a * (row i . x) on the active rows (non-active entries are
        overwritten afterwards)"""
        lv = self.cd.finest
        return ocd.apply_scaled_add(lv.row_ptr, lv.cols, vals, self.cd.active(), x, y, a)

    def assemble(self):
        self._assemble_stiffness(self.t)
        lv = self.cd.finest
        na = lv.n_active
        rhs = self.cd.rhs[-1]
        A, M = self.cd.vals[-1], self.mass[-1]
        td = rhs.copy()
        tau = self.tau
        if self.scheme == "bdf_two" and not self.pre_stage_bdf:
            td[:na] = td[:na] * (BDF[2] * tau)
            td = self._mult_active(M, self.sol_m1, td, BDF[0])
            td = self._mult_active(M, self.sol_m2, td, BDF[1])
            factor = tau * BDF[2]
        elif self.scheme == "backward_euler" or self.pre_stage_bdf:
            td[:na] = td[:na] * tau
            td = self._mult_active(M, self.sol_m1, td, 1.0)
            factor = tau
        else:  # crank_nicolson
            td[:na] = td[:na] * (0.5 * tau)
            td[:na] = td[:na] + (0.5 * tau) * self.old_rhs[:na]
            td = self._mult_active(M, self.sol_m1, td, 1.0)
            td = self._mult_active(A, self.sol_m1, td, -0.5 * tau)
            factor = tau * 0.5
        self.old_rhs = rhs.copy()
        td[na:] = rhs[na:]
        self.sol[na:] = rhs[na:]
        self.rhs_td = td
        # prepare_system_matrix: factor * A + M on the entries of active rows
        for l in range(len(self.cd.levels)):
            ne = self._active_entries(l)
            S = self.cd.vals[l]
            S[:ne] = S[:ne] * factor + self.mass[l][:ne]
        self.factor = factor

    def solve(self, solver="multigrid", mg=None, tol=1e-15, reduction=0.0, max_it=100, restart=20):
        """the solve with the system matrices; mg: keyword arguments of
        OracleCD.build_mg (multigrid only)"""
        lv = self.cd.finest
        if solver == "direct":
            n = lv.n_dofs
            S = np.zeros((n, n))
            rows = np.repeat(np.arange(n), np.diff(lv.row_ptr))
            S[rows, lv.cols] = self.cd.vals[-1]
            self.sol = np.linalg.solve(S, self.rhs_td)
            self.last_it = 1
        else:
            self.cd.rhs[-1] = self.rhs_td
            self.cd.build_mg(**(mg or {}))
            self.sol, self.last_it, res, hist, st = self.cd.solve("fgmres", tol, reduction, max_it, 0, restart,
                                                                 sol0=self.sol)
        # reset_linear_matrices: (S - M) / factor on the active entries
        inv = 1.0 / self.factor
        for l in range(len(self.cd.levels)):
            ne = self._active_entries(l)
            S = self.cd.vals[l]
            S[:ne] = (S[:ne] - self.mass[l][:ne]) * inv
        self.factor = None
        self.sol_m2 = self.sol_m1
        self.sol_m1 = self.sol.copy()
