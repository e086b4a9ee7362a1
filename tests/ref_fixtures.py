"""Loading the fixtures made by the compiled reference (tests/golden/ref_*.npz,
generated by tests/golden/make_ref_fixtures.py) and mapping their
configuration onto the library's and the oracle's arguments."""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"

# the reference's quadrature rule of a tensor element of order k:
# degree = (2 if INTERNAL_PROBLEM_LINEAR else 3) * k, then
# QF{Quad,Hexa}FromDegree (src/FE/FEDatabase2D.C:1629-1647,
# src/FE/FEDatabase3D.C:977-994): degree 0-2 Gauss2, 3-5 Gauss3, 6-7 Gauss4
_POINTS = {0: 2, 1: 2, 2: 2, 3: 3, 4: 3, 5: 3, 6: 4, 7: 4}


def names() -> list[str]:
    """the convection-diffusion cases"""
    return sorted(p.stem[len("ref_"):] for p in GOLDEN.glob("ref_*.npz")
                  if not p.stem.startswith(("ref_stokes", "ref_nse")))


def stokes_names() -> list[str]:
    return sorted(p.stem[len("ref_"):] for p in GOLDEN.glob("ref_stokes*.npz"))


def nse_names(solver: str | None = None) -> list[str]:
    """the Navier-Stokes cases (of one solver: direct, mg or none)"""
    out = sorted(p.stem[len("ref_"):] for p in GOLDEN.glob("ref_nse*.npz"))
    return [n for n in out if solver is None or NseRefCase(n).solver == solver]


class RefCase:
    def __init__(self, name: str):
        self.name = name
        self.z = np.load(GOLDEN / f"ref_{name}.npz")
        cfg = [int(v) for v in self.z["config"]]
        dim, nref, order, nlev, quad_linear, restart = cfg[:6]
        eps, b1, b2, b3, reduction = (float(v) for v in self.z["coeffs"])
        self.dim, self.n_refine, self.order, self.n_levels = dim, nref, order, nlev
        self.restart, self.reduction = restart, reduction
        self.eps, self.b = eps, (b1, b2, b3)
        # unit square (quads) / unit cube (hexahedra) / unit cube (tetrahedra)
        self.geometry = cfg[6] if len(cfg) > 6 else (0 if dim == 2 else 1)
        if self.geometry == 2:
            # P1 / P2 (library elements 11 / 12); QFTetraFromDegree: degree 3 -> P4Tetra
            # (11 points), 6 -> P5Tetra (15 points); 2 x order: P2Tetra / P4Tetra
            self.elem = 10 + order
            degree = (2 if quad_linear else 3) * order
            self.quad_points = 11 if degree in (3, 4) else 15 if degree in (5, 6) else 4
        else:
            self.elem = order
            self.quad_points = _POINTS[(2 if quad_linear else 3) * order]
        # the reference's own example (0 = SineLaplace, Neumann side x = 1) or -1
        self.example = int(self.z["example"]) if "example" in self.z.files else -1
        self.neumann_sides = 2 if self.example == 0 else 0
        self.errors = self.z["errors"] if "errors" in self.z.files else None
        self.iterations = int(self.z["iterations"])
        self.initial_residual = float(self.z["initial_residual"])
        self.final_residual = float(self.z["final_residual"])

    def has(self, key: str) -> bool:
        return key in self.z.files

    def level(self, l: int) -> dict:
        p = f"L{l}_"
        d = {k[len(p):]: self.z[k] for k in self.z.files if k.startswith(p)}
        cells, nloc, n_dofs, active, nnz = (int(v) for v in d["sizes"])
        d.update(cells=cells, nloc=nloc, n_dofs=n_dofs, active=active, nnz=nnz)
        return d

    def compare(self, key_prefix: str, got_full: np.ndarray, level: int | None = None) -> float:
        """largest difference of `got_full` to the reference's entries (full or
        sampled), relative to the reference's largest magnitude"""
        pre = f"L{level}_" if level is not None else ""
        ref = self.z[pre + key_prefix]
        idx_key = pre + key_prefix + "_idx"
        got = got_full[self.z[idx_key]] if idx_key in self.z.files else got_full
        assert got.shape == ref.shape, (got.shape, ref.shape)
        return float(np.abs(got - ref).max() / float(self.z[pre + key_prefix + "_max"]))


def digest(a: np.ndarray, dtype) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=dtype).tobytes()).hexdigest()


class StokesRefCase:
    """a Stokes fixture: NavierStokes<3> (Stokes, P2/P1, example -3) of the
    reference on Default_UnitCube_Tetra"""

    def __init__(self, name: str):
        self.name = name
        self.z = np.load(GOLDEN / f"ref_{name}.npz")
        self.n_refine, self.n_levels = (int(v) for v in self.z["config"])

    def has(self, key: str) -> bool:
        return key in self.z.files

    def level(self, l: int) -> dict:
        p = f"L{l}_"
        d = {k[len(p):]: self.z[k] for k in self.z.files if k.startswith(p)}
        cells, nu, nua, np_, npa, nnz = (int(v) for v in d["sizes"])
        d.update(cells=cells, nu=nu, nu_active=nua, np=np_, np_active=npa, nnz=nnz)
        return d

    def compare_matrix(self, l: int, rp: np.ndarray, ci: np.ndarray, vals: np.ndarray) -> float:
        """largest difference between the reference's combined matrix of level
        l (pressure projection applied, exact zeros removed) and the given
        projected CSR matrix, relative to the reference's largest entry; the
        given matrix's entries outside the reference's pattern count as
        differences from zero"""
        d = self.level(l)
        n = rp.size - 1
        ours_row = np.repeat(np.arange(n, dtype=np.int64), np.diff(rp))
        ours_key = ours_row * n + ci
        if "rows" in d:
            ref_row = np.repeat(np.arange(d["rows"].size - 1, dtype=np.int64), np.diff(d["rows"]))
            ref_key, ref_val = ref_row * n + d["cols"], d["vals"]
            # every entry of ours: the reference's value or zero
            pos = np.searchsorted(ref_key, ours_key)
            pos_c = np.minimum(pos, ref_key.size - 1)
            hit = ref_key[pos_c] == ours_key
            diff_ours = np.abs(vals - np.where(hit, ref_val[pos_c], 0.0)).max()
        else:
            ref_key = d["sample_rows"].astype(np.int64) * n + d["sample_cols"]
            ref_val = d["sample_vals"]
            diff_ours = 0.0
        # every entry of the reference: ours must hold it
        pos = np.searchsorted(ours_key, ref_key)
        pos_c = np.minimum(pos, ours_key.size - 1)
        assert np.all(ours_key[pos_c] == ref_key), "an entry of the reference is outside the pattern"
        diff_ref = np.abs(vals[pos_c] - ref_val).max()
        return float(max(diff_ours, diff_ref) / float(d["vals_max"]))


class NseRefCase(StokesRefCase):
    """a Navier-Stokes fixture: NavierStokes<3> (problem_type 5, convective
    form, example -3) of the reference through the nonlinear loop of
    test/nse3d_solvers_test.c++ (solver direct or mg: residuals of every step,
    linear iterations, solution, errors), or one assemble_nonlinear_term with
    a fixed finest velocity (solver none: every level's matrix and velocity)"""

    def __init__(self, name: str):
        self.name = name
        self.z = np.load(GOLDEN / f"ref_{name}.npz")
        self.n_refine, self.n_levels, self.maxit = (int(v) for v in self.z["config"])
        self.reynolds, self.epsilon = (float(v) for v in self.z["params"])
        self.solver = str(self.z["solver"])
        # nse_nonlinear_form: convective or skew_symmetric
        self.form = str(self.z["form"]) if "form" in self.z.files else "convective"

    def level(self, l: int) -> dict:
        p = f"L{l}_"
        d = {k[len(p):]: self.z[k] for k in self.z.files if k.startswith(p)}
        cells, nu, nua, np_, nnz = (int(v) for v in d["sizes"])
        d.update(cells=cells, nu=nu, nu_active=nua, np=np_, nnz=nnz)
        return d

    def fixed_velocity(self, nu: int, n: int) -> np.ndarray:
        """the finest solution the nonlinear assembly case starts from:
        u_b[i] = sin(0.7 i + 1.3 b + 0.1), pressure 0"""
        x = np.zeros(n)
        i = np.arange(nu)
        for b in range(3):
            x[b * nu:(b + 1) * nu] = np.sin(0.7 * i + 1.3 * b + 0.1)
        return x

    def full_solution(self, n: int):
        """(indices, values) of the stored solution"""
        if "solution_idx" in self.z.files:
            return self.z["solution_idx"], self.z["solution"]
        return np.arange(n), self.z["solution"]
