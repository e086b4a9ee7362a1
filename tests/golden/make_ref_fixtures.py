"""Generate the golden fixtures that pin the solve path against the reference
itself (ParMooN compiled by oracle/ref/build_ref.py; run where the reference
sources are present).

For each case the reference's own ConvectionDiffusion<d> (driver
oracle/ref/ref_cd.C) builds the mesh hierarchy, the FE spaces and the CSR
structures, assembles every multigrid level and solves with FGMRES +
multigrid. The fixture keeps, per level:
  * SHA-256 digests of GlobalNumbers (cell order, BeginIndex = c * nloc), the
    CSR row pointers and column indices and the cell vertex coordinates - the
    bit-exact contract;
  * the assembled entries and the right-hand side: in full for the small cases,
    as a fixed sample (SAMPLES indices) plus the largest magnitude for the
    full-size ones;
and for the solve: the FGMRES iteration count, the initial and final residual
of the reference's LoopInfo and the solution (full or sampled).

The sine_* cases run the reference's own SineLaplace example (Example_CD2D
number 0, include/Examples/CD_2D/SineLaplace.h: u = sin(pi x) sin(pi y),
eps = 1, Neumann boundary on x = 1) instead of the driver's sine problem, and
keep the L2, H1-semi, SD and L_inf errors of ConvectionDiffusion::output.

The stokes_* cases run the driver oracle/ref/ref_stokes.C: the reference's
NavierStokes<3> as a Stokes problem with P2/P1 elements on
Default_UnitCube_Tetra and its example -3 (test_u_2_p_1). Per level: digests
of the cell vertices and of the velocity and pressure GlobalNumbers, and the
combined matrix of BlockFEMatrix::get_combined_matrix (the pressure
projection applied, exact zeros removed) with the right-hand side; on the
smallest mesh also the direct solve's solution.

The nse_* cases run the same driver in its Navier-Stokes mode: problem_type 5,
the convective form and the reference's own example -3 (whose coefficients
hold the convective term) at a Reynolds number, through the nonlinear loop of
the reference's test/nse3d_solvers_test.c++ (assemble_linear_terms,
stop_it(0), then solve / assemble_nonlinear_term / stop_it(k)). They keep the
impuls, mass and full residual of every nonlinear step, the FGMRES iterations
of every solve (multigrid cases), the final solution and get_errors(). The
nse_*_nl case instead sets a fixed finest velocity, calls
assemble_nonlinear_term once and keeps every level's restricted velocity and
combined matrix (the convective term and GridTransfer::RestrictFunction).

    python tests/golden/make_ref_fixtures.py            # all cases
    python tests/golden/make_ref_fixtures.py cd3d_q2_8  # one case
"""
from __future__ import annotations

import hashlib
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "oracle" / "ref"))

SAMPLES = 4096

# name: (dim, n_refine, element order, levels, eps, b, quadrature degree 2 x
#        order (1) or the default 3 x order (0), restart, residual reduction, full arrays
#        [, the reference's example number (-1: the sine problem) [, "tetra"]])
CASES = {
    # 3D Q2 32^3 convection-diffusion, 4 levels, FGMRES(30), 1e-8, Gauss 3x3x3
    "cd3d_q2_32": (3, 5, 2, 4, 1e-2, (1.0, 0.5, 0.25), 1, 30, 1e-8, False),
    # 2D Q1 128^2 convection-diffusion, 4 levels, FGMRES(20), 1e-10, Gauss 3x3
    "cd2d_q1_128": (2, 7, 1, 4, 0.1, (1.0, 0.0, 0.0), 0, 20, 1e-10, False),
    # smaller cases (the last three with every array in full)
    "cd3d_q2_8": (3, 3, 2, 3, 0.1, (1.0, 0.5, 0.25), 1, 30, 1e-10, False),
    "cd3d_q2_4": (3, 2, 2, 2, 0.1, (1.0, 0.5, 0.25), 1, 30, 1e-10, True),
    "cd3d_q1_8": (3, 3, 1, 3, 0.05, (0.3, -1.0, 0.5), 1, 30, 1e-10, True),
    "cd2d_q2_16": (2, 4, 2, 3, 0.02, (1.0, 0.5, 0.0), 1, 20, 1e-10, True),
    # SineLaplace with its Neumann side: the 4 x 4 mesh of test/cd2d_test.c++
    # (2 refinements of UnitSquare) and larger meshes
    "sine_q1_4": (2, 2, 1, 2, 1.0, (0.0, 0.0, 0.0), 0, 20, 1e-12, True, 0),
    "sine_q2_4": (2, 2, 2, 2, 1.0, (0.0, 0.0, 0.0), 0, 20, 1e-12, True, 0),
    "sine_q1_64": (2, 6, 1, 4, 1.0, (0.0, 0.0, 0.0), 0, 20, 1e-10, False, 0),
    "sine_q2_32": (2, 5, 2, 3, 1.0, (0.0, 0.0, 0.0), 0, 20, 1e-10, False, 0),
    # P1 / P2 on Default_UnitCube_Tetra (the tetrahedral half of test/cd3d_solvers_test.c++)
    "tet_p1_8": (3, 3, 1, 3, 0.1, (1.0, 0.5, 0.25), 0, 30, 1e-10, True, -1, "tetra"),
    "tet_p2_4": (3, 2, 2, 2, 0.1, (1.0, 0.5, 0.25), 0, 30, 1e-10, True, -1, "tetra"),
    "tet_p2_16": (3, 4, 2, 3, 0.05, (1.0, 0.5, 0.25), 0, 30, 1e-10, False, -1, "tetra"),
}


# name: (refinements of Default_UnitCube_Tetra, levels, full arrays, direct solve)
STOKES_CASES = {
    "stokes_p2p1_4": (2, 2, True, True),
    "stokes_p2p1_8": (3, 3, False, False),
}

# name: (refinements, levels, solver (direct | mg | none), Reynolds number,
#        nonlinloop_epsilon, nonlinloop_maxit[, nse_nonlinear_form])
NSE_CASES = {
    "nse_p2p1_4": (2, 1, "direct", 1.0, 1e-10, 10),
    "nse_p2p1_4_re100": (2, 1, "direct", 100.0, 1e-10, 30),
    "nse_p2p1_8_mg": (3, 3, "mg", 10.0, 1e-10, 10),
    "nse_p2p1_8_nl": (3, 3, "none", 1.0, 1e-10, 10),
    # the skew-symmetric form (1/2) [((u.grad) u, v) - ((u.grad) v, u)]
    "nse_p2p1_4_skew_re100": (2, 1, "direct", 100.0, 1e-10, 30, "skew_symmetric"),
    "nse_p2p1_8_nl_skew": (3, 3, "none", 1.0, 1e-10, 10, "skew_symmetric"),
}


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def sample_idx(n: int) -> np.ndarray:
    if n <= SAMPLES:
        return np.arange(n, dtype=np.int64)
    rng = np.random.default_rng(n)
    return np.unique(np.concatenate([np.linspace(0, n - 1, SAMPLES // 2).astype(np.int64),
                                     rng.integers(0, n, SAMPLES // 2)]))


def run_case(name: str) -> None:
    import build_ref
    dim, nref, order, nlev, eps, b, quad_linear, restart, reduction, full = CASES[name][:10]
    example = CASES[name][10] if len(CASES[name]) > 10 else -1
    geometry = CASES[name][11] if len(CASES[name]) > 11 else ("square" if dim == 2 else "hexa")
    exe = build_ref.link_program(str(dim), build_ref.HERE / "ref_cd.C", build_ref.OUT / f"ref_cd{dim}d")
    with tempfile.TemporaryDirectory() as tmp:
        cmd = [str(exe), tmp, str(nref), str(order), str(nlev), repr(eps), *map(repr, b), str(quad_linear),
               "fgmres_mg", str(restart), repr(reduction)] + ([str(example)] if example >= 0 or geometry == "tetra" else [])
        if geometry == "tetra":
            cmd.append("tetra")
        subprocess.run(cmd, check=True, capture_output=True)
        meta = {}
        for line in Path(tmp, "meta.txt").read_text().splitlines():
            k, v = line.split(None, 1)
            meta[k] = v
        out: dict[str, np.ndarray] = {
            "config": np.array([dim, nref, order, nlev, quad_linear, restart,
                                {"square": 0, "hexa": 1, "tetra": 2}[geometry]], dtype=np.int64),
            "coeffs": np.array([eps, *b, reduction], dtype=np.float64),
            "iterations": np.array(int(meta["iterations"])),
            "initial_residual": np.array(float(meta["initial_residual"])),
            "final_residual": np.array(float(meta["final_residual"])),
            "example": np.array(example, dtype=np.int64),
        }
        if example >= 0:
            out["errors"] = np.array([float(v) for v in meta["errors"].split()])
        for rl in range(nlev):
            lvl = nlev - 1 - rl  # 0 = coarsest, as the library counts levels
            info = meta[f"L{rl}"].split()
            kv = dict(zip(info[0::2], map(int, info[1::2])))
            rd = lambda n, t: np.fromfile(Path(tmp, f"L{rl}_{n}"), dtype=t)
            dm, rows, cols = rd("dofmap.i32", np.int32), rd("rows.i32", np.int32), rd("cols.i32", np.int32)
            verts, vals, rhs = rd("verts.f64", np.float64), rd("vals.f64", np.float64), rd("rhs.f64", np.float64)
            p = f"L{lvl}_"
            out[p + "sizes"] = np.array([kv["cells"], kv["nloc"], kv["n_dofs"], kv["active"], kv["nnz"]], np.int64)
            out[p + "digests"] = np.array([digest(dm), digest(rows), digest(cols), digest(verts)])
            for key, arr in (("vals", vals), ("rhs", rhs)):
                out[p + key + "_max"] = np.array(np.abs(arr).max())
                if full:
                    out[p + key] = arr
                else:
                    idx = sample_idx(arr.size)
                    out[p + key + "_idx"] = idx
                    out[p + key] = arr[idx]
            if full:
                out[p + "dofmap"], out[p + "rows"], out[p + "cols"] = dm, rows, cols
        sol = np.fromfile(Path(tmp, "solution.f64"), dtype=np.float64)
        out["solution_max"] = np.array(np.abs(sol).max())
        if full:
            out["solution"] = sol
        else:
            idx = sample_idx(sol.size)
            out["solution_idx"], out["solution"] = idx, sol[idx]
    np.savez_compressed(HERE / f"ref_{name}.npz", **out)
    print(f"{name}: {int(out['iterations'])} iterations, final residual {float(out['final_residual']):.3e}")


def run_stokes_case(name: str) -> None:
    import build_ref
    nref, nlev, full, direct = STOKES_CASES[name]
    exe = build_ref.link_program("3", build_ref.HERE / "ref_stokes.C", build_ref.OUT / "ref_stokes3d")
    out: dict[str, np.ndarray] = {"config": np.array([nref, nlev], dtype=np.int64)}
    with tempfile.TemporaryDirectory() as tmp:
        subprocess.run([str(exe), tmp, str(nref), str(nlev), "none"], check=True, capture_output=True)
        meta = {}
        for line in Path(tmp, "meta.txt").read_text().splitlines():
            k, v = line.split(None, 1)
            meta[k] = v
        for rl in range(nlev):
            lvl = nlev - 1 - rl
            info = meta[f"L{rl}"].split()
            kv = dict(zip(info[0::2], map(int, info[1::2])))
            rd = lambda n, t: np.fromfile(Path(tmp, f"L{rl}_{n}"), dtype=t)
            udm, pdm, verts = rd("u_dofmap.i32", np.int32), rd("p_dofmap.i32", np.int32), rd("verts.f64", np.float64)
            rows, cols, vals, rhs = (rd("rows.i32", np.int32), rd("cols.i32", np.int32), rd("vals.f64", np.float64),
                                     rd("rhs.f64", np.float64))
            p = f"L{lvl}_"
            out[p + "sizes"] = np.array([kv["cells"], kv["u_n_dofs"], kv["u_active"], kv["p_n_dofs"], kv["p_active"],
                                         kv["nnz"]], np.int64)
            out[p + "digests"] = np.array([digest(udm), digest(pdm), digest(verts)])
            out[p + "vals_max"] = np.array(np.abs(vals).max())
            out[p + "rhs_max"] = np.array(np.abs(rhs).max())
            out[p + "rhs"] = rhs
            if full:
                out[p + "rows"], out[p + "cols"], out[p + "vals"] = rows, cols, vals
            else:
                # a fixed sample of the combined matrix's entries as (row, column, value)
                idx = sample_idx(vals.size)
                row_of = np.repeat(np.arange(rows.size - 1, dtype=np.int32), np.diff(rows))
                out[p + "sample_rows"], out[p + "sample_cols"] = row_of[idx], cols[idx]
                out[p + "sample_vals"] = vals[idx]
    if direct:
        with tempfile.TemporaryDirectory() as tmp:
            subprocess.run([str(exe), tmp, str(nref), "1", "direct"], check=True, capture_output=True)
            out["solution"] = np.fromfile(Path(tmp, "solution.f64"), dtype=np.float64)
    np.savez_compressed(HERE / f"ref_{name}.npz", **out)
    print(f"{name}: {nlev} levels" + (", direct solution" if direct else ""))


def run_nse_case(name: str) -> None:
    import build_ref
    nref, nlev, solver, re, eps, maxit = NSE_CASES[name][:6]
    form = NSE_CASES[name][6] if len(NSE_CASES[name]) > 6 else "convective"
    exe = build_ref.link_program("3", build_ref.HERE / "ref_stokes.C", build_ref.OUT / "ref_stokes3d")
    out: dict[str, np.ndarray] = {"config": np.array([nref, nlev, maxit], dtype=np.int64),
                                  "params": np.array([re, eps]), "solver": np.array(solver),
                                  "form": np.array(form)}
    with tempfile.TemporaryDirectory() as tmp:
        subprocess.run([str(exe), tmp, str(nref), str(nlev), solver, "nse", repr(re), repr(eps), str(maxit), form],
                       check=True, capture_output=True)
        lines = Path(tmp, "meta.txt").read_text().splitlines()
        if solver == "none":
            for rl in range(nlev):
                lvl = nlev - 1 - rl
                info = next(l for l in lines if l.startswith(f"L{rl} ")).split()[1:]
                kv = dict(zip(info[0::2], map(int, info[1::2])))
                rd = lambda n, t: np.fromfile(Path(tmp, f"L{rl}_{n}"), dtype=t)
                rows, cols, vals = rd("rows.i32", np.int32), rd("cols.i32", np.int32), rd("vals.f64", np.float64)
                p = f"L{lvl}_"
                out[p + "sizes"] = np.array([kv["cells"], kv["u_n_dofs"], kv["u_active"], kv["p_n_dofs"], kv["nnz"]],
                                            np.int64)
                out[p + "velocity"] = rd("velocity.f64", np.float64)
                out[p + "vals_max"] = np.array(np.abs(vals).max())
                if lvl == 0:
                    out[p + "rows"], out[p + "cols"], out[p + "vals"] = rows, cols, vals
                else:
                    idx = sample_idx(vals.size)
                    row_of = np.repeat(np.arange(rows.size - 1, dtype=np.int32), np.diff(rows))
                    out[p + "sample_rows"], out[p + "sample_cols"] = row_of[idx], cols[idx]
                    out[p + "sample_vals"] = vals[idx]
        else:
            res = [list(map(float, l.split()[2:])) for l in lines if l.startswith("res ")]
            lin = [int(l.split()[2]) for l in lines if l.startswith("lin ")]
            out["residuals"] = np.array(res)
            # the solver's LoopInfo counts iterations over all solves
            out["linear_iterations"] = np.diff(np.array([0] + lin, dtype=np.int64))
            out["errors"] = np.array([float(v) for v in next(l for l in lines if l.startswith("errors")).split()[1:]])
            sol = np.fromfile(Path(tmp, "solution.f64"), dtype=np.float64)
            if sol.size <= 4 * SAMPLES:
                out["solution"] = sol
            else:
                idx = sample_idx(sol.size)
                out["solution_idx"], out["solution"] = idx, sol[idx]
    np.savez_compressed(HERE / f"ref_{name}.npz", **out)
    if "residuals" in out:
        print(f"{name}: {len(out['residuals']) - 1} nonlinear steps, residual {out['residuals'][-1][2]:.3e}")
    else:
        print(f"{name}: {nlev} levels after one nonlinear assembly")


if __name__ == "__main__":
    for n in (sys.argv[1:] or list(CASES) + list(STOKES_CASES) + list(NSE_CASES)):
        if n in STOKES_CASES:
            run_stokes_case(n)
        elif n in NSE_CASES:
            run_nse_case(n)
        else:
            run_case(n)
