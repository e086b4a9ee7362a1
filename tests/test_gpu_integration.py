"""The C++ drop-in for ParMooN's Solver (integration/GpuSolver.C) drives the
GPU solve with the reference's semantics: the reference's own level matrices
and right-hand side (tests/golden/ref_cd2d_q2_16.npz, from ParMooN's
ConvectionDiffusion<2>) go in through BlockFEMatrix / BlockVector, the
multigrid hierarchy is handed over coarsest first, solve() starts from the
solution vector, and the result matches the reference's solution within
1e-10 with the iteration count within one; a wrong vector length comes back
as std::runtime_error (ErrThrow). Compiled here with g++ against the stand-in
headers of tests/gpusolver_standin/ (the reference sources are not needed)."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from ref_fixtures import RefCase

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def test_drop_in_solver_reproduces_the_reference_solve(tmp_path):
    rc = RefCase("cd2d_q2_16")
    for l in range(rc.n_levels):
        lv = rc.level(l)
        lv["rows"].astype(np.int32).tofile(tmp_path / f"L{l}_rows.i32")
        lv["cols"].astype(np.int32).tofile(tmp_path / f"L{l}_cols.i32")
        lv["vals"].astype(np.float64).tofile(tmp_path / f"L{l}_vals.f64")
        np.array([lv["active"]], np.int32).tofile(tmp_path / f"L{l}_active.i32")
    rc.level(rc.n_levels - 1)["rhs"].astype(np.float64).tofile(tmp_path / "rhs.f64")
    exe = tmp_path / "drive"
    lib = ROOT / "mymoonmd_gb300" / "libpmgpu.so"
    cmd = ["g++", "-std=c++11", "-O2", "-I", str(ROOT / "tests" / "gpusolver_standin"), "-I",
           str(ROOT / "integration"), "-I", str(ROOT / "include"), str(ROOT / "integration" / "GpuSolver.C"),
           str(ROOT / "tests" / "gpusolver_standin" / "drive.C"), str(lib), f"-Wl,-rpath,{lib.parent}",
           "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe), str(tmp_path), str(rc.n_levels), str(rc.geometry), str(rc.n_refine),
                        str(rc.order), str(rc.restart), repr(rc.reduction)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    first = r.stdout.splitlines()[0].split()
    its, init = int(first[1]), float(first[3])
    assert abs(its - rc.iterations) <= 1, (its, rc.iterations)
    assert abs(init - rc.initial_residual) <= 1e-12 * rc.initial_residual
    assert "runtime_error" in r.stdout and "length" in r.stdout
    sol = np.fromfile(tmp_path / "solution.f64", dtype=np.float64)
    assert rc.compare("solution", sol) <= 1e-10
