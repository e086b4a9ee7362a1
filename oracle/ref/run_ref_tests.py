"""Compile and run the reference's own known-answer test programs for the solve
path against the oracle's build of the reference (test infrastructure only).

Each program is compiled from the reference's test/ directory where it lies
and linked with oracle/_ref/libparmoon_{2,3}d.a (oracle/ref/build_ref.py),
with the arguments the reference's test/CMakeLists.txt registers. A program
that exits 0 has reproduced every golden value it checks (error norms,
exact polynomial solutions, known SpMV results), so this pins the build that
generates the fixtures of tests/golden/ref_*.npz.

    python oracle/ref/run_ref_tests.py          # all, prints one line each
    python oracle/ref/run_ref_tests.py cd2d     # the ones whose name contains "cd2d"
"""
from __future__ import annotations

import subprocess
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

import build_ref  # noqa: E402

# (name, dimension, source under test/, arguments) as test/CMakeLists.txt
# registers them; the programs that exercise the solve path
PROGRAMS = [
    ("matrix", "2", "matrix_test.c++", []),
    ("block_matrix", "2", "block_matrix_test.c++", []),
    ("block_fe_matrix", "2", "block_fe_matrix_test.c++", []),
    ("direct_solver", "2", "direct_solver_test.c++", []),
    ("iterative_solver", "2", "iterative_solver_test.c++", []),
    ("multigrid_2d", "2", "multigrid_test.c++", []),
    ("multigrid_3d", "3", "multigrid_test.c++", []),
    ("cd2d", "2", "cd2d_test.c++", []),
    ("cd3d_umfpack", "3", "cd3d_solvers_test.c++", ["umfpack"]),
    ("cd3d_jacobi", "3", "cd3d_solvers_test.c++", ["jacobi"]),
    ("cd3d_multigrid", "3", "cd3d_solvers_test.c++", ["multigrid"]),
    ("tcd3d_umfpack", "3", "tcd3d_solvers_test.c++", ["umfpack"]),
    ("tcd3d_multigrid", "3", "tcd3d_solvers_test.c++", ["multigrid"]),
    ("nse3d_umfpack", "3", "nse3d_solvers_test.c++", ["umfpack"]),
    ("nse3d_multigrid", "3", "nse3d_solvers_test.c++", ["multigrid"]),
    ("nse3d_cell_vanka_jacobi", "3", "nse3d_solvers_test.c++", ["cell_vanka_jacobi"]),
]


def run(name: str, timeout: float = 1800.0) -> tuple[int, float, str]:
    """returns (exit code, seconds, last lines of output)"""
    prog = next(p for p in PROGRAMS if p[0] == name)
    _, dim, src, args = prog
    exe = build_ref.OUT / ("t_" + Path(src).stem + f"_{dim}d")
    build_ref.link_program(dim, build_ref.REF / "test" / src, exe)
    workdir = build_ref.OUT / "run" / name
    workdir.mkdir(parents=True, exist_ok=True)
    t0 = time.perf_counter()
    r = subprocess.run([str(exe), *args], cwd=workdir, capture_output=True, text=True, timeout=timeout)
    tail = "\n".join((r.stdout + r.stderr).strip().splitlines()[-5:])
    return r.returncode, time.perf_counter() - t0, tail


def main(argv: list[str]) -> int:
    pick = [p[0] for p in PROGRAMS if not argv or any(a in p[0] for a in argv)]
    bad = 0
    for name in pick:
        rc, secs, tail = run(name)
        print(f"{name:28s} exit {rc}  {secs:7.1f} s")
        if rc:
            bad += 1
            print("    " + tail.replace("\n", "\n    "))
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
