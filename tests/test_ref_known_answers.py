"""The reference's own known-answer test programs, compiled from the reference
sources against the oracle's build of the reference (oracle/ref/), exit 0:
every golden value they hold is reproduced by the build that generates
tests/golden/ref_*.npz (cd2d_test's L2/H1/SD/L-infinity error norms for Q1-Q8
and P1-P6 with the direct, FGMRES+SSOR and FGMRES+multigrid solvers;
cd3d_solvers_test's exact polynomial solutions with UMFPACK, Jacobi and
multigrid; tcd3d_solvers_test; nse3d_solvers_test with UMFPACK, multigrid and
cell Vanka; the matrix, block matrix, solver and multigrid unit tests).

Runs where the reference sources are present and its build exists
(oracle/_ref, made by __graft_entry__.build() or oracle/ref/build_ref.py);
skipped elsewhere.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle" / "ref"))


def _available() -> bool:
    try:
        import build_ref
    except Exception:
        return False
    return build_ref.REF.is_dir() and all((build_ref.OUT / f"libparmoon_{d}d.a").exists() for d in "23")


@pytest.mark.skipif(not _available(), reason="the reference sources or its oracle build are not present")
@pytest.mark.parametrize("name", [p[0] for p in __import__("run_ref_tests").PROGRAMS] if _available() else [])
def test_reference_known_answer_program_passes(name):
    import run_ref_tests
    rc, secs, tail = run_ref_tests.run(name, timeout=600)
    assert rc == 0, tail
