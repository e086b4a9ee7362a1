"""The C++ drop-in for ParMooN's Solver (integration/GpuSolver.{h,C}) and the
example main program (integration/example_cd.C) compile against the
reference's own headers and link with the reference's library and
libpmgpu.so (CPU only; the GPU run is tests/test_gpu_integration.py).

Where the reference sources or their oracle build are absent, the drop-in is
still compiled against the stand-in headers of tests/gpusolver_standin/."""
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle" / "ref"))


def _reference():
    try:
        import build_ref
    except Exception:
        return None
    if not build_ref.REF.is_dir() or not all((build_ref.OUT / f"libparmoon_{d}d.a").exists() for d in "23"):
        return None
    return build_ref


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.skipif(_reference() is None, reason="the reference sources or its oracle build are not present")
@pytest.mark.parametrize("dim", ["2", "3"])
def test_drop_in_compiles_and_links_in_the_reference_tree(dim, tmp_path):
    b = _reference()
    lib = ROOT / "mymoonmd_gb300" / "libpmgpu.so"
    if not lib.exists():
        pytest.skip("libpmgpu.so is not built")
    flags = ["g++", "-std=c++11", "-O1", "-Wall", "-Wextra", f"-D__{dim}D__", *b.FORCED_INCLUDES,
             *b.include_flags(), "-I", str(ROOT / "include"), "-I", str(ROOT / "integration")]
    objs = []
    for src in ("GpuSolver.C", "example_cd.C"):
        obj = tmp_path / (src + ".o")
        _run([*flags, "-c", str(ROOT / "integration" / src), "-o", str(obj)])
        objs.append(str(obj))
    blas = b.openblas()
    _run(["g++", *objs, str(b.build_lib(dim)), *map(str, b.build_shims()), str(blas),
          f"-Wl,-rpath,{blas.parent}", str(lib), "-o", str(tmp_path / "example_cd")])


def test_drop_in_compiles_against_the_stand_in_headers():
    _run(["g++", "-std=c++11", "-Wall", "-Wextra", "-fsyntax-only", "-I", str(ROOT / "tests" / "gpusolver_standin"),
          "-I", str(ROOT / "integration"), "-I", str(ROOT / "include"), str(ROOT / "integration" / "GpuSolver.C"),
          str(ROOT / "tests" / "gpusolver_standin" / "drive.C")])
