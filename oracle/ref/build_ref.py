"""Recipe that compiles the reference (ParMooN) itself into oracle/_ref/.

Test infrastructure only: the compiled reference generates the golden fixtures
under tests/golden/ (numbering, CSR structure, assembled entries, iteration
counts and solutions of the reference's own classes) and runs the reference's
own known-answer test programs. Nothing in the product links it, and the
reference sources are compiled where they lie; nothing is copied.

What the reference's CMake build would do, restated:
  * the source lists PARMOON_SOURCES_2D / PARMOON_SOURCES_3D of
    cmake/sources_*.cmake, minus the files that are absent from the snapshot,
    the Fortran file (no gfortran here), the reduced-order models (Boost) and
    three files that do not compile in this snapshot (src/System/Brinkman2D.C,
    src/System/Brinkman3D.C, and src/Geometry/AdaptiveRefine.C in 2D, which
    includes a missing Vector.h) - none of them is on the solve path;
  * g++ -std=c++11 -O2 -DNDEBUG -D__2D__ | -D__3D__ (SEQUENTIAL build);
  * the two configure-time headers (ParMooN_repository_info.h,
    all_defines_external_libraries.h) are written by this script with fixed
    content: a sequential build with UMFPACK;
  * UMFPACK is replaced by the dense-LU stand-in oracle/ref/umfpack_dense.c
    behind the published interface (oracle/ref/umfpack.h), and LAPACK by
    oracle/ref/lapack_shim.c, which forwards to scipy's bundled OpenBLAS.

Usage: python oracle/ref/build_ref.py [2|3 ...] (default both). Needs the
reference sources (REFERENCE_ROOT, default /root/reference) and scipy.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"
REF = Path(os.environ.get("REFERENCE_ROOT", "/root/reference"))

CXXFLAGS = ["-std=c++11", "-O2", "-DNDEBUG", "-w"]
# Parameter.C / PDECoefficients.C use std::numeric_limits and std::ostream
# without including their headers (a GCC 13 difference from the compilers the
# reference was written against).
FORCED_INCLUDES = ["-include", "limits", "-include", "ostream"]
EXCLUDED = ("/ReducedOrderModels/", "/System/Brinkman2D.C", "/System/Brinkman3D.C", ".f90", ".f")
EXCLUDED_2D = ("/Geometry/AdaptiveRefine.C",)

REPO_INFO_H = """#ifndef PARMOON__REPOSITORY_INFO
#define PARMOON__REPOSITORY_INFO
namespace parmoon
{
constexpr const char * hg_revision = "unknown";
constexpr const char * hg_branch = "unknown";
constexpr const bool hg_local_changes = false;
constexpr const char * parallel_type = "SEQUENTIAL";
constexpr const char * build_type = "Release";
constexpr const char * source_directory = "reference";
}
#endif
"""

DEFINES_H = """// configure-time switches of the oracle's sequential build of the reference
#define PARMOON_WITH_BLAS
#define PARMOON_WITH_LAPACK
#define PARMOON_WITH_UMFPACK
"""


def source_lists() -> dict[str, list[str]]:
    """PARMOON_SOURCES_2D/3D as cmake/sources_*.cmake append them."""
    vars_: dict[str, list[str]] = {}
    for f in sorted((REF / "cmake").glob("sources_*.cmake")):
        txt = f.read_text(encoding="utf-8-sig")
        for m in re.finditer(r"list\s*\(\s*APPEND\s+(\w+)\s+([^)]*)\)", txt):
            out: list[str] = []
            for it in m.group(2).split():
                it = it.strip('"')
                mv = re.fullmatch(r"\$\{(\w+)\}", it)
                if mv:
                    out += vars_.get(mv.group(1), [])
                else:
                    out.append(it.replace("${PROJECT_SOURCE_DIR}", str(REF))
                               .replace("${CMAKE_SOURCE_DIR}", str(REF)))
            vars_.setdefault(m.group(1), []).extend(out)
    return {"2": vars_["PARMOON_SOURCES_2D"], "3": vars_["PARMOON_SOURCES_3D"]}


def include_flags() -> list[str]:
    dirs = [REF / "include"] + sorted(p for p in (REF / "include").rglob("*") if p.is_dir())
    flags = ["-I", str(OUT / "cfg"), "-I", str(HERE)]
    for d in dirs:
        flags += ["-I", str(d)]
    return flags


def _run(cmd: list[str]) -> tuple[int, str]:
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.returncode, r.stderr[-3000:]


def _compile(args: tuple[str, str, Path]) -> tuple[str, int, str]:
    src, dim, obj = args
    if obj.exists() and obj.stat().st_mtime >= Path(src).stat().st_mtime:
        return src, 0, ""
    cmd = ["g++", *CXXFLAGS, f"-D__{dim}D__", *FORCED_INCLUDES, *include_flags(), "-c", src,
           "-o", str(obj)]
    rc, err = _run(cmd)
    return src, rc, err


def openblas() -> Path:
    import scipy
    libs = Path(scipy.__file__).resolve().parent.parent / "scipy.libs"
    cands = sorted(libs.glob("libscipy_openblas*.so"))
    if not cands:
        raise RuntimeError(f"no scipy OpenBLAS under {libs}")
    return cands[0]


def build_lib(dim: str, jobs: int = 0) -> Path:
    """Compile one dimension's library into oracle/_ref/libparmoon_{dim}d.a."""
    (OUT / "cfg").mkdir(parents=True, exist_ok=True)
    for name, text in (("ParMooN_repository_info.h", REPO_INFO_H),
                       ("all_defines_external_libraries.h", DEFINES_H)):
        p = OUT / "cfg" / name
        if not p.exists() or p.read_text() != text:
            p.write_text(text)
    objdir = OUT / f"obj{dim}d"
    objdir.mkdir(exist_ok=True)
    srcs = []
    for s in source_lists()[dim]:
        if s.endswith(EXCLUDED) or "/ReducedOrderModels/" in s or (dim == "2" and s.endswith(EXCLUDED_2D)):
            continue
        if not Path(s).exists():  # listed in the cmake files, absent from the snapshot
            continue
        rel = Path(s).relative_to(REF / "src")
        srcs.append((s, dim, objdir / (str(rel).replace("/", "__") + ".o")))
    jobs = jobs or (os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        res = list(ex.map(_compile, srcs))
    bad = [r for r in res if r[1]]
    if bad:
        raise RuntimeError("reference sources failed to compile:\n" +
                           "\n".join(f"{s}:\n{e}" for s, _, e in bad))
    lib = OUT / f"libparmoon_{dim}d.a"
    newest = max(o.stat().st_mtime for _, _, o in srcs)
    if not lib.exists() or lib.stat().st_mtime < newest:
        if lib.exists():
            lib.unlink()
        rc, err = _run(["ar", "rcs", str(lib), *[str(o) for _, _, o in srcs]])
        if rc:
            raise RuntimeError(err)
    return lib


def build_shims() -> list[Path]:
    outs = []
    for name in ("umfpack_dense.c", "lapack_shim.c"):
        src = HERE / name
        obj = OUT / (name + ".o")
        if not obj.exists() or obj.stat().st_mtime < src.stat().st_mtime:
            rc, err = _run(["gcc", "-O2", "-std=c99", "-c", str(src), "-o", str(obj)])
            if rc:
                raise RuntimeError(err)
        outs.append(obj)
    return outs


def link_program(dim: str, src: Path, exe: Path) -> Path:
    """Compile a driver (ours, or one of the reference's test programs where it
    lies) against the compiled reference."""
    lib = build_lib(dim)
    shims = build_shims()
    deps = [src, lib, *shims]
    if exe.exists() and exe.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return exe
    blas = openblas()
    cmd = ["g++", *CXXFLAGS, f"-D__{dim}D__", *FORCED_INCLUDES, *include_flags(), str(src),
           str(lib), *map(str, shims), str(blas), f"-Wl,-rpath,{blas.parent}", "-o", str(exe)]
    rc, err = _run(cmd)
    if rc:
        raise RuntimeError(f"link of {src.name} failed:\n{err}")
    return exe


def main(argv: list[str]) -> None:
    dims = [a for a in argv if a in ("2", "3")] or ["2", "3"]
    for d in dims:
        print(build_lib(d))
    print(build_shims())


if __name__ == "__main__":
    main(sys.argv[1:])
