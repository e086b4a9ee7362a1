"""Build recipe of the oracle's C restatement (test infrastructure only):
gcc -O2 -shared oracle/oracle.c -> oracle/_build/liboracle.so.

The reference itself is not compiled: its solve path needs CMake-generated
headers and external LAPACK/UMFPACK libraries, so it is treated as
unbuildable and the oracle restates it in C instead.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle.c"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "liboracle.so"


def build() -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    if LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off", str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build())
