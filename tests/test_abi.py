"""The C-ABI library loads and exports every symbol include/pmgpu.h declares
(no compute calls; no GPU needed)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared():
    text = (ROOT / "include" / "pmgpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pm_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from mymoonmd_gb300 import _lib
    lib = ctypes.CDLL(str(_lib._LIB_PATH))
    names = declared()
    assert len(names) >= 50
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # every declared function has a ctypes signature in the Python binding
    assert set(names) <= set(_lib.declared_symbols())


def test_version_and_error_paths_without_gpu():
    from mymoonmd_gb300 import _lib
    assert _lib.lib.pm_version() >= 1
    out = ctypes.c_void_p()
    rc = _lib.lib.pm_disc_create(7, 1, 1, 1, 0, 1, ctypes.byref(out))
    assert rc != 0 and b"" != _lib.lib.pm_last_error(None)


def test_parameter_database_defaults():
    from mymoonmd_gb300 import ParameterDatabase
    db = ParameterDatabase.solve_path_database()
    assert db["solver_type"] == "direct"
    assert db["gmres_restart"] == 20 and db["residual_tolerance"] == 1e-8
    assert db["multigrid_n_levels"] == 2 and db["multigrid_coarse_residual"] == 0.1
    db["preconditioner"] = "multigrid"
    try:
        db["preconditioner"] = "not_a_preconditioner"
        raise AssertionError("invalid choice accepted")
    except ValueError:
        pass
    assert "multigrid_cycle_type: V" in db.to_text()
