"""ParameterDatabase mirror: typed keys with the reference's names, defaults and
allowed values for the solve path.

Defaults follow Solver<>::default_solver_database (src/Solver/Solver.C:21-115)
and Multigrid::default_multigrid_database (src/Multigrid/Multigrid.C:422-514).
New keys with defaults here: `gpu_precision` (fp64 | mixed), `gpu_mixed_fallback`
(0 | 1) and `gpu_mixed_coarse` (fp32 | fp64); `gpu_gram_schmidt` and `gpu_cuda_graphs` can be
added with `add`.
"""
from __future__ import annotations

from typing import Any

_SOLVER_DEFAULTS: dict[str, tuple[Any, tuple | None]] = {
    "solver_type": ("direct", ("direct", "iterative", "petsc")),
    "direct_solver_type": ("umfpack", ("umfpack", "pardiso", "mumps")),
    "iterative_solver_type": ("fgmres", ("jacobi", "sor", "ssor", "richardson", "cg", "cgs",
                                         "bi_cgstab", "left_gmres", "right_gmres", "fgmres")),
    "max_n_iterations": (100, None),
    "min_n_iterations": (0, None),
    "residual_tolerance": (1.0e-8, None),
    "residual_reduction": (0.0, None),
    "divergence_factor": (1.0e10, None),
    "gmres_restart": (20, None),
    "preconditioner": ("no_preconditioner", ("no_preconditioner", "jacobi", "sor", "ssor",
                                             "multigrid", "vanka_cell", "vanka_nodal",
                                             "vanka_cell_jacobi")),
    "sor_omega": (1.5, None),
    "damping_factor": (1.0, None),
}

_MG_DEFAULTS: dict[str, tuple[Any, tuple | None]] = {
    "multigrid_n_levels": (2, None),
    "multigrid_type": ("standard", ("standard", "mdml")),
    "multigrid_cycle_type": ("V", ("V", "W", "F")),
    # the reference's choices, plus "nodal_vanka_jacobi" (additive nodal Vanka,
    # the CELL_JACOBI treatment on nodal patches), which only this library has
    "multigrid_smoother": ("nodal_vanka", ("jacobi", "sor", "ssor", "nodal_vanka", "cell_vanka",
                                           "patch_vanka", "cell_vanka_jacobi", "nodal_vanka_store",
                                           "cell_vanka_store", "patch_vanka_store", "nodal_vanka_jacobi")),
    "multigrid_smoother_coarse": ("direct_solve", ("direct_solve", "jacobi", "sor", "ssor",
                                                   "nodal_vanka", "cell_vanka", "patch_vanka",
                                                   "cell_vanka_jacobi", "nodal_vanka_jacobi")),
    "multigrid_correction_damp_factor": (1.0, None),
    "multigrid_n_pre_smooth": (1, None),
    "multigrid_n_post_smooth": (1, None),
    "multigrid_coarse_residual": (1.0e-1, None),
    "multigrid_coarse_max_n_iterations": (10, None),
    "multigrid_vanka_damp_factor": (1.0, None),
    "jacobi_damp": (1.0, None),
}

_GPU_DEFAULTS: dict[str, tuple[Any, tuple | None]] = {
    "gpu_precision": ("fp64", ("fp64", "mixed")),
    # mixed form: the multigrid switches to FP64 for the rest of a solve when
    # the FP64 residual falls by less than half over 10 FGMRES iterations
    "gpu_mixed_fallback": (1, (0, 1)),
    # mixed form: the coarse direct solve with an FP32 inverse or with the
    # FP64 inverse (FP32 vectors in and out, FP64 products and sums)
    "gpu_mixed_coarse": ("fp32", ("fp32", "fp64")),
}

# TimeDiscretization::default_TimeDiscretization_database
# (src/TimeDiscRoutines/TimeDiscretizations.C:23-56); fractional_step is not
# implemented on the GPU
_TIME_DEFAULTS: dict[str, tuple[Any, tuple | None]] = {
    "time_start": (0.0, None),
    "time_end": (1.0, None),
    "time_step_length": (0.05, None),
    "time_discretization": ("backward_euler", ("backward_euler", "crank_nicolson", "bdf_two")),
}


class ParameterDatabase:
    """Typed key/value store; unknown keys may be added with `add`."""

    def __init__(self, name: str = "database"):
        self.name = name
        self._values: dict[str, Any] = {}
        self._choices: dict[str, tuple | None] = {}

    def add(self, key: str, value: Any, choices: tuple | None = None) -> None:
        self._values[key] = value
        self._choices[key] = choices

    def __contains__(self, key: str) -> bool:
        return key in self._values

    def __getitem__(self, key: str) -> Any:
        if key not in self._values:
            raise KeyError(f"parameter {key} is not in the database {self.name}")
        return self._values[key]

    def __setitem__(self, key: str, value: Any) -> None:
        if key not in self._values:
            raise KeyError(f"parameter {key} is not in the database {self.name}")
        choices = self._choices.get(key)
        old = self._values[key]
        if isinstance(old, bool):
            value = bool(value)
        elif isinstance(old, int) and not isinstance(value, str):
            value = int(value)
        elif isinstance(old, float) and not isinstance(value, str):
            value = float(value)
        if choices is not None and value not in choices:
            raise ValueError(f"value {value!r} of {key} is not one of {choices}")
        self._values[key] = value

    def merge(self, other: "ParameterDatabase", create_new: bool = True) -> None:
        for k, v in other._values.items():
            if k in self._values:
                self._values[k] = v
            elif create_new:
                self.add(k, v, other._choices.get(k))

    def keys(self):
        return self._values.keys()

    def to_text(self) -> str:
        lines = []
        for k, v in self._values.items():
            if isinstance(v, float):
                lines.append(f"{k}: {v!r}")
            else:
                lines.append(f"{k}: {v}")
        return "\n".join(lines) + "\n"

    @staticmethod
    def _from(defaults: dict, name: str) -> "ParameterDatabase":
        db = ParameterDatabase(name)
        for k, (v, ch) in defaults.items():
            db.add(k, v, ch)
        return db

    @staticmethod
    def default_solver_database() -> "ParameterDatabase":
        return ParameterDatabase._from(_SOLVER_DEFAULTS, "default solver database")

    @staticmethod
    def default_multigrid_database() -> "ParameterDatabase":
        return ParameterDatabase._from(_MG_DEFAULTS, "default multigrid database")

    @staticmethod
    def default_gpu_database() -> "ParameterDatabase":
        return ParameterDatabase._from(_GPU_DEFAULTS, "gpu database")

    @staticmethod
    def default_time_database() -> "ParameterDatabase":
        return ParameterDatabase._from(_TIME_DEFAULTS, "default time discretization database")

    @staticmethod
    def solve_path_database() -> "ParameterDatabase":
        db = ParameterDatabase.default_solver_database()
        db.merge(ParameterDatabase.default_multigrid_database())
        db.merge(ParameterDatabase.default_gpu_database())
        db.name = "solve path database"
        return db
