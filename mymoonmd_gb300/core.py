"""Python mirror of the reference's matrix / vector / solver classes over the C ABI.

Context       - one GPU, one CUDA stream (pm_ctx)
DeviceVector  - FP64 (or FP32) array on the device; BlockVector storage
FEMatrix      - TMatrix/FEMatrix/BlockFEMatrix in CSR on the device (pm_matrix)
Solver        - Solver<BlockFEMatrix, BlockVector> driven by a ParameterDatabase
Discretization, ConvectionDiffusion - the set-up and system classes of the
convection-diffusion solve path (ConvectionDiffusion<d>, src/System/ConvectionDiffusion.C)
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from ._lib import CdCoeffs, PmError, check, lib
from .parameter_database import ParameterDatabase

GEO_SQUARE_QUAD = 0
GEO_CUBE_HEXA = 1
GEO_CUBE_TETRA = 2
KIND_CD = 0
KIND_STOKES = 1


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class Context:
    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib.pm_ctx_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def close(self) -> None:
        if self.handle:
            lib.pm_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self) -> None:
        check(lib.pm_ctx_synchronize(self.handle), self.handle)

    def set_option(self, key: str, value: int) -> None:
        check(lib.pm_ctx_set_option(self.handle, key.encode(), int(value)), self.handle)

    def kernel_launches(self) -> int:
        v = C.c_uint64()
        check(lib.pm_ctx_kernel_launches(self.handle, C.byref(v)))
        return int(v.value)

    def time_begin(self) -> None:
        check(lib.pm_ctx_time_begin(self.handle), self.handle)

    def time_end(self) -> float:
        ms = C.c_float()
        check(lib.pm_ctx_time_end(self.handle, C.byref(ms)), self.handle)
        return float(ms.value)

    def probe(self, nnz: int) -> None:
        """bracket SpMV-family launches on matrices with `nnz` nonzeros by events (0 = off)"""
        check(lib.pm_ctx_probe(self.handle, int(nnz)), self.handle)

    def probe_result(self) -> tuple[int, float, float]:
        n, ms, b = C.c_int(), C.c_double(), C.c_double()
        check(lib.pm_ctx_probe_result(self.handle, C.byref(n), C.byref(ms), C.byref(b)), self.handle)
        return n.value, ms.value, b.value


class PinnedArray:
    """page-locked host array (cudaMallocHost through the library)"""

    def __init__(self, ctx: Context, n: int, dtype=np.float64):
        self.ctx = ctx
        dt = np.dtype(dtype)
        p = C.c_void_p()
        check(lib.pm_host_alloc(ctx.handle, max(1, n * dt.itemsize), C.byref(p)), ctx.handle)
        self.ptr = p
        buf = (C.c_byte * max(1, n * dt.itemsize)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dt, count=n)

    def free(self) -> None:
        if self.ptr:
            self.array = None
            lib.pm_host_free(self.ctx.handle, self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            if self.ptr and self.ctx.handle:
                self.free()
        except Exception:
            pass


class DeviceVector:
    """Device array (FP64 by default) owned by Python."""

    def __init__(self, ctx: Context, n: int, dtype=np.float64):
        self.ctx = ctx
        self.n = int(n)
        self.dtype = np.dtype(dtype)
        p = C.c_void_p()
        check(lib.pm_dev_alloc(ctx.handle, max(1, self.n * self.dtype.itemsize), C.byref(p)), ctx.handle)
        self.ptr = p
        self.zero()

    @classmethod
    def from_numpy(cls, ctx: Context, a: np.ndarray) -> "DeviceVector":
        a = np.ascontiguousarray(a)
        v = cls(ctx, a.size, a.dtype)
        v.upload(a)
        return v

    def upload(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=self.dtype)
        if a.size != self.n:
            raise ValueError("length mismatch")
        check(lib.pm_memcpy_h2d(self.ctx.handle, self.ptr, _ptr(a), a.nbytes), self.ctx.handle)

    def numpy(self) -> np.ndarray:
        out = np.empty(self.n, dtype=self.dtype)
        check(lib.pm_memcpy_d2h(self.ctx.handle, _ptr(out), self.ptr, out.nbytes), self.ctx.handle)
        return out

    def zero(self) -> None:
        check(lib.pm_memset_dev(self.ctx.handle, self.ptr, 0, max(1, self.n * self.dtype.itemsize)),
              self.ctx.handle)

    def norm(self) -> float:
        out = C.c_double()
        check(lib.pm_norm(self.ctx.handle, self.n, self.ptr, C.byref(out)), self.ctx.handle)
        return out.value

    def dot(self, other: "DeviceVector") -> float:
        out = C.c_double()
        check(lib.pm_dot(self.ctx.handle, self.n, self.ptr, other.ptr, C.byref(out)), self.ctx.handle)
        return out.value

    def add_scaled(self, x: "DeviceVector", a: float) -> None:
        check(lib.pm_axpy(self.ctx.handle, self.n, a, x.ptr, self.ptr), self.ctx.handle)

    def scale(self, a: float) -> None:
        check(lib.pm_scal(self.ctx.handle, self.n, a, self.ptr), self.ctx.handle)

    def free(self) -> None:
        if self.ptr:
            lib.pm_dev_free(self.ctx.handle, self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            if self.ptr and self.ctx.handle:
                self.free()
        except Exception:
            pass


class FEMatrix:
    """CSR matrix with an active bound on the device (TMatrix/FEMatrix/BlockFEMatrix)."""

    def __init__(self, ctx: Context, handle, owned: bool = True):
        self.ctx = ctx
        self.handle = handle
        self.owned = owned

    @classmethod
    def from_csr(cls, ctx: Context, row_ptr, cols, vals=None, n_active: Optional[int] = None,
                 n_cols: Optional[int] = None) -> "FEMatrix":
        rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
        ci = np.ascontiguousarray(cols, dtype=np.int32)
        n = rp.size - 1
        nc = n if n_cols is None else int(n_cols)
        na = n if n_active is None else int(n_active)
        vv = None if vals is None else np.ascontiguousarray(vals, dtype=np.float64)
        h = C.c_void_p()
        check(lib.pm_matrix_create_csr(ctx.handle, n, nc, na, _ptr(rp), _ptr(ci),
                                       _ptr(vv) if vv is not None else None, C.byref(h)), ctx.handle)
        return cls(ctx, h)

    def set_blocks(self, lengths, actives) -> None:
        ln = np.ascontiguousarray(lengths, dtype=np.int32)
        ac = np.ascontiguousarray(actives, dtype=np.int32)
        check(lib.pm_matrix_set_blocks(self.handle, ln.size, _ptr(ln), _ptr(ac)), self.ctx.handle)

    def info(self) -> tuple[int, int, int, int]:
        r, c, a = C.c_int(), C.c_int(), C.c_int()
        z = C.c_int64()
        check(lib.pm_matrix_info(self.handle, C.byref(r), C.byref(c), C.byref(a), C.byref(z)))
        return r.value, c.value, a.value, int(z.value)

    @property
    def n_rows(self) -> int:
        return self.info()[0]

    @property
    def nnz(self) -> int:
        return self.info()[3]

    def values(self) -> np.ndarray:
        out = np.empty(self.nnz, dtype=np.float64)
        check(lib.pm_matrix_get_values(self.handle, _ptr(out)), self.ctx.handle)
        return out

    def set_values(self, vals) -> None:
        v = np.ascontiguousarray(vals, dtype=np.float64)
        check(lib.pm_matrix_set_values(self.handle, _ptr(v)), self.ctx.handle)

    def structure(self) -> tuple[np.ndarray, np.ndarray]:
        n, _, _, nnz = self.info()
        rp = np.empty(n + 1, dtype=np.int32)
        ci = np.empty(nnz, dtype=np.int32)
        check(lib.pm_matrix_get_structure(self.handle, _ptr(rp), _ptr(ci)), self.ctx.handle)
        return rp, ci

    def apply_scaled_add(self, x: DeviceVector, y: DeviceVector, a: float = 1.0) -> None:
        check(lib.pm_matrix_apply_scaled_add(self.handle, x.ptr, y.ptr, a), self.ctx.handle)

    def apply(self, x: DeviceVector, y: DeviceVector) -> None:
        check(lib.pm_matrix_apply(self.handle, x.ptr, y.ptr), self.ctx.handle)

    def get_diagonal(self) -> np.ndarray:
        n = self.n_rows
        d = DeviceVector(self.ctx, n)
        check(lib.pm_matrix_get_diagonal(self.handle, d.ptr), self.ctx.handle)
        return d.numpy()

    def make_fp32(self) -> None:
        check(lib.pm_matrix_make_fp32(self.handle), self.ctx.handle)

    def make_sliced64(self) -> None:
        check(lib.pm_matrix_make_sliced64(self.handle), self.ctx.handle)

    def apply_f32(self, x: DeviceVector, y: DeviceVector) -> None:
        check(lib.pm_matrix_apply_f32(self.handle, x.ptr, y.ptr), self.ctx.handle)

    def set_kernel(self, lanes: int = 0, unroll: int = 0) -> None:
        check(lib.pm_matrix_set_kernel(self.handle, lanes, unroll), self.ctx.handle)

    def bench_apply(self, x: DeviceVector, y: DeviceVector, reps: int, fp32: bool = False):
        ms = C.c_float()
        b = C.c_double()
        check(lib.pm_matrix_bench_apply(self.handle, int(fp32), x.ptr, y.ptr, reps, C.byref(ms),
                                        C.byref(b)), self.ctx.handle)
        return float(ms.value), float(b.value)

    def close(self) -> None:
        # after Context.close() the native context is gone; the handle is dropped
        if self.owned and self.handle and self.ctx.handle:
            lib.pm_matrix_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _db_text(db) -> str:
    if db is None:
        return ""
    if isinstance(db, ParameterDatabase):
        return db.to_text()
    if isinstance(db, dict):
        return "".join(f"{k}: {v}\n" for k, v in db.items())
    return str(db)


class Solver:
    """Solver<BlockFEMatrix, BlockVector> (include/Solver/Solver.h:31-127)."""

    def __init__(self, ctx: Context, db, handle=None, owned: bool = True):
        self.ctx = ctx
        if handle is None:
            h = C.c_void_p()
            check(lib.pm_solver_create(ctx.handle, _db_text(db).encode(), C.byref(h)), ctx.handle)
            handle = h
        self.handle = handle
        self.owned = owned
        self._keep = []

    @staticmethod
    def default_solver_database() -> ParameterDatabase:
        return ParameterDatabase.default_solver_database()

    def set_multigrid_level(self, level: int, n_levels: int, A: FEMatrix, P=None) -> None:
        """Multigrid::initialize: level 0 = coarsest; P = (row_ptr, cols, vals, n_rows)
        prolongation from this level to the next finer one."""
        if P is None:
            check(lib.pm_solver_set_multigrid_level(self.handle, level, n_levels, A.handle, 0, 0,
                                                    None, None, None), self.ctx.handle)
        else:
            rp, ci, v = (np.ascontiguousarray(P[0], dtype=np.int32), np.ascontiguousarray(P[1], dtype=np.int32),
                         np.ascontiguousarray(P[2], dtype=np.float64))
            check(lib.pm_solver_set_multigrid_level(self.handle, level, n_levels, A.handle, rp.size - 1,
                                                    A.n_rows, _ptr(rp), _ptr(ci), _ptr(v)), self.ctx.handle)
        self._keep.append(A)

    def update_matrix(self, A: FEMatrix) -> None:
        check(lib.pm_solver_update_matrix(self.handle, A.handle), self.ctx.handle)
        self._keep.append(A)

    def solve(self, rhs, sol) -> None:
        """solve(rhs, sol): device vectors, or numpy arrays (solution written back)."""
        if isinstance(rhs, DeviceVector):
            check(lib.pm_solver_solve(self.handle, rhs.ptr, sol.ptr), self.ctx.handle)
        else:
            r = np.ascontiguousarray(rhs, dtype=np.float64)
            if not (isinstance(sol, np.ndarray) and sol.dtype == np.float64 and sol.flags.c_contiguous):
                raise TypeError("host solution must be a contiguous float64 numpy array")
            check(lib.pm_solver_solve_host(self.handle, _ptr(r), _ptr(sol), r.size), self.ctx.handle)

    def apply_preconditioner(self, z: DeviceVector, r: DeviceVector) -> None:
        check(lib.pm_solver_apply_preconditioner(self.handle, z.ptr, r.ptr), self.ctx.handle)

    def last_info(self) -> tuple[int, float, float]:
        it, res, init = C.c_int(), C.c_double(), C.c_double()
        check(lib.pm_solver_last_info(self.handle, C.byref(it), C.byref(res), C.byref(init)))
        return it.value, res.value, init.value

    def residual_history(self) -> np.ndarray:
        cnt = C.c_int()
        buf = np.empty(100000, dtype=np.float64)
        check(lib.pm_solver_residual_history(self.handle, _ptr(buf), buf.size, C.byref(cnt)))
        return buf[: min(cnt.value, buf.size)].copy()

    def close(self) -> None:
        if self.owned and self.handle and self.ctx.handle:
            lib.pm_solver_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Discretization:
    """Mesh hierarchy + FE spaces + structures + transfer (host set-up)."""

    def __init__(self, geometry: int, root_n: int, n_refine: int, n_levels: int, kind: int = KIND_CD,
                 elem: int = 1, neumann_sides: int = 0, ctx: Optional["Context"] = None):
        """neumann_sides: bit mask of the unit square's sides (0 y=0, 1 x=1,
        2 y=1, 3 x=0) with Neumann conditions; the others are Dirichlet.
        ctx: build the structure and the gather plans on that context's GPU
        (pm_disc_create_device); the same discretisation as without"""
        h = C.c_void_p()
        if ctx is not None:
            check(lib.pm_disc_create_device(ctx.handle, geometry, root_n, n_refine, n_levels, kind, elem,
                                            neumann_sides, C.byref(h)), ctx.handle)
        else:
            check(lib.pm_disc_create_bc(geometry, root_n, n_refine, n_levels, kind, elem, neumann_sides,
                                        C.byref(h)))
        self.handle = h
        self.geometry, self.root_n, self.n_refine, self.n_levels = geometry, root_n, n_refine, n_levels
        self.kind, self.elem, self.neumann_sides = kind, elem, neumann_sides
        self.dim = 2 if geometry == GEO_SQUARE_QUAD else 3

    def level_info(self, level: int, space: int = 0) -> dict:
        nc, nl, nd, na = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        nz = C.c_int64()
        check(lib.pm_disc_level_info(self.handle, level, space, C.byref(nc), C.byref(nl), C.byref(nd),
                                     C.byref(na), C.byref(nz)))
        return dict(n_cells=nc.value, nloc=nl.value, n_dofs=nd.value, n_active=na.value, nnz=int(nz.value))

    def dofmap(self, level: int, space: int = 0) -> np.ndarray:
        i = self.level_info(level, space)
        out = np.empty(i["n_cells"] * i["nloc"], dtype=np.int32)
        check(lib.pm_disc_dofmap(self.handle, level, space, _ptr(out)))
        return out.reshape(i["n_cells"], i["nloc"])

    def cell_vertices(self, level: int) -> np.ndarray:
        i = self.level_info(level)
        nv = 4 if self.geometry in (GEO_SQUARE_QUAD, GEO_CUBE_TETRA) else 8
        out = np.empty(i["n_cells"] * nv * self.dim, dtype=np.float64)
        check(lib.pm_disc_cell_vertices(self.handle, level, _ptr(out)))
        return out.reshape(i["n_cells"], nv, self.dim)

    def structure(self, level: int) -> tuple[np.ndarray, np.ndarray]:
        i = self.level_info(level)
        n = i["n_dofs"]
        if self.kind == KIND_STOKES:  # combined [u1 | u2 | u3 | p] system
            n = 3 * n + self.level_info(level, 1)["n_dofs"]
        rp = np.empty(n + 1, dtype=np.int32)
        ci = np.empty(i["nnz"], dtype=np.int32)
        check(lib.pm_disc_structure(self.handle, level, _ptr(rp), _ptr(ci)))
        return rp, ci

    def prolongation(self, level: int) -> tuple[np.ndarray, np.ndarray, np.ndarray, int, int]:
        r, c = C.c_int(), C.c_int()
        z = C.c_int64()
        check(lib.pm_disc_prolongation_info(self.handle, level, C.byref(r), C.byref(c), C.byref(z)))
        rp = np.empty(r.value + 1, dtype=np.int32)
        ci = np.empty(int(z.value), dtype=np.int32)
        v = np.empty(int(z.value), dtype=np.float64)
        check(lib.pm_disc_prolongation(self.handle, level, _ptr(rp), _ptr(ci), _ptr(v)))
        return rp, ci, v, r.value, c.value

    def close(self) -> None:
        if self.handle:
            lib.pm_disc_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cd_coeffs(eps: float, b=(0.0, 0.0, 0.0), c: float = 0.0, manufactured: bool = True,
              f_const: float = 0.0, poly=None, poly_src=None) -> CdCoeffs:
    """poly: the ten coefficients of a quadratic exact solution (1, x, y, z, x^2,
    y^2, z^2, xy, xz, yz); f and the Dirichlet values then come from it;
    poly_src (same monomials) is added to f"""
    cf = CdCoeffs()
    if poly is not None:
        p = list(poly) + [0.0] * (10 - len(poly))
        q = [] if poly_src is None else list(poly_src)
        q = q + [0.0] * (10 - len(q))
        for i in range(10):
            cf.poly[i] = p[i]
            cf.poly_src[i] = q[i]
    cf.eps = eps
    bb = list(b) + [0.0] * (3 - len(b))
    for i in range(3):
        cf.b[i] = bb[i]
    cf.c = c
    cf.manufactured = 2 if poly is not None else (1 if manufactured else 0)
    cf.f_const = f_const
    return cf


def assemble_cd(ctx: Context, disc: Discretization, level: int, coeffs: CdCoeffs, quad_points: int,
                A: FEMatrix, rhs: DeviceVector) -> None:
    """Assemble2D/Assemble3D with the ConvDiff Galerkin local form, on the device."""
    check(lib.pm_assemble_cd(ctx.handle, disc.handle, level, C.byref(coeffs), quad_points, A.handle,
                             rhs.ptr), ctx.handle)


class ConvectionDiffusion:
    """ConvectionDiffusion<d> on one GPU: assemble() and solve() as in
    src/System/ConvectionDiffusion.C:174-209."""

    def __init__(self, ctx: Context, disc: Discretization, coeffs: CdCoeffs, db, quad_points: int = 0):
        self.ctx = ctx
        self.disc = disc
        self.coeffs = coeffs
        h = C.c_void_p()
        check(lib.pm_problem_create_cd(ctx.handle, disc.handle, C.byref(coeffs), quad_points,
                                       _db_text(db).encode(), C.byref(h)), ctx.handle)
        self.handle = h

    def assemble(self) -> None:
        check(lib.pm_problem_assemble(self.handle), self.ctx.handle)

    def solve(self) -> None:
        check(lib.pm_problem_solve(self.handle), self.ctx.handle)

    def reset_solution(self) -> None:
        check(lib.pm_problem_reset_solution(self.handle), self.ctx.handle)

    def size(self) -> tuple[int, int]:
        n, na = C.c_int(), C.c_int()
        check(lib.pm_problem_size(self.handle, C.byref(n), C.byref(na)))
        return n.value, na.value

    def solution(self) -> np.ndarray:
        out = np.empty(self.size()[0], dtype=np.float64)
        check(lib.pm_problem_get_solution(self.handle, _ptr(out)), self.ctx.handle)
        return out

    def set_solution(self, x: np.ndarray) -> None:
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.size != self.size()[0]:
            raise ValueError("solution of the wrong length")
        check(lib.pm_problem_set_solution(self.handle, _ptr(x)), self.ctx.handle)

    def rhs(self) -> np.ndarray:
        out = np.empty(self.size()[0], dtype=np.float64)
        check(lib.pm_problem_get_rhs(self.handle, _ptr(out)), self.ctx.handle)
        return out

    def matrix(self, level: int = -1) -> FEMatrix:
        if level < 0:
            level = self.disc.n_levels + level
        h = C.c_void_p()
        check(lib.pm_problem_matrix(self.handle, level, C.byref(h)))
        return FEMatrix(self.ctx, h, owned=False)

    def solver(self) -> Solver:
        h = C.c_void_p()
        check(lib.pm_problem_solver(self.handle, C.byref(h)))
        return Solver(self.ctx, None, handle=h, owned=False)

    def assemble_level_noalloc(self, level: int, vals: DeviceVector, rhs: DeviceVector,
                               coeffs: Optional[CdCoeffs] = None) -> None:
        """pm_assemble_cd_noalloc: one level into caller-owned device arrays, no device allocation"""
        check(lib.pm_assemble_cd_noalloc(self.handle, level, C.byref(coeffs) if coeffs is not None else None,
                                         vals.ptr, rhs.ptr), self.ctx.handle)

    def last_info(self) -> tuple[int, float, float]:
        it, res, init = C.c_int(), C.c_double(), C.c_double()
        check(lib.pm_problem_last_info(self.handle, C.byref(it), C.byref(res), C.byref(init)))
        return it.value, res.value, init.value

    def errors(self) -> tuple[float, float, float, float]:
        """(L2, H1-semi, SD, L_inf) errors of the solution against the exact
        solution, as ConvectionDiffusion<d>::output computes them"""
        out = np.zeros(4, dtype=np.float64)
        check(lib.pm_problem_errors(self.handle, _ptr(out)), self.ctx.handle)
        return tuple(float(v) for v in out)

    def run_host(self, coeffs: Optional[CdCoeffs], level_verts, sol_out: np.ndarray) -> None:
        """one request end to end from host memory (pm_problem_run_host)"""
        arr = None
        if level_verts is not None:
            arr = (C.c_void_p * len(level_verts))(*[C.c_void_p(v.ctypes.data) if v is not None else None
                                                    for v in level_verts])
        check(lib.pm_problem_run_host(self.handle, C.byref(coeffs) if coeffs is not None else None,
                                      arr, _ptr(sol_out)), self.ctx.handle)

    def close(self) -> None:
        if self.handle and self.ctx.handle:
            lib.pm_problem_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass



def solve_batched(problems, slots: int = 8) -> list:
    """pm_problem_solve_batched: assembled ConvectionDiffusion problems of one
    set-up and one context solved together, at most `slots` in lockstep (every
    kernel of an Arnoldi step runs once for all of them). Returns the status of
    each problem; last_info() and solution() hold each result."""
    n = len(problems)
    arr = (C.c_void_p * n)(*[p.handle for p in problems])
    st = (C.c_int * n)()
    check(lib.pm_problem_solve_batched(arr, n, slots, st), problems[0].ctx.handle)
    return list(st)


class TimeConvectionDiffusion(ConvectionDiffusion):
    """TimeConvectionDiffusion<d> on one GPU (src/System/TimeConvectionDiffusion.C)
    with TimeDiscretization's backward_euler, crank_nicolson and bdf_two. The
    database carries the solver keys and time_discretization,
    time_step_length, time_start, time_end. poly_time = (P1, P2) makes the
    exact solution u = P0 + t P1 + t^2 P2 (P0 = the coefficients' poly).

    The time loop of the reference's tests:
        tcd.assemble_initial_time()
        while tcd.current_time < tcd.end_time - 1e-10:
            tcd.next_time_step(); tcd.assemble(); tcd.solve()
    """

    def __init__(self, ctx: Context, disc: Discretization, coeffs: CdCoeffs, db, quad_points: int = 0,
                 poly_time=None):
        self.ctx = ctx
        self.disc = disc
        self.coeffs = coeffs
        text = _db_text(db)
        pt = None
        if poly_time is not None:
            p1, p2 = [list(v) + [0.0] * (10 - len(v)) for v in poly_time]
            pt = np.ascontiguousarray(p1 + p2, dtype=np.float64)
        self._pt = pt
        h = C.c_void_p()
        check(lib.pm_tcd_create(ctx.handle, disc.handle, C.byref(coeffs), None if pt is None else _ptr(pt),
                                quad_points, text.encode(), C.byref(h)), ctx.handle)
        self.tcd = h
        ph = C.c_void_p()
        check(lib.pm_tcd_problem(self.tcd, C.byref(ph)))
        self.handle = ph
        prm = dict(line.split(":", 1) for line in text.splitlines() if ":" in line)
        self.end_time = float(prm.get("time_end", 1.0))

    def assemble_initial_time(self) -> None:
        check(lib.pm_tcd_assemble_initial_time(self.tcd), self.ctx.handle)

    def next_time_step(self) -> None:
        check(lib.pm_tcd_next_step(self.tcd), self.ctx.handle)

    def assemble(self) -> None:
        check(lib.pm_tcd_assemble(self.tcd), self.ctx.handle)

    def solve(self) -> None:
        check(lib.pm_tcd_solve(self.tcd), self.ctx.handle)

    @property
    def current_time(self) -> float:
        t, k = C.c_double(), C.c_int()
        check(lib.pm_tcd_state(self.tcd, C.byref(t), C.byref(k)))
        return t.value

    @property
    def current_step(self) -> int:
        t, k = C.c_double(), C.c_int()
        check(lib.pm_tcd_state(self.tcd, C.byref(t), C.byref(k)))
        return k.value

    def close(self) -> None:
        if self.tcd and self.ctx.handle:
            lib.pm_tcd_destroy(self.tcd)
        self.tcd = None
        self.handle = None

class StokesProblem(ConvectionDiffusion):
    """NavierStokes<3> (P2/P1 on tetrahedra) on one GPU: the Stokes problem, or
    with "problem_type": 5 in the database the Navier-Stokes problem in
    convective form (nu = 1 / Reynolds number; example -3). assemble() and
    solve() as NavierStokes::assemble_linear_terms / solve
    (src/System/NavierStokes.C:407, 878), the pressure of the solution projected
    into L2_0. Vector layout [u1 | u2 | u3 | p]."""

    def __init__(self, ctx: Context, disc: Discretization, nu: float, db):
        self.ctx = ctx
        self.disc = disc
        self.nu = nu
        h = C.c_void_p()
        check(lib.pm_problem_create_stokes(ctx.handle, disc.handle, nu, _db_text(db).encode(), C.byref(h)),
              ctx.handle)
        self.handle = h

    def blocks(self) -> tuple[int, int, int]:
        """(velocity DOFs per component, active velocity DOFs, pressure DOFs)"""
        lv = self.disc.n_levels - 1
        v, p = self.disc.level_info(lv, 0), self.disc.level_info(lv, 1)
        return v["n_dofs"], v["n_active"], p["n_dofs"]

    def assemble_linear_terms(self) -> None:
        """NavierStokes::assemble_linear_terms (the same as assemble())"""
        self.assemble()

    def assemble_nonlinear_term(self) -> None:
        """NavierStokes::assemble_nonlinear_term (src/System/NavierStokes.C:573):
        the finest velocity restricted to every level, the velocity blocks
        reassembled with the convective term (problem_type 5 only)"""
        check(lib.pm_problem_assemble_nonlinear(self.handle), self.ctx.handle)

    def residuals(self) -> tuple[float, float, float]:
        """NavierStokes::compute_residuals: (impuls, mass, full) residual of the
        current solution, the pressure defect projected into L2_0"""
        out = np.zeros(3)
        check(lib.pm_problem_residuals(self.handle, out.ctypes.data_as(C.c_void_p)), self.ctx.handle)
        return float(out[0]), float(out[1]), float(out[2])

    def solve_nonlinear(self, max_records: int = 1000) -> np.ndarray:
        """The nonlinear loop of test/nse3d_solvers_test.c++ (stop_it(0), then
        solve / assemble_nonlinear_term / stop_it(k)) with the nonlinloop_*
        keys of the problem's database; call after assemble(). Returns the
        (impuls, mass, full) residuals of steps 0..n (n solves)."""
        res = np.zeros((max_records, 3))
        n = C.c_int()
        check(lib.pm_problem_solve_nonlinear(self.handle, max_records, res.ctypes.data_as(C.c_void_p),
                                             C.byref(n)), self.ctx.handle)
        return res[: min(n.value + 1, max_records)].copy()


class Server:
    """Request executor (pm_server_*): independent convection-diffusion and
    Stokes solves on one GPU by `n_workers` threads, each with its own stream
    and a cache of device-resident problems per set-up; the cached footprint is
    kept under `hbm_cap_bytes` by evicting least recently used problems."""

    def __init__(self, device: int = 0, n_workers: int = 4, db_cd=None, db_stokes=None,
                 hbm_cap_bytes: int = 150 * 10**9):
        from ._lib import Request, Result
        self._Request, self._Result = Request, Result
        h = C.c_void_p()
        check(lib.pm_server_create(device, n_workers, _db_text(db_cd).encode() if db_cd is not None else b"",
                                   _db_text(db_stokes).encode() if db_stokes is not None else b"",
                                   hbm_cap_bytes, C.byref(h)))
        self.handle = h
        self._outputs = {}

    def submit(self, kind: int, geometry: int, root_n: int, n_refine: int, n_levels: int, elem: int,
               coeffs: Optional[CdCoeffs] = None, nu: float = 1.0, solution_out: Optional[np.ndarray] = None,
               tag: int = 0) -> None:
        rq = self._Request()
        rq.kind, rq.geometry, rq.root_n, rq.n_refine, rq.n_levels, rq.elem = (kind, geometry, root_n, n_refine,
                                                                           n_levels, elem)
        if coeffs is not None:
            rq.coeffs = coeffs
        rq.nu = nu
        if solution_out is not None:
            if solution_out.dtype != np.float64 or not solution_out.flags.c_contiguous:
                raise TypeError("solution_out must be a contiguous float64 array")
            rq.solution_out = solution_out.ctypes.data_as(C.POINTER(C.c_double))
            self._outputs[tag] = solution_out  # kept alive until its result is polled
        rq.tag = tag
        check(lib.pm_server_submit(self.handle, C.byref(rq)))

    def poll(self, max_results: int = 1024, min_results: int = 0) -> list:
        buf = (self._Result * max_results)()
        n = C.c_int()
        check(lib.pm_server_poll(self.handle, buf, max_results, min_results, C.byref(n)))
        out = []
        for r in buf[: n.value]:
            d = {f: getattr(r, f) for f, _ in self._Result._fields_}
            self._outputs.pop(d["tag"], None)
            out.append(d)
        return out

    def drain(self) -> None:
        check(lib.pm_server_drain(self.handle))

    def stats(self) -> dict:
        b, s, e = C.c_size_t(), C.c_uint64(), C.c_uint64()
        check(lib.pm_server_stats(self.handle, C.byref(b), C.byref(s), C.byref(e)))
        return {"cached_bytes": b.value, "served": s.value, "evictions": e.value}

    def close(self) -> None:
        if self.handle:
            lib.pm_server_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = ["Context", "Server", "StokesProblem", "DeviceVector", "FEMatrix", "Solver", "Discretization", "ConvectionDiffusion",
           "ParameterDatabase", "PmError", "cd_coeffs", "assemble_cd", "GEO_SQUARE_QUAD", "GEO_CUBE_HEXA",
           "GEO_CUBE_TETRA", "KIND_CD", "KIND_STOKES"]
