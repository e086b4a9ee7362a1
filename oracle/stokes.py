"""Oracle Stokes P2/P1 driver (test infrastructure only).

Restates the NSE3D Stokes set-up of the solve path with numpy and drives the C
restatement in oracle.c:

  spaces      : velocity C_T_P2_3D with Dirichlet boundary, pressure C_T_P1_3D
                with Neumann boundary (all pressure DOFs active), numbered as
                TFESpace3D::ConstructSpace (src/FE/FESpace3D.C:506-2092)
  combined    : BlockFEMatrix::NSE3D_Type4 Stokes blocks (A11 = A22 = A33,
                B^T, B; src/Matrix/BlockFEMatrix.C:616-664) flattened as
                get_combined_matrix ([u1 | u2 | u3 | p] ordering,
                BlockFEMatrix.C:1168-1345); non-active rows hold a unit
                diagonal
  projection  : first pressure row replaced by a unit row
                (get_combined_submatrix with pressure projection)
  Vanka       : patches = sorted combined DOFs of a cell
                (VankaSmoother::set_up_cell_patches, src/Multigrid/VankaSmoother.C:305)
                plus a greedy cell colouring for the colour-ordered sweep
  multigrid   : block-diagonal transfer, P2 for the velocity components and
                P1 for the pressure (GridTransfer on each space)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import refsetup
from .cd import _p, lib as _cd_lib

SM_JAC, SM_DIR, SM_VANKA, SM_VANKA_JAC, SM_VANKA_COLOR = 0, 1, 2, 3, 4
# smoother name -> (code, patches): "cell" patches are the 34 combined DOFs of a
# cell (VankaType::CELL / CELL_JACOBI), "nodal" patches one pressure DOF with
# the velocity nodes it couples to through B (VankaType::NODAL). Sweeps: in
# patch order (the reference), additive with averaged corrections (jacobi),
# or by colour (the GPU's multiplicative order).
VANKA_TYPES = {"cell": (SM_VANKA, "cell"), "cell_jacobi": (SM_VANKA_JAC, "cell"),
               "cell_color": (SM_VANKA_COLOR, "cell"), "nodal": (SM_VANKA, "nodal"),
               "nodal_jacobi": (SM_VANKA_JAC, "nodal"), "nodal_color": (SM_VANKA_COLOR, "nodal"),
               "direct_solve": (SM_DIR, None), "jacobi": (SM_JAC, None)}


def lib() -> C.CDLL:
    L = _cd_lib()
    if not getattr(L, "_stokes_sigs", False):
        vp, i32, f64 = C.c_void_p, C.c_int, C.c_double
        L.orc_assemble_stokes.argtypes = [i32, vp, f64, vp, i32, vp, vp, vp, vp, vp]
        L.orc_assemble_stokes.restype = i32
        L.orc_assemble_stokes_ex.argtypes = [i32, vp, f64, vp, i32, vp, vp, vp, vp, vp, i32]
        L.orc_assemble_stokes_ex.restype = i32
        L.orc_vanka_sweep.argtypes = [i32, i32, vp, i32, vp, vp, vp, vp, vp, f64, vp, vp, i32, vp]
        L.orc_mg_set_smoothers.argtypes = [vp, i32, i32, f64]
        L.orc_mg_set_vanka.argtypes = [vp, i32, vp, vp, vp, vp, i32, vp, vp, i32, vp, vp]
        L.orc_vanka_sweep_var.argtypes = [i32, i32, vp, vp, i32, vp, vp, vp, vp, vp, f64, vp, vp, i32, vp, vp]
        L.orc_mg_finalize.argtypes = [vp]
        L.orc_mg_finalize.restype = i32
        L.orc_mg_set_transfer_block.argtypes = [vp, i32, i32, i32, i32, i32, i32, i32, i32, vp, vp, vp, vp, vp,
                                                i32, i32]
        L._stokes_sigs = True
    return L


def _nonzero_pattern() -> np.ndarray:
    """34x34 local coupling pattern of the Stokes blocks"""
    blk = np.array([m // 10 if m < 30 else 3 for m in range(34)])
    bm, bk = blk[:, None], blk[None, :]
    return np.where((bm < 3) & (bk < 3), bm == bk, ~((bm == 3) & (bk == 3)))


class StokesLevel:
    def __init__(self, verts_lattice, parent, scale):
        geo = refsetup.GEO_CUBE_TETRA
        self.verts_lattice = verts_lattice
        self.parent = None if parent is None else parent.astype(np.int32)
        self.n_cells = verts_lattice.shape[0]
        self.verts = (verts_lattice * (1.0 / scale)).astype(np.float64)
        self.udofmap, self.nu, self.nu_active, self.ucoords = refsetup.number_dofs(
            refsetup.local_nodes(geo, 12, verts_lattice), scale, dirichlet=True)
        self.pdofmap, self.np_, _, self.pcoords = refsetup.number_dofs(
            refsetup.local_nodes(geo, 11, verts_lattice), scale, dirichlet=False)
        nu, np_ = self.nu, self.np_
        self.n = 3 * nu + np_
        self.cdof = np.concatenate([self.udofmap + b * nu for b in range(3)] + [self.pdofmap + 3 * nu],
                                   axis=1).astype(np.int32)
        act = np.ones(self.n, dtype=np.uint8)
        for b in range(3):
            act[b * nu + self.nu_active: (b + 1) * nu] = 0
        self.active = act
        self.p0 = 3 * nu
        self._structure()
        self._projected()
        self.patch = np.ascontiguousarray(np.sort(self.cdof, axis=1), dtype=np.int32)
        # a cell's local matrix is singular when the 3 rows of each active
        # velocity node cannot control the pressures of the cell: 4 of them, or
        # 3 when the cell holds p0, whose row is a unit row of the projected
        # matrix. The pressures of such cells are frozen.
        n_act = self.active[self.udofmap].sum(axis=1).astype(np.int64)
        need = np.where((self.pdofmap == 0).any(axis=1), 3, 4)
        self.n_freeze = np.ascontiguousarray(np.where(3 * n_act < need, 4, 0), dtype=np.int32)
        self._colouring()

    def _structure(self):
        pat = _nonzero_pattern()
        mm, kk = np.nonzero(pat)
        rows = self.cdof[:, mm].ravel().astype(np.int64)
        cols = self.cdof[:, kk].ravel().astype(np.int64)
        keep = self.active[rows] == 1
        rows, cols = rows[keep], cols[keep]
        d = np.nonzero(self.active == 0)[0].astype(np.int64)
        rows = np.concatenate([rows, d])
        cols = np.concatenate([cols, d])
        key = np.unique(rows * self.n + cols)
        r = key // self.n
        self.cols = (key % self.n).astype(np.int32)
        rp = np.zeros(self.n + 1, dtype=np.int64)
        np.add.at(rp, r + 1, 1)
        self.row_ptr = np.cumsum(rp).astype(np.int32)

    def _projected(self):
        rp, ci = self.row_ptr, self.cols
        lens = np.diff(rp).astype(np.int64)
        lens[self.p0] = 1
        self.vrow_ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
        src = np.concatenate([np.arange(rp[i], rp[i + 1]) if i != self.p0 else np.array([-1])
                              for i in range(self.n)]).astype(np.int64)
        self.vsrc = src
        vc = np.where(src >= 0, ci[np.maximum(src, 0)], self.p0)
        self.vcols = np.ascontiguousarray(vc, dtype=np.int32)

    def project(self, vals: np.ndarray) -> np.ndarray:
        return np.where(self.vsrc >= 0, vals[np.maximum(self.vsrc, 0)], 1.0)

    def _colouring(self):
        """greedy colouring in cell order: the smallest colour not used by an
        earlier cell that shares a DOF"""
        nc = self.n_cells
        flat = self.cdof.ravel()
        order = np.argsort(flat, kind="stable")
        sorted_dofs = flat[order]
        starts = np.searchsorted(sorted_dofs, np.arange(self.n))
        ends = np.searchsorted(sorted_dofs, np.arange(self.n), side="right")
        cells_of = [order[starts[d]:ends[d]] // 34 for d in range(self.n)]
        color = np.full(nc, -1, dtype=np.int64)
        n_colors = 0
        for c in range(nc):
            nb = np.unique(np.concatenate([cells_of[d] for d in self.cdof[c]]))
            nb = nb[nb < c]
            used = set(color[nb].tolist())
            col = 0
            while col in used:
                col += 1
            color[c] = col
            n_colors = max(n_colors, col + 1)
        self.color_ptr = np.zeros(n_colors + 1, dtype=np.int32)
        np.add.at(self.color_ptr, color + 1, 1)
        self.color_ptr = np.cumsum(self.color_ptr).astype(np.int32)
        self.color_cells = np.argsort(color, kind="stable").astype(np.int32)
        self.n_colors = n_colors


def _greedy_colours(members: list, n_shared: int):
    """greedy colouring in patch order: the smallest colour not used by an
    earlier patch sharing an entry of `members` (arrays of shared ids)"""
    owners = [[] for _ in range(n_shared)]
    for p, mem in enumerate(members):
        for d in mem:
            owners[d].append(p)
    color = np.full(len(members), -1, dtype=np.int64)
    n_colors = 0
    for p, mem in enumerate(members):
        used = {color[q] for d in mem for q in owners[d] if q < p}
        col = 0
        while col in used:
            col += 1
        color[p] = col
        n_colors = max(n_colors, col + 1)
    cp = np.zeros(n_colors + 1, dtype=np.int64)
    np.add.at(cp, color + 1, 1)
    return (np.cumsum(cp).astype(np.int32), np.argsort(color, kind="stable").astype(np.int32), n_colors)


def _lattice_colours(members: list, n_shared: int, coords: np.ndarray):
    """the periodic colouring (i mod 3) + 3 (j mod 3) + 9 (k mod 3) of patches
    whose anchors lie on a lattice (coords: integer lattice coordinates of each
    patch's anchor), or None where two patches of one colour share an entry
    of `members`; colours in ascending order, patches in patch order inside"""
    spacing = int(np.gcd.reduce(coords.ravel().astype(np.int64)))
    if spacing <= 0:
        return None
    ijk = coords.astype(np.int64) // spacing
    color = (ijk[:, 0] % 3) + 3 * (ijk[:, 1] % 3) + 9 * (ijk[:, 2] % 3)
    owner = np.full((27, n_shared), False)
    for p, mem in enumerate(members):
        if owner[color[p], mem].any():
            return None
        owner[color[p], mem] = True
    used = np.unique(color)
    remap = np.full(27, -1)
    remap[used] = np.arange(used.size)
    color = remap[color]
    n_colors = int(used.size)
    cp = np.zeros(n_colors + 1, dtype=np.int64)
    np.add.at(cp, color + 1, 1)
    return (np.cumsum(cp).astype(np.int32), np.argsort(color, kind="stable").astype(np.int32), n_colors)


def nodal_patches(lv: "StokesLevel"):
    """VankaType::NODAL patches (VankaSmoother::set_up_pressure_patches /
    set_up_velocity_patches, src/Multigrid/VankaSmoother.C:302-420): pressure
    DOF i with the velocity nodes in row i of the coupling block B1, all three
    components; returns (ptr, dofs, colour_ptr, colour_patches, n_colours) with
    the library's colouring of the patches for the colour-ordered sweep"""
    if getattr(lv, "_nodal", None) is None:
        nu, rp, ci = lv.nu, lv.row_ptr, lv.cols
        vel, dofs, ptr = [], [], [0]
        for i in range(lv.np_):
            r = 3 * nu + i
            cols = ci[rp[r]:rp[r + 1]]
            vn = cols[cols < nu]
            vel.append(vn)
            dofs.append(np.concatenate([vn + k * nu for k in range(3)] + [np.array([r])]))
            ptr.append(ptr[-1] + dofs[-1].size)
        # the library's colouring: periodic on the vertex lattice where that is
        # conflict-free (27 colours of equal size), greedy otherwise
        lat = _lattice_colours(vel, nu, lv.pcoords)
        cptr, cpat, nc = lat if lat is not None else _greedy_colours(vel, nu)
        lv._nodal = (np.array(ptr, dtype=np.int32), np.ascontiguousarray(np.concatenate(dofs), dtype=np.int32),
                     cptr, cpat, nc)
    return lv._nodal


def stokes_levels(root_n: int, n_refine: int, n_levels: int):
    meshes, parents, scale = refsetup.hierarchy(refsetup.GEO_CUBE_TETRA, root_n, n_refine)
    first = n_refine + 1 - n_levels
    return [StokesLevel(meshes[l], parents[l], scale) for l in range(first, n_refine + 1)]


def vanka_sweep(kind: str, lv: StokesLevel, pvals: np.ndarray, b: np.ndarray, x: np.ndarray,
                damp: float = 1.0, freeze: bool = True) -> np.ndarray:
    """one VankaSmoother::smooth sweep on the projected matrix; returns the new x
    (freeze=False builds every local matrix as the reference does)"""
    x = np.array(x, dtype=np.float64, copy=True)
    pv = np.ascontiguousarray(pvals, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    code, patches = VANKA_TYPES[kind]
    t = {SM_VANKA: 0, SM_VANKA_JAC: 1, SM_VANKA_COLOR: 2}[code]
    if patches == "cell":
        args = (lv.n_cells, None, _p(lv.patch), lv.n, _p(lv.vrow_ptr), _p(lv.vcols), _p(pv), _p(b), _p(x), damp,
                _p(lv.color_ptr), _p(lv.color_cells), lv.n_colors, _p(lv.n_freeze) if freeze else None)
    else:
        ptr, dofs, cptr, cpat, nc = nodal_patches(lv)
        args = (lv.np_, _p(ptr), _p(dofs), lv.n, _p(lv.vrow_ptr), _p(lv.vcols), _p(pv), _p(b), _p(x), damp,
                _p(cptr), _p(cpat), nc, None)
    lib().orc_vanka_sweep_var(t, *args, None)
    return x


class OracleStokes:
    """NavierStokes<3> (Stokes, Laplace form) restated on the CPU."""

    def __init__(self, root_n: int, n_refine: int, n_levels: int, nu: float = 1.0, example: int = 0):
        """example 0: the manufactured sine velocity; -3: the polynomial
        solution u = (y^2, xz, -y^2), p = x + y + z - 3/2 of
        include/Examples/NSE_3D/test_u_2_p_1.h with its Dirichlet values"""
        self.levels = stokes_levels(root_n, n_refine, n_levels)
        self.nu = nu
        self.example = example
        self.vals, self.pvals, self.rhs = [], [], []
        self._mg = None
        self._keep = []

    @property
    def finest(self) -> StokesLevel:
        return self.levels[-1]

    def assemble(self) -> None:
        L = lib()
        self.vals, self.pvals, self.rhs = [], [], []
        for lv in self.levels:
            vals = np.zeros(lv.cols.size)
            rhs = np.zeros(lv.n)
            rc = L.orc_assemble_stokes_ex(lv.n_cells, _p(lv.verts), self.nu, _p(lv.cdof), lv.n, _p(lv.active),
                                          _p(lv.row_ptr), _p(lv.cols), _p(vals), _p(rhs), self.example)
            if rc != 0:
                raise RuntimeError(f"oracle Stokes assembly failed ({rc})")
            if self.example == -3:
                # Dirichlet values: the exact velocity at the non-active nodes
                X = lv.ucoords[lv.nu_active:] / lv.ucoords.max()
                x, y, z = X[:, 0], X[:, 1], X[:, 2]
                for b, val in enumerate((y * y, x * z, -y * y)):
                    rhs[b * lv.nu + lv.nu_active: (b + 1) * lv.nu] = val
            self.vals.append(vals)
            self.pvals.append(np.ascontiguousarray(lv.project(vals)))
            self.rhs.append(rhs)

    def build_mg(self, smoother="cell_jacobi", coarse_smoother="direct_solve", n_pre=2, n_post=2,
                 vanka_damp=1.0, correction_damp=1.0, cycle="V", coarse_max_it=10, coarse_residual=0.1,
                 n_mg_levels=None):
        L = lib()
        if self._mg:
            L.orc_mg_destroy(self._mg)
        nl = len(self.levels) if n_mg_levels is None else n_mg_levels
        off = len(self.levels) - nl
        coarse_direct = coarse_smoother == "direct_solve"
        mg = L.orc_mg_create(nl, n_pre, n_post, 1.0, correction_damp, {"V": 0, "W": 1, "F": 2}[cycle],
                             int(coarse_direct), coarse_max_it, coarse_residual)
        (fine_code, fine_kind), (coarse_code, coarse_kind) = VANKA_TYPES[smoother], VANKA_TYPES[coarse_smoother]
        L.orc_mg_set_smoothers(mg, fine_code, coarse_code, vanka_damp)
        keep = []
        for l in range(nl):
            lv = self.levels[off + l]
            L.orc_mg_set_level(mg, l, lv.n, _p(lv.active), _p(lv.row_ptr), _p(lv.cols), _p(self.vals[off + l]))
            kind = coarse_kind if l == 0 else fine_kind
            if kind == "nodal":
                ptr, dofs, cptr, cpat, nc = nodal_patches(lv)
                L.orc_mg_set_vanka(mg, l, _p(lv.vrow_ptr), _p(lv.vcols), _p(self.pvals[off + l]), _p(dofs), lv.np_,
                                   _p(cptr), _p(cpat), nc, None, _p(ptr))
            else:
                L.orc_mg_set_vanka(mg, l, _p(lv.vrow_ptr), _p(lv.vcols), _p(self.pvals[off + l]), _p(lv.patch),
                                   lv.n_cells, _p(lv.color_ptr), _p(lv.color_cells), lv.n_colors, _p(lv.n_freeze),
                                   None)
        for l in range(nl - 1):
            cl, fl = self.levels[off + l], self.levels[off + l + 1]
            cv = np.ascontiguousarray(cl.verts)
            fv = np.ascontiguousarray(fl.verts)
            par = np.ascontiguousarray(fl.parent)
            fu = np.ascontiguousarray(fl.udofmap, dtype=np.int32)
            cu = np.ascontiguousarray(cl.udofmap, dtype=np.int32)
            fp = np.ascontiguousarray(fl.pdofmap, dtype=np.int32)
            cp = np.ascontiguousarray(cl.pdofmap, dtype=np.int32)
            keep += [cv, fv, par, fu, cu, fp, cp]
            for b in range(3):
                L.orc_mg_set_transfer_block(mg, l, b, b * fl.nu, b * cl.nu, 3, 12, fl.n_cells, 10, _p(fu), _p(cu),
                                            _p(par), _p(fv), _p(cv), fl.nu, cl.nu)
            L.orc_mg_set_transfer_block(mg, l, 3, 3 * fl.nu, 3 * cl.nu, 3, 11, fl.n_cells, 4, _p(fp), _p(cp),
                                        _p(par), _p(fv), _p(cv), fl.np_, cl.np_)
        if L.orc_mg_finalize(mg) != 0:
            raise RuntimeError("oracle coarse factorisation failed")
        self._mg = mg
        self._keep = keep
        return mg

    def mg_apply(self, z: np.ndarray) -> np.ndarray:
        z = np.ascontiguousarray(z, dtype=np.float64)
        r = np.zeros_like(z)
        lib().orc_mg_apply(self._mg, _p(z), _p(r))
        return r

    def solve(self, tol: float = 0.0, reduction: float = 1e-8, max_it: int = 100, restart: int = 20):
        """FGMRES with the multigrid preconditioner; returns
        (solution, iterations, residual, history, status)"""
        lv = self.finest
        rhs = self.rhs[-1]
        sol = np.zeros(lv.n)
        sol[lv.active == 0] = rhs[lv.active == 0]
        it, res, nh = C.c_int(), C.c_double(), C.c_int()
        hist = np.zeros(100000)
        st = lib().orc_krylov_solve(0, lv.n, _p(lv.active), _p(lv.row_ptr), _p(lv.cols), _p(self.vals[-1]),
                                    self._mg, tol, reduction, max_it, 0, restart, _p(rhs), _p(sol),
                                    C.byref(it), C.byref(res), _p(hist), hist.size, C.byref(nh))
        return sol, it.value, res.value, hist[: nh.value].copy(), st

    def close(self):
        if self._mg:
            lib().orc_mg_destroy(self._mg)
            self._mg = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
