"""Oracle set-up (test infrastructure only): uniform mesh hierarchies, DOF
numbering and CSR patterns of ParMooN's solve path, restated with numpy.

  cell order   : depth-first walk of the refinement tree
                 (src/Geometry/It_LE.C:17-55, TDomain::RegRefineAll Domain.C:1045-1062)
  refinement   : DatChildVertex of src/Refinement/RefQuadRegDesc.C:9,
                 RefHexaRegDesc.C:17, RefTetraRegDesc.C:13
  root meshes  : TDomain::UnitSquare (src/Geometry/Tests.C:449),
                 initialize_cube_hexa_mesh / initialize_cube_tetra_mesh (Tests.C:1815-1912)
                 with the Default_UnitCube boundary planes (Tests.C:1767)
  numbering    : TFESpace3D::ConstructSpace (src/FE/FESpace3D.C:506-2092). The
                 mapper (src/FE/FE3DMapper.C:34-190) links the local DOFs of
                 neighbouring cells into classes whose representative is the
                 smallest position BeginIndex[cell]+local; the renumbering pass
                 (FESpace3D.C:1750-1910) walks positions in order and numbers each
                 class when it meets its representative, inner classes first
                 and Dirichlet classes after them. On a conforming mesh a class
                 is a geometric node, so the result is first-touch order over
                 (cell, local DOF), inner nodes, then boundary nodes. With
                 Neumann sides (2D, SineLaplace's BoundCondition) the boundary
                 splits into Neumann nodes (all their sides Neumann, active)
                 numbered before the Dirichlet nodes (TFESpace2D::ConstructSpace,
                 src/FE/FESpace2D.C).
  structure    : TStructure(space) (src/Matrix/Structure.C:829-1283), Sort (:2681)
"""
from __future__ import annotations

import numpy as np

GEO_SQUARE_QUAD, GEO_CUBE_HEXA, GEO_CUBE_TETRA = 0, 1, 2

QUAD_CHILD = np.array([[0, 4, 8, 7], [1, 5, 8, 4], [2, 6, 8, 5], [3, 7, 8, 6]])
QUAD_NEW = [(0, 1), (1, 2), (2, 3), (3, 0), (0, 1, 2, 3)]
HEX_CHILD = np.array([[0, 8, 12, 11, 15, 16, 26, 24], [1, 9, 12, 8, 13, 19, 26, 16],
                      [2, 10, 12, 9, 17, 22, 26, 19], [3, 11, 12, 10, 20, 24, 26, 22],
                      [4, 23, 25, 14, 15, 24, 26, 16], [5, 14, 25, 18, 13, 16, 26, 19],
                      [6, 18, 25, 21, 17, 19, 26, 22], [7, 21, 25, 23, 20, 22, 26, 24]])
# refined hexa vertices 8..26: children that share them (DatVertexChild)
HEX_NEW = [(0, 1), (1, 2), (2, 3), (0, 3), (0, 1, 2, 3), (1, 5), (4, 5), (0, 4), (0, 1, 4, 5),
           (2, 6), (5, 6), (1, 2, 5, 6), (3, 7), (6, 7), (2, 3, 6, 7), (4, 7), (0, 3, 4, 7),
           (4, 5, 6, 7), (0, 1, 2, 3, 4, 5, 6, 7)]
TET_CHILD = np.array([[0, 4, 6, 7], [4, 1, 5, 8], [6, 5, 2, 9], [7, 8, 9, 3],
                      [4, 6, 7, 8], [5, 6, 4, 8], [6, 7, 8, 9], [8, 5, 6, 9]])
TET_NEW = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]
CUBE = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
KUHN = np.array([[0, 1, 2, 6], [0, 5, 1, 6], [0, 2, 3, 6], [0, 3, 7, 6], [0, 4, 5, 6], [0, 7, 4, 6]])


def root_mesh(geometry: int, root_n: int, unit: int) -> np.ndarray:
    cells = []
    if geometry == GEO_SQUARE_QUAD:
        sq = np.array([[0, 0], [1, 0], [1, 1], [0, 1]])
        for j in range(root_n):
            for i in range(root_n):
                cells.append((sq + [i, j]) * unit)
    else:
        for k in range(root_n):
            for j in range(root_n):
                for i in range(root_n):
                    if geometry == GEO_CUBE_HEXA:
                        cells.append((CUBE + [i, j, k]) * unit)
                    else:
                        for t in KUHN:
                            cells.append((CUBE[t] + [i, j, k]) * unit)
    return np.array(cells, dtype=np.int64)


def refine(geometry: int, v: np.ndarray) -> np.ndarray:
    """children of every cell, in cell order then child order"""
    if geometry == GEO_SQUARE_QUAD:
        new, child = QUAD_NEW, QUAD_CHILD
    elif geometry == GEO_CUBE_HEXA:
        new, child = HEX_NEW, HEX_CHILD
    else:
        new, child = TET_NEW, TET_CHILD
    ext = [v]
    for grp in new:
        s = sum(v[:, g, :] for g in grp)
        assert np.all(s % len(grp) == 0)
        ext.append((s // len(grp))[:, None, :])
    ref = np.concatenate(ext, axis=1)  # (n_cells, n_refined_vertices, dim)
    out = ref[:, child, :]             # (n_cells, n_children, nv, dim)
    return out.reshape(-1, v.shape[1], v.shape[2])


def hierarchy(geometry: int, root_n: int, n_refine: int):
    unit = 2 << n_refine
    scale = unit * root_n
    levels = [root_mesh(geometry, root_n, unit)]
    for _ in range(n_refine):
        levels.append(refine(geometry, levels[-1]))
    nchild = 4 if geometry == GEO_SQUARE_QUAD else 8
    parents = [None] + [np.repeat(np.arange(levels[l].shape[0]), nchild) for l in range(n_refine)]
    return levels, parents, scale


def local_nodes(geometry: int, elem: int, v: np.ndarray) -> np.ndarray:
    """lattice coordinates of the local DOF nodes (n_cells, nloc, dim)"""
    if geometry in (GEO_SQUARE_QUAD, GEO_CUBE_HEXA):
        k = elem
        e1 = v[:, 1] - v[:, 0]
        e2 = v[:, 3] - v[:, 0]
        e3 = v[:, 4] - v[:, 0] if geometry == GEO_CUBE_HEXA else None
        nodes = []
        rng_c = range(k + 1) if geometry == GEO_CUBE_HEXA else [0]
        for c in rng_c:
            for b in range(k + 1):
                for a in range(k + 1):
                    x = v[:, 0] + e1 * a // k + e2 * b // k
                    if e3 is not None:
                        x = x + e3 * c // k
                    nodes.append(x)
        return np.stack(nodes, axis=1)
    if elem == 11:
        return v.copy()
    pairs = [(0, 0), (0, 1), (1, 1), (0, 2), (1, 2), (2, 2), (0, 3), (1, 3), (2, 3), (3, 3)]
    return np.stack([(v[:, a] + v[:, b]) // 2 for a, b in pairs], axis=1)


def square_sides(c: np.ndarray, scale: int) -> np.ndarray:
    """bit mask of the unit square's sides (0 y=0, 1 x=1, 2 y=1, 3 x=0, the
    boundary components of UnitSquare) that each lattice point lies on"""
    return ((c[:, 1] == 0) * 1 + (c[:, 0] == scale) * 2 + (c[:, 1] == scale) * 4 +
            (c[:, 0] == 0) * 8).astype(np.int64)


def number_dofs(nodes: np.ndarray, scale: int, dirichlet: bool = True, neumann_sides: int = 0):
    """first-touch numbering, inner nodes first, then Neumann nodes (active),
    then Dirichlet nodes; returns (dofmap, n_dofs, n_active, coords)"""
    n_cells, nloc, dim = nodes.shape
    flat = nodes.reshape(-1, dim)
    w = scale + 1
    key = flat[:, 0] + w * flat[:, 1] + (w * w * flat[:, 2] if dim == 3 else 0)
    uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")           # unique nodes in first-touch order
    ucoord = flat[first]
    on_bnd = np.any((ucoord == 0) | (ucoord == scale), axis=1)
    neumann = np.zeros(uniq.size, dtype=bool)
    if neumann_sides:
        sides = square_sides(ucoord, scale)
        neumann = on_bnd & ((sides & neumann_sides) == sides)
    inner = order[~on_bnd[order]]
    neu = order[neumann[order]]
    bnd = order[(on_bnd & ~neumann)[order]]
    number = np.empty(uniq.size, dtype=np.int64)
    number[inner] = np.arange(inner.size)
    number[neu] = inner.size + np.arange(neu.size)
    number[bnd] = inner.size + neu.size + np.arange(bnd.size)
    dofmap = number[inv].reshape(n_cells, nloc).astype(np.int32)
    coords = np.empty((uniq.size, dim), dtype=np.int64)
    coords[number] = ucoord
    n_active = inner.size + neu.size if dirichlet else uniq.size
    return dofmap, uniq.size, n_active, coords


def structure(dofmap: np.ndarray, n_dofs: int, n_active: int):
    """square CSR pattern: active rows couple to all DOFs of their cells, sorted;
    non-active rows hold the diagonal only"""
    n_cells, nloc = dofmap.shape
    rows = np.repeat(dofmap, nloc, axis=1).ravel().astype(np.int64)
    cols = np.tile(dofmap, (1, nloc)).ravel().astype(np.int64)
    keep = rows < n_active
    rows, cols = rows[keep], cols[keep]
    d = np.arange(n_active, n_dofs, dtype=np.int64)
    rows = np.concatenate([rows, d])
    cols = np.concatenate([cols, d])
    key = np.unique(rows * n_dofs + cols)
    r = key // n_dofs
    c = (key % n_dofs).astype(np.int32)
    rp = np.zeros(n_dofs + 1, dtype=np.int64)
    np.add.at(rp, r + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    return rp, c


class Level:
    def __init__(self, geometry, elem, verts_lattice, parent, scale, neumann_sides=0):
        self.verts_lattice = verts_lattice
        self.scale = scale
        self.parent = None if parent is None else parent.astype(np.int32)
        self.n_cells = verts_lattice.shape[0]
        inv = 1.0 / scale if (scale & (scale - 1)) == 0 else None
        self.verts = (verts_lattice * inv if inv is not None else verts_lattice / scale).astype(np.float64)
        nodes = local_nodes(geometry, elem, verts_lattice)
        self.dofmap, self.n_dofs, self.n_active, self.coords = number_dofs(nodes, scale,
                                                                           neumann_sides=neumann_sides)
        self.nloc = self.dofmap.shape[1]
        self.row_ptr, self.cols = structure(self.dofmap, self.n_dofs, self.n_active)
        self.node_coords = self.coords / scale


def cd_levels(geometry: int, root_n: int, n_refine: int, n_levels: int, elem: int, neumann_sides: int = 0):
    """the kept multigrid levels (coarsest first) of a convection-diffusion set-up"""
    meshes, parents, scale = hierarchy(geometry, root_n, n_refine)
    first = n_refine + 1 - n_levels
    out = []
    for l in range(first, n_refine + 1):
        out.append(Level(geometry, elem, meshes[l], parents[l], scale, neumann_sides))
    return out
