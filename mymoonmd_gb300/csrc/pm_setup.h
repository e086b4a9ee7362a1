// Host-side set-up of the solve path: uniform mesh hierarchies, finite element
// spaces (global DOF numbering), CSR structures and grid-transfer operators.
//
// Everything here restates ParMooN's set-up for the configurations the solve
// path is driven with (unit square / unit cube, regular refinement):
//   * cell order            : depth-first walk of the refinement tree
//                             (src/Geometry/It_LE.C:17-55, Domain.C:1045-1062)
//   * child cells / vertices: DatChildVertex tables of
//                             src/Refinement/RefQuadRegDesc.C:9,
//                             src/Refinement/RefHexaRegDesc.C:17,
//                             src/Refinement/RefTetraRegDesc.C:13
//   * DOF numbering         : TFESpace{2,3}D::ConstructSpace
//                             (src/FE/FESpace3D.C:506-2092) with the mapper
//                             union-find of src/FE/FE3DMapper.C:34-190
//   * CSR structure         : TStructure(space) (src/Matrix/Structure.C:829)
//                             followed by Sort() (Structure.C:2681)
//   * transfer              : GridTransfer::Prolongate / DefectRestriction
//                             (src/Multigrid/GridTransfer.C:665-1216)
//
// Coordinates are kept on an integer lattice (units of half the finest cell
// width) so that vertex midpoints, DOF nodes and node identification are exact.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace pmsetup {

enum Geometry { GEO_SQUARE_QUAD = 0, GEO_CUBE_HEXA = 1, GEO_CUBE_TETRA = 2 };
enum Element { EL_Q1 = 1, EL_Q2 = 2, EL_P1 = 11, EL_P2 = 12 };
enum BoundaryKind { BND_DIRICHLET = 0, BND_NEUMANN = 1 };

struct Level {
  int n_cells = 0;
  std::vector<int64_t> vtx;  // n_cells * nvc * dim lattice coordinates
  std::vector<int> parent;   // parent cell on the previous level, -1 on level 0
  std::vector<int> child_no; // index of the cell among its parent's children
};

struct Space {
  int elem = 0, nloc = 0, n_dofs = 0, n_active = 0;
  int boundary = BND_DIRICHLET;
  int neumann_sides = 0;  // 2D sides with Neumann conditions (bit s: side s)
  int n_neumann = 0;      // Neumann DOFs n_active - n_neumann .. n_active-1
  std::vector<int> dofmap;   // n_cells * nloc  (GlobalNumbers, BeginIndex = c*nloc)
  std::vector<int64_t> node; // n_dofs * dim lattice coordinates of each DOF
};

struct Csr {
  int n_rows = 0, n_cols = 0, n_active = 0;
  std::vector<int> row_ptr, cols;
  std::vector<double> vals;
};

struct Hierarchy {
  int geometry = 0, dim = 0, nvc = 0, root_n = 1, n_refine = 0;
  int64_t scale = 0;  // lattice units per unit length
  std::vector<Level> levels;  // 0 = root mesh ... n_refine = finest
};

int element_nloc(int elem);
// local DOFs of `elem` on the cells of `geometry` (Qk on quadrilaterals or
// hexahedra, Pk on tetrahedra)
int space_nloc(int geometry, int elem);
int element_dim(int elem);

// Builds the root mesh (root_n cells per side; root_n = 1 is ParMooN's default
// UnitSquare / Default_UnitCube_Hexa / Default_UnitCube_Tetra) and refines it
// regularly n_refine times, keeping every level.
Hierarchy build_hierarchy(int geometry, int root_n, int n_refine);
// the same hierarchy with the root mesh only (its lattice scale already that
// of n_refine refinements): the start of a refinement done elsewhere
Hierarchy root_hierarchy(int geometry, int root_n, int n_refine);

// Sides of the unit square as the boundary components of UnitSquare number
// them (Default_UnitSquare): 0 y=0, 1 x=1, 2 y=1, 3 x=0.
enum SquareSide { SIDE_Y0 = 1, SIDE_X1 = 2, SIDE_Y1 = 4, SIDE_X0 = 8 };

// Bit mask of the square's sides that lattice point x lies on (0 inside).
int square_sides(int64_t scale, const int64_t* x);

// Numbers the DOFs of `elem` on one level: inner DOFs in order of first touch
// (cells in collection order, local DOFs in local order), then boundary DOFs of
// the given kind in the same order. Dirichlet DOFs are non-active.
//
// With boundary == BND_DIRICHLET and a non-zero neumann_sides (2D only) the
// sides in the mask carry Neumann conditions: DOFs whose every side is a
// Neumann side are numbered after the inner DOFs and stay active, the rest of
// the boundary (the corners between a Neumann and a Dirichlet side among
// them) after those, non-active: inner, Neumann, Dirichlet, each in order of
// first touch (TFESpace2D::ConstructSpace, src/FE/FESpace2D.C).
Space build_space(const Hierarchy& h, int level, int elem, int boundary, int neumann_sides = 0);

// Boundary edges of one 2D level on the Neumann sides: for each, the cell,
// the local edge m (vertices m and m+1 mod 4) and the side, in cell order then
// edge order.
struct NeumannEdge {
  int cell, edge, side;
};
std::vector<NeumannEdge> neumann_edges(const Hierarchy& h, int level, int neumann_sides);

// Square CSR pattern of one space: active rows couple to every DOF of every
// cell containing them, rows sorted ascending; non-active rows hold only the
// diagonal.
Csr build_structure(const Space& s, int n_cells);

// Rectangular CSR pattern (test space rows x ansatz space columns) on one mesh.
// Rows of non-active test DOFs are empty.
Csr build_structure_rect(const Space& test, const Space& ansatz, int n_cells);

// Prolongation P (fine rows x coarse columns, empty rows for fine non-active
// DOFs) and restriction R (coarse rows x fine columns) of the nodal
// interpolation between two consecutive levels.
void build_transfer(const Hierarchy& h, int fine_level, const Space& coarse,
                    const Space& fine, Csr& P, Csr& R);

// Physical coordinates (double) of the cell vertices of one level.
std::vector<double> cell_vertices(const Hierarchy& h, int level);

}  // namespace pmsetup
