// Discretisation hierarchy (host): the levels a multigrid solve uses, each with
// its FE space(s), system CSR pattern, gather plans for the device assembly and
// the prolongation to the next finer level.
#pragma once
#include <functional>
#include <memory>
#include <vector>

#include "pm_setup.h"

namespace pm {

enum ProblemKind { KIND_CD = 0, KIND_STOKES = 1 };

struct DiscLevel {
  int level_in_hierarchy = 0;
  int n_cells = 0;
  pmsetup::Space space;     // CD scalar space / Stokes velocity component space
  pmsetup::Space pspace;    // Stokes pressure space (unused for CD)
  pmsetup::Csr sys;         // system pattern (combined blocks for Stokes)
  std::vector<double> verts;  // cell vertex coordinates
  // assembly gather plan: for each CSR entry of an active row, the positions
  // (cell * nloc * nloc + m * nloc + k) of the element-matrix entries that add
  // to it, in cell order (the order Assemble3D.C:346-370 adds them)
  std::vector<int> gat_ptr, gat_idx;
  // right-hand side gather plan: for each active DOF, positions cell*nloc + m
  std::vector<int> rgat_ptr, rgat_idx;
  // Dirichlet rows: CSR position of the diagonal entry
  std::vector<int> diag_pos;
  // physical coordinates (x, y, z; z = 0 in 2D) of the non-active DOFs
  // n_active .. n_dofs-1 of `space` (for Stokes the velocity component space),
  // the points of the nodal functionals the Dirichlet values are taken at
  std::vector<double> bnd_xyz;
  // Neumann boundary integral plan (2D): the active DOFs that lie on a
  // Neumann edge (ascending) and, per DOF, its (cell, code) pairs in cell
  // order; code = edge | side << 2 | local DOF << 4
  std::vector<int> nm_dof, nm_ptr, nm_cell, nm_code;
  // prolongation to the next finer level (rows of the finer level)
  pmsetup::Csr P;
  // Stokes block layout of the combined vector [u1 | u2 | u3 | p]
  int n_blocks = 1;
  int block_len[4] = {0, 0, 0, 0};
  int block_active[4] = {0, 0, 0, 0};
  // Stokes: combined local DOFs per cell (3 x 10 velocity + 4 pressure,
  // global combined indices) and the element storage per cell (10x10 A block
  // + 3 x 4x10 B blocks)
  std::vector<int> cdof;  // n_cells * 34
  int elem_stride = 0;    // doubles of element-matrix storage per cell
  int rhs_stride = 0;     // doubles of element right-hand side per cell
  // Vanka: per cell, its 34 combined DOFs sorted ascending (DofPatch order),
  // and a colouring of the cells such that cells of one colour share no DOF
  std::vector<int> patch_dofs;  // n_cells * 34
  std::vector<int> color_ptr, color_cells;
  // position of the first pressure row's diagonal in `sys` (pressure projection)
  int pressure_row0 = -1;
};

struct Disc {
  int kind = KIND_CD;
  int geometry = 0, root_n = 1, n_refine = 0, n_levels = 1, elem = 1;
  int neumann_sides = 0;  // 2D convection-diffusion: sides with Neumann conditions
  pmsetup::Hierarchy h;
  std::vector<DiscLevel> levels;  // 0 = coarsest kept level
  int dim() const { return h.dim; }
  int nvc() const { return h.nvc; }
};

// The parts of the set-up that can come from elsewhere (the GPU set-up,
// pm_devsetup.cu); each gives the same arrays as the host construction it
// replaces. hierarchy: the mesh hierarchy (build_hierarchy); space: a level's
// numbering (build_space); structure: a convection-diffusion level's `sys`,
// gather plans and diag_pos from its space.
struct SetupParts {
  std::function<pmsetup::Hierarchy(int geometry, int root_n, int n_refine)> hierarchy;
  std::function<pmsetup::Space(const pmsetup::Hierarchy&, int level, int elem, int boundary, int neumann_sides)>
      space;
  std::function<void(DiscLevel&)> structure;
  // a Stokes level's combined `sys`, gather plans and diag_pos from its cdof
  // and the active flags of the combined DOFs
  std::function<void(DiscLevel&, const std::vector<char>& active)> stokes_structure;
};

// the Stokes element's local coupling: (local row m, local column k) pairs of
// the 34 combined local DOFs (3 x 10 velocity, then 4 pressure) that carry a
// block entry, in row-major order, with their position in the 220-entry
// element storage (A 10 x 10, then B_0, B_1, B_2 4 x 10; B^T read transposed)
struct StokesLocal {
  int n = 0;
  int m[540], k[540], pos[540];
};
const StokesLocal& stokes_local();

std::unique_ptr<Disc> build_disc(int geometry, int root_n, int n_refine, int n_levels, int kind, int elem,
                                 int neumann_sides = 0, const SetupParts* parts = nullptr);

}  // namespace pm

struct pm_disc {
  std::unique_ptr<pm::Disc> d;
};
