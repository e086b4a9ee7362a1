// Stokes P2/P1 on tetrahedra: element assembly, the projected combined matrix
// used by the Vanka smoother and the coarse direct solve, and cell Vanka.
#pragma once
#include "pm_disc.h"
#include "pm_linalg.cuh"

namespace pm {

// reference-element data of P2/P1 on the P4Tetra rule (11 points)
struct DevStokesTables {
  DBuf<double> data;  // S (6 x 100), D (3 x 40), phi2 (11 x 10), w (11), xi (11 x 3)
  void upload(pm_ctx* c);
};

// device copy of one Stokes level's assembly inputs
struct DevStokesLevel {
  int n_cells = 0, n = 0;
  DBuf<double> verts;
  DBuf<int> gat_ptr, gat_idx, rgat_ptr, rgat_idx, diag_pos;
  void upload(pm_ctx* c, const DiscLevel& L);
};

// element matrices (220 doubles per cell) and element right-hand sides (34)
// of -nu Lap u + grad p = f, div u = 0 with f from the manufactured
// velocity u = curl(psi (1,1,1)), psi = (sin pi x sin pi y sin pi z)^2 and
// pressure p = x + y + z - 3/2; then gather into the combined CSR
void assemble_stokes_level(pm_ctx* c, const DevStokesLevel& L, const DevStokesTables& t, double nu,
                           DevCsr& A, double* rhs, double* K, double* F);

// get_combined_submatrix: the combined matrix with the first pressure row
// replaced by the unit row (pressure projection, all-Dirichlet velocity)
struct ProjectedMatrix {
  DevCsr csr;          // structure of the system with row p0 = {p0}
  DBuf<int> src;       // value source in the system matrix, -1 = unit diagonal
  void build(pm_ctx* c, const pmsetup::Csr& sys, int p0, const BlockMask& mask);
  void refresh(pm_ctx* c, const DevCsr& sys, bool fp32);  // copy values from the system
};

// rank of the coupling int psi_j grad phi_n between the P1 pressures j and
// the P2 velocity nodes n set in `mask` (bit n = local node n) on the
// reference tetrahedron; an affine map keeps the rank
int stokes_coupling_rank(unsigned mask);

// cell Vanka (src/Multigrid/VankaSmoother.C:110-292) with stored local inverses.
// A cell whose active velocity rows couple to its four pressures with rank < 4
// has a singular local matrix (the reference's LAPACK LU throws or returns a
// blown-up correction there): its pressures are frozen - unit rows and
// columns in the local matrix and no update.
struct DevVanka {
  int n_cells = 0, n = 0;
  DBuf<int> patch;        // n_cells x 34 sorted combined DOFs
  DBuf<int> freeze;       // per cell: trailing pressure entries frozen (0 or 4)
  int n_frozen = 0;
  DBuf<double> inv;       // n_cells x 34 x 34, column-major per cell
  DBuf<float> inv32;
  DBuf<int> inc_ptr, inc_idx;  // per DOF: positions cell*34+k in cell order
  DBuf<int> count;             // patches containing each DOF
  std::vector<int> color_ptr;  // host: colour ranges into color_cells
  DBuf<int> color_cells;
  DBuf<double> sol;  // n_cells x 34 local corrections
  DBuf<float> sol32;
  DBuf<int> flag;
  void setup(pm_ctx* c, const DiscLevel& L);
  // local matrices from the projected matrix, inverted on the device
  void factor(pm_ctx* c, const DevCsr& V, bool fp32);
  // one additive sweep (CELL_JACOBI): x += average of damp * A_loc^{-1} r_loc
  void sweep_jacobi(pm_ctx* c, const DevCsr& V, const double* b, double* x, double* r, double damp);
  void sweep_jacobi32(pm_ctx* c, const DevCsr& V, const float* b, float* x, float* r, float damp);
  // one multiplicative sweep (CELL), cells grouped by colour
  void sweep_colored(pm_ctx* c, const DevCsr& V, const double* b, double* x, double damp);
  void sweep_colored32(pm_ctx* c, const DevCsr& V, const float* b, float* x, float damp);
};

}  // namespace pm
