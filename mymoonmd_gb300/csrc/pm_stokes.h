// Stokes P2/P1 on tetrahedra: element assembly, the projected combined matrix
// used by the Vanka smoother and the coarse direct solve, and cell Vanka.
#pragma once
#include "pm_disc.h"
#include "pm_linalg.cuh"

namespace pm {

// reference-element data of P2/P1 on a tetrahedral rule: P4Tetra (11 points)
// for the Stokes problem, P5Tetra (15 points) for the Navier-Stokes problem
// (FEDatabase3D.C:1153-1219: degree 2 x 2 for linear problems, 3 x 2
// otherwise)
struct DevStokesTables {
  int qn = 11;
  // S (6 x 100), D (3 x 40), phi2 (qn x 10), w (qn), xi (qn x 3), and the
  // convection tensor C[a][i][j][k] = sum_q w phi_i d_a phi_j phi_k (3 x 1000;
  // with skew its antisymmetric part in i, j: the skew-symmetric form)
  DBuf<double> data;
  void upload(pm_ctx* c, int qn = 11, bool skew = false);
};

// device copy of one Stokes level's assembly inputs
struct DevStokesLevel {
  int n_cells = 0, n = 0;
  int nvel = 0, nvel_active = 0;  // DOFs and active DOFs of one velocity component
  int np = 0;                     // pressure DOFs
  DBuf<double> verts;
  DBuf<double> bnd_xyz;  // coordinates of the non-active velocity DOFs
  DBuf<int> gat_ptr, gat_idx, rgat_ptr, rgat_idx, diag_pos;
  DBuf<int> udof;        // velocity GlobalNumbers (n_cells x 10)
  // P1 pressure: integral weights (sum over the cells of a DOF of |K| / 4)
  // and the measure of the domain, for the projection into L2_0
  DBuf<double> pweight;
  double measure = 0.0;
  // restriction of a velocity from the next finer level (coarse levels):
  // the 8 children of each cell, and per velocity DOF its (cell * 10 + k)
  // positions in cell order
  DBuf<int> children, vinc_ptr, vinc_idx;
  void upload(pm_ctx* c, const DiscLevel& L);
  void set_children(pm_ctx* c, const pmsetup::Level& fine, const DiscLevel& L);
};

// element matrices (220 doubles per cell) and element right-hand sides (34)
// of -nu Lap u + grad p = f, div u = 0 with f from the manufactured
// velocity u = curl(psi (1,1,1)), psi = (sin pi x sin pi y sin pi z)^2 and
// pressure p = x + y + z - 3/2 (example 0), or from the polynomial solution
// u = (y^2, xz, -y^2), p = x + y + z - 3/2 of the reference's example -3
// (include/Examples/NSE_3D/test_u_2_p_1.h, u in P2, p in P1) with its
// Dirichlet values u(node); then gather into the combined CSR
void assemble_stokes_level(pm_ctx* c, const DevStokesLevel& L, const DevStokesTables& t, double nu,
                           DevCsr& A, double* rhs, double* K, double* F, int example = 0);

// Navier-Stokes (problem_type 5, convective form, NSTYPE 4, LAPLACETYPE 0):
// NavierStokesAll / NavierStokesNL of src/AssembleRoutinesSaddle/
// NSE_local_assembling_routines.C with NSNonlinearTerm_convective, which adds
//   N_ij = sum_q w |det J| (u . grad phi_j) phi_i
// to each of A11, A22, A33 for the current velocity u = [u1 | u2 | u3] of the
// level (nullptr: u = 0). With rhs == nullptr only the matrix is assembled
// (assemble_nonlinear_term, NavierStokes.C:573-750); otherwise also the
// right-hand side of the reference's example -3, whose body force holds the
// convective term: f = -nu Lap u + (u . grad) u + grad p.
void assemble_nse_level(pm_ctx* c, const DevStokesLevel& L, const DevStokesTables& t, double nu, DevCsr& A,
                        const double* u, double* rhs, double* K, double* F);

// the restriction matrices of P2 on the 8 children of the regular tetrahedral
// refinement (TFEDatabase3D::GetRestrictionMatrix3D, FEDatabase3D.C:1771-1890):
// Q_j = G^{-1} R_j, G the mass matrix of the parent's basis, R_j the products
// of the parent's and child j's basis over child j; 8 x 10 x 10, Q_j[k][l]
void build_p2_restriction(const pmsetup::Hierarchy& h, std::vector<double>& q);

// GridTransfer::RestrictFunction (src/Multigrid/GridTransfer.C:1218-1501) of
// the three velocity components from `fine` to `coarse`: per coarse cell the
// sum over its children of Q_j times the child's values, then each coarse DOF
// the average over its cells. cellval: coarse n_cells x 30 doubles scratch
void restrict_velocity(pm_ctx* c, const DevStokesLevel& coarse, const DevStokesLevel& fine, const double* q,
                       const double* u_fine, double* u_coarse, double* cellval);

// TFEFunction3D::project_into_L20 (src/FE/FEFunction3D.C:1678) of a P1
// pressure: p -= (integral of p) / measure
void project_pressure_l20(pm_ctx* c, const DevStokesLevel& L, double* p);

// NavierStokes::compute_residuals (NavierStokes.C:820-870): d = rhs - A x,
// the pressure part of d projected into L2_0, then the squared norms of the
// blocks u1, u2, u3, p of d into out4[0..3] (device; out4 holds
// kResidualScratch doubles, the rest partial sums)
constexpr int kResidualScratch = 4 + 4 * 256;
void nse_residuals(pm_ctx* c, const DevStokesLevel& L, const DevCsr& A, const double* rhs, const double* x,
                   double* d, double* out4);

// get_combined_submatrix: the combined matrix with the first pressure row
// replaced by the unit row (pressure projection, all-Dirichlet velocity)
struct ProjectedMatrix {
  DevCsr csr;          // structure of the system with row p0 = {p0}
  DBuf<int> src;       // value source in the system matrix, -1 = unit diagonal
  void build(pm_ctx* c, const pmsetup::Csr& sys, int p0, const BlockMask& mask);
  void refresh(pm_ctx* c, const DevCsr& sys, bool fp32);  // copy values from the system
};

// cell Vanka (src/Multigrid/VankaSmoother.C:110-292) with stored local inverses.
// A cell whose active velocity nodes are too few to control its pressures
// (3 rows per node against 4 pressures, or 3 when the cell holds the first
// pressure DOF, a unit row of the projected matrix) has a singular local
// matrix; the reference's LAPACK LU throws or returns a blown-up correction
// there. Such cells have their pressures frozen: unit rows and columns in the
// local matrix and no update.
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

// nodal Vanka (VankaType::NODAL, src/Multigrid/VankaSmoother.C:302-420): one
// patch per pressure DOF i, holding i and, in all three velocity components,
// the velocity nodes of row i of the coupling block B1. The local system
//   A u_k + bt_k p = r_k (k = 0, 1, 2),   sum_k b_k . u_k + c p = r_p
// is solved through the Schur complement of its single pressure:
//   w_k = A^{-1} r_k,  p = (r_p - sum_k b_k . w_k) / S,  u_k = w_k - t_k p,
//   t_k = A^{-1} bt_k, S = c - sum_k b_k . t_k,
// with one stored inverse A^{-1} of the velocity block (the three diagonal
// blocks are the same matrix in the Laplace-form Stokes system; the
// off-diagonal velocity blocks are zero). The reference factorises the whole
// (3n+1) x (3n+1) local matrix with LAPACK; the solution is the same up to
// rounding.
constexpr int kNodalMaxNodes = 96;

struct DevNodalVanka {
  int np = 0, nu = 0, n = 0, max_nodes = 0;
  int64_t ainv_len = 0;
  DBuf<int> vptr, vidx;      // per pressure DOF: velocity nodes (sorted)
  DBuf<int64_t> aoff;        // offsets of the n_i x n_i inverses
  DBuf<double> ainv;         // column-major inverses of the velocity blocks
  DBuf<float> ainv32;
  DBuf<double> tb;           // per patch at 6 vptr[i]: t_0, t_1, t_2, b_0, b_1, b_2 (n_i each)
  DBuf<float> tb32;
  DBuf<double> sinv;         // 1 / S per patch
  DBuf<float> sinv32;
  DBuf<int> inc_ptr, inc_idx, count;  // per combined DOF: positions in the local storage
  std::vector<int> color_ptr;          // host: colour ranges into color_patches
  // host, per colour: matrix entries of the patches' rows, the rows (3 m + 1
  // per patch), the velocity nodes m and the inverse entries m^2 (the launch
  // probe's algorithmic bytes)
  std::vector<int64_t> color_entries, color_rows, color_nodes, color_msq;
  DBuf<int> color_patches;
  DBuf<double> sol;  // local corrections / residuals: patch i at 3 vptr[i] + i, 3 n_i + 1 entries
  DBuf<float> sol32;
  DBuf<int> flag;
  // the rows of every patch as a sliced-ELL copy of the projected matrix,
  // colour by colour (the layout of the sliced SpMV, four lanes per row):
  // the local residuals of one colour are one SpMV-shaped launch over its
  // slices, rs_perm mapping each sliced row to its slot in the local storage.
  // Slices of colour k: color_slice[k] .. color_slice[k+1]. bslot: the global
  // row of each slot (the smoother's right-hand side gathered once per sweep)
  bool rs_ok = false;
  int rs_lanes = 0;  // lanes per row of the copy (4 or 8)
  std::vector<int> color_slice;
  int64_t rs_entries = 0;
  DBuf<int> rs_perm, rs_off, rs_cols, rs_src, bslot;
  DBuf<float> rs_vals32, bloc32;
  DBuf<double> rs_vals, bloc;
  void setup(pm_ctx* c, const DiscLevel& L);
  void build_row_slices(pm_ctx* c, const pmsetup::Csr& S, int p0, const std::vector<int>& vp,
                        const std::vector<int>& vi, const std::vector<int>& cp);
  void factor(pm_ctx* c, const DevCsr& V, bool fp32);
  // additive sweep: x += average of damp * local corrections from one residual
  void sweep_jacobi(pm_ctx* c, const DevCsr& V, const double* b, double* x, double* r, double damp);
  void sweep_jacobi32(pm_ctx* c, const DevCsr& V, const float* b, float* x, float* r, float damp);
  // multiplicative sweep, patches grouped by colour
  void sweep_colored(pm_ctx* c, const DevCsr& V, const double* b, double* x, double damp);
  void sweep_colored32(pm_ctx* c, const DevCsr& V, const float* b, float* x, float damp);
};

}  // namespace pm
