// Device assembly of convection-diffusion levels (see pm_assemble.cu).
#pragma once
#include <vector>

#include "pm_disc.h"
#include "pm_linalg.cuh"

namespace pm {

// reference-element tables of a Qk element on a tensor Gauss rule
struct RefTables {
  int dim = 0, nb = 0, nq = 0;
  std::vector<double> w, xi, phi, dphi;
};
void build_qk_tables(int dim, int k, int qn, RefTables& t);
// P1 (elem 11) / P2 (elem 12) on a tetrahedral rule of qn = 11 or 15 points
void build_pk_tables(int elem, int qn, RefTables& t);
// the tables of `elem` (Qk: k = 1, 2 on qn Gauss points per direction; Pk on
// tetrahedra: elem 11, 12 on a rule of qn points)
void build_element_tables(int dim, int elem, int qn, RefTables& t);

struct DevRefTables {
  int nb = 0, nq = 0, nt = 0;
  DBuf<double> data;
  // reference tensors of the bilinear form (sum over the quadrature points
  // of the reference element): stiffness S_ab (a<=b, S_ab+S_ba for a<b),
  // convection C_a[i][j] = sum_q w phi_i d_a phi_j, mass M; nt x nb x nb
  DBuf<double> tensors;
  void upload(pm_ctx* c, const RefTables& t);
};
// number of reference tensors: dim*(dim+1)/2 + dim + 1
inline int n_ref_tensors(int dim) { return dim * (dim + 1) / 2 + dim + 1; }
void build_ref_tensors(const RefTables& t, std::vector<double>& out);

// device copy of one level's assembly inputs
struct DevAssemblyLevel {
  int n_cells = 0, nloc = 0, n_dofs = 0, n_active = 0;
  DBuf<double> verts;
  DBuf<double> bnd_xyz;  // coordinates of the non-active DOFs (3 per DOF)
  DBuf<int> gat_ptr, gat_idx, rgat_ptr, rgat_idx, diag_pos;
  DBuf<int> nm_dof, nm_ptr, nm_cell, nm_code;  // Neumann boundary integral plan
  void upload(pm_ctx* c, const DiscLevel& L, int dim, int nvc);
  void scratch_sizes(size_t& k_elems, size_t& f_elems) const;
};

// value of the quadratic polynomial p (1, x, y, z, x^2, y^2, z^2, xy, xz, yz)
// at x (the evaluation the device kernels use)
double poly_value_host(const double* p, const double* x);

// Dirichlet values of the quadratic exact solution (manufactured = 2) into the
// non-active entries of rhs; nothing for the other coefficient kinds
void launch_dirichlet_values(pm_ctx* c, const DevAssemblyLevel& L, const pm_cd_coeffs& cf, double* rhs);

// Neumann boundary integrals of the exact solution's flux eps grad u . n added
// to the active entries of rhs on the Neumann edges; nothing without Neumann
// sides or for a constant right-hand side (homogeneous Neumann data)
void launch_neumann_values(pm_ctx* c, const DevAssemblyLevel& L, const pm_cd_coeffs& cf, double* rhs);

// L2, H1-semi, SD and L_inf errors of the FE function u (dofmap: n_cells x
// nloc) against the exact solution of cf, over the tensor Gauss rule with qn
// points per direction; partial holds error_blocks(n_cells) * 4 doubles, out
// receives the four errors (device pointers)
int error_blocks(int n_cells);
void launch_cd_errors(pm_ctx* c, int dim, int k, int qn, int n_cells, const double* verts, const int* dofmap,
                      const double* u, const DevRefTables& rt, const pm_cd_coeffs& cf, double* partial,
                      double* out);

// element matrices and element right-hand sides of one level into K and F, by
// the kernel the context's assembly_quadrature_loop option selects
void launch_cd_elements(pm_ctx* c, const DevAssemblyLevel& L, int dim, int k, int qn,
                        const pm_cd_coeffs& cf, const DevRefTables& rt, double* K, double* F);

// assemble matrix values and right-hand side of one level; K and F are scratch
// arrays of n_cells*nloc*nloc and n_cells*nloc doubles
void assemble_cd_level(pm_ctx* c, const DevAssemblyLevel& L, int dim, int elem, int qn,
                       const pm_cd_coeffs& cf, const DevRefTables& rt, DevCsr& A, double* rhs,
                       double* K, double* F);

}  // namespace pm
