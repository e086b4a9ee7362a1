/*
 * pmgpu.h - C ABI of the GB300-native finite element solve path.
 *
 * The library replaces, for one GPU, the element assembly, CSR SpMV, geometric
 * multigrid and Krylov kernels behind ParMooN's (nahmedwias/MyMooNMD) solver
 * interface. Every entry point names the reference interface it stands in for.
 *
 * Conventions
 *   - All functions return a status (PM_OK == 0). The message of the last
 *     failure of a context is returned by pm_last_error(). They never throw.
 *     The reference reports the same failures by ErrThrow -> std::runtime_error
 *     (include/General/MooNMD_Io.h:210).
 *   - Host arrays are copied in; the caller keeps ownership. Pointers named
 *     *_dev are device pointers (allocated with pm_dev_alloc or any CUDA
 *     allocation on the context's device). Device buffers of handles belong to
 *     the library and are freed by the matching *_destroy call.
 *   - One context owns one CUDA stream. Calls on one context must be serialised
 *     by the caller; different contexts may be used from different threads.
 *   - Vectors are contiguous FP64 arrays laid out like BlockVector
 *     (include/Matrix/BlockVector.h:43): blocks one after another, the
 *     non-active (Dirichlet) DOFs at the tail of each block.
 */
#ifndef PMGPU_H
#define PMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define PM_OK 0
#define PM_E_INVALID 1     /* bad argument (ErrThrow on wrong sizes/keys)          */
#define PM_E_OOM 2         /* device allocation failed / admission refused         */
#define PM_E_DIVERGED 3    /* IterativeMethod::converged divergence branch         */
#define PM_E_BREAKDOWN 4   /* FGMRES unhappy breakdown, BiCGStab omega == 0, zero pivot */
#define PM_E_MAXIT 5       /* reserved: iteration cap (reported through info, not as failure) */
#define PM_E_CUDA 6        /* CUDA runtime error                                   */
#define PM_E_TIMEOUT 7     /* a bounded device wait gave up                        */
#define PM_E_UNSUPPORTED 8 /* configuration outside what this library implements   */

typedef struct pm_ctx pm_ctx;
typedef struct pm_matrix pm_matrix;
typedef struct pm_solver pm_solver;
typedef struct pm_disc pm_disc;
typedef struct pm_problem pm_problem;
typedef struct pm_server pm_server;

/* ------------------------------------------------------------ context ---- */
int pm_ctx_create(int device, pm_ctx** out);
void pm_ctx_destroy(pm_ctx* ctx);
const char* pm_last_error(const pm_ctx* ctx);
int pm_ctx_synchronize(pm_ctx* ctx);
/* number of kernels this context launched since creation */
int pm_ctx_kernel_launches(const pm_ctx* ctx, uint64_t* out);
/* CUDA events on the context's stream, for timing (ms between two records) */
int pm_ctx_time_begin(pm_ctx* ctx);
int pm_ctx_time_end(pm_ctx* ctx, float* ms);
int pm_version(void);
/* Context options (no reference counterpart):
 *   "assembly_quadrature_loop" 0|1 - element matrices by the per-quadrature-
 *   point loop of LocalAssembling instead of the reference-tensor contraction
 *   (same quadrature, different summation order);
 *   "probe_epilogue" -1..5 - the launch probe below brackets only launches of
 *   this SpMV epilogue (0 y+=aAx, 1 y=Ax, 2 defect, 3 damped Jacobi sweep,
 *   4 restriction, 5 prolongation add; -1 = all);
 *   "probe_precision" 0|4|8 - only launches whose matrix values have this
 *   size in bytes (0 = all);
 *   "probe_nodal" 0|1 - the launch probe brackets instead the residual and
 *   local-solve pair of every colour of the multiplicative nodal Vanka
 *   sweeps (counted as one launch, with the pair's algorithmic bytes);
 *   "nodal_sliced" 0|4|8 - the local residuals of a colour of the
 *   multiplicative nodal Vanka sweep by one sliced-ELL launch over a copy of
 *   its patches' rows with 4 or 8 lanes per row (8, default; 1 = 4; the copy
 *   holds every patch row once, laid out when a problem sets up its
 *   smoothers, values refreshed with the Vanka factors) or by one block per
 *   patch over the CSR rows (0);
 *   "fp32_sliced_spmv" 0|100 L + 10 U + P - FP32 SpMV-family launches on
 *   matrices with more than 16 entries per row by the sliced-ELL kernel: L
 *   lanes per row (1, 2, 4, 8), U steps in flight (4, 8), P = 1 issues the next
 *   steps' loads before the current gathers; accepted: 140 141 180 240 241 280
 *   440 441 480 481 840 841 881; 0 = the row-group kernel on the CSR arrays.
 *   Default 481. The sliced copy (rows sorted by length in windows of 1024,
 *   slices of 32/L rows, padded to the slice's longest row) is laid out when
 *   the FP32 values are made (pm_matrix_make_fp32, the multigrid update) for
 *   the shape's L. Shapes with the same L give the same bits;
 *   "pdl" 0|1 - launches of the sliced-ELL sweeps with programmatic stream
 *   serialization (a sweep loads its slice layout and first values while the
 *   previous kernel finishes, and waits for it before reading vectors; default
 *   1: on GB300 the 3D Q2 request took 26.9 ms with 1, 27.6 ms with 0);
 *   "fp64_sliced_spmv" 0|441|481|841 - the same for FP64 values (the Krylov
 *   SpMV, the FP64 multigrid); used when its L equals the layout's (default 441);
 *   "jacobi_zero_start" 0|1 - the first damped Jacobi sweep of a multigrid level
 *   whose iterate is exactly zero (coarse levels after their reset; the finest
 *   level inside FGMRES when the initial residual has zero non-actives) as the
 *   diagonal scaling x = w b / d, which gives the sweep's bits (default 1). */
int pm_ctx_set_option(pm_ctx* ctx, const char* key, int value);
/* Launch probe (no reference counterpart; measurement only): while enabled
 * (nnz != 0), every SpMV-family launch (apply, defect, Jacobi sweep, transfer)
 * on a matrix with exactly `nnz` nonzeros is bracketed by CUDA events on the
 * context's stream. pm_ctx_probe_result returns the number of probed launches,
 * their summed device time and their summed algorithmic bytes. */
int pm_ctx_probe(pm_ctx* ctx, int64_t nnz);
int pm_ctx_probe_result(pm_ctx* ctx, int* launches, double* total_ms, double* total_bytes);

int pm_dev_alloc(pm_ctx* ctx, size_t bytes, void** out_dev);
int pm_dev_free(pm_ctx* ctx, void* dev);
int pm_memcpy_h2d(pm_ctx* ctx, void* dst_dev, const void* src_host, size_t bytes);
int pm_memcpy_d2h(pm_ctx* ctx, void* dst_host, const void* src_dev, size_t bytes);
int pm_memset_dev(pm_ctx* ctx, void* dst_dev, int value, size_t bytes);
/* page-locked host memory for the host<->device copies of requests */
int pm_host_alloc(pm_ctx* ctx, size_t bytes, void** out_host);
int pm_host_free(pm_ctx* ctx, void* host);

/* ------------------------------------------------------------ matrices --- */
/* TMatrix / FEMatrix (include/Matrix/Matrix.h:47, include/Matrix/FEMatrix.h:27):
 * CSR with ascending column indices per row (TStructure ColOrder = 1). Rows
 * [n_active, n_rows) are non-active; FE matrices store a unit diagonal there
 * (src/AssembleRoutines/Assemble3D.C:396-404). vals may be NULL (zeros). */
int pm_matrix_create_csr(pm_ctx* ctx, int n_rows, int n_cols, int n_active,
                         const int* row_ptr, const int* cols, const double* vals,
                         pm_matrix** out);
void pm_matrix_destroy(pm_matrix* A);
/* BlockFEMatrix block layout of a combined square matrix
 * (src/Matrix/BlockFEMatrix.C:1168 get_combined_submatrix): n_blocks <= 4
 * blocks of the given lengths, the first actives[b] rows of block b active. */
int pm_matrix_set_blocks(pm_matrix* A, int n_blocks, const int* lengths, const int* actives);
int pm_matrix_info(const pm_matrix* A, int* n_rows, int* n_cols, int* n_active, int64_t* nnz);
int pm_matrix_set_values(pm_matrix* A, const double* vals_host);
int pm_matrix_get_values(const pm_matrix* A, double* vals_host);
int pm_matrix_get_structure(const pm_matrix* A, int* row_ptr_host, int* cols_host);
/* BlockFEMatrix::apply_scaled_add (src/Matrix/BlockFEMatrix.C:863):
 * y += a*A*x on active rows, y += a*x on non-active rows. */
int pm_matrix_apply_scaled_add(pm_matrix* A, const double* x_dev, double* y_dev, double a);
/* BlockFEMatrix::apply (src/Matrix/BlockFEMatrix.C:855): y = A*x */
int pm_matrix_apply(pm_matrix* A, const double* x_dev, double* y_dev);
/* TMatrix::get_diagonal (src/Matrix/Matrix.C:298) */
int pm_matrix_get_diagonal(pm_matrix* A, double* diag_dev);
/* FP32 copy of the values for the mixed-precision preconditioner, and its SpMV
 * y = A32*x (FP32 values, vectors and accumulation). */
int pm_matrix_make_fp32(pm_matrix* A);
/* Sliced-ELL copy of the FP64 values for the context's "fp64_sliced_spmv"
 * shape (no reference counterpart): FP64 SpMV-family launches on A use it from
 * then on; writers of the values keep it current. Solvers make it in their
 * update. */
int pm_matrix_make_sliced64(pm_matrix* A);
int pm_matrix_apply_f32(pm_matrix* A, const float* x_dev, float* y_dev);
/* Launch shape of the CSR kernels of this matrix (no reference counterpart;
 * tuning only): lanes per row (1, 2, 4, 8, 16, 32) and entries per lane per chunk
 * (2, 4, 8, 16) of the per-row-group kernel (the default); (0, 0) selects the
 * row-block streaming kernel. */
int pm_matrix_set_kernel(pm_matrix* A, int lanes, int unroll);
/* Timed SpMV loop: `reps` applications y = A x on the context's stream, timed
 * with CUDA events; returns ms per application and the algorithmic bytes. */
int pm_matrix_bench_apply(pm_matrix* A, int fp32, const void* x_dev, void* y_dev, int reps,
                          float* ms_per_apply, double* bytes_per_apply);

/* ------------------------------------------------------------- BLAS-1 ---- */
/* Ddot / Dnorm / Daxpy / Dscal (src/FE/Blas1.C:14-115) on device vectors;
 * reductions use a fixed tree and are deterministic. */
int pm_dot(pm_ctx* ctx, int n, const double* x_dev, const double* y_dev, double* out);
int pm_norm(pm_ctx* ctx, int n, const double* x_dev, double* out);
int pm_axpy(pm_ctx* ctx, int n, double a, const double* x_dev, double* y_dev);
int pm_scal(pm_ctx* ctx, int n, double a, double* x_dev);

/* --------------------------------------------------------------- solver --- */
/* Solver<BlockFEMatrix, BlockVector> (include/Solver/Solver.h:31-127), driven
 * by ParameterDatabase keys given as text, one "key: value" per line, with the
 * reference's names and meaning (src/Solver/Solver.C:21-115,
 * src/Multigrid/Multigrid.C:422-514), e.g.
 *   solver_type: iterative       iterative_solver_type: fgmres
 *   preconditioner: multigrid    residual_reduction: 1e-8
 * Implemented: iterative_solver_type fgmres (right_gmres), cg, bi_cgstab,
 * jacobi, sor, ssor, richardson (x += damping_factor P^-1 (b - A x),
 * src/Solver/Iteration_richardson.C), cgs (src/Solver/Iteration_cgs.C),
 * left_gmres (Iteration_gmres::left_gmres, preconditioned residual); preconditioner no_preconditioner, jacobi, sor, ssor,
 * multigrid; multigrid_smoother(_coarse) jacobi, sor, ssor, cell_vanka,
 * cell_vanka_jacobi, nodal_vanka, nodal_vanka_jacobi, direct_solve (coarse).
 * SOR and SSOR (TMatrix::sor_sweep, src/Matrix/Matrix.C:943, omega =
 * sor_omega) sweep the rows in multicolour order: a greedy colouring of the
 * matrix graph in row order, rows grouped by colour; rows of one colour are
 * updated in parallel, which equals the sequential sweep over that order.
 * New keys (no reference counterpart):
 *   gpu_precision {fp64, mixed}: mixed = FP32 multigrid inside FP64 FGMRES;
 *   gpu_mixed_fallback {1, 0}: in the mixed form, the multigrid switches to
 *     FP64 for the rest of a solve once the FP64 residual has fallen by less
 *     than half over 10 iterations (FGMRES is flexible);
 *   gpu_gram_schmidt {mgs, cgs2, cgs2_cond}: Arnoldi orthogonalisation; mgs is
 *     the reference's (default for fp64), cgs2 two batched classical passes
 *     (default for mixed), cgs2_cond the second pass only when the first lost
 *     more than a factor 1/sqrt(2) of the norm;
 *   gpu_cuda_graphs {1, 0}: Arnoldi steps captured as CUDA graphs.
 * Unknown keys are ignored like ParameterDatabase::merge(.., false). */
int pm_solver_create(pm_ctx* ctx, const char* params, pm_solver** out);
void pm_solver_destroy(pm_solver* s);
/* Solver::update_matrix (src/Solver/Solver.C:261). With preconditioner
 * multigrid the finest level is `A`; coarser levels come from
 * pm_solver_set_multigrid_level (Multigrid::initialize, coarsest -> finest). */
int pm_solver_update_matrix(pm_solver* s, pm_matrix* A);
/* Multigrid level `level` (0 = coarsest) with its matrix and the prolongation
 * from this level to the next finer one (fine rows x this level's columns,
 * empty rows for non-active fine DOFs) - the operator GridTransfer::Prolongate
 * applies (src/Multigrid/GridTransfer.C:665); restriction uses its transpose
 * (GridTransfer::DefectRestriction, :943). The finest level passes P = NULL. */
int pm_solver_set_multigrid_level(pm_solver* s, int level, int n_levels, pm_matrix* A,
                                  int p_rows, int p_cols, const int* p_row_ptr,
                                  const int* p_cols_idx, const double* p_vals);
/* Solver::solve (src/Solver/Solver.C:415,493) on device vectors. */
int pm_solver_solve(pm_solver* s, const double* rhs_dev, double* sol_dev);
/* Same on host vectors (host->device copy in, device->host copy out). */
int pm_solver_solve_host(pm_solver* s, const double* rhs_host, double* sol_host, int n);
/* LoopInfo of the last solve: iterations and final residual. */
int pm_solver_last_info(const pm_solver* s, int* iterations, double* residual,
                        double* initial_residual);
/* Residual history of the last solve (up to cap entries), returns count. */
int pm_solver_residual_history(const pm_solver* s, double* out, int cap, int* count);
/* Iteration_multigrid::apply (src/Solver/Iteration_multigrid.C:22): one
 * multigrid cycle with rhs z, result r. */
int pm_solver_apply_preconditioner(pm_solver* s, const double* z_dev, double* r_dev);

/* ------------------------------------------------ discretisation set-up --- */
/* Mesh hierarchy + FE spaces + CSR structures + transfer operators, restating
 * TDomain refinement (src/Geometry/Domain.C:1045), TFESpace3D::ConstructSpace
 * (src/FE/FESpace3D.C:506) and TStructure (src/Matrix/Structure.C:829).
 * geometry: 0 unit square (quadrilaterals), 1 unit cube (hexahedra),
 *           2 unit cube (tetrahedra, 6 per cube as Default_UnitCube_Tetra)
 * root_n: root cells per side (1 = the reference's default meshes)
 * n_refine: regular refinements; the finest n_levels levels are kept for MG.
 * kind: 0 convection-diffusion (elem 1 = Q1, 2 = Q2 on quads/hexes),
 *       1 Stokes P2/P1 Taylor-Hood on tetrahedra (elem ignored). */
int pm_disc_create(int geometry, int root_n, int n_refine, int n_levels, int kind, int elem,
                   pm_disc** out);
/* pm_disc_create with Neumann conditions on some sides of the unit square
 * (convection-diffusion, geometry 0): bit s of neumann_sides marks side s in
 * the numbering of UnitSquare's boundary components (Default_UnitSquare):
 * 0 y=0, 1 x=1, 2 y=1, 3 x=0; the other sides stay Dirichlet. The example's
 * BoundCondition (e.g. include/Examples/CD_2D/SineLaplace.h: side 1 Neumann)
 * in mask form. DOFs are numbered inner, Neumann, Dirichlet, each in order of
 * first touch (TFESpace2D::ConstructSpace); a DOF is Neumann when every side it
 * lies on is, so corners next to a Dirichlet side are Dirichlet. Neumann DOFs
 * are active. Assembly adds the boundary integral of the exact solution's flux
 * eps grad u . n over the Neumann edges (Assemble2D.C:716-757); with a constant
 * right-hand side (no exact solution) the Neumann data are zero. */
int pm_disc_create_bc(int geometry, int root_n, int n_refine, int n_levels, int kind, int elem,
                      int neumann_sides, pm_disc** out);
/* pm_disc_create_bc with the set-up on the context's GPU: the regular
 * refinement of the root mesh (the RefQuadRegDesc / RefHexaRegDesc /
 * RefTetraRegDesc children, one thread per child cell), the first-touch DOF
 * numbering of every kept convection-diffusion level (TFESpace{2,3}D::
 * ConstructSpace: two radix sorts, of the local DOF positions by node and of
 * the distinct nodes by class and first touch) and its CSR structure
 * (TStructure(space), src/Matrix/Structure.C:829-1283, sorted) with the
 * assembly gather plans (one stable radix sort of the element entries by
 * (row, column)); for a Stokes set-up the refinement, the numbering of both
 * spaces and the combined structure of the NSTYPE 4 blocks with its gather
 * plans. The result is the same discretisation, array for array; the grid
 * transfer stays on the host. The context's
 * stream is synchronised; temporary device memory of about 40 bytes per
 * element-matrix entry of the finest level is freed before the call returns. */
int pm_disc_create_device(pm_ctx* ctx, int geometry, int root_n, int n_refine, int n_levels, int kind,
                          int elem, int neumann_sides, pm_disc** out);
void pm_disc_destroy(pm_disc* d);
/* per level (0 = coarsest kept level): cells, local DOFs per cell, DOFs,
 * active DOFs and nnz of the level matrix (space 0 = velocity/scalar,
 * space 1 = pressure for Stokes) */
int pm_disc_level_info(const pm_disc* d, int level, int space, int* n_cells, int* nloc,
                       int* n_dofs, int* n_active, int64_t* nnz);
/* GlobalNumbers of the level (n_cells * nloc, BeginIndex[c] = c*nloc) */
int pm_disc_dofmap(const pm_disc* d, int level, int space, int* out);
/* cell vertex coordinates (n_cells * vertices * dim) */
int pm_disc_cell_vertices(const pm_disc* d, int level, double* out);
/* CSR pattern of the level system matrix (combined blocks for Stokes) */
int pm_disc_structure(const pm_disc* d, int level, int* row_ptr, int* cols);
/* prolongation from `level` to `level+1` (rows of level+1) */
int pm_disc_prolongation_info(const pm_disc* d, int level, int* rows, int* cols, int64_t* nnz);
int pm_disc_prolongation(const pm_disc* d, int level, int* row_ptr, int* cols, double* vals);

/* ------------------------------------------------------------ assembly --- */
/* Coefficients of the convection-diffusion problem
 *   -eps Laplace(u) + b.grad(u) + c u = f, u = g on the boundary:
 *   manufactured = 1: f from the exact solution u = prod_d sin(pi x_d), g = 0
 *     (Example_CD2D/3D sine examples);
 *   manufactured = 0: f = f_const, g = 0;
 *   manufactured = 2: f from the quadratic exact solution
 *     u = poly[0] + poly[1] x + poly[2] y + poly[3] z + poly[4] x^2 + poly[5] y^2
 *         + poly[6] z^2 + poly[7] xy + poly[8] xz + poly[9] yz,
 *     g = u at the Dirichlet DOFs (the point values of the Lagrange nodal
 *     functionals, Assemble3D.C:640-665). The examples test_p0 / test_p1 /
 *     test_p2 of Example_CD3D.C:164-193 (exact solution in Q1 / Q2).
 *     With manufactured = 2, poly_src (same monomials) is added to f: the time
 *     derivative of a time-dependent exact solution (zero for stationary
 *     problems).
 * poly and poly_src are read only with manufactured = 2 (a caller built
 * against a header without them passes the smaller struct safely with 0 or 1). */
typedef struct pm_cd_coeffs {
  double eps;
  double b[3];
  double c;
  int manufactured;
  double f_const;
  double poly[10];
  double poly_src[10];
} pm_cd_coeffs;

/* Assemble2D / Assemble3D with LocalAssembling (ConvDiff Galerkin,
 * src/AssembleRoutines/Assemble3D.C:37, LocalAssembling.C:669,
 * ConvDiff.C:1794-1856) of one level on the device: element matrices over the
 * quadrature points, gathered into the CSR in cell order; Dirichlet rows get a
 * unit diagonal and zero right-hand side. quad_points: points per direction of
 * the tensor Gauss rule (2..4); 0 picks the reference's default. */
int pm_assemble_cd(pm_ctx* ctx, const pm_disc* d, int level, const pm_cd_coeffs* coeffs,
                   int quad_points, pm_matrix* A, double* rhs_dev);

/* Assembly of level `level` of a convection-diffusion problem into device
 * arrays the caller owns (vals_dev: the level's nnz matrix values in CSR
 * order, rhs_dev: its n_dofs right-hand side), allocating no device memory.
 * No counterpart in the reference: it serves callers that cannot call
 * cudaMalloc at this point (a serving worker that must not stall concurrent
 * requests with an allocation, code bound to memory reserved up front). The
 * element-matrix scratch lives in a static 32 MiB device array per GPU, so
 * levels needing more than 4 Mi doubles (n_cells*nloc*(nloc+1)) are rejected
 * with PM_E_INVALID. The first call on a device looks the array up and should
 * come before any stream capture; calls that overlap on the GPU race on the
 * shared array. coeffs == NULL keeps the problem's coefficients. The element
 * kernels are those pm_assemble_cd runs under the same context options, so
 * both entry points give the same bits. Stokes problems are refused with
 * PM_E_UNSUPPORTED. */
int pm_assemble_cd_noalloc(pm_problem* p, int level, const pm_cd_coeffs* coeffs, double* vals_dev,
                           double* rhs_dev);

/* ----------------------------------------------------- problem (system) --- */
/* ConvectionDiffusion<d> / NavierStokes<3> (Stokes) system on the device: the
 * level hierarchy of `disc`, assembled matrices, right-hand side and the solver
 * built from `params`. */
int pm_problem_create_cd(pm_ctx* ctx, const pm_disc* d, const pm_cd_coeffs* coeffs,
                         int quad_points, const char* params, pm_problem** out);
void pm_problem_destroy(pm_problem* p);
/* NavierStokes<3> with FLOW_PROBLEM_TYPE Stokes (src/System/NavierStokes.C:407,
 * 878) on a Stokes discretisation (P2/P1 on tetrahedra): -nu Lap u + grad p =
 * f, div u = 0, no-slip walls, f from the manufactured velocity
 * u = curl(psi (1,1,1)), psi = (sin pi x sin pi y sin pi z)^2, and pressure
 * p = x + y + z - 3/2. Vector layout [u1 | u2 | u3 | p]. The multigrid levels
 * get the projected combined matrices and cell-Vanka data
 * (multigrid_smoother cell_vanka | cell_vanka_jacobi, VankaSmoother.C). */
int pm_problem_create_stokes(pm_ctx* ctx, const pm_disc* d, double nu, const char* params,
                             pm_problem** out);
/* The Navier-Stokes problem (NavierStokes<3> with problem_type 5, the
 * convective form, NSTYPE 4, LAPLACETYPE 0, Galerkin) is the same handle,
 * created with "problem_type: 5" and "example: -3" in params (the reference's
 * example -3, include/Examples/NSE_3D/test_u_2_p_1.h, whose body force holds
 * the convective term; nu = 1 / reynolds_number). Its assembly uses the
 * P5Tetra rule (degree 3 x 2 for nonlinear problems, FEDatabase3D.C:1153-1219)
 * and adds the convective term (u . grad u_j, phi_i) of each level's current
 * velocity to A11, A22 and A33 (NSNonlinearTerm_convective,
 * src/AssembleRoutinesSaddle/NSE_local_assembling_routines.C); with
 * "nse_nonlinear_form: skew_symmetric" its skew-symmetric form (1/2)
 * [(u . grad phi_j, phi_i) - (u . grad phi_i, phi_j)] (NSNonlinearTerm_
 * skew_symmetric). The rotational, divergence and emac forms couple the
 * velocity components and return PM_E_UNSUPPORTED. */
/* ConvectionDiffusion::assemble (src/System/ConvectionDiffusion.C:174);
 * NavierStokes::assemble_linear_terms (src/System/NavierStokes.C:407) for a
 * Stokes / Navier-Stokes problem */
int pm_problem_assemble(pm_problem* p);
/* NavierStokes::assemble_nonlinear_term (src/System/NavierStokes.C:573): the
 * finest velocity restricted to every coarser level
 * (GridTransfer::RestrictFunctionRepeatedly, src/Multigrid/GridTransfer.C:1506;
 * per coarse cell the L2 projection of its children's values, averaged over
 * the cells of each DOF) and the velocity blocks of every level reassembled
 * with the convective term of that level's velocity. Navier-Stokes only. */
int pm_problem_assemble_nonlinear(pm_problem* p);
/* NavierStokes::compute_residuals (src/System/NavierStokes.C:820): d = rhs -
 * A x on the finest level, the pressure part of d projected into L2_0; out[0]
 * = |d_u1| + |d_u2| + |d_u3| (impuls: BlockVector::norm over blocks sums the
 * blocks' 2-norms, src/Matrix/BlockVector.C:293), out[1] = |d_p| (mass),
 * out[2] = the full residual sqrt(out[0]^2 + out[1]^2). Stokes or
 * Navier-Stokes problems. */
int pm_problem_residuals(pm_problem* p, double* out);
/* The nonlinear loop of the reference's test/nse3d_solvers_test.c++:
 * stop_it(0); then solve / assemble_nonlinear_term / stop_it(k) until stop_it
 * (src/System/NavierStokes.C:753) says so, with the params keys
 * nonlinloop_maxit (100), nonlinloop_minit (1), nonlinloop_epsilon (1e-10),
 * nonlinloop_damping_factor (1.0), nonlinloop_slowfactor (1e10),
 * nonlinloop_scale_epsilon_with_size and nonlinloop_residual_relative_to_rhs
 * (false). Call after pm_problem_assemble. residuals (3 doubles per step,
 * steps 0..n_steps, at most max_records steps, or NULL) receives the impuls,
 * mass and full residual of every stop_it; n_steps the number of solves. */
int pm_problem_solve_nonlinear(pm_problem* p, int max_records, double* residuals, int* n_steps);
/* ConvectionDiffusion::solve (src/System/ConvectionDiffusion.C:191). Like the
 * reference, the solve starts from the current solution vector. For a Stokes /
 * Navier-Stokes problem NavierStokes::solve (src/System/NavierStokes.C:878):
 * afterwards the pressure is projected into L2_0 (TFEFunction3D::
 * project_into_L20, src/FE/FEFunction3D.C:1678). */
int pm_problem_solve(pm_problem* p);
/* Zero initial guess for the next request (the state after construction,
 * ConvectionDiffusion.C:73). */
int pm_problem_reset_solution(pm_problem* p);
int pm_problem_size(const pm_problem* p, int* n_dofs, int* n_active);
int pm_problem_get_solution(const pm_problem* p, double* sol_host);
/* the finest-level solution vector from host memory (an initial guess or a
 * given velocity for the nonlinear assembly: NavierStokes::get_solution()) */
int pm_problem_set_solution(pm_problem* p, const double* sol_host);
int pm_problem_get_rhs(const pm_problem* p, double* rhs_host);
int pm_problem_matrix(pm_problem* p, int level, pm_matrix** out);
int pm_problem_solver(pm_problem* p, pm_solver** out);
int pm_problem_solution_dev(pm_problem* p, double** sol_dev, double** rhs_dev);
/* One request end to end from host memory: new coefficients, the cell vertex
 * coordinates of every kept level (level_verts[l], NULL = keep the current
 * geometry) copied to the device, assembly of all levels, solve (for a
 * Navier-Stokes problem the nonlinear loop of pm_problem_solve_nonlinear), and
 * the finest-level solution copied back into sol_host. */
int pm_problem_run_host(pm_problem* p, const pm_cd_coeffs* coeffs, const double* const* level_verts,
                        double* sol_host);
/* Errors of the finest-level solution against the exact solution of the
 * problem's coefficients, as ConvectionDiffusion<d>::output computes them
 * (src/System/ConvectionDiffusion.C:213-283 with conv_diff_l2_h1_linf_error,
 * src/AssembleRoutines/ConvDiff.C:2134-2185): errors[0] L2, errors[1]
 * H1-semi, errors[2] SD (eps |grad e|^2 + c e^2 + delta (b . grad e)^2 with
 * the SUPG delta of the reference's default parameters), errors[3] L_inf over
 * the quadrature points, on the assembly's quadrature rule (the rule
 * TFEDatabase{2,3}D::GetOrig picks). With a constant right-hand side the exact
 * solution is zero and these are norms of the solution. Convection-diffusion
 * problems only. */
int pm_problem_errors(pm_problem* p, double* errors);
/* Solver statistics of the problem's last solve. */
int pm_problem_last_info(const pm_problem* p, int* iterations, double* residual,
                         double* initial_residual);
/* Batched solve (no reference counterpart; the reference solves one system
 * per Solver::solve, src/Solver/Solver.C:415): n_problems assembled
 * convection-diffusion problems of one set-up (the same pm_disc) and one
 * context, solved by FGMRES(m <= 32) with the multigrid preconditioner (damped
 * Jacobi smoothing, direct coarse solve) in lockstep, at most `slots` (<= 16)
 * at a time: every kernel of an Arnoldi step and of the V-cycle runs once for
 * all slots. Problems join at restart-cycle boundaries and leave when their
 * residual test passes; each problem's iterates are those of its lone
 * pm_problem_solve, bit for bit, except that the mixed form keeps its FP32
 * cycle throughout (the lone solve may switch to FP64 when the residual
 * stalls). status_out (n_problems, or NULL): per problem PM_OK, PM_E_MAXIT,
 * PM_E_DIVERGED or PM_E_BREAKDOWN; pm_problem_last_info and the solution
 * vectors hold each problem's result. */
int pm_problem_solve_batched(pm_problem* const* probs, int n_problems, int slots, int* status_out);

/* ------------------------------------------- time-dependent problem ------ */
/* TimeConvectionDiffusion<d> (src/System/TimeConvectionDiffusion.C) with
 * TimeDiscretization (src/TimeDiscRoutines/TimeDiscretizations.C):
 * backward_euler, crank_nicolson, bdf_two. params: the solver keys of
 * pm_problem_create_cd plus time_discretization, time_step_length,
 * time_start, time_end. poly_time (20 doubles or NULL): P1, P2 of the exact
 * solution u = P0 + t P1 + t^2 P2 with coeffs->manufactured = 2 (P0 =
 * coeffs->poly); f and the Dirichlet values follow from u at the current time.
 * The time loop of the reference's test programs
 * (test/tcd3d_solvers_test.c++:76-92) reads:
 *   pm_tcd_assemble_initial_time(s);
 *   while (time < time_end - 1e-10) { pm_tcd_next_step(s); pm_tcd_assemble(s); pm_tcd_solve(s); } */
typedef struct pm_tcd pm_tcd;
int pm_tcd_create(pm_ctx* ctx, const pm_disc* d, const pm_cd_coeffs* coeffs, const double* poly_time,
                  int quad_points, const char* params, pm_tcd** out);
void pm_tcd_destroy(pm_tcd* s);
/* assemble_initial_time: stiffness, mass, rhs; solution = initial condition */
int pm_tcd_assemble_initial_time(pm_tcd* s);
/* current_step_++, set_time_disc_parameters, current_time += tau */
int pm_tcd_next_step(pm_tcd* s);
/* assemble: stiffness and rhs at the current time, time-discrete rhs, system matrices */
int pm_tcd_assemble(pm_tcd* s);
/* solve, then reset_linear_matrices and the old solutions */
int pm_tcd_solve(pm_tcd* s);
int pm_tcd_state(const pm_tcd* s, double* time, int* step);
/* the underlying problem: solution, matrices, solver statistics */
int pm_tcd_problem(pm_tcd* s, pm_problem** out);

/* ---------------------------------------------------------------------------
 * Request executor (no reference counterpart: the batched stream and the
 * serving loop). Independent solves run on one GPU by n_workers host threads,
 * each with its own context (CUDA stream). A worker keeps the device-resident
 * problem of every set-up it has served (mesh, spaces, structures, level
 * matrices, solver and its captured graphs) and reuses it for later requests
 * with the same set-up; new coefficients are assembled on the device. Set-ups
 * (host mesh hierarchies) are shared between the workers. The estimated device
 * footprint of the cached problems is kept under hbm_cap_bytes by evicting the
 * least recently used ones of the worker that needs room; a problem whose own
 * footprint exceeds the cap is solved and then released instead of being kept
 * (0 = no cap). A device allocation failure is reported as PM_E_OOM in the
 * result. params_cd / params_stokes: the solver parameters of
 * the two problem kinds (ParameterDatabase text, as pm_solver_create; the
 * number of multigrid levels comes from the request). */
typedef struct {
  int kind;     /* 0 convection-diffusion, 1 Stokes */
  int geometry; /* as pm_disc_create: 0 square, 1 cube (hexahedra), 2 cube (tetrahedra) */
  int root_n, n_refine, n_levels, elem;
  pm_cd_coeffs coeffs; /* convection-diffusion */
  double nu;           /* Stokes viscosity */
  double* solution_out; /* host buffer for the finest-level solution, or NULL */
  uint64_t tag;         /* caller's identifier, returned in the result */
} pm_request;

typedef struct {
  uint64_t tag;
  int status;      /* PM_OK converged; PM_E_MAXIT stopped at the iteration cap; other codes on failure */
  int iterations;
  double residual, initial_residual;
  int n_dofs;
  int worker;
  int cache_hit;   /* 1 if the worker's problem for this set-up was reused */
  double queue_ms; /* submit -> start on a worker (host clock) */
  double setup_ms; /* set-up and problem creation, 0 on a cache hit */
  double run_ms;   /* assembly + solve + solution copy */
  double latency_ms; /* submit -> completion */
} pm_result;

int pm_server_create(int device, int n_workers, const char* params_cd, const char* params_stokes,
                     size_t hbm_cap_bytes, pm_server** out);
void pm_server_destroy(pm_server* s);
/* enqueue (non-blocking, first in first out) */
int pm_server_submit(pm_server* s, const pm_request* req);
/* completed results in completion order; blocks until at least min_results
 * are available (0 = do not block) and returns at most max_results */
int pm_server_poll(pm_server* s, pm_result* out, int max_results, int min_results, int* n_out);
/* blocks until every submitted request has completed */
int pm_server_drain(pm_server* s);
/* bytes held by cached problems (estimate), requests served, evictions */
int pm_server_stats(pm_server* s, size_t* cached_bytes, uint64_t* served, uint64_t* evictions);

#ifdef __cplusplus
}
#endif
#endif /* PMGPU_H */
