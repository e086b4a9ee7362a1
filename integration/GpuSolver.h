// GpuSolver.h - drop-in for ParMooN's Solver<BlockFEMatrix, BlockVector>
// (include/Solver/Solver.h:31-127) that runs the solve on one GPU through
// libpmgpu (include/pmgpu.h).
//
// A maintainer adds this file and GpuSolver.C to the ParMooN tree (for
// instance under src/Solver/) and links libpmgpu.so. The call sites keep the
// reference's names and meaning:
//   GpuSolver solver(db);                // Solver(const ParameterDatabase&)
//   solver.update_matrix(A);             // Solver::update_matrix (Solver.C:261)
//   solver.solve(rhs, sol);              // Solver::solve (Solver.C:415), starts from sol
//   solver.solve(A, rhs, sol);           // Solver::solve (Solver.C:493)
//   solver.get_solver_loop_info();       // LoopInfo of the last solve
// The database keys are the reference's (solver_type, iterative_solver_type,
// preconditioner, residual_tolerance, residual_reduction, gmres_restart,
// multigrid_*, ...); they travel as ParameterDatabase::write's text.
//
// Multigrid: the reference's Multigrid::initialize takes the level matrices
// coarsest to finest (src/Multigrid/Multigrid.C:106) and transfers between
// levels with GridTransfer on the FE spaces. The library applies the same
// transfer as a prolongation matrix, which its own set-up builds for the
// uniform unit square / unit cube meshes (pm_disc_create; its numbering is
// identical to TFESpace2D/3D::ConstructSpace's), so set_multigrid_levels
// takes the mesh description with the matrices.
//
// Failures are thrown as the reference throws them: ErrThrow ->
// std::runtime_error (include/General/MooNMD_Io.h:210).
#ifndef GPU_SOLVER_H
#define GPU_SOLVER_H

#include <list>
#include <string>
#include <vector>

#include <LoopInfo.h>

#include "pmgpu.h"

class BlockFEMatrix;
class BlockVector;
class ParameterDatabase;

class GpuSolver
{
  public:
    /// Solver(const ParameterDatabase&): the database is handed to the library
    /// as the text ParameterDatabase::write produces
    explicit GpuSolver(const ParameterDatabase& db, int device = 0);
    ~GpuSolver();
    GpuSolver(const GpuSolver&) = delete;
    GpuSolver& operator=(const GpuSolver&) = delete;

    /// Solver::update_matrix: copies the combined CSR matrix to the device
    void update_matrix(const BlockFEMatrix& matrix);
    /// Solver::solve(rhs, solution): solution is the initial iterate and the result
    void solve(const BlockVector& rhs, BlockVector& solution);
    /// Solver::solve(matrix, rhs, solution) = update_matrix + solve
    void solve(const BlockFEMatrix& matrix, const BlockVector& rhs, BlockVector& solution);

    bool is_using_multigrid() const { return using_multigrid; }
    /// Multigrid::initialize equivalent: level matrices coarsest to finest on
    /// the library's mesh hierarchy (geometry, root_n, n_refine as
    /// pm_disc_create takes them; 0 unit square, 1 unit cube of hexahedra).
    /// The finest matrix becomes the solver's operator.
    void set_multigrid_levels(const std::list<const BlockFEMatrix*>& matrices, int geometry,
                              int root_n, int n_refine, int element_order);

    const LoopInfo& get_solver_loop_info() const { return loop_info; }
    /// the database text the library received
    const std::string& get_parameters() const { return params; }

  private:
    pm_ctx* ctx = nullptr;
    pm_solver* solver = nullptr;
    std::vector<pm_matrix*> levels;  // multigrid levels (coarsest first) or the one operator
    pm_disc* disc = nullptr;
    std::string params;
    bool using_multigrid = false;
    LoopInfo loop_info;

    pm_matrix* upload(const BlockFEMatrix& matrix) const;
    void check(int status) const;
    void release_levels();
};

#endif
