// GpuSolver.C - see GpuSolver.h. Compiled inside a ParMooN tree
// (-D__2D__ or -D__3D__ and its include directories) and linked with
// libpmgpu.so.
#include "GpuSolver.h"

#include <sstream>
#include <stdexcept>

#include <BlockFEMatrix.h>
#include <BlockVector.h>
#include <Matrix.h>
#include <MooNMD_Io.h>
#include <ParameterDatabase.h>

namespace
{
// the value of `key` in ParameterDatabase::write's "key: value" lines
std::string value_of(const std::string& text, const std::string& key)
{
  std::istringstream in(text);
  std::string line;
  while(std::getline(in, line))
  {
    const auto sep = line.find(':');
    if(line.empty() || line[0] == '#' || sep == std::string::npos)
      continue;
    std::string k = line.substr(0, sep), v = line.substr(sep + 1);
    k.erase(0, k.find_first_not_of(" \t"));
    k.erase(k.find_last_not_of(" \t") + 1);
    v.erase(0, v.find_first_not_of(" \t"));
    v.erase(v.find_last_not_of(" \t\r") + 1);
    if(k == key)
      return v;
  }
  return "";
}
}

GpuSolver::GpuSolver(const ParameterDatabase& db, int device)
 : loop_info("gpu solver")
{
  std::ostringstream os;
  db.write(os, false);  // the reference's keys and values, unchanged
  params = os.str();
  using_multigrid = value_of(params, "solver_type") == "iterative"
                    && value_of(params, "preconditioner") == "multigrid";
  check(pm_ctx_create(device, &ctx));
  check(pm_solver_create(ctx, params.c_str(), &solver));
}

GpuSolver::~GpuSolver()
{
  pm_solver_destroy(solver);
  release_levels();
  if(disc)
    pm_disc_destroy(disc);
  pm_ctx_destroy(ctx);
}

void GpuSolver::check(int status) const
{
  if(status != PM_OK)
    ErrThrow("libpmgpu: ", pm_last_error(ctx));
}

void GpuSolver::release_levels()
{
  for(pm_matrix* m : levels)
    pm_matrix_destroy(m);
  levels.clear();
}

pm_matrix* GpuSolver::upload(const BlockFEMatrix& matrix) const
{
  // BlockFEMatrix::get_combined_matrix (src/Matrix/BlockFEMatrix.C:1168):
  // one CSR over all blocks, Dirichlet rows already unit rows
  std::shared_ptr<TMatrix> A = matrix.get_combined_matrix();
  const size_t nb = matrix.get_n_cell_rows();
  if(nb > 4)
    ErrThrow("GpuSolver: at most four block rows are supported, not ", nb);
  std::vector<int> lengths(nb), actives(nb);
  int n_active = 0;
  for(size_t b = 0; b < nb; ++b)
  {
    lengths[b] = matrix.get_row_space(b)->GetN_DegreesOfFreedom();
    actives[b] = matrix.get_row_space(b)->GetActiveBound();
    n_active += actives[b];
  }
  pm_matrix* m = nullptr;
  check(pm_matrix_create_csr(ctx, A->GetN_Rows(), A->GetN_Columns(), nb == 1 ? actives[0] : n_active,
                             A->GetRowPtr(), A->GetKCol(), A->GetEntries(), &m));
  if(nb > 1)
  {
    const int status = pm_matrix_set_blocks(m, int(nb), lengths.data(), actives.data());
    if(status != PM_OK)
    {
      pm_matrix_destroy(m);
      check(status);
    }
  }
  return m;
}

void GpuSolver::update_matrix(const BlockFEMatrix& matrix)
{
  if(using_multigrid && !levels.empty())
  {
    // the finest level gets the new values; the coarser ones stay
    std::shared_ptr<TMatrix> A = matrix.get_combined_matrix();
    check(pm_matrix_set_values(levels.back(), A->GetEntries()));
    check(pm_solver_update_matrix(solver, levels.back()));
    return;
  }
  if(using_multigrid)
    ErrThrow("GpuSolver: multigrid needs set_multigrid_levels before update_matrix");
  release_levels();
  levels.push_back(upload(matrix));
  check(pm_solver_update_matrix(solver, levels.back()));
}

void GpuSolver::set_multigrid_levels(const std::list<const BlockFEMatrix*>& matrices, int geometry,
                                     int root_n, int n_refine, int element_order)
{
  const int n_levels = int(matrices.size());
  if(disc)
    pm_disc_destroy(disc);
  disc = nullptr;
  check(pm_disc_create(geometry, root_n, n_refine, n_levels, 0, element_order, &disc));
  release_levels();
  int l = 0;
  for(const BlockFEMatrix* M : matrices)
  {
    levels.push_back(upload(*M));
    std::vector<int> rp, ci;
    std::vector<double> v;
    int rows = 0, cols = 0;
    if(l + 1 < n_levels)
    {
      int64_t nnz = 0;
      check(pm_disc_prolongation_info(disc, l, &rows, &cols, &nnz));
      rp.resize(size_t(rows) + 1);
      ci.resize(size_t(nnz));
      v.resize(size_t(nnz));
      check(pm_disc_prolongation(disc, l, rp.data(), ci.data(), v.data()));
    }
    check(pm_solver_set_multigrid_level(solver, l, n_levels, levels.back(), rows, cols,
                                        rp.empty() ? nullptr : rp.data(),
                                        ci.empty() ? nullptr : ci.data(),
                                        v.empty() ? nullptr : v.data()));
    ++l;
  }
  check(pm_solver_update_matrix(solver, levels.back()));
}

void GpuSolver::solve(const BlockVector& rhs, BlockVector& solution)
{
  if(levels.empty())
    ErrThrow("GpuSolver: no matrix; call update_matrix first");
  if(rhs.length() != solution.length())
    ErrThrow("GpuSolver: rhs and solution have different lengths");
  check(pm_solver_solve_host(solver, rhs.get_entries(), solution.get_entries(), int(rhs.length())));
  int iterations = 0;
  double residual = 0.0, initial = 0.0;
  check(pm_solver_last_info(solver, &iterations, &residual, &initial));
  loop_info.restart("gpu " + value_of(params, "iterative_solver_type"), initial);
  loop_info.finish(unsigned(iterations), residual);
}

void GpuSolver::solve(const BlockFEMatrix& matrix, const BlockVector& rhs, BlockVector& solution)
{
  update_matrix(matrix);
  solve(rhs, solution);
}
