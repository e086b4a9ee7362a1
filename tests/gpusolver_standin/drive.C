// Drives integration/GpuSolver.C the way ParMooN's ConvectionDiffusion<d>
// drives Solver: the multigrid hierarchy (coarsest first), update_matrix,
// solve from a zero iterate with the Dirichlet values copied from the rhs.
// Inputs come from a directory of raw arrays written by
// tests/test_gpu_integration.py (the reference's own level matrices and
// right-hand side from tests/golden/). Test infrastructure.
//
// usage: drive DIR N_LEVELS GEOMETRY N_REFINE ORDER RESTART REDUCTION
#include <cstdio>
#include <stdexcept>
#include <cstdlib>
#include <fstream>
#include <list>
#include <memory>
#include <string>
#include <vector>

#include "BlockFEMatrix.h"
#include "BlockVector.h"
#include "GpuSolver.h"
#include "ParameterDatabase.h"

template <class T>
std::vector<T> load(const std::string& path) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  const size_t n = size_t(f.tellg()) / sizeof(T);
  f.seekg(0);
  std::vector<T> v(n);
  f.read(reinterpret_cast<char*>(v.data()), std::streamsize(n * sizeof(T)));
  return v;
}

int main(int argc, char** argv) {
  if (argc < 8) return 2;
  const std::string dir = argv[1];
  const int n_levels = std::atoi(argv[2]), geometry = std::atoi(argv[3]), n_refine = std::atoi(argv[4]),
            order = std::atoi(argv[5]);
  ParameterDatabase db("Solver parameters");
  db.set("solver_type", "iterative");
  db.set("iterative_solver_type", "fgmres");
  db.set("preconditioner", "multigrid");
  db.set("residual_tolerance", "0");
  db.set("residual_reduction", argv[7]);
  db.set("max_n_iterations", "1000");
  db.set("gmres_restart", argv[6]);
  db.set("multigrid_n_levels", std::to_string(n_levels));
  db.set("multigrid_cycle_type", "V");
  db.set("multigrid_smoother", "jacobi");
  db.set("multigrid_smoother_coarse", "direct_solve");
  db.set("jacobi_damp", "0.8");
  db.set("multigrid_n_pre_smooth", "2");
  db.set("multigrid_n_post_smooth", "2");
  std::vector<std::unique_ptr<BlockFEMatrix>> mats;
  std::list<const BlockFEMatrix*> hierarchy;
  for (int l = 0; l < n_levels; ++l) {
    const std::string p = dir + "/L" + std::to_string(l) + "_";
    auto rows = load<int>(p + "rows.i32");
    const int n = int(rows.size()) - 1;
    const int active = load<int>(p + "active.i32")[0];
    auto A = std::make_shared<TMatrix>(n, n, rows, load<int>(p + "cols.i32"), load<double>(p + "vals.f64"));
    mats.emplace_back(new BlockFEMatrix(A, active));
    hierarchy.push_back(mats.back().get());
  }
  try {
    GpuSolver solver(db);
    solver.set_multigrid_levels(hierarchy, geometry, 1, n_refine, order);
    auto rhs_v = load<double>(dir + "/rhs.f64");
    BlockVector rhs(rhs_v.size()), sol(rhs_v.size());
    const int active = load<int>(dir + "/L" + std::to_string(n_levels - 1) + "_active.i32")[0];
    for (size_t i = 0; i < rhs_v.size(); ++i) rhs.get_entries()[i] = rhs_v[i];
    for (size_t i = size_t(active); i < rhs_v.size(); ++i) sol.get_entries()[i] = rhs_v[i];
    solver.update_matrix(*mats.back());
    solver.solve(rhs, sol);
    std::ofstream(dir + "/solution.f64", std::ios::binary)
        .write(reinterpret_cast<const char*>(sol.get_entries()), std::streamsize(sol.length() * sizeof(double)));
    const LoopInfo& info = solver.get_solver_loop_info();
    std::printf("iterations %u initial %.17g final %.17g\n", info.get_n_previous_iterations(),
                info.get_initial_residual(), info.get_previous_residual());
    // a failure comes back as the reference's exception type
    BlockVector wrong(3);
    try {
      solver.solve(rhs, wrong);
      std::printf("no exception\n");
      return 1;
    } catch (const std::runtime_error& e) {
      std::printf("runtime_error: %s\n", e.what());
    }
  } catch (const std::exception& e) {
    std::printf("failed: %s\n", e.what());
    return 1;
  }
  return 0;
}
