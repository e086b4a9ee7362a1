// The device-resident convection-diffusion system behind the pm_problem handle:
// level matrices, assembly inputs, right-hand side, solution and solver.
#pragma once
#include <vector>

#include "pm_assemble.h"
#include "pm_solver.h"

struct pm_problem {
  pm_ctx* ctx = nullptr;
  const pm_disc* disc = nullptr;
  pm_cd_coeffs coeffs{};
  int qn = 3;
  std::vector<pm_matrix*> mats;
  std::vector<pm::DevAssemblyLevel> alev;
  pm::DevRefTables ref;
  pm::DBuf<double> K, F, rhs, sol, rhs_coarse;
  pm_solver* solver = nullptr;
  bool solver_ready = false;
  ~pm_problem();
};
