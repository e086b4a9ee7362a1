// The device-resident convection-diffusion system behind the pm_problem handle:
// level matrices, assembly inputs, right-hand side, solution and solver.
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "pm_assemble.h"
#include "pm_solver.h"
#include "pm_stokes.h"

struct pm_problem {
  pm_ctx* ctx = nullptr;
  const pm_disc* disc = nullptr;
  int kind = 0;  // 0 convection-diffusion, 1 Stokes
  pm_cd_coeffs coeffs{};
  double nu = 1.0;  // Stokes viscosity
  int stokes_example = 0;  // 0: manufactured sine velocity; -3: polynomial (test_u_2_p_1)
  int problem_type = 3;    // Stokes kind: 3 Stokes, 5 Navier-Stokes (convective form)
  // Navier-Stokes: restricted velocities of the coarser levels, the P2
  // restriction matrices, scratch, the defect and its blocks' squared norms
  std::vector<pm::DBuf<double>> ulev;
  pm::DBuf<double> rq, cellval, defect, res2;
  std::string params_text;  // the creation parameters (nonlinloop_* keys)
  int qn = 3;
  std::vector<pm::DevStokesLevel> slev;
  pm::DevStokesTables stab;
  std::vector<std::unique_ptr<pm::ProjectedMatrix>> proj;
  std::vector<std::unique_ptr<pm::DevVanka>> vanka;
  std::vector<std::unique_ptr<pm::DevNodalVanka>> nodal;  // built when a nodal smoother is chosen
  std::vector<pm_matrix*> mats;
  std::vector<pm::DevAssemblyLevel> alev;
  pm::DevRefTables ref;
  pm::DBuf<double> K, F, rhs, sol, rhs_coarse;
  pm_solver* solver = nullptr;
  bool solver_ready = false;
  // error functional: reference tables of its quadrature rule, the finest
  // level's dofmap and the four results (set up by the first pm_problem_errors)
  int err_qn = 0;
  pm::DevRefTables err_ref;
  pm::DBuf<int> err_dofmap;
  pm::DBuf<double> err_out;
  ~pm_problem();
};
