// ref_stokes.C - driver of the oracle's build of the reference (test
// infrastructure only; compiled with -D__3D__ against oracle/_ref/libparmoon_3d.a
// by oracle/ref/build_ref.py).
//
// Runs the reference's own NavierStokes<3> class as a Stokes problem
// (problem_type 3, NSTYPE 4, LAPLACETYPE 0, Galerkin) with P2/P1 Taylor-Hood
// elements on Default_UnitCube_Tetra with the solution of the reference's
// example -3 (include/Examples/NSE_3D/test_u_2_p_1.h: u = (y^2, xz, -y^2),
// p = x + y + z - 3/2, viscosity 1) and the Stokes body force
// f = -Laplace(u) + grad(p) (the example's own coefficients add the convective
// term of the Navier-Stokes equations), and dumps, per multigrid level (finest
// first, as NavierStokes keeps its systems): the cell vertices in collection
// order, the GlobalNumbers of the velocity and the pressure space, their
// ActiveBounds, the combined matrix [A11 A12 A13 B1T; ...; B1 B2 B3 C] as CSR
// (BlockFEMatrix::get_combined_matrix) and the right-hand side; with SOLVER
// direct, the direct solve's solution of the finest level.
//
// usage: ref_stokes OUTDIR N_REFINE N_LEVELS SOLVER [MODE RE EPS MAXIT FORM]
//   SOLVER direct (one level) | none (assemble only; N_LEVELS levels) |
//          mg (FGMRES with a nodal Vanka multigrid, N_LEVELS levels)
//   MODE stokes (default) | nse: the Navier-Stokes problem (problem_type 5,
//   convective form) with the reference's own example -3 (whose coefficients
//   hold the convective term) at Reynolds number RE, run as the reference's
//   nse3d_solvers_test runs it (assemble_linear_terms, stop_it(0), then
//   solve / assemble_nonlinear_term / stop_it(k) until stop_it says so, with
//   nonlinloop_epsilon EPS and nonlinloop_maxit MAXIT, and the nonlinear form
//   FORM, nse_nonlinear_form: convective (default) or skew_symmetric); dumps the residuals
//   of every nonlinear step, the linear iterations of every solve, the final
//   solution and get_errors(). With SOLVER none, MODE nse sets the finest
//   solution to u_b[i] = sin(0.7 i + 1.3 b + 0.1) (velocity component b, DOF
//   i; pressure 0) and calls assemble_nonlinear_term once, then dumps every
//   level as above plus every level's (restricted) velocity.
#include <BaseCell.h>
#include <Database.h>
#include <Domain.h>
#include <Example_NSE3D.h>
#include <FEDatabase3D.h>
#include <LocalAssembling.h>
#include <LoopInfo.h>
#include <Multigrid.h>
#include <NavierStokes.h>
#include <Solver.h>
#include <Vertex.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

namespace {

template <class T>
void dump(const std::string& path, const T* p, size_t n) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(p), std::streamsize(n * sizeof(T)));
}

// u = (y^2, xz, -y^2), p = x + y + z - 3/2: value, d/dx, d/dy, d/dz, Laplacian
void exact_u1(double, double y, double, double* v) { v[0] = y * y; v[1] = 0; v[2] = 2 * y; v[3] = 0; v[4] = 2; }
void exact_u2(double x, double, double z, double* v) { v[0] = x * z; v[1] = z; v[2] = 0; v[3] = x; v[4] = 0; }
void exact_u3(double, double y, double, double* v) { v[0] = -y * y; v[1] = 0; v[2] = -2 * y; v[3] = 0; v[4] = -2; }
void exact_p(double x, double y, double z, double* v) { v[0] = x + y + z - 1.5; v[1] = v[2] = v[3] = 1; v[4] = 0; }
void bc_velocity(double, double, double, BoundCond& c) { c = DIRICHLET; }
void bc_pressure(double, double, double, BoundCond& c) { c = NEUMANN; }
void bv_u1(double, double y, double, double& v) { v = y * y; }
void bv_u2(double x, double, double z, double& v) { v = x * z; }
void bv_u3(double, double y, double, double& v) { v = -y * y; }
void bv_zero(double, double, double, double& v) { v = 0; }
void stokes_coeffs(int n, double* x, double* y, double* z, double**, double** c) {
  for (int i = 0; i < n; ++i) {
    double u1[5], u2[5], u3[5], p[5];
    exact_u1(x[i], y[i], z[i], u1);
    exact_u2(x[i], y[i], z[i], u2);
    exact_u3(x[i], y[i], z[i], u3);
    exact_p(x[i], y[i], z[i], p);
    c[i][0] = 1.0;
    c[i][1] = -u1[4] + p[1];
    c[i][2] = -u2[4] + p[2];
    c[i][3] = -u3[4] + p[3];
    c[i][4] = 0;
    c[i][5] = 0;
  }
}
Example_NSE3D make_example() {
  return Example_NSE3D({exact_u1, exact_u2, exact_u3, exact_p}, {bc_velocity, bc_velocity, bc_velocity, bc_pressure},
                       {bv_u1, bv_u2, bv_u3, bv_zero}, stokes_coeffs);
}

// access to the systems of every level
struct RefStokes : public NavierStokes<3> {
  RefStokes(const TDomain& dom, const ParameterDatabase& db, const Example_NSE3D& ex)
      : NavierStokes<3>(dom, db, ex) {}
  using NavierStokes<3>::systems;
  using NavierStokes<3>::solver;
};

void dump_space(const std::string& pre, const TFESpace3D& space, std::FILE* meta, const char* name) {
  const TCollection* coll = space.GetCollection();
  const int n_cells = coll->GetN_Cells();
  const int* begin = space.GetBeginIndex();
  const int* numbers = space.GetGlobalNumbers();
  std::vector<int> dofmap;
  for (int c = 0; c < n_cells; ++c)
    for (int k = begin[c]; k < begin[c + 1]; ++k) dofmap.push_back(numbers[k]);
  dump(pre + "_" + name + "_dofmap.i32", dofmap.data(), dofmap.size());
  std::fprintf(meta, " %s_nloc %d %s_n_dofs %d %s_active %d", name, begin[1] - begin[0], name,
               space.GetN_DegreesOfFreedom(), name, space.GetActiveBound());
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s OUTDIR N_REFINE N_LEVELS SOLVER [MODE RE EPS MAXIT]\n", argv[0]);
    return 2;
  }
  const std::string out = argv[1];
  const size_t n_refine = size_t(std::atoi(argv[2]));
  const size_t n_levels = size_t(std::atoi(argv[3]));
  const std::string solver = argv[4];
  const bool nse_mode = argc > 5 && std::string(argv[5]) == "nse";
  const double reynolds = argc > 6 ? std::atof(argv[6]) : 1.0;
  const double nl_eps = argc > 7 ? std::atof(argv[7]) : 1e-10;
  const size_t nl_maxit = argc > 8 ? size_t(std::atoi(argv[8])) : 10;
  const std::string nl_form = argc > 9 ? argv[9] : "convective";

  Output::setVerbosity(1);
  TDatabase database;
  TFEDatabase3D fe_database;
  ParameterDatabase db = ParameterDatabase::parmoon_default_database();
  db.merge(Solver<>::default_solver_database());
  db.merge(Multigrid::default_multigrid_database());
  db.merge(ParameterDatabase::default_nonlinit_database());
  db.merge(LocalAssembling3D::default_local_assembling_database());
  db.merge(Example_NSE3D::default_example_database());
  db["problem_type"].set<size_t>(nse_mode ? 5 : 3);
  db["example"] = -3;
  if (nse_mode) {
    db["nse_nonlinear_form"] = nl_form;
    db["reynolds_number"] = reynolds;
    db["nonlinloop_epsilon"] = nl_eps;
    db["nonlinloop_maxit"] = nl_maxit;
  }
  db["space_discretization_type"] = "galerkin";
  db.add("boundary_file", "Default_UnitCube", "");
  db.add("geo_file", "Default_UnitCube_Tetra", "");
  db.add("refinement_n_initial_steps", n_refine, "");
  if (solver == "direct") {
    db["solver_type"] = "direct";
  } else {
    // a multigrid solver makes NavierStokes keep a system per level
    db["solver_type"] = "iterative";
    db["iterative_solver_type"] = "fgmres";
    db["preconditioner"] = "multigrid";
    db["multigrid_n_levels"] = n_levels;
    db["multigrid_smoother"] = "nodal_vanka";
    db["multigrid_smoother_coarse"] = "direct_solve";
    if (solver == "mg") {
      db["gmres_restart"] = size_t(20);
      db["max_n_iterations"] = size_t(100);
      db["residual_tolerance"] = 1e-12;
      db["residual_reduction"] = 0.0;
      db["multigrid_cycle_type"] = "V";
      db["multigrid_n_pre_smooth"] = size_t(1);
      db["multigrid_n_post_smooth"] = size_t(1);
      db["multigrid_vanka_damp_factor"] = 1.0;
      db["multigrid_correction_damp_factor"] = 1.0;
    }
  }
  TDatabase::ParamDB->VELOCITY_SPACE = 2;
  TDatabase::ParamDB->PRESSURE_SPACE = -4711;
  TDatabase::ParamDB->NSTYPE = 4;
  TDatabase::ParamDB->LAPLACETYPE = 0;
  TDatabase::ParamDB->FLOW_PROBLEM_TYPE = nse_mode ? 5 : 3;
  TDatabase::ParamDB->SC_NONLIN_ITE_TYPE_SADDLE = 0;
  check_parameters_consistency_NSE(db);

  TDomain domain(db);
  domain.refine_and_get_hierarchy_of_collections(db);
  RefStokes nse(domain, db, nse_mode ? Example_NSE3D(db) : make_example());
  nse.assemble_linear_terms();

  if (nse_mode && solver != "none") {
    // the nonlinear loop of the reference's nse3d_solvers_test
    std::FILE* meta = std::fopen((out + "/meta.txt").c_str(), "w");
    std::fprintf(meta, "n_refine %zu\nlevels %zu\n", n_refine, nse.systems.size());
    nse.stop_it(0);
    std::fprintf(meta, "res 0 %.17g %.17g %.17g\n", nse.get_impuls_residual(), nse.get_mass_residual(),
                 nse.get_full_residual());
    for (unsigned k = 1;; ++k) {
      nse.solve();
      const unsigned lin = solver == "mg" ? nse.solver.get_solver_loop_info().get_n_previous_iterations() : 0;
      nse.assemble_nonlinear_term();
      const bool stop = nse.stop_it(k);
      std::fprintf(meta, "res %u %.17g %.17g %.17g\nlin %u %u\n", k, nse.get_impuls_residual(),
                   nse.get_mass_residual(), nse.get_full_residual(), k, lin);
      if (stop) break;
    }
    nse.output();
    const auto e = nse.get_errors();
    std::fprintf(meta, "errors");
    for (double v : e) std::fprintf(meta, " %.17g", v);
    std::fprintf(meta, "\n");
    const auto& s = nse.systems.front();
    dump(out + "/solution.f64", s.solution.get_entries(), s.solution.length());
    std::fclose(meta);
    return 0;
  }
  if (nse_mode) {
    // a fixed finest velocity, restricted to every level by the nonlinear
    // assembly
    auto& f = nse.systems.front().solution;
    for (int b = 0; b < 3; ++b) {
      double* u = f.block(b);
      for (size_t i = 0; i < f.length(b); ++i) u[i] = std::sin(0.7 * double(i) + 1.3 * b + 0.1);
    }
    nse.assemble_nonlinear_term();
    int level = 0;
    for (auto& s : nse.systems) {
      dump(out + "/L" + std::to_string(level) + "_velocity.f64", s.solution.get_entries(),
           3 * s.solution.length(0));
      ++level;
    }
  }

  std::FILE* meta = std::fopen((out + "/meta.txt").c_str(), "w");
  std::fprintf(meta, "n_refine %zu\nlevels %zu\n", n_refine, nse.systems.size());
  int level = 0;
  for (auto& s : nse.systems) {  // finest first
    const std::string pre = out + "/L" + std::to_string(level);
    const TCollection* coll = s.velocity_space->GetCollection();
    const int n_cells = coll->GetN_Cells();
    std::vector<double> verts;
    for (int c = 0; c < n_cells; ++c) {
      const TBaseCell* cell = coll->GetCell(c);
      for (int v = 0; v < cell->GetN_Vertices(); ++v) {
        double x, y, z;
        cell->GetVertex(v)->GetCoords(x, y, z);
        verts.push_back(x);
        verts.push_back(y);
        verts.push_back(z);
      }
    }
    dump(pre + "_verts.f64", verts.data(), verts.size());
    std::fprintf(meta, "L%d cells %d", level, n_cells);
    dump_space(pre, *s.velocity_space, meta, "u");
    dump_space(pre, *s.pressure_space, meta, "p");
    auto A = s.matrix.get_combined_matrix();
    const int nr = A->GetN_Rows();
    const int nnz = A->GetN_Entries();
    dump(pre + "_rows.i32", A->GetRowPtr(), size_t(nr) + 1);
    dump(pre + "_cols.i32", A->GetKCol(), size_t(nnz));
    dump(pre + "_vals.f64", A->GetEntries(), size_t(nnz));
    dump(pre + "_rhs.f64", s.rhs.get_entries(), s.rhs.length());
    std::fprintf(meta, " rows %d nnz %d\n", nr, nnz);
    ++level;
  }
  if (solver == "direct") {
    nse.solve();
    const auto& s = nse.systems.front();
    dump(out + "/solution.f64", s.solution.get_entries(), s.solution.length());
  }
  std::fclose(meta);
  return 0;
}
