// ref_cd.C - driver of the oracle's build of the reference (test
// infrastructure only; compiled with -D__2D__ or -D__3D__ against
// oracle/_ref/libparmoon_{2,3}d.a by oracle/ref/build_ref.py).
//
// Runs the reference's own ConvectionDiffusion<d> class on the unit square
// (UnitSquare, quadrilaterals) or the unit cube (Default_UnitCube_Hexa) for
//   -eps Laplace(u) + b.grad(u) = f,  u = 0 on the boundary,
//   f from u = prod_d sin(pi x_d)
// and dumps, per multigrid level (finest first, as ConvectionDiffusion keeps
// its systems): the cell vertices in collection order, GlobalNumbers,
// ActiveBound, the CSR arrays of the assembled matrix and the right-hand side;
// after the solve: iterations, initial and final residual, and the solution.
//
// usage: ref_cd OUTDIR N_REFINE ANSATZ_ORDER N_LEVELS EPS B1 B2 B3 QUAD_LINEAR
//               SOLVER RESTART REDUCTION
//   QUAD_LINEAR 1 sets INTERNAL_PROBLEM_LINEAR (quadrature degree 2 x the
//   element degree, e.g. Gauss3 for Q2), 0 keeps the default (3 x);
//   SOLVER fgmres_mg | direct | none (assemble only).
//   optional GEOMETRY (after EXAMPLE; 3D only): tetra for Default_UnitCube_Tetra
//   (P1 / P2 for ANSATZ_ORDER 1 / 2), hexa (default) for Default_UnitCube_Hexa.
//   optional EXAMPLE: the reference's own example of that number
//   (Example_CD2D/3D from the database, e.g. 0 = SineLaplace in 2D, whose
//   boundary part 1 is a Neumann boundary) instead of the sine problem above;
//   the errors of ConvectionDiffusion::output are dumped as well.
#include <BaseCell.h>
#include <ConvectionDiffusion.h>
#include <Vertex.h>
#include <Database.h>
#include <Domain.h>
#include <LoopInfo.h>
#include <Multigrid.h>
#include <Solver.h>
#ifdef __2D__
#include <Example_CD2D.h>
#include <FEDatabase2D.h>
#else
#include <Example_CD3D.h>
#include <FEDatabase3D.h>
#endif

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

namespace {

double g_eps = 1.0, g_b[3] = {0.0, 0.0, 0.0};
const double kPi = 3.14159265358979323846;

template <class T>
void dump(const std::string& path, const T* p, size_t n) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(p), std::streamsize(n * sizeof(T)));
}

#ifdef __2D__
constexpr int D = 2;
void exact(double x, double y, double* v) {
  const double sx = std::sin(kPi * x), sy = std::sin(kPi * y);
  v[0] = sx * sy;
  v[1] = kPi * std::cos(kPi * x) * sy;
  v[2] = kPi * sx * std::cos(kPi * y);
  v[3] = -2.0 * kPi * kPi * sx * sy;
}
void bound_cond(int, double, BoundCond& c) { c = DIRICHLET; }
void bound_value(int, double, double& v) { v = 0.0; }
void coeffs(int n, double* x, double* y, double**, double** c) {
  double v[4];
  for (int i = 0; i < n; ++i) {
    exact(x[i], y[i], v);
    c[i][0] = g_eps;
    c[i][1] = g_b[0];
    c[i][2] = g_b[1];
    c[i][3] = 0.0;
    c[i][4] = -g_eps * v[3] + g_b[0] * v[1] + g_b[1] * v[2];
  }
}
using Example = Example_CD2D;
Example make_example() { return Example({exact}, {bound_cond}, {bound_value}, coeffs); }
#else
constexpr int D = 3;
void exact(double x, double y, double z, double* v) {
  const double sx = std::sin(kPi * x), sy = std::sin(kPi * y), sz = std::sin(kPi * z);
  v[0] = sx * sy * sz;
  v[1] = kPi * std::cos(kPi * x) * sy * sz;
  v[2] = kPi * sx * std::cos(kPi * y) * sz;
  v[3] = kPi * sx * sy * std::cos(kPi * z);
  v[4] = -3.0 * kPi * kPi * sx * sy * sz;
}
void bound_cond(double, double, double, BoundCond& c) { c = DIRICHLET; }
void bound_value(double, double, double, double& v) { v = 0.0; }
void coeffs(int n, double* x, double* y, double* z, double**, double** c) {
  double v[5];
  for (int i = 0; i < n; ++i) {
    exact(x[i], y[i], z[i], v);
    c[i][0] = g_eps;
    c[i][1] = g_b[0];
    c[i][2] = g_b[1];
    c[i][3] = g_b[2];
    c[i][4] = 0.0;
    c[i][5] = -g_eps * v[4] + g_b[0] * v[1] + g_b[1] * v[2] + g_b[2] * v[3];
  }
}
using Example = Example_CD3D;
Example make_example() { return Example({exact}, {bound_cond}, {bound_value}, coeffs); }
#endif

// access to the systems of every level and to the solver
struct RefCD : public ConvectionDiffusion<D> {
  RefCD(const TDomain& dom, const ParameterDatabase& db, const Example& ex)
      : ConvectionDiffusion<D>(dom, db, ex) {}
  using ConvectionDiffusion<D>::systems;
  using ConvectionDiffusion<D>::solver;
};

}  // namespace

int main(int argc, char** argv) {
  if (argc < 13) {
    std::fprintf(stderr, "usage: %s OUTDIR N_REFINE ANSATZ_ORDER N_LEVELS EPS B1 B2 B3 QUAD_LINEAR SOLVER "
                         "RESTART REDUCTION\n", argv[0]);
    return 2;
  }
  const std::string out = argv[1];
  const size_t n_refine = size_t(std::atoi(argv[2]));
  const int order = std::atoi(argv[3]);
  const size_t n_levels = size_t(std::atoi(argv[4]));
  g_eps = std::atof(argv[5]);
  g_b[0] = std::atof(argv[6]);
  g_b[1] = std::atof(argv[7]);
  g_b[2] = std::atof(argv[8]);
  const int quad_linear = std::atoi(argv[9]);
  const std::string solver = argv[10];
  const int restart = std::atoi(argv[11]);
  const double reduction = std::atof(argv[12]);
  const int builtin_example = argc > 13 ? std::atoi(argv[13]) : -1;
  const std::string geometry = argc > 14 ? argv[14] : "hexa";

  Output::setVerbosity(1);
  TDatabase database;
#ifdef __2D__
  TFEDatabase2D fe_database;
#else
  TFEDatabase3D fe_database;
#endif
  ParameterDatabase db = ParameterDatabase::parmoon_default_database();
  db.merge(Solver<>::default_solver_database());
  db.merge(Multigrid::default_multigrid_database());
  db.merge(ParameterDatabase::default_output_database());
#ifdef __2D__
  db.merge(Example2D::default_example_database());
#else
  db.merge(Example3D::default_example_database());
#endif
  if (builtin_example >= 0) {
    db["example"] = builtin_example;
    db["output_compute_errors"] = true;
  }
  db["problem_type"] = 1;
#ifdef __2D__
  db.add("boundary_file", "Default_UnitSquare", "");
  db.add("geo_file", "UnitSquare", "");
#else
  db.add("boundary_file", "Default_UnitCube", "");
  db.add("geo_file", geometry == "tetra" ? "Default_UnitCube_Tetra" : "Default_UnitCube_Hexa", "");
#endif
  db.add("refinement_n_initial_steps", n_refine, "");
  if (solver == "direct" || solver == "none") {
    db["solver_type"] = "direct";
  } else {
    db["solver_type"] = "iterative";
    db["iterative_solver_type"] = "fgmres";
    db["preconditioner"] = "multigrid";
    db["gmres_restart"] = size_t(restart);
    db["max_n_iterations"] = size_t(1000);
    db["residual_tolerance"] = 0.0;
    db["residual_reduction"] = reduction;
    db["multigrid_n_levels"] = n_levels;
    db["multigrid_cycle_type"] = "V";
    db["multigrid_smoother"] = "jacobi";
    db["multigrid_smoother_coarse"] = "direct_solve";
    db["jacobi_damp"] = 0.8;
    db["multigrid_n_pre_smooth"] = size_t(2);
    db["multigrid_n_post_smooth"] = size_t(2);
    db["multigrid_correction_damp_factor"] = 1.0;
  }
  TDatabase::ParamDB->ANSATZ_ORDER = order;
  TDatabase::ParamDB->INTERNAL_PROBLEM_LINEAR = quad_linear;

  TDomain domain(db);
  domain.refine_and_get_hierarchy_of_collections(db);
  RefCD cd(domain, db, builtin_example >= 0 ? Example(db) : make_example());
  cd.assemble();

  std::FILE* meta = std::fopen((out + "/meta.txt").c_str(), "w");
  std::fprintf(meta, "dim %d\nn_refine %zu\norder %d\nlevels %zu\n", D, n_refine, order, cd.systems.size());
  int level = 0;
  for (auto& s : cd.systems) {  // finest first
    const auto& space = *s.fe_space;
    const TCollection* coll = space.GetCollection();
    const int n_cells = coll->GetN_Cells();
    const int* begin = space.GetBeginIndex();
    const int* numbers = space.GetGlobalNumbers();
    const int nloc = begin[1] - begin[0];
    std::vector<int> dofmap;
    std::vector<double> verts;
    for (int c = 0; c < n_cells; ++c) {
      if (begin[c + 1] - begin[c] != nloc) {
        std::fprintf(stderr, "cells with different local DOF counts\n");
        return 1;
      }
      for (int k = 0; k < nloc; ++k) dofmap.push_back(numbers[begin[c] + k]);
      const TBaseCell* cell = coll->GetCell(c);
      for (int v = 0; v < cell->GetN_Vertices(); ++v) {
        double x, y, z = 0.0;
#ifdef __2D__
        cell->GetVertex(v)->GetCoords(x, y);
#else
        cell->GetVertex(v)->GetCoords(x, y, z);
#endif
        verts.push_back(x);
        verts.push_back(y);
        if (D == 3) verts.push_back(z);
      }
    }
    auto A = s.matrix.get_blocks()[0];
    const int nr = A->GetN_Rows();
    const int nnz = A->GetN_Entries();
    const std::string pre = out + "/L" + std::to_string(level);
    dump(pre + "_dofmap.i32", dofmap.data(), dofmap.size());
    dump(pre + "_verts.f64", verts.data(), verts.size());
    dump(pre + "_rows.i32", A->GetRowPtr(), size_t(nr) + 1);
    dump(pre + "_cols.i32", A->GetKCol(), size_t(nnz));
    dump(pre + "_vals.f64", A->GetEntries(), size_t(nnz));
    dump(pre + "_rhs.f64", s.rhs.get_entries(), s.rhs.length());
    std::fprintf(meta, "L%d cells %d nloc %d n_dofs %d active %d nnz %d\n", level, n_cells, nloc,
                 space.GetN_DegreesOfFreedom(), space.GetActiveBound(), nnz);
    ++level;
  }
  if (solver != "none") {
    Chrono timer;
    cd.solve();
    const double t = timer.elapsed_time();
    const auto& s = cd.systems.front();
    dump(out + "/solution.f64", s.solution.get_entries(), s.solution.length());
    if (solver != "direct") {
      const LoopInfo& info = cd.solver.get_solver_loop_info();
      std::fprintf(meta, "iterations %u\ninitial_residual %.17g\nfinal_residual %.17g\n",
                   info.get_n_previous_iterations(), info.get_initial_residual(),
                   info.get_previous_residual());
    }
    std::fprintf(meta, "solve_seconds %.6f\n", t);
    if (builtin_example >= 0) {
      cd.output();
      std::fprintf(meta, "errors %.17g %.17g %.17g %.17g\n", cd.get_L2_error(), cd.get_H1_semi_error(),
                   cd.get_SD_error(), cd.get_L_inf_error());
    }
  }
  std::fclose(meta);
  return 0;
}
