// example_cd.C - a ParMooN main program whose solve runs on the GPU through
// GpuSolver (the pattern of 2DPrograms/CD2D_ParMooN.C and
// 3DPrograms/CD3D_ParMooN.C with the solver swapped). Compiled with -D__2D__
// or -D__3D__ in a ParMooN tree and linked with libpmgpu.so.
//
// The reference's ConvectionDiffusion<d> builds the mesh hierarchy, the FE
// spaces and the matrices of every level and assembles them; GpuSolver takes
// the level matrices (coarsest first, as Multigrid::initialize does) and
// solves the finest system.
#include <BaseCell.h>
#include <ConvectionDiffusion.h>
#include <Database.h>
#include <Domain.h>
#include <Multigrid.h>
#include <Solver.h>
#ifdef __2D__
#include <FEDatabase2D.h>
#else
#include <FEDatabase3D.h>
#endif

#include <list>

#include "GpuSolver.h"

#ifdef __2D__
constexpr int D = 2;
#else
constexpr int D = 3;
#endif

// gives GpuSolver the systems of all levels
struct CDLevels : public ConvectionDiffusion<D> {
  using ConvectionDiffusion<D>::ConvectionDiffusion;
  using ConvectionDiffusion<D>::systems;
};

int main(int, char** argv) {
  TDatabase database;
#ifdef __2D__
  TFEDatabase2D fe_database;
#else
  TFEDatabase3D fe_database;
#endif
  ParameterDatabase db = ParameterDatabase::parmoon_default_database();
  db.merge(Solver<>::default_solver_database());
  db.merge(Multigrid::default_multigrid_database());
  db.merge(CDLevels::Example_CD::default_example_database());
  db.read(argv[1]);  // geometry, refinement, example, solver and multigrid keys
  TDomain domain(db);
  domain.refine_and_get_hierarchy_of_collections(db);
  CDLevels cd(domain, db);
  cd.assemble();

  GpuSolver solver(db);
  if (solver.is_using_multigrid()) {
    std::list<const BlockFEMatrix*> levels;  // systems are kept finest first
    for (auto& s : cd.systems) levels.push_front(&s.matrix);
    const int geometry = D == 2 ? 0 : 1;  // UnitSquare / Default_UnitCube_Hexa
    solver.set_multigrid_levels(levels, geometry, 1, int(size_t(db["refinement_n_initial_steps"])),
                                TDatabase::ParamDB->ANSATZ_ORDER);
  } else {
    solver.update_matrix(cd.get_matrix());
  }
  solver.solve(cd.get_rhs(), cd.get_solution());
  cd.output();
  return 0;
}
