// Multigrid (V/W/F cycles, damped-Jacobi / direct coarse) and Krylov solvers
// (FGMRES, CG, BiCGStab, Jacobi iteration) on device vectors, driven by
// ParameterDatabase keys.
#pragma once
#include <map>
#include <string>
#include <vector>

#include "pm_linalg.cuh"
#include "pm_stokes.h"

struct pm_matrix {
  pm_ctx* ctx = nullptr;
  pm::DevCsr csr;
  bool owned_by_problem = false;
};

namespace pm {

// "key: value" parameter text (ParameterDatabase::read semantics for the keys
// this library consumes, src/General/ParameterDatabase.C:1078)
struct Params {
  std::map<std::string, std::string> kv;
  static Params parse(const char* text);
  bool has(const std::string& k) const { return kv.count(k) != 0; }
  std::string str(const std::string& k, const std::string& def) const;
  double num(const std::string& k, double def) const;
  long integer(const std::string& k, long def) const;
};

enum Smoother {
  SM_JACOBI = 0, SM_DIRECT = 1, SM_CELL_VANKA = 2, SM_CELL_VANKA_JACOBI = 3, SM_NONE = 4,
  SM_NODAL_VANKA = 5, SM_NODAL_VANKA_JACOBI = 6,
  SM_SOR = 7, SM_SSOR = 8  // SORSmoother (src/Multigrid/SORSmoother.C), forward / forward + backward
};
enum Dir { DIR_DUMMY = 0, DIR_DOWN = 1, DIR_UP = 2, DIR_END = 3 };

struct MGLevel {
  pm_matrix* A = nullptr;  // level matrix (not owned)
  DevCsr P;                // prolongation to the next finer level (fine rows)
  DevCsr R;                // restriction from the next finer level (this level's rows)
  DBuf<double> rhs, sol, alt, defect;
  DBuf<float> rhs32, sol32, alt32, defect32;
  double* cur = nullptr;   // current iterate (sol or alt)
  double* oth = nullptr;
  float* cur32 = nullptr;
  float* oth32 = nullptr;
  int smoother = SM_JACOBI;
  DenseInverse coarse;
  DBuf<double> coarse_rhs64, coarse_sol64;
  SorColours sor;  // the level's multicolour SOR order
  // saddle point levels: the projected combined matrix (Vanka, direct solve)
  // and the cell Vanka data; owned by the problem
  ProjectedMatrix* proj = nullptr;
  DevVanka* vanka = nullptr;
  DevNodalVanka* nodal = nullptr;
};

// CycleControl (src/Multigrid/CycleControl.C:17-110)
std::vector<int> cycle_control(const std::string& type, int n_levels);

struct Multigrid {
  std::vector<MGLevel> levels;  // 0 = coarsest
  std::vector<int> control;
  int n_pre = 1, n_post = 1;
  double jacobi_damp = 1.0, correction_damp = 1.0, coarse_residual = 0.1, vanka_damp = 1.0, sor_omega = 1.5;
  int coarse_max_it = 10;
  int smoother = SM_JACOBI, smoother_coarse = SM_DIRECT;
  std::string cycle_type = "V";
  bool mixed = false;       // the precision the cycle runs in now
  bool mixed_cfg = false;   // the precision the database asked for
  // mixed form: the coarse direct solve with the FP64 inverse (FP32 vectors,
  // FP64 products and sums) instead of an FP32 inverse (gpu_mixed_coarse)
  bool coarse64 = false;
  bool fp64_smoothers = false;  // FP64 Vanka factors exist for the current matrices
  bool ready = false;

  void configure(const Params& p);
  void update(pm_ctx* c);                                  // Multigrid::update
  // queue the coarse direct solver's factorisation (FP32 in the mixed form,
  // else FP64) on the context's side stream as soon as the coarsest matrix is
  // assembled (a direct coarse solve on a plain system matrix); update()
  // completes it
  void start_coarse(pm_ctx* c);
  // Iteration_multigrid::apply; rhs_nonactive_zero: the caller guarantees
  // exact zeros in the non-active entries of rhs (FGMRES basis vectors whose
  // initial residual had them), so the finest iterate starts at exact zero
  void apply(pm_ctx* c, const double* rhs, double* sol, bool rhs_nonactive_zero = false);
  // pieces of one cycle (Multigrid::cycle_step)
  void smooth(pm_ctx* c, int l);
  // the first smoothing step from an iterate that is exactly zero: a damped
  // Jacobi sweep reduces to x = w (b / d) with the sweep's bits (A*0 sums to
  // +0); other smoothers sweep as usual
  void smooth_from_zero(pm_ctx* c, int l);
  void defect(pm_ctx* c, int l);
  void restrict_to(pm_ctx* c, int l);  // from l to l-1
  void prolongate_from(pm_ctx* c, int l);  // from l to l+1
  void coarse_solve(pm_ctx* c);
  // switch the cycle between FP32 and FP64 (FGMRES is flexible, so the
  // preconditioner may change between iterations); FP64 Vanka factors are
  // computed on the first switch after an update
  void set_mixed(pm_ctx* c, bool on);
  // iterative coarsest level (Multigrid::cycle_step): at most coarse_max_it
  // sweeps, each followed by the defect, stopping once its norm is at or below
  // coarse_residual; the test runs on the device (a flag that turns the
  // remaining sweeps into no-ops), so the cycle needs no host round trip
  void coarse_iterate(pm_ctx* c);
  DBuf<int> coarse_flag;
  DBuf<double> coarse_part;
};

}  // namespace pm

struct pm_solver {
  pm_ctx* ctx = nullptr;
  pm::Params params;
  std::string solver_type = "iterative";
  std::string method = "fgmres";
  std::string prec = "no_preconditioner";
  double tol = 1e-8, reduction = 0.0, divergence = 1e10, stagnation = 1e10, damping = 1.0;
  long max_it = 100, min_it = 0, restart = 20;
  bool mixed = false;
  // Arnoldi orthogonalisation: "mgs" (the reference's modified Gram-Schmidt),
  // "cgs2" (classical Gram-Schmidt, two passes, batched; FP64 as well) or
  // "cgs2_cond" (the second pass only when the first lost more than a factor
  // 1/sqrt(2) of the norm, the DGKS criterion, decided on the device)
  std::string gram_schmidt = "mgs";
  // mixed form: switch the multigrid to FP64 for the rest of a solve when
  // the FP64 residual has fallen by less than half over 10 iterations
  bool mixed_fallback = true;
  pm_matrix* A = nullptr;
  pm::Multigrid mg;
  bool use_mg = false;
  pm::DenseInverse direct;
  bool direct_ready = false;
  // "sor" / "ssor" preconditioner (Iteration_sor, src/Solver/Iteration_sor.C)
  pm::SorColours sor;
  double sor_omega = 1.5;
  // Krylov work space
  pm::DBuf<double> work;  // vectors
  size_t work_n = 0;
  pm::DBuf<double> gm;    // FGMRES H, s, cs, sn, y
  pm::DBuf<int> flags;
  // one captured CUDA graph per Arnoldi index i (preconditioner, SpMV,
  // Gram-Schmidt, Givens rotation, residual read-back); rebuilt whenever the
  // buffers they reference are reallocated
  std::vector<cudaGraphExec_t> arnoldi_graphs;
  std::vector<uint64_t> arnoldi_launches;  // kernels inside each graph
  bool use_graphs = true;
  size_t graphs_signature = 0;  // addresses the captured graphs were built with
  size_t layout_signature() const;
  void drop_graphs();
  ~pm_solver();
  // loop information of the last solve
  int last_it = 0;
  double last_res = 0.0, init_res = 0.0, prev_res = 0.0;
  std::vector<double> history;
  // host scalars
  void ensure_work(size_t n_vectors, int n);
  bool converged(double r, unsigned it);
  void solve(const double* rhs, double* sol);
  void precondition(const double* z, double* r, bool z_nonactive_zero = false);
  void fgmres(const double* rhs, double* sol);
  void cg(const double* rhs, double* sol);
  void bicgstab(const double* rhs, double* sol);
  void jacobi_iter(const double* rhs, double* sol);
  void sor_iter(const double* rhs, double* sol, bool symmetric);
  void richardson(const double* rhs, double* sol);
  void cgs(const double* rhs, double* sol);
  void left_gmres(const double* rhs, double* sol);
};
