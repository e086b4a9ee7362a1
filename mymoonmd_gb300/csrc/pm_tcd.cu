// Time-dependent convection-diffusion on the device:
// TimeConvectionDiffusion<d> (src/System/TimeConvectionDiffusion.C:252-386)
// with the theta-free schemes of TimeDiscretization
// (src/TimeDiscRoutines/TimeDiscretizations.C:106-232, 341-380): backward
// Euler, Crank-Nicolson and BDF2 (its first step by backward Euler).
//
// The stiffness matrices of every level are the pm_problem's; they are turned
// into the system matrices tau' A + M in place before the solve and back
// after it, as the reference does. Mass matrices are assembled once, at the
// initial time. Element-wise arithmetic of the time discretisation uses
// separately rounded products and sums (__dmul_rn, __dadd_rn), the operations
// FEMatrix::scaleActive / addActive and BlockVector::scaleActive /
// addScaledActive perform.
#include <cmath>
#include <string>
#include <vector>

#include "pm_problem.h"

using namespace pm;

#define TCD_TRY try {
#define TCD_CATCH(c)                      \
  }                                       \
  catch (const pm::Error& e) {            \
    (c)->last_error = e.what();           \
    return e.code;                        \
  }                                       \
  catch (const std::exception& e) {       \
    (c)->last_error = e.what();           \
    return PM_E_INVALID;                  \
  }

struct pm_tcd {
  pm_problem* p = nullptr;  // stiffness matrices, rhs, solution, solver
  std::vector<DevCsr> mass;  // per level, the stiffness matrices' structure
  std::vector<int64_t> active_entries;  // entries of the active rows per level
  DBuf<double> old_rhs, rhs_td, sol_m1, sol_m2;
  pm_cd_coeffs base{};
  double ptime[20] = {};  // u = P0 + t P1 + t^2 P2: P1, P2 (P0 is base.poly)
  std::string scheme = "backward_euler";
  double tau = 0.05, t_start = 0.0, t_end = 1.0, t = 0.0;
  int step = 0;
  bool pre_stage_bdf = false;
  bool initial_done = false;
  double factor_used = 0.0;  // the factor the system matrices were built with
  const double bdf[3] = {4. / 3., -1. / 3., 2. / 3.};
  ~pm_tcd() { pm_problem_destroy(p); }
};

namespace {

__global__ void k_tcd_system(int64_t n, double* __restrict__ a, const double* __restrict__ m, double factor) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    a[i] = __dadd_rn(__dmul_rn(a[i], factor), m[i]);
}

__global__ void k_tcd_reset(int64_t n, double* __restrict__ a, const double* __restrict__ m, double inv) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    a[i] = __dmul_rn(__dsub_rn(a[i], m[i]), inv);
}

// y[i] = y[i] * s (+ a * x[i] when x) for the active entries i < n
__global__ void k_tcd_scale_add(int n, double* __restrict__ y, double s, const double* __restrict__ x, double a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = __dmul_rn(y[i], s);
  if (x) v = __dadd_rn(v, __dmul_rn(a, x[i]));
  y[i] = v;
}

int grid_of(pm_ctx* c, int64_t n) {
  return int(std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, int64_t(c->num_sms) * 8)));
}

// the exact solution's spatial polynomial at time t, and its time derivative
void time_polys(const pm_tcd* s, double t, double* q, double* r) {
  for (int i = 0; i < 10; ++i) {
    const double p0 = s->base.poly[i], p1 = s->ptime[i], p2 = s->ptime[10 + i];
    q[i] = p0 + t * p1 + (t * t) * p2;
    r[i] = p1 + (2.0 * t) * p2;
  }
}

pm_cd_coeffs coeffs_at(const pm_tcd* s, double t) {
  pm_cd_coeffs cf = s->base;
  if (cf.manufactured == 2) time_polys(s, t, cf.poly, cf.poly_src);
  return cf;
}

// assembly of the stiffness matrix and rhs of every level at time t
// (call_assembling_routine with TCDStiffRhs)
void assemble_stiffness(pm_tcd* s, double t) {
  pm_problem* p = s->p;
  pm_ctx* c = p->ctx;
  const Disc& D = *p->disc->d;
  const pm_cd_coeffs cf = coeffs_at(s, t);
  const int nl = int(D.levels.size());
  for (int l = 0; l < nl; ++l) {
    double* r = (l == nl - 1) ? p->rhs.p : p->rhs_coarse.p;
    assemble_cd_level(c, p->alev[l], D.dim(), D.elem, p->qn, cf, p->ref, p->mats[l]->csr, r, p->K.p, p->F.p);
  }
}

// TimeDiscretization factor of the stiffness part of the system matrix
double system_factor(const pm_tcd* s) {
  if (s->scheme == "backward_euler" || s->pre_stage_bdf) return s->tau;
  if (s->scheme == "bdf_two") return s->tau * s->bdf[2];
  return s->tau * 0.5;  // crank_nicolson
}

}  // namespace

/* Creates the time-dependent problem: the convection-diffusion problem of
 * pm_problem_create_cd plus the keys time_discretization (backward_euler |
 * crank_nicolson | bdf_two), time_step_length, time_start, time_end
 * (TimeDiscretization::default_TimeDiscretization_database). poly_time: the
 * coefficients P1, P2 (20 doubles, NULL = 0) of the exact solution
 * u = P0 + t P1 + t^2 P2 when cf->manufactured = 2 (P0 = cf->poly). */
extern "C" int pm_tcd_create(pm_ctx* c, const pm_disc* d, const pm_cd_coeffs* cf, const double* poly_time,
                             int quad_points, const char* params, pm_tcd** out) {
  if (!c || !d || !cf || !out) return PM_E_INVALID;
  TCD_TRY
  if (d->d->kind != KIND_CD) throw Error(PM_E_INVALID, "the discretisation is not a convection-diffusion set-up");
  auto* s = new pm_tcd();
  try {
    s->base = *cf;
    if (poly_time)
      for (int i = 0; i < 20; ++i) s->ptime[i] = poly_time[i];
    const Params prm = Params::parse(params ? params : "");
    s->scheme = prm.str("time_discretization", "backward_euler");
    if (s->scheme != "backward_euler" && s->scheme != "crank_nicolson" && s->scheme != "bdf_two")
      throw Error(PM_E_UNSUPPORTED, "time_discretization '" + s->scheme + "' is not implemented on the GPU");
    s->tau = prm.num("time_step_length", 0.05);
    s->t_start = prm.num("time_start", 0.0);
    s->t_end = prm.num("time_end", 1.0);
    s->t = s->t_start;
    // TimeDiscretization constructor: BDF2 starts with its pre-stage
    s->pre_stage_bdf = s->scheme == "bdf_two";
    int rc = pm_problem_create_cd(c, d, cf, quad_points, params, &s->p);
    if (rc != PM_OK) throw Error(rc, c->last_error);
    const Disc& D = *d->d;
    const int nl = int(D.levels.size());
    s->mass.resize(nl);
    s->active_entries.resize(nl);
    for (int l = 0; l < nl; ++l) {
      const DiscLevel& L = D.levels[l];
      s->mass[l].upload(c, L.sys.n_rows, L.sys.n_cols, L.space.n_active, L.sys.row_ptr.data(), L.sys.cols.data(),
                        nullptr);
      s->mass[l].mask = s->p->mats[l]->csr.mask;
      s->active_entries[l] = L.sys.row_ptr[size_t(L.space.n_active)];
    }
    const int n = D.levels.back().sys.n_rows;
    s->old_rhs.alloc(n);
    s->rhs_td.alloc(n);
    s->sol_m1.alloc(n);
    s->sol_m2.alloc(n);
  } catch (...) {
    delete s;
    throw;
  }
  *out = s;
  return PM_OK;
  TCD_CATCH(c)
}

extern "C" void pm_tcd_destroy(pm_tcd* s) { delete s; }

/* TimeConvectionDiffusion::assemble_initial_time (:252-292) at time_start:
 * stiffness and mass matrices of every level and the rhs; the solution is the
 * initial condition (the exact solution's nodal values with manufactured = 2,
 * else zero), solution_m1 = solution_m2 = solution, old_rhs = rhs. */
extern "C" int pm_tcd_assemble_initial_time(pm_tcd* s) {
  if (!s) return PM_E_INVALID;
  pm_ctx* c = s->p->ctx;
  TCD_TRY
  pm_problem* p = s->p;
  const Disc& D = *p->disc->d;
  s->t = s->t_start;
  s->step = 0;
  s->pre_stage_bdf = s->scheme == "bdf_two";
  assemble_stiffness(s, s->t);
  // mass matrices: the c u v term of the same element kernels (eps = 0, b = 0,
  // c = 1, f = 0); their non-active rows are never used
  pm_cd_coeffs mc{};
  mc.c = 1.0;
  const int nl = int(D.levels.size());
  for (int l = 0; l < nl; ++l)
    assemble_cd_level(c, p->alev[l], D.dim(), D.elem, p->qn, mc, p->ref, s->mass[l], p->rhs_coarse.p, p->K.p,
                      p->F.p);
  // initial condition: the interpolant of the exact solution at time_start
  const DiscLevel& top = D.levels.back();
  const int n = top.sys.n_rows;
  std::vector<double> u0(static_cast<size_t>(n), 0.0);
  if (s->base.manufactured == 2) {
    double q[10], r[10];
    time_polys(s, s->t, q, r);
    const int dim = D.dim();
    const int64_t S = D.h.scale;
    const bool pow2 = (S & (S - 1)) == 0;
    for (int i = 0; i < n; ++i) {
      double x[3] = {0.0, 0.0, 0.0};
      for (int k = 0; k < dim; ++k) {
        const double v = double(top.space.node[size_t(i) * dim + k]);
        x[k] = pow2 ? v * (1.0 / double(S)) : v / double(S);
      }
      u0[size_t(i)] = poly_value_host(q, x);
    }
  }
  PM_CUDA(cudaMemcpyAsync(p->sol.p, u0.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));  // u0 is a host temporary
  vcopy(c, n, p->rhs.p, s->old_rhs.p);
  vcopy(c, n, p->sol.p, s->sol_m1.p);
  vcopy(c, n, s->sol_m1.p, s->sol_m2.p);
  p->solver_ready = false;
  s->initial_done = true;
  return PM_OK;
  TCD_CATCH(c)
}

/* The time loop's bookkeeping (test/tcd3d_solvers_test.c++:78-86):
 * current_step_++, set_time_disc_parameters (BDF2 leaves its pre-stage from
 * the second step on), current_time += time_step_length. */
extern "C" int pm_tcd_next_step(pm_tcd* s) {
  if (!s) return PM_E_INVALID;
  s->step += 1;
  if (s->scheme == "bdf_two" && s->step >= 2) s->pre_stage_bdf = false;
  s->t += s->tau;
  return PM_OK;
}

/* TimeConvectionDiffusion::assemble (:294-352): stiffness matrices and rhs at
 * the current time, the rhs of the time discretisation
 * (prepare_rhs_from_time_disc), old_rhs = rhs, the non-active rhs and
 * solution entries from the new rhs, and the system matrices
 * factor * A + M on every level (prepare_system_matrix). */
extern "C" int pm_tcd_assemble(pm_tcd* s) {
  if (!s) return PM_E_INVALID;
  pm_ctx* c = s->p->ctx;
  TCD_TRY
  if (!s->initial_done) throw Error(PM_E_INVALID, "assemble_initial_time first");
  pm_problem* p = s->p;
  const int nl = int(s->mass.size());
  assemble_stiffness(s, s->t);
  DevCsr& A = p->mats.back()->csr;
  const DevCsr& M = s->mass.back();
  const int n = A.n_rows, na = A.n_active;
  vcopy(c, n, p->rhs.p, s->rhs_td.p);
  const int gb = std::max(1, (na + 255) / 256);
  const bool bdf2 = s->scheme == "bdf_two" && !s->pre_stage_bdf;
  if (bdf2) {
    k_tcd_scale_add<<<gb, 256, 0, c->stream>>>(na, s->rhs_td.p, s->bdf[2] * s->tau, nullptr, 0.0);
    csr_apply(c, M, EPI_AXPY, s->sol_m1.p, s->rhs_td.p, nullptr, s->bdf[0]);
    csr_apply(c, M, EPI_AXPY, s->sol_m2.p, s->rhs_td.p, nullptr, s->bdf[1]);
  } else if (s->scheme == "backward_euler" || s->pre_stage_bdf) {
    k_tcd_scale_add<<<gb, 256, 0, c->stream>>>(na, s->rhs_td.p, s->tau, nullptr, 0.0);
    csr_apply(c, M, EPI_AXPY, s->sol_m1.p, s->rhs_td.p, nullptr, 1.0);
  } else {  // crank_nicolson
    k_tcd_scale_add<<<gb, 256, 0, c->stream>>>(na, s->rhs_td.p, 0.5 * s->tau, s->old_rhs.p, 0.5 * s->tau);
    csr_apply(c, M, EPI_AXPY, s->sol_m1.p, s->rhs_td.p, nullptr, 1.0);
    csr_apply(c, A, EPI_AXPY, s->sol_m1.p, s->rhs_td.p, nullptr, -0.5 * s->tau);
  }
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
  vcopy(c, n, p->rhs.p, s->old_rhs.p);
  if (n > na) {
    PM_CUDA(cudaMemcpyAsync(s->rhs_td.p + na, p->rhs.p + na, sizeof(double) * (n - na), cudaMemcpyDeviceToDevice,
                            c->stream));
    PM_CUDA(cudaMemcpyAsync(p->sol.p + na, p->rhs.p + na, sizeof(double) * (n - na), cudaMemcpyDeviceToDevice,
                            c->stream));
  }
  const double factor = system_factor(s);
  for (int l = 0; l < nl; ++l) {
    DevCsr& Al = p->mats[l]->csr;
    const int64_t ne = s->active_entries[l];
    if (ne) {
      k_tcd_system<<<grid_of(c, ne), 256, 0, c->stream>>>(ne, Al.vals.p, s->mass[l].vals.p, factor);
      PM_CHECK_LAUNCH();
      c->kernel_launches++;
    }
    Al.values_changed(c);
  }
  s->factor_used = factor;
  p->solver_ready = false;
  return PM_OK;
  TCD_CATCH(c)
}

/* TimeConvectionDiffusion::solve (:354-386): the solver on the system
 * matrices with the time-discrete rhs, then reset_linear_matrices (system
 * matrix minus mass, scaled by 1/factor) and solution_m2 = solution_m1,
 * solution_m1 = solution. */
extern "C" int pm_tcd_solve(pm_tcd* s) {
  if (!s) return PM_E_INVALID;
  pm_ctx* c = s->p->ctx;
  TCD_TRY
  pm_problem* p = s->p;
  if (s->factor_used == 0.0) throw Error(PM_E_INVALID, "pm_tcd_assemble first");
  if (!p->solver_ready) {
    int rc = pm_solver_update_matrix(p->solver, p->mats.back());
    if (rc != PM_OK) return rc;
    p->solver_ready = true;
  }
  p->solver->solve(s->rhs_td.p, p->sol.p);
  const double inv = 1. / s->factor_used;
  for (size_t l = 0; l < s->mass.size(); ++l) {
    DevCsr& Al = p->mats[l]->csr;
    const int64_t ne = s->active_entries[l];
    if (ne) {
      k_tcd_reset<<<grid_of(c, ne), 256, 0, c->stream>>>(ne, Al.vals.p, s->mass[l].vals.p, inv);
      PM_CHECK_LAUNCH();
      c->kernel_launches++;
    }
    Al.values_changed(c);
  }
  s->factor_used = 0.0;
  p->solver_ready = false;
  const int n = p->mats.back()->csr.n_rows;
  vcopy(c, n, s->sol_m1.p, s->sol_m2.p);
  vcopy(c, n, p->sol.p, s->sol_m1.p);
  PM_CUDA(cudaStreamSynchronize(c->stream));
  return PM_OK;
  TCD_CATCH(c)
}

extern "C" int pm_tcd_state(const pm_tcd* s, double* time, int* step) {
  if (!s) return PM_E_INVALID;
  if (time) *time = s->t;
  if (step) *step = s->step;
  return PM_OK;
}

extern "C" int pm_tcd_problem(pm_tcd* s, pm_problem** out) {
  if (!s || !out) return PM_E_INVALID;
  *out = s->p;
  return PM_OK;
}
