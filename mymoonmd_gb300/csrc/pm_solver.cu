// Multigrid cycle and Krylov methods on the device.
//
// The control flow restates src/Multigrid/Multigrid.C:157-420 (cycle,
// cycle_step, restriction, damped prolongation), src/Solver/Iteration_gmres.C
// :376-532 (flexible GMRES with modified Gram-Schmidt and Givens rotations),
// Iteration_cg.C:22-79, Iteration_bicgstab.C:28-206, Iteration_jacobi.C:31-105
// and the stopping test of include/Solver/IterativeMethod.h:81-140. All vector
// work stays on the device; FGMRES keeps H, the Givens state and the scalars
// of Gram-Schmidt on the device and reads back one residual per iteration for
// the host-side stopping test.
#include <algorithm>
#include <cmath>
#include <sstream>

#include "pm_solver.h"
#include "pm_batch.h"

namespace pm {

// ---------------------------------------------------------------- params ---
static std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\"'");
  size_t b = s.find_last_not_of(" \t\r\"'");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

Params Params::parse(const char* text) {
  Params p;
  if (!text) return p;
  std::istringstream in(text);
  std::string line;
  while (std::getline(in, line)) {
    size_t hash = line.find('#');
    if (hash != std::string::npos) line = line.substr(0, hash);
    size_t sep = line.find(':');
    if (sep == std::string::npos) sep = line.find('=');
    if (sep == std::string::npos) continue;
    std::string k = trim(line.substr(0, sep)), v = trim(line.substr(sep + 1));
    if (!k.empty()) p.kv[k] = v;
  }
  return p;
}

std::string Params::str(const std::string& k, const std::string& def) const {
  auto it = kv.find(k);
  return it == kv.end() ? def : it->second;
}
double Params::num(const std::string& k, double def) const {
  auto it = kv.find(k);
  if (it == kv.end()) return def;
  // ParameterDatabase::write prints bool parameters as true / false
  if (it->second == "true") return 1.0;
  if (it->second == "false") return 0.0;
  char* end = nullptr;
  double v = strtod(it->second.c_str(), &end);
  if (end == it->second.c_str()) throw Error(PM_E_INVALID, "parameter " + k + " is not a number");
  return v;
}
long Params::integer(const std::string& k, long def) const {
  return long(num(k, double(def)));
}

// ------------------------------------------------------- cycle control -----
static void fill_recursively(std::vector<int>& out, std::vector<int>& rec, int level, int n_levels,
                             bool fcycle) {
  if (level == 0) {
    out.push_back(DIR_UP);
    return;
  }
  for (int j = 0; j < rec[level]; ++j) {
    out.push_back(DIR_DOWN);
    fill_recursively(out, rec, level - 1, n_levels, fcycle);
  }
  if (fcycle) rec[level] = 1;
  out.push_back(level == n_levels - 1 ? DIR_END : DIR_UP);
}

std::vector<int> cycle_control(const std::string& type, int n_levels) {
  std::vector<int> rec(n_levels, type == "V" ? 1 : 2);
  rec[n_levels - 1] = 1;
  std::vector<int> out{DIR_DUMMY};
  fill_recursively(out, rec, n_levels - 1, n_levels, type == "F");
  return out;
}

// ------------------------------------------------------------ multigrid ----
static int smoother_code(const std::string& s) {
  if (s == "jacobi") return SM_JACOBI;
  if (s == "direct_solve") return SM_DIRECT;
  if (s == "cell_vanka") return SM_CELL_VANKA;
  if (s == "cell_vanka_jacobi") return SM_CELL_VANKA_JACOBI;
  // the reference's *_store variants keep the local factorisations; here they
  // are always kept
  if (s == "cell_vanka_store") return SM_CELL_VANKA;
  if (s == "cell_vanka_jacobi_store") return SM_CELL_VANKA_JACOBI;
  if (s == "nodal_vanka" || s == "nodal_vanka_store") return SM_NODAL_VANKA;
  // additive nodal Vanka (the CELL_JACOBI treatment on nodal patches)
  if (s == "nodal_vanka_jacobi") return SM_NODAL_VANKA_JACOBI;
  // SOR / SSOR in multicolour order (the sequential sweep over the rows
  // ordered by colour)
  if (s == "sor") return SM_SOR;
  if (s == "ssor") return SM_SSOR;
  throw Error(PM_E_UNSUPPORTED, "multigrid smoother '" + s + "' is not implemented on the GPU");
}

void Multigrid::configure(const Params& p) {
  n_pre = int(p.integer("multigrid_n_pre_smooth", 1));
  n_post = int(p.integer("multigrid_n_post_smooth", 1));
  jacobi_damp = p.num("jacobi_damp", 1.0);
  sor_omega = p.num("sor_omega", 1.5);
  vanka_damp = p.num("multigrid_vanka_damp_factor", 1.0);
  correction_damp = p.num("multigrid_correction_damp_factor", 1.0);
  coarse_residual = p.num("multigrid_coarse_residual", 0.1);
  coarse_max_it = int(p.integer("multigrid_coarse_max_n_iterations", 10));
  cycle_type = p.str("multigrid_cycle_type", "V");
  if (cycle_type != "V" && cycle_type != "W" && cycle_type != "F") cycle_type = "V";
  smoother = smoother_code(p.str("multigrid_smoother", "jacobi"));
  smoother_coarse = smoother_code(p.str("multigrid_smoother_coarse", "direct_solve"));
  std::string type = p.str("multigrid_type", "standard");
  if (type != "standard") throw Error(PM_E_UNSUPPORTED, "only standard multigrid is implemented");
  mixed = p.str("gpu_precision", "fp64") == "mixed";
  mixed_cfg = mixed;
  const std::string cp = p.str("gpu_mixed_coarse", "fp32");
  if (cp != "fp32" && cp != "fp64") throw Error(PM_E_INVALID, "gpu_mixed_coarse is fp32 or fp64");
  coarse64 = cp == "fp64";
}

void Multigrid::set_mixed(pm_ctx* c, bool on) {
  if (on == mixed) return;
  if (on && !mixed_cfg) throw Error(PM_E_INVALID, "the multigrid was not set up for the mixed form");
  if (!on && !fp64_smoothers) {
    for (auto& lv : levels) {
      const bool vanka = lv.smoother == SM_CELL_VANKA || lv.smoother == SM_CELL_VANKA_JACOBI;
      const bool nodal = lv.smoother == SM_NODAL_VANKA || lv.smoother == SM_NODAL_VANKA_JACOBI;
      if (vanka) lv.vanka->factor(c, lv.proj->csr, false);
      if (nodal) lv.nodal->factor(c, lv.proj->csr, false);
      // the mixed cycle built only the FP32 coarse inverse
      if (lv.smoother == SM_DIRECT && !lv.coarse.has64) lv.coarse.build(c, lv.proj ? lv.proj->csr : lv.A->csr);
    }
    fp64_smoothers = true;
  }
  mixed = on;
}

void Multigrid::start_coarse(pm_ctx* c) {
  if (levels.size() < 2 || !levels[0].A || levels[0].proj) return;
  if (smoother_coarse != SM_DIRECT) return;
  // the side stream starts after the assembly queued so far on the main one
  PM_CUDA(cudaEventRecord(c->side_event, c->stream));
  PM_CUDA(cudaStreamWaitEvent(c->side, c->side_event, 0));
  if (mixed_cfg && !coarse64) levels[0].coarse.launch32(c, levels[0].A->csr, c->side);
  else levels[0].coarse.launch64(c, levels[0].A->csr, c->side);
}

void Multigrid::update(pm_ctx* c) {
  mixed = mixed_cfg;
  fp64_smoothers = !mixed;
  const int L = int(levels.size());
  if (L < 2) throw Error(PM_E_INVALID, "for multigrid you need at least two multigrid levels");
  for (int l = 0; l < L; ++l)
    if (!levels[l].A) throw Error(PM_E_INVALID, "multigrid level " + std::to_string(l) + " has no matrix");
  control = cycle_control(cycle_type, L);
  // the coarse loop's device flag and partial sums (allocated here: the cycle
  // itself may run inside a graph capture, where allocation is not allowed)
  coarse_flag.ensure(1);
  coarse_part.ensure(kRedBlocks);
  for (int l = 0; l < L; ++l) {
    MGLevel& lv = levels[l];
    DevCsr& A = lv.A->csr;
    lv.smoother = (l == 0) ? smoother_coarse : smoother;
    const bool vanka = lv.smoother == SM_CELL_VANKA || lv.smoother == SM_CELL_VANKA_JACOBI;
    const bool nodal = lv.smoother == SM_NODAL_VANKA || lv.smoother == SM_NODAL_VANKA_JACOBI;
    if ((vanka && (!lv.vanka || !lv.proj)) || (nodal && (!lv.nodal || !lv.proj)))
      throw Error(PM_E_UNSUPPORTED, "Vanka smoothers need the Stokes problem set-up");
    // get_combined_matrix of this level (values copied from the system matrix)
    if (lv.proj) lv.proj->refresh(c, A, mixed);
    if (vanka) lv.vanka->factor(c, lv.proj->csr, mixed);
    if (nodal) lv.nodal->factor(c, lv.proj->csr, mixed);
    const bool sor = lv.smoother == SM_SOR || lv.smoother == SM_SSOR;
    if (lv.smoother == SM_JACOBI || sor) A.make_diag(c);
    if (sor) {
      lv.sor.build(c, A);
      sor_check_diagonal(c, A);
    }
    A.make_sliced64(c);  // FP64 sweeps, defects and the Krylov SpMV on the sliced copy
    const int n = A.n_rows;
    if (l < L - 1) {
      if (!lv.P.row_ptr.p) throw Error(PM_E_INVALID, "missing prolongation of level " + std::to_string(l));
      lv.P.mask = levels[l + 1].A->csr.mask;
      lv.R.mask = A.mask;
      lv.R.make_sliced64(c);
    }
    if (mixed) {
      // the FP32 copy of this update's values: the matrix may have been
      // re-assembled (new coefficients or geometry) since the last update
      A.make_fp32(c);
      if (l < L - 1) {
        lv.P.make_fp32(c);
        lv.R.make_fp32(c);
      }
      lv.rhs32.ensure(n);
      lv.sol32.ensure(n);
      lv.alt32.ensure(n);
      lv.defect32.ensure(n);
    }
    // FP64 buffers (kept at the same addresses across updates, so captured
    // graphs stay valid)
    lv.rhs.ensure(n);
    lv.sol.ensure(n);
    lv.alt.ensure(n);
    lv.defect.ensure(n);
    if (lv.smoother == SM_DIRECT) {
      // DirectSolver factorises get_combined_matrix (with the pressure projection);
      // the mixed cycle solves with an FP32 inverse (the FP64 one is made on a
      // fallback to FP64)
      if (mixed && !coarse64 && lv.coarse.pending32) lv.coarse.complete32(c, A);  // queued by start_coarse
      else if (mixed && !coarse64) lv.coarse.build32(c, lv.proj ? lv.proj->csr : A);
      else if (lv.coarse.pending64) lv.coarse.complete64(c);
      else lv.coarse.build(c, lv.proj ? lv.proj->csr : A);
      if (mixed) {
        lv.coarse_rhs64.ensure(n);
        lv.coarse_sol64.ensure(n);
      }
    }
  }
  ready = true;
}

void Multigrid::smooth(pm_ctx* c, int l) {
  MGLevel& lv = levels[l];
  const DevCsr& A = lv.A->csr;
  if (lv.smoother == SM_JACOBI) {
    if (mixed) {
      csr_apply32(c, A, EPI_JACOBI, lv.cur32, lv.oth32, lv.rhs32.p, float(jacobi_damp));
      std::swap(lv.cur32, lv.oth32);
    } else {
      csr_apply(c, A, EPI_JACOBI, lv.cur, lv.oth, lv.rhs.p, jacobi_damp);
      std::swap(lv.cur, lv.oth);
    }
  } else if (lv.smoother == SM_SOR || lv.smoother == SM_SSOR) {
    // SORSmoother::smooth: one sweep of Iteration_sor::apply_smoother on the
    // current iterate (SSOR: forward, then backward)
    if (mixed) {
      sor_sweep32(c, A, lv.sor, lv.rhs32.p, lv.cur32, float(sor_omega), false);
      if (lv.smoother == SM_SSOR) sor_sweep32(c, A, lv.sor, lv.rhs32.p, lv.cur32, float(sor_omega), true);
    } else {
      sor_sweep(c, A, lv.sor, lv.rhs.p, lv.cur, sor_omega, false);
      if (lv.smoother == SM_SSOR) sor_sweep(c, A, lv.sor, lv.rhs.p, lv.cur, sor_omega, true);
    }
  } else if (lv.smoother == SM_DIRECT) {
    coarse_solve(c);
  } else if (lv.smoother == SM_CELL_VANKA_JACOBI) {
    // additive cell Vanka, in place; the level's defect buffer holds the residual
    if (mixed) lv.vanka->sweep_jacobi32(c, lv.proj->csr, lv.rhs32.p, lv.cur32, lv.defect32.p, float(vanka_damp));
    else lv.vanka->sweep_jacobi(c, lv.proj->csr, lv.rhs.p, lv.cur, lv.defect.p, vanka_damp);
  } else if (lv.smoother == SM_CELL_VANKA) {
    if (mixed) lv.vanka->sweep_colored32(c, lv.proj->csr, lv.rhs32.p, lv.cur32, float(vanka_damp));
    else lv.vanka->sweep_colored(c, lv.proj->csr, lv.rhs.p, lv.cur, vanka_damp);
  } else if (lv.smoother == SM_NODAL_VANKA_JACOBI) {
    if (mixed) lv.nodal->sweep_jacobi32(c, lv.proj->csr, lv.rhs32.p, lv.cur32, lv.defect32.p, float(vanka_damp));
    else lv.nodal->sweep_jacobi(c, lv.proj->csr, lv.rhs.p, lv.cur, lv.defect.p, vanka_damp);
  } else if (lv.smoother == SM_NODAL_VANKA) {
    if (mixed) lv.nodal->sweep_colored32(c, lv.proj->csr, lv.rhs32.p, lv.cur32, float(vanka_damp));
    else lv.nodal->sweep_colored(c, lv.proj->csr, lv.rhs.p, lv.cur, vanka_damp);
  }
}

void Multigrid::smooth_from_zero(pm_ctx* c, int l) {
  MGLevel& lv = levels[l];
  const DevCsr& A = lv.A->csr;
  if (lv.smoother != SM_JACOBI || !c->jacobi_zero_start) {
    smooth(c, l);
    return;
  }
  // the iterate stays in its buffer (the sweep's swap of the two buffers is
  // not needed: x0 is not read)
  if (mixed) jacobi_from_zero32(c, A.n_rows, lv.rhs32.p, A.diag32.p, float(jacobi_damp), lv.cur32);
  else jacobi_from_zero(c, A.n_rows, lv.rhs.p, A.diag.p, jacobi_damp, lv.cur);
}

void Multigrid::coarse_solve(pm_ctx* c) {
  MGLevel& lv = levels[0];
  const DevCsr& A = lv.A->csr;
  if (mixed && coarse64) {
    lv.coarse.solve_mixed(c, lv.rhs32.p, lv.cur32);
  } else if (mixed) {
    // the coarse rhs comes from the restriction with its non-actives reset
    lv.coarse.solve32(c, lv.rhs32.p, lv.cur32);
  } else {
    // the coarse rhs comes from the restriction with its non-actives reset
    lv.coarse.solve(c, A, lv.rhs.p, lv.cur, true);
  }
}

// sum of squares of x in kRedBlocks partial sums (fixed order)
template <class T>
__global__ void __launch_bounds__(256) k_sumsq_partials(int n, const T* __restrict__ x,
                                                        double* __restrict__ part) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = double(x[i]);
    s += v * v;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (int(threadIdx.x) < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// res = sqrt(sum of the partials); the loop goes on while res > tol
__global__ void k_stop_if_small(const double* __restrict__ part, int n_part, double tol, int* __restrict__ flag) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n_part; i += blockDim.x) s += part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (int(threadIdx.x) < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0 && !(sqrt(sh[0]) > tol)) *flag = 1;
}

void Multigrid::coarse_iterate(pm_ctx* c) {
  MGLevel& lv = levels[0];
  const int n = lv.A->csr.n_rows;
  PM_CUDA(cudaMemsetAsync(coarse_flag.p, 0, sizeof(int), c->stream));
  c->guard = coarse_flag.p;
  try {
    for (int i = 0; i < coarse_max_it; ++i) {
      smooth(c, 0);
      defect(c, 0);
      if (mixed) k_sumsq_partials<float><<<kRedBlocks, 256, 0, c->stream>>>(n, lv.defect32.p, coarse_part.p);
      else k_sumsq_partials<double><<<kRedBlocks, 256, 0, c->stream>>>(n, lv.defect.p, coarse_part.p);
      k_stop_if_small<<<1, 256, 0, c->stream>>>(coarse_part.p, kRedBlocks, coarse_residual, coarse_flag.p);
      PM_CHECK_LAUNCH();
      c->kernel_launches += 2;
    }
  } catch (...) {
    c->guard = nullptr;
    throw;
  }
  c->guard = nullptr;
}

void Multigrid::defect(pm_ctx* c, int l) {
  MGLevel& lv = levels[l];
  if (mixed) csr_apply32(c, lv.A->csr, EPI_DEFECT, lv.cur32, lv.defect32.p, lv.rhs32.p, 1.0f);
  else csr_apply(c, lv.A->csr, EPI_DEFECT, lv.cur, lv.defect.p, lv.rhs.p, 1.0);
}

void Multigrid::restrict_to(pm_ctx* c, int l) {
  MGLevel& fine = levels[l];
  MGLevel& crs = levels[l - 1];
  // DefectRestriction followed by ResetNonActive of the coarse rhs
  if (mixed) csr_apply32(c, crs.R, EPI_RESTRICT, fine.defect32.p, crs.rhs32.p, nullptr, 1.0f);
  else csr_apply(c, crs.R, EPI_RESTRICT, fine.defect.p, crs.rhs.p, nullptr, 1.0);
}

void Multigrid::prolongate_from(pm_ctx* c, int l) {
  MGLevel& crs = levels[l];
  MGLevel& fine = levels[l + 1];
  if (mixed)
    csr_apply32(c, crs.P, EPI_PROLONG, crs.cur32, fine.cur32, nullptr, float(correction_damp));
  else
    csr_apply(c, crs.P, EPI_PROLONG, crs.cur, fine.cur, nullptr, correction_damp);
}

void Multigrid::apply(pm_ctx* c, const double* rhs, double* sol, bool rhs_nonactive_zero) {
  if (!ready) throw Error(PM_E_INVALID, "multigrid used before update()");
  // a factorisation queued by a new assembly (a caller applying the cycle
  // without the update that follows an assembly): wait for it
  if (levels[0].coarse.pending32) levels[0].coarse.complete32(c, levels[0].A->csr);
  if (levels[0].coarse.pending64) levels[0].coarse.complete64(c);
  const int L = int(levels.size());
  const int finest = L - 1;
  MGLevel& top = levels[finest];
  const int nf = top.A->csr.n_rows;
  for (auto& lv : levels) {
    lv.cur = lv.sol.p;
    lv.oth = lv.alt.p;
    lv.cur32 = lv.sol32.p;
    lv.oth32 = lv.alt32.p;
  }
  // set_finest_rhs / set_finest_sol; cycle(): solution := 0, copy_nonactive(rhs)
  if (mixed) {
    vcvt_d2f(c, nf, rhs, top.rhs32.p);
    init_solution32(c, nf, top.A->csr.mask, top.rhs32.p, top.cur32);
  } else {
    vcopy(c, nf, rhs, top.rhs.p);
    init_solution(c, nf, top.A->csr.mask, top.rhs.p, top.cur);
  }
  // levels whose iterate is exactly zero now: the finest one when its rhs has
  // zero non-actives (init_solution copies them), the coarser ones after their
  // reset below (their rhs has its non-actives reset by the restriction)
  std::vector<char> zero(L, 0);
  zero[finest] = rhs_nonactive_zero ? 1 : 0;
  const int n_steps = int(control.size()) - 1;
  int level = finest;
  for (int step = 1; step <= n_steps && level >= 0; ++step) {
    if (level == 0) {
      // coarsest level: with the direct solver one application solves exactly;
      // the defects the reference computes around it only feed its loop test
      if (levels[0].smoother == SM_DIRECT) coarse_solve(c);
      else coarse_iterate(c);
      zero[0] = 0;
      prolongate_from(c, 0);
      zero[1] = 0;
      level = 1;
      continue;
    }
    const bool from_below = control[step - 1] == DIR_UP;
    const bool up = control[step] == DIR_UP;
    const bool down = control[step] == DIR_DOWN;
    if (from_below)
      for (int i = 0; i < n_post; ++i) smooth(c, level);
    if (down) {
      for (int i = 0; i < n_pre; ++i) {
        if (i == 0 && zero[level]) smooth_from_zero(c, level);
        else smooth(c, level);
        zero[level] = 0;
      }
      defect(c, level);
      MGLevel& crs = levels[level - 1];
      const int nc = crs.A->csr.n_rows;
      // the coarse iterate starts at zero; the reset is skipped where the
      // level's first step writes every entry without reading it (a Jacobi
      // sweep from zero, the direct coarse solve)
      const bool written = (level - 1 > 0 && crs.smoother == SM_JACOBI && n_pre >= 1 && c->jacobi_zero_start) ||
                           (level - 1 == 0 && crs.smoother == SM_DIRECT);
      if (!written) {
        if (mixed) PM_CUDA(cudaMemsetAsync(crs.cur32, 0, sizeof(float) * nc, c->stream));
        else PM_CUDA(cudaMemsetAsync(crs.cur, 0, sizeof(double) * nc, c->stream));
      }
      zero[level - 1] = 1;
      restrict_to(c, level);
      level -= 1;
    } else if (up) {
      prolongate_from(c, level);
      zero[level + 1] = 0;
      level += 1;
    } else {
      level = -1;
    }
  }
  if (mixed) vcvt_f2d(c, nf, top.cur32, sol);
  else vcopy(c, nf, top.cur, sol);
}

static int grid_blocks_for(int n) { return std::max(1, std::min((n + 255) / 256, 1216)); }

// ------------------------------------------------------ FGMRES kernels -----
// every block sums the partials of the previous reduction in the same order
__device__ __forceinline__ double sum_partials(const double* __restrict__ part, double* sh) {
  const int t = threadIdx.x;
  double s = 0.0;
  for (int i = t; i < kRedBlocks; i += blockDim.x) s += part[i];
  sh[t] = s;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (t < k) sh[t] += sh[t + k];
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ void block_partial(double v, double* sh, double* out) {
  const int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (t < k) sh[t] += sh[t + k];
    __syncthreads();
  }
  if (t == 0) out[blockIdx.x] = sh[0];
}

// H(k,i) = <r, v_k>; r -= H(k,i) v_k; partial sums of <r, next>
__global__ void __launch_bounds__(256) k_fg_mgs(int n, int ldh, int k, int i, double* __restrict__ r,
                                                const double* __restrict__ vk,
                                                const double* __restrict__ next,
                                                const double* __restrict__ part_in,
                                                double* __restrict__ part_out, double* __restrict__ H) {
  __shared__ double sh[256];
  const double h = sum_partials(part_in, sh);
  if (blockIdx.x == 0 && threadIdx.x == 0) H[k + (size_t)ldh * i] = h;
  double acc = 0.0;
  const double mh = -h;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const double ri = r[idx] + mh * vk[idx];
    r[idx] = ri;
    const double nx = (next == r) ? ri : next[idx];
    acc += ri * nx;
  }
  block_partial(acc, sh, part_out);
}

// H(i+1,i) = |r|; v_{i+1} = r * (1/H(i+1,i))
__device__ __forceinline__ void fg_normalize_body(int n, int ldh, int i, const double* __restrict__ r,
                                                      double* __restrict__ v,
                                                      const double* __restrict__ part_in,
                                                      double* __restrict__ H, int* __restrict__ flag) {
  pdl_enter();
  __shared__ double sh[256];
  const double hn = sqrt(sum_partials(part_in, sh));
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    H[(i + 1) + (size_t)ldh * i] = hn;
    if (hn == 0.0) flag[0] = 1;
  }
  const double sc = hn != 0.0 ? 1.0 / hn : 0.0;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x)
    v[idx] = r[idx] * sc;
}
__global__ void __launch_bounds__(256) k_fg_normalize(int n, int ldh, int i, const double* __restrict__ r,
                                                      double* __restrict__ v,
                                                      const double* __restrict__ part_in,
                                                      double* __restrict__ H, int* __restrict__ flag) {
  fg_normalize_body(n, ldh, i, r, v, part_in, H, flag);
}

// beta = |r|; v_0 = r * (1/beta); s = (beta, 0, ...)
__device__ __forceinline__ void fg_start_body(int n, int m, const double* __restrict__ r,
                                                  double* __restrict__ v0,
                                                  const double* __restrict__ part_in,
                                                  double* __restrict__ s, double* __restrict__ beta_out) {
  __shared__ double sh[256];
  const double beta = sqrt(sum_partials(part_in, sh));
  if (blockIdx.x == 0) {
    for (int k = threadIdx.x; k <= m; k += blockDim.x) s[k] = (k == 0) ? beta : 0.0;
    if (threadIdx.x == 0) *beta_out = beta;
  }
  const double sc = 1.0 / beta;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x)
    v0[idx] = r[idx] * sc;
}
__global__ void __launch_bounds__(256) k_fg_start(int n, int m, const double* __restrict__ r,
                                                  double* __restrict__ v0,
                                                  const double* __restrict__ part_in,
                                                  double* __restrict__ s, double* __restrict__ beta_out) {
  fg_start_body(n, m, r, v0, part_in, s, beta_out);
}

// Classical Gram-Schmidt with one re-orthogonalisation (CGS2), the batched
// alternative to the modified Gram-Schmidt loop: the i+1 projections of one
// pass are computed in one sweep over the vectors and subtracted in another.
// Partial sums: part[k * kRedBlocks + block], CH accumulators per sweep.
// with_rr: also <r, r> into slot nk (the norm before the pass, for the
// conditional second pass); guard: a set flag skips the launch
template <int CH>
__global__ void __launch_bounds__(256) k_multidot(int n, int nk, const double* __restrict__ r,
                                                  const double* __restrict__ V, size_t ld,
                                                  double* __restrict__ part, int with_rr,
                                                  const int* __restrict__ guard) {
  __shared__ double sh[256];
  if (guarded(guard)) return;  // uniform for the whole grid
  if (with_rr) {
    double acc = 0.0;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
      const double ri = r[idx];
      acc += ri * ri;
    }
    block_partial(acc, sh, part + (size_t)nk * kRedBlocks);
  }
  for (int k0 = 0; k0 < nk; k0 += CH) {
    double acc[CH];
#pragma unroll
    for (int u = 0; u < CH; ++u) acc[u] = 0.0;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
      const double ri = r[idx];
#pragma unroll
      for (int u = 0; u < CH; ++u)
        if (k0 + u < nk) acc[u] += ri * V[(size_t)(k0 + u) * ld + idx];
    }
#pragma unroll
    for (int u = 0; u < CH; ++u)
      if (k0 + u < nk) block_partial(acc[u], sh, part + (size_t)(k0 + u) * kRedBlocks);
  }
}

// h[k] = sum of the partials of projection k (one block per k); with hsum,
// also H(k, col) = hsum[k] + h[k]
// guard set (second pass skipped): h[k] = 0 and H(k, col) = hsum[k]
__device__ __forceinline__ void reduce_proj_body(const double* __restrict__ part, double* __restrict__ h,
                                                     const double* __restrict__ hsum, double* __restrict__ H,
                                                     int ldh, int col, const int* __restrict__ guard) {
  pdl_enter();
  __shared__ double sh[256];
  const int k = blockIdx.x;
  if (guarded(guard)) {  // uniform for the whole grid
    if (threadIdx.x == 0) {
      h[k] = 0.0;
      if (hsum) H[k + (size_t)ldh * col] = hsum[k];
    }
    return;
  }
  const double s = sum_partials(part + (size_t)k * kRedBlocks, sh);
  if (threadIdx.x == 0) {
    h[k] = s;
    if (hsum) H[k + (size_t)ldh * col] = hsum[k] + s;
  }
}
__global__ void __launch_bounds__(256) k_reduce_proj(const double* __restrict__ part, double* __restrict__ h,
                                                     const double* __restrict__ hsum, double* __restrict__ H,
                                                     int ldh, int col, const int* __restrict__ guard) {
  reduce_proj_body(part, h, hsum, H, ldh, col, guard);
}

// r -= sum_k h[k] V_k, subtracted in k order
__global__ void __launch_bounds__(256) k_cgs_update(int n, int nk, double* __restrict__ r,
                                                    const double* __restrict__ V, size_t ld,
                                                    const double* __restrict__ h, const int* __restrict__ guard) {
  __shared__ double hs[64];
  if (guarded(guard)) return;  // uniform for the whole grid
  for (int k = threadIdx.x; k < nk; k += blockDim.x) hs[k] = h[k];
  __syncthreads();
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    double ri = r[idx];
    for (int k = 0; k < nk; ++k) ri -= hs[k] * V[(size_t)k * ld + idx];
    r[idx] = ri;
  }
}

// CGS2 for up to kCgsFused basis vectors in three sweeps over V: projections
// of pass 1 (k_mdot), the pass-1 update fused with the projections of pass 2
// (k_cgs_update_mdot), the pass-2 update fused with the partial sums of |r|^2
// (k_cgs_update_norm). The FP64 pipe bounds these sweeps on GB300 (about one
// FP64 FMA per clock per SM), so they run 16 warps per SM and keep the update
// chains short: V is read in chunks of 8 vectors, the pass-2 projections read
// the chunk again (from L1/L2) after the update. 256 threads per block, grid
// kRedBlocks; partial sums per block in a fixed order: each thread in index
// order, warps by xor shuffles, warps in order.
constexpr int kCgsFused = 32;
constexpr int kCgsChunk = 8;

// Reduce-scatter of W accumulators over the lanes of a warp by recursive
// halving (W = 32: offsets 16..1, afterwards lane l holds the warp's sum of
// accumulator l); W - 1 FP64 additions per lane instead of 5 W for a
// butterfly on every accumulator, which on GB300's FP64 pipe cost as much as
// the projections themselves
template <int W>
__device__ __forceinline__ double warp_halving(double (&a)[W], int lane) {
#pragma unroll
  for (int o = W / 2; o >= 1; o >>= 1) {
    const bool hi = (lane & o) != 0;
#pragma unroll
    for (int j = 0; j < o; ++j) {
      const double keep = hi ? a[o + j] : a[j];
      const double send = hi ? a[j] : a[o + j];
      a[j] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  return a[0];
}

// the block's partial sums of NK accumulators (NK = 16 or 32) into
// part[k * kRedBlocks + block], k < nk
template <int NK>
__device__ __forceinline__ void block_partials_multi(double (&acc)[NK], double* red, double* __restrict__ part,
                                                     int nk) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if constexpr (NK == 16) {
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], 16);
  }
  const double v = warp_halving<NK>(acc, lane);  // lane l (mod NK): accumulator l
  if (lane < NK) red[warp * NK + lane] = v;
  __syncthreads();
  const int k = threadIdx.x;
  if (k < NK && k < nk) {
    double sum = 0.0;
    for (int w = 0; w < nw; ++w) sum += red[w * NK + k];
    part[(size_t)k * kRedBlocks + blockIdx.x] = sum;
  }
  __syncthreads();
}

// Per basis chunk c (8 vectors) f(c, rem) with rem = nk - 8c >= 1: exactly
// min(8, rem) loads and FMAs; the bodies run full chunks unpredicated and the
// last partial chunk predicated (uniform tests). The loop is unrolled, so c is
// a constant in every body and the accumulator indices stay static.
template <int NK, class F>
__device__ __forceinline__ void cgs_chunks(int nk, F&& f) {
#pragma unroll
  for (int c = 0; c < NK / kCgsChunk; ++c)
    if (c * kCgsChunk < nk) f(c, nk - c * kCgsChunk);
}

// acc[8c + u] += ri * V_{8c+u}(idx) for the chunk's vectors
template <int NK>
__device__ __forceinline__ void cgs_dot_chunk(double (&acc)[NK], int c, int rem, double ri, int idx,
                                              const double* __restrict__ V, size_t ld) {
  if (rem >= kCgsChunk) {
    double v[kCgsChunk];
#pragma unroll
    for (int u = 0; u < kCgsChunk; ++u) v[u] = V[(size_t)(c * kCgsChunk + u) * ld + idx];
#pragma unroll
    for (int u = 0; u < kCgsChunk; ++u) acc[c * kCgsChunk + u] += ri * v[u];
  } else {
#pragma unroll
    for (int u = 0; u < kCgsChunk; ++u)
      if (u < rem) acc[c * kCgsChunk + u] += ri * V[(size_t)(c * kCgsChunk + u) * ld + idx];
  }
}

// partials of <r, V_k>, k < nk <= NK, in one sweep
template <int NK>
__device__ __forceinline__ void mdot_body(int n, int nk, const double* __restrict__ r,
                                                 const double* __restrict__ V, size_t ld, double* __restrict__ part) {
  pdl_enter();
  __shared__ double red[8 * NK];
  double acc[NK];
#pragma unroll
  for (int u = 0; u < NK; ++u) acc[u] = 0.0;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const double ri = r[idx];
    cgs_chunks<NK>(nk, [&](int c, int rem) { cgs_dot_chunk<NK>(acc, c, rem, ri, idx, V, ld); });
  }
  block_partials_multi<NK>(acc, red, part, nk);
}
template <int NK>
__global__ void __launch_bounds__(256, 2) k_mdot(int n, int nk, const double* __restrict__ r,
                                                 const double* __restrict__ V, size_t ld, double* __restrict__ part) {
  mdot_body<NK>(n, nk, r, V, ld, part);
}

// ri -= sum_k h[k] V_k(idx) in k order (the operations of k_cgs_update)
template <int NK>
__device__ __forceinline__ double cgs_update_entry(double ri, int idx, int nk, const double* __restrict__ V,
                                                   size_t ld, const double* hs) {
  cgs_chunks<NK>(nk, [&](int c, int rem) {
    double v[kCgsChunk];
    if (rem >= kCgsChunk) {
#pragma unroll
      for (int u = 0; u < kCgsChunk; ++u) v[u] = V[(size_t)(c * kCgsChunk + u) * ld + idx];
#pragma unroll
      for (int u = 0; u < kCgsChunk; ++u) ri -= hs[c * kCgsChunk + u] * v[u];
    } else {
#pragma unroll
      for (int u = 0; u < kCgsChunk; ++u) v[u] = u < rem ? V[(size_t)(c * kCgsChunk + u) * ld + idx] : 0.0;
#pragma unroll
      for (int u = 0; u < kCgsChunk; ++u)
        if (u < rem) ri -= hs[c * kCgsChunk + u] * v[u];
    }
  });
  return ri;
}

// r -= sum_k h[k] V_k, then the partials of <r_new, V_k> (nk <= NK)
template <int NK>
__device__ __forceinline__ void cgs_update_mdot_body(int n, int nk, double* __restrict__ r,
                                                            const double* __restrict__ V, size_t ld,
                                                            const double* __restrict__ h, double* __restrict__ part) {
  pdl_enter();
  __shared__ double hs[NK];
  __shared__ double red[8 * NK];
  if (threadIdx.x < NK) hs[threadIdx.x] = int(threadIdx.x) < nk ? h[threadIdx.x] : 0.0;
  __syncthreads();
  double acc[NK];
#pragma unroll
  for (int u = 0; u < NK; ++u) acc[u] = 0.0;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const double ri = cgs_update_entry<NK>(r[idx], idx, nk, V, ld, hs);
    r[idx] = ri;
    cgs_chunks<NK>(nk, [&](int c, int rem) { cgs_dot_chunk<NK>(acc, c, rem, ri, idx, V, ld); });
  }
  block_partials_multi<NK>(acc, red, part, nk);
}
template <int NK>
__global__ void __launch_bounds__(256, 2) k_cgs_update_mdot(int n, int nk, double* __restrict__ r,
                                                            const double* __restrict__ V, size_t ld,
                                                            const double* __restrict__ h, double* __restrict__ part) {
  cgs_update_mdot_body<NK>(n, nk, r, V, ld, h, part);
}

// r -= sum_k h[k] V_k, then the block's partial sum of |r_new|^2
__device__ __forceinline__ void cgs_update_norm_body(int n, int nk, double* __restrict__ r,
                                                         const double* __restrict__ V, size_t ld,
                                                         const double* __restrict__ h, double* __restrict__ part) {
  pdl_enter();
  constexpr int NK = kCgsFused;
  __shared__ double hs[NK];
  __shared__ double red[8];
  if (threadIdx.x < NK) hs[threadIdx.x] = int(threadIdx.x) < nk ? h[threadIdx.x] : 0.0;
  __syncthreads();
  double acc = 0.0;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const double ri = cgs_update_entry<NK>(r[idx], idx, nk, V, ld, hs);
    r[idx] = ri;
    acc += ri * ri;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) sum += red[w];
    part[blockIdx.x] = sum;
  }
}
__global__ void __launch_bounds__(256, 2) k_cgs_update_norm(int n, int nk, double* __restrict__ r,
                                                         const double* __restrict__ V, size_t ld,
                                                         const double* __restrict__ h, double* __restrict__ part) {
  cgs_update_norm_body(n, nk, r, V, ld, h, part);
}

// DGKS test after the first classical Gram-Schmidt pass: the second pass is
// needed only if |r after| < |r before| / sqrt(2); flag = 1 skips it
__global__ void k_cgs_decide(const double* __restrict__ part_after, const double* __restrict__ rr_before,
                             int* __restrict__ flag) {
  __shared__ double sh[256];
  const double after = sum_partials(part_after, sh);
  if (threadIdx.x == 0) *flag = (after >= 0.5 * rr_before[0]) ? 1 : 0;
}

__device__ void gen_rot(double dx, double dy, double& cs, double& sn) {
  // GeneratePlaneRotation (src/Solver/Iteration_gmres.C:123)
  if (dy == 0.0) {
    cs = 1.0;
    sn = 0.0;
  } else if (fabs(dy) > fabs(dx)) {
    double t = dx / dy;
    sn = 1.0 / sqrt(1.0 + t * t);
    cs = t * sn;
  } else {
    double t = dy / dx;
    cs = 1.0 / sqrt(1.0 + t * t);
    sn = t * cs;
  }
}
__device__ void app_rot(double& dx, double& dy, double cs, double sn) {
  // ApplyPlaneRotation (src/Solver/Iteration_gmres.C:144)
  double t = cs * dx + sn * dy;
  dy = -sn * dx + cs * dy;
  dx = t;
}

__device__ __forceinline__ void fg_givens_body(int ldh, int i, double* __restrict__ H, double* __restrict__ cs,
                            double* __restrict__ sn, double* __restrict__ s, double* __restrict__ resid) {
  pdl_enter();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double* col = H + (size_t)ldh * i;
  for (int k = 0; k < i; ++k) app_rot(col[k], col[k + 1], cs[k], sn[k]);
  gen_rot(col[i], col[i + 1], cs[i], sn[i]);
  app_rot(col[i], col[i + 1], cs[i], sn[i]);
  app_rot(s[i], s[i + 1], cs[i], sn[i]);
  *resid = fabs(s[i + 1]);
}
__global__ void k_fg_givens(int ldh, int i, double* __restrict__ H, double* __restrict__ cs,
                            double* __restrict__ sn, double* __restrict__ s, double* __restrict__ resid) {
  fg_givens_body(ldh, i, H, cs, sn, s, resid);
}

// Update (src/Solver/Iteration_gmres.C:152): back-solve H y = s
__device__ __forceinline__ void fg_backsolve_body(int ldh, int k, const double* __restrict__ H,
                               const double* __restrict__ s, double* __restrict__ y) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int i = 0; i <= k; ++i) y[i] = s[i];
  for (int i = k; i >= 0; --i) {
    y[i] /= H[i + (size_t)ldh * i];
    for (int j = i - 1; j >= 0; --j) y[j] -= H[j + (size_t)ldh * i] * y[i];
  }
}
__global__ void k_fg_backsolve(int ldh, int k, const double* __restrict__ H,
                               const double* __restrict__ s, double* __restrict__ y) {
  fg_backsolve_body(ldh, k, H, s, y);
}

// x += sum_j y_j z_j  (accumulated in j order, then added)
__device__ __forceinline__ void fg_combine_body(int n, int k, const double* __restrict__ Z, size_t ldz,
                                                    const double* __restrict__ y, double* __restrict__ x) {
  __shared__ double ys[64];
  for (int j = threadIdx.x; j <= k; j += blockDim.x) ys[j] = y[j];
  __syncthreads();
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j <= k; ++j) acc += ys[j] * Z[(size_t)j * ldz + idx];
    x[idx] += acc;
  }
}
__global__ void __launch_bounds__(256) k_fg_combine(int n, int k, const double* __restrict__ Z, size_t ldz,
                                                    const double* __restrict__ y, double* __restrict__ x) {
  fg_combine_body(n, k, Z, ldz, y, x);
}


// ---- batched FGMRES launches (pm_batch.h): every pointer is slot 0's and
// moves by bt.stride to the slot blockIdx.y; the bodies are the kernels' own
#define PM_SLOT(p) (p) = slot_ptr((p), bt)

__global__ void __launch_bounds__(256) kb_fg_start(int n, int m, const double* __restrict__ r, double* __restrict__ v0,
                                                   const double* __restrict__ part_in, double* __restrict__ s,
                                                   double* __restrict__ beta_out, Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  PM_SLOT(r); PM_SLOT(v0); PM_SLOT(part_in); PM_SLOT(s); PM_SLOT(beta_out);
  fg_start_body(n, m, r, v0, part_in, s, beta_out);
}
template <int NK>
__global__ void __launch_bounds__(256, 2) kb_mdot(int n, int nk, const double* __restrict__ r,
                                                  const double* __restrict__ V, size_t ld, double* __restrict__ part,
                                                  Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  PM_SLOT(r); PM_SLOT(V); PM_SLOT(part);
  mdot_body<NK>(n, nk, r, V, ld, part);
}
__global__ void __launch_bounds__(256) kb_reduce_proj(const double* __restrict__ part, double* __restrict__ h,
                                                      const double* __restrict__ hsum, double* __restrict__ H, int ldh,
                                                      int col, Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  PM_SLOT(part); PM_SLOT(h); PM_SLOT(hsum); PM_SLOT(H);
  reduce_proj_body(part, h, hsum, H, ldh, col, nullptr);
}
template <int NK>
__global__ void __launch_bounds__(256, 2) kb_cgs_update_mdot(int n, int nk, double* __restrict__ r,
                                                             const double* __restrict__ V, size_t ld,
                                                             const double* __restrict__ h, double* __restrict__ part,
                                                             Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  PM_SLOT(r); PM_SLOT(V); PM_SLOT(h); PM_SLOT(part);
  cgs_update_mdot_body<NK>(n, nk, r, V, ld, h, part);
}
__global__ void __launch_bounds__(256, 2) kb_cgs_update_norm(int n, int nk, double* __restrict__ r,
                                                             const double* __restrict__ V, size_t ld,
                                                             const double* __restrict__ h, double* __restrict__ part,
                                                             Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  PM_SLOT(r); PM_SLOT(V); PM_SLOT(h); PM_SLOT(part);
  cgs_update_norm_body(n, nk, r, V, ld, h, part);
}
__global__ void __launch_bounds__(256) kb_fg_normalize(int n, int ldh, int i, const double* __restrict__ r,
                                                       double* __restrict__ v, const double* __restrict__ part_in,
                                                       double* __restrict__ H, int* __restrict__ flag, Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  PM_SLOT(r); PM_SLOT(v); PM_SLOT(part_in); PM_SLOT(H); PM_SLOT(flag);
  fg_normalize_body(n, ldh, i, r, v, part_in, H, flag);
}
__global__ void kb_fg_givens(int ldh, int i, double* __restrict__ H, double* __restrict__ cs, double* __restrict__ sn,
                             double* __restrict__ s, double* __restrict__ resid, Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  PM_SLOT(H); PM_SLOT(cs); PM_SLOT(sn); PM_SLOT(s); PM_SLOT(resid);
  fg_givens_body(ldh, i, H, cs, sn, s, resid);
}
__global__ void kb_fg_backsolve(int ldh, int k, const double* __restrict__ H, const double* __restrict__ s,
                                double* __restrict__ y, Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  PM_SLOT(H); PM_SLOT(s); PM_SLOT(y);
  fg_backsolve_body(ldh, k, H, s, y);
}
__global__ void __launch_bounds__(256) kb_fg_combine(int n, int k, const double* __restrict__ Z, size_t ldz,
                                                     const double* __restrict__ y, double* __restrict__ x, Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  PM_SLOT(Z); PM_SLOT(y); PM_SLOT(x);
  fg_combine_body(n, k, Z, ldz, y, x);
}
#undef PM_SLOT

void fg_start_batch(pm_ctx* c, int ns, const Batch& bt, int n, int m, const double* r, double* v0,
                    const double* part, double* s, double* beta_out) {
  kb_fg_start<<<dim3(kRedBlocks, unsigned(ns)), 256, 0, c->stream>>>(n, m, r, v0, part, s, beta_out, bt);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

// the fused CGS2 branch of pm_solver::fgmres for i + 1 <= kCgsFused
void fg_cgs2_batch(pm_ctx* c, int ns, const Batch& bt, int n, int i, int ldh, double* r, const double* V, size_t ld,
                   double* cgs_part, double* h1, double* h2, double* H, double* part_norm) {
  const int nk = i + 1;
  if (nk > kCgsFused) throw Error(PM_E_UNSUPPORTED, "batched FGMRES needs gmres_restart <= 32");
  const dim3 rb = dim3(kRedBlocks, unsigned(ns)), pk = dim3(unsigned(nk), unsigned(ns)), t256 = dim3(256);
  if (nk <= 16) kb_mdot<16><<<rb, t256, 0, c->stream>>>(n, nk, r, V, ld, cgs_part, bt);
  else kb_mdot<kCgsFused><<<rb, t256, 0, c->stream>>>(n, nk, r, V, ld, cgs_part, bt);
  kb_reduce_proj<<<pk, t256, 0, c->stream>>>(cgs_part, h1, nullptr, H, ldh, i, bt);
  if (nk <= 16) kb_cgs_update_mdot<16><<<rb, t256, 0, c->stream>>>(n, nk, r, V, ld, h1, cgs_part, bt);
  else kb_cgs_update_mdot<kCgsFused><<<rb, t256, 0, c->stream>>>(n, nk, r, V, ld, h1, cgs_part, bt);
  kb_reduce_proj<<<pk, t256, 0, c->stream>>>(cgs_part, h2, h1, H, ldh, i, bt);
  kb_cgs_update_norm<<<rb, t256, 0, c->stream>>>(n, nk, r, V, ld, h2, part_norm, bt);
  PM_CHECK_LAUNCH();
  c->kernel_launches += 5;
}

void fg_normalize_batch(pm_ctx* c, int ns, const Batch& bt, int n, int ldh, int i, const double* r, double* v,
                        const double* part, double* H, int* flag) {
  kb_fg_normalize<<<dim3(kRedBlocks, unsigned(ns)), 256, 0, c->stream>>>(n, ldh, i, r, v, part, H, flag, bt);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

void fg_givens_batch(pm_ctx* c, int ns, const Batch& bt, int ldh, int i, double* H, double* cs, double* sn, double* s,
                     double* resid) {
  kb_fg_givens<<<dim3(1, unsigned(ns)), 32, 0, c->stream>>>(ldh, i, H, cs, sn, s, resid, bt);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

void fg_update_batch(pm_ctx* c, int ns, const Batch& bt, int n, int ldh, int k, const double* H, const double* s,
                     double* y, const double* Z, size_t ldz, double* x) {
  kb_fg_backsolve<<<dim3(1, unsigned(ns)), 32, 0, c->stream>>>(ldh, k, H, s, y, bt);
  kb_fg_combine<<<dim3(unsigned(grid_blocks_for(n)), unsigned(ns)), 256, 0, c->stream>>>(n, k, Z, ldz, y, x, bt);
  PM_CHECK_LAUNCH();
  c->kernel_launches += 2;
}

}  // namespace pm

using namespace pm;

// ------------------------------------------------------------- solver ------
void pm_solver::ensure_work(size_t n_vectors, int n) {
  const size_t need = n_vectors * size_t(n);
  if (work.n < need || work_n != size_t(n)) {
    drop_graphs();
    if (work.n < need) work.alloc(need);
  }
  work_n = size_t(n);
}

void pm_solver::drop_graphs() {
  for (auto& g : arnoldi_graphs)
    if (g) cudaGraphExecDestroy(g);
  arnoldi_graphs.clear();
  arnoldi_launches.clear();
}

pm_solver::~pm_solver() { drop_graphs(); }

// hash of every device address a captured Arnoldi step reads or writes
size_t pm_solver::layout_signature() const {
  size_t h = 1469598103934665603ull;
  auto mix = [&h](const void* p) {
    h ^= reinterpret_cast<size_t>(p);
    h *= 1099511628211ull;
  };
  // the sliced copies are chosen per launch by the context's kernel options
  auto mix_csr = [&mix](const DevCsr& M) {
    mix(M.vals.p); mix(M.vals32.p); mix(M.diag.p); mix(M.diag32.p);
    mix(M.row_ptr.p); mix(M.cols.p); mix(M.rblock.p);
    mix(M.sell_perm.p); mix(M.sell_off.p); mix(M.sell_cols.p); mix(M.sell_vals.p); mix(M.sell_vals64.p);
  };
  mix(A);
  if (A) mix_csr(A->csr);
  for (const auto& lv : mg.levels) {
    mix(lv.A);
    if (lv.A) mix_csr(lv.A->csr);
    if (lv.proj) mix_csr(lv.proj->csr);
    mix_csr(lv.P);
    mix_csr(lv.R);
    mix(lv.rhs.p); mix(lv.sol.p); mix(lv.alt.p); mix(lv.defect.p);
    mix(lv.rhs32.p); mix(lv.sol32.p); mix(lv.alt32.p); mix(lv.defect32.p);
    mix(lv.coarse.inv.p); mix(lv.coarse.act.p); mix(lv.coarse.pos.p); mix(lv.coarse.tmp.p);
    mix(lv.coarse.inv32.p);
    mix(lv.coarse_rhs64.p); mix(lv.coarse_sol64.p);
    mix(lv.sor.rows.p);
    h ^= lv.sor.ptr.size();
  }
  // the SOR preconditioner's colours (a new structure gives new launches)
  mix(sor.rows.p);
  h ^= sor.ptr.size() * 977;
  mix(work.p); mix(gm.p); mix(flags.p);
  mix(ctx->partials.p); mix(ctx->host_scalars);
  h ^= size_t(restart) * 31 + size_t(work_n);
  h = h * 1099511628211ull ^ size_t(ctx->sell_shape);
  h = h * 1099511628211ull ^ (size_t(ctx->sell_shape64) * 8 + size_t(ctx->pdl) * 2 + size_t(ctx->jacobi_zero_start));
  return h;
}

bool pm_solver::converged(double r, unsigned it) {
  if (it == 0) {
    init_res = r;
    prev_res = r;
    history.clear();
  }
  history.push_back(r);
  const bool small = r < tol;
  const bool red = r < reduction * init_res;
  const bool enough = it > (unsigned long)min_it || min_it == 0;
  const bool stag = r > stagnation * prev_res;
  const bool div = r > divergence * init_res;
  bool conv = (small || red || stag || div) && enough;
  if (it == (unsigned long)max_it) conv = true;
  prev_res = r;
  last_it = int(it);
  last_res = r;
  if (div)
    throw Error(PM_E_DIVERGED, "Execution of the code stopped because of solver divergence.");
  if (!std::isfinite(r)) throw Error(PM_E_DIVERGED, "residual is not finite");
  return conv;
}

void pm_solver::precondition(const double* z, double* r, bool z_nonactive_zero) {
  const int n = A->csr.n_rows;
  if (use_mg) {
    mg.apply(ctx, z, r, z_nonactive_zero);
  } else if (prec == "jacobi") {
    // Iteration_jacobi::apply: r = z / diag
    vcopy(ctx, n, z, r);
    vdiv(ctx, n, A->csr.diag.p, r);
  } else if (prec == "sor" || prec == "ssor") {
    // Iteration_sor::apply (src/Solver/Iteration_sor.C:75): r = 0, one sweep
    vset(ctx, n, r, 0.0);
    sor_sweep(ctx, A->csr, sor, z, r, sor_omega, false);
    if (prec == "ssor") sor_sweep(ctx, A->csr, sor, z, r, sor_omega, true);
  } else {
    vcopy(ctx, n, z, r);
  }
}

void pm_solver::fgmres(const double* rhs, double* sol) {
  pm_ctx* c = ctx;
  const DevCsr& M = A->csr;
  const int n = M.n_rows;
  const int m = int(restart);
  if (m > 60) throw Error(PM_E_UNSUPPORTED, "gmres_restart above 60");
  const int ldh = m + 1;
  ensure_work(size_t(2 * m + 2), n);
  double* r = work.p;
  double* V = work.p + work_n;                     // m+1 vectors
  double* Z = work.p + work_n * size_t(m + 2);     // m vectors
  const size_t ld = work_n;
  const size_t gm_need = size_t(ldh) * m + 4 * size_t(m + 1) + 8 + 64 * size_t(kRedBlocks) + 128;
  if (gm.n != gm_need) {
    drop_graphs();
    gm.alloc(gm_need);
  }
  double* H = gm.p;
  double* s = H + size_t(ldh) * m;
  double* cs = s + (m + 1);
  double* sn = cs + (m + 1);
  double* y = sn + (m + 1);
  double* dres = y + (m + 1);
  double* cgs_part = dres + 8;                 // 64 x kRedBlocks partial sums
  double* h1 = cgs_part + 64 * size_t(kRedBlocks);
  double* h2 = h1 + 64;
  if (flags.n < 3) {  // [0] breakdown, [1] skip of the second Gram-Schmidt pass, [2] non-zero non-actives
    drop_graphs();
    flags.alloc(3);
  }
  PM_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(int), c->stream));
  PM_CUDA(cudaMemsetAsync(H, 0, sizeof(double) * size_t(ldh) * m, c->stream));
  double* partA = c->partials.p;
  double* partB = c->partials.p + kRedBlocks;
  if (use_mg && mg.mixed_cfg) mg.set_mixed(c, true);  // every solve starts in the mixed form
  std::vector<double> res_hist;  // residual after each iteration (for the fallback test)

  csr_apply(c, M, EPI_DEFECT, sol, r, rhs, 1.0);  // r = rhs - A sol
  // exact zeros in the non-active entries of the initial residual carry over
  // to every basis vector (A's non-active rows are unit rows and the
  // multigrid copies non-actives through): the cycles may then start the
  // finest level from an exactly zero iterate
  PM_CUDA(cudaMemsetAsync(flags.p + 2, 0, sizeof(int), c->stream));
  nonactive_nonzero(c, M.mask, r, flags.p + 2);
  dot_partials(c, n, r, r, partA);
  finish_sum(c, partA, dres, true);
  PM_CUDA(cudaMemcpyAsync(c->host_scalars, dres, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaMemcpyAsync(reinterpret_cast<int*>(c->host_scalars + 2), flags.p + 2, sizeof(int),
                          cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));
  double resid = c->host_scalars[0];
  const bool na_zero = *reinterpret_cast<int*>(c->host_scalars + 2) == 0;
  {
    // the captured Arnoldi steps depend on the buffers and on na_zero
    const size_t sig = layout_signature() * 1099511628211ull ^ (na_zero ? 0x9e3779b9ull : 0ull);
    if (sig != graphs_signature) {
      drop_graphs();
      graphs_signature = sig;
    }
  }
  if (converged(resid, 0)) return;

  const int grid = kRedBlocks;
  const bool cgs_cond = gram_schmidt == "cgs2_cond";
  const bool cgs2 = gram_schmidt == "cgs2" || cgs_cond;
  unsigned j = 1;
  while (j <= (unsigned long)max_it) {
    // v_0 = r / beta, s = (beta, 0, ...)   (partA holds <r,r>)
    k_fg_start<<<grid, 256, 0, c->stream>>>(n, m, r, V, partA, s, dres + 1);
    PM_CHECK_LAUNCH();
    c->kernel_launches++;
    int i = 0;
    bool done = false;
    bool restart_fp64 = false;
    for (; i < m && j <= (unsigned long)max_it; ++i, ++j) {
      // one Arnoldi step: z_i = M^-1 v_i, r = A z_i, modified Gram-Schmidt,
      // H(i+1,i), v_{i+1}, Givens rotation, residual copied to the host
      auto arnoldi_step = [&]() {
        double* vi = V + ld * i;
        double* zi = Z + ld * i;
        precondition(vi, zi, na_zero);
        csr_apply(c, M, EPI_SET, zi, r, nullptr, 1.0);  // r = A z_i
        double* pin = partA;
        if (cgs2 && !cgs_cond && i + 1 <= kCgsFused) {
          // two classical Gram-Schmidt passes in three sweeps over the basis;
          // H(:,i) = h1 + h2, |r|^2 partials into partA
          const int nk = i + 1;
          const dim3 rb(kRedBlocks), t256(256);
          const double* Vc = V;
          const double* nul = nullptr;
          const int* inul = nullptr;
          if (nk <= 16) launch_k(c, k_mdot<16>, rb, t256, 0, n, nk, (const double*)r, Vc, ld, cgs_part);
          else launch_k(c, k_mdot<kCgsFused>, rb, t256, 0, n, nk, (const double*)r, Vc, ld, cgs_part);
          launch_k(c, k_reduce_proj, dim3(nk), t256, 0, (const double*)cgs_part, h1, nul, H, ldh, i, inul);
          if (nk <= 16) launch_k(c, k_cgs_update_mdot<16>, rb, t256, 0, n, nk, r, Vc, ld, (const double*)h1, cgs_part);
          else launch_k(c, k_cgs_update_mdot<kCgsFused>, rb, t256, 0, n, nk, r, Vc, ld, (const double*)h1, cgs_part);
          launch_k(c, k_reduce_proj, dim3(nk), t256, 0, (const double*)cgs_part, h2, (const double*)h1, H, ldh, i,
                     inul);
          launch_k(c, k_cgs_update_norm, rb, t256, 0, n, nk, r, Vc, ld, (const double*)h2, partA);
        } else if (cgs2) {
          // two passes of classical Gram-Schmidt; H(:,i) = h1 + h2. With the
          // conditional variant the second pass runs only when the first lost
          // more than a factor 1/sqrt(2) of the norm (decided on the device)
          const int nk = i + 1;
          const int ub = grid_blocks_for(n);
          k_multidot<8><<<kRedBlocks, 256, 0, c->stream>>>(n, nk, r, V, ld, cgs_part, cgs_cond ? 1 : 0, nullptr);
          k_reduce_proj<<<nk + (cgs_cond ? 1 : 0), 256, 0, c->stream>>>(cgs_part, h1, nullptr, H, ldh, i, nullptr);
          k_cgs_update<<<ub, 256, 0, c->stream>>>(n, nk, r, V, ld, h1, nullptr);
          const int* skip = nullptr;
          if (cgs_cond) {
            dot_partials(c, n, r, r, partB);
            k_cgs_decide<<<1, 256, 0, c->stream>>>(partB, h1 + nk, flags.p + 1);
            c->kernel_launches++;
            skip = flags.p + 1;
          }
          k_multidot<8><<<kRedBlocks, 256, 0, c->stream>>>(n, nk, r, V, ld, cgs_part, 0, skip);
          k_reduce_proj<<<nk, 256, 0, c->stream>>>(cgs_part, h2, h1, H, ldh, i, skip);
          k_cgs_update<<<ub, 256, 0, c->stream>>>(n, nk, r, V, ld, h2, skip);
          PM_CHECK_LAUNCH();
          c->kernel_launches += 6;
          dot_partials(c, n, r, r, partA);
        } else {
          // modified Gram-Schmidt in the reference's order (Iteration_gmres.C:452-461)
          dot_partials(c, n, r, V, partA);                   // <r, v_0>
          double* pout = partB;
          for (int k = 0; k <= i; ++k) {
            const double* next = (k < i) ? V + ld * (k + 1) : r;
            k_fg_mgs<<<grid, 256, 0, c->stream>>>(n, ldh, k, i, r, V + ld * k, next, pin, pout, H);
            PM_CHECK_LAUNCH();
            c->kernel_launches++;
            std::swap(pin, pout);
          }
        }
        launch_k(c, k_fg_normalize, dim3(grid), dim3(256), 0, n, ldh, i, (const double*)r, V + ld * (i + 1),
                   (const double*)pin, H, flags.p);
        launch_k(c, k_fg_givens, dim3(1), dim3(32), 0, ldh, i, H, cs, sn, s, dres);
        PM_CUDA(cudaMemcpyAsync(c->host_scalars, dres, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        PM_CUDA(cudaMemcpyAsync(reinterpret_cast<int*>(c->host_scalars + 1), flags.p, sizeof(int),
                                cudaMemcpyDeviceToHost, c->stream));
      };
      // the probe brackets launches with events one by one: no graphs then
      const bool graphs = use_graphs && c->probe_nnz == 0 && !c->probe_nodal;
      // one graph per Arnoldi index and multigrid precision
      const int gi = i + ((use_mg && !mg.mixed && mg.mixed_cfg) ? m : 0);
      if (graphs) {
        if (arnoldi_graphs.size() != size_t(2 * m)) {
          drop_graphs();
          arnoldi_graphs.assign(2 * m, nullptr);
          arnoldi_launches.assign(2 * m, 0);
        }
        if (!arnoldi_graphs[gi]) {
          const uint64_t before = c->kernel_launches;
          cudaGraph_t g = nullptr;
          PM_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
          try {
            arnoldi_step();
          } catch (...) {
            cudaStreamEndCapture(c->stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
          }
          PM_CUDA(cudaStreamEndCapture(c->stream, &g));
          cudaGraphExec_t ex = nullptr;
          cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
          cudaGraphDestroy(g);
          PM_CUDA(e);
          arnoldi_graphs[gi] = ex;
          arnoldi_launches[gi] = c->kernel_launches - before;
          c->kernel_launches = before;
        }
        PM_CUDA(cudaGraphLaunch(arnoldi_graphs[gi], c->stream));
        c->kernel_launches += arnoldi_launches[gi];
      } else {
        arnoldi_step();
      }
      PM_CUDA(cudaStreamSynchronize(c->stream));
      resid = c->host_scalars[0];
      if (*reinterpret_cast<int*>(c->host_scalars + 1))
        throw Error(PM_E_BREAKDOWN, "Unhappy breakdown in flexible gmres Iteration " + std::to_string(j));
      if (!std::isfinite(resid) && use_mg && mg.mixed && mixed_fallback) {
        // the FP32 cycle overflowed: the cycle's Krylov basis is lost; restart
        // from the current solution with the FP64 multigrid
        mg.set_mixed(c, false);
        restart_fp64 = true;
        break;
      }
      res_hist.push_back(resid);
      if (use_mg && mg.mixed && mixed_fallback && res_hist.size() > 10 &&
          !(resid <= 0.5 * res_hist[res_hist.size() - 11]))
        mg.set_mixed(c, false);  // the FP32 cycle stalled: FP64 from the next iteration on
      if (converged(resid, j)) {
        k_fg_backsolve<<<1, 32, 0, c->stream>>>(ldh, i, H, s, y);
        k_fg_combine<<<grid_blocks_for(n), 256, 0, c->stream>>>(n, i, Z, ld, y, sol);
        PM_CHECK_LAUNCH();
        c->kernel_launches += 2;
        done = true;
        break;
      }
    }
    if (done) return;
    if (restart_fp64) {
      // the solution is unchanged since the start of this cycle
      csr_apply(c, M, EPI_DEFECT, sol, r, rhs, 1.0);
      dot_partials(c, n, r, r, partA);
      finish_sum(c, partA, dres, true);
      PM_CUDA(cudaMemcpyAsync(c->host_scalars, dres, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      PM_CUDA(cudaStreamSynchronize(c->stream));
      resid = c->host_scalars[0];
      if (converged(resid, j)) return;
      ++j;  // the lost iteration counts
      continue;
    }
    k_fg_backsolve<<<1, 32, 0, c->stream>>>(ldh, m - 1, H, s, y);
    k_fg_combine<<<grid_blocks_for(n), 256, 0, c->stream>>>(n, m - 1, Z, ld, y, sol);
    PM_CHECK_LAUNCH();
    c->kernel_launches += 2;
    csr_apply(c, M, EPI_DEFECT, sol, r, rhs, 1.0);
    dot_partials(c, n, r, r, partA);
    if (converged(resid, j)) return;
  }
}


// Iteration_cg::iterate (src/Solver/Iteration_cg.C:22-79)
void pm_solver::cg(const double* rhs, double* sol) {
  pm_ctx* c = ctx;
  const DevCsr& M = A->csr;
  const int n = M.n_rows;
  ensure_work(4, n);
  double *r = work.p, *z = r + work_n, *p = z + work_n, *q = p + work_n;
  csr_apply(c, M, EPI_DEFECT, sol, r, rhs, 1.0);
  double normb = std::sqrt(dot_host(c, n, rhs, rhs));
  if (normb == 0.0) normb = 1.0;
  double resid = std::sqrt(dot_host(c, n, r, r)) / normb;
  if (converged(resid, 0)) return;
  double rho_1 = 0.0;
  for (unsigned i = 1; i <= (unsigned long)max_it; ++i) {
    precondition(r, z);
    const double rho = dot_host(c, n, r, z);
    if (i == 1) vcopy(c, n, z, p);
    else vaxpby(c, n, 1.0, z, rho / rho_1, p);  // p = beta p + z
    csr_apply(c, M, EPI_SET, p, q, nullptr, 1.0);
    const double alpha = rho / dot_host(c, n, p, q);
    vaxpy(c, n, alpha, p, sol);
    vaxpy(c, n, -alpha, q, r);
    resid = std::sqrt(dot_host(c, n, r, r)) / normb;
    if (converged(resid, i)) return;
    rho_1 = rho;
  }
}

// Iteration_bicgstab::iterate (src/Solver/Iteration_bicgstab.C:28-206)
void pm_solver::bicgstab(const double* rhs, double* sol) {
  pm_ctx* c = ctx;
  const DevCsr& M = A->csr;
  const int n = M.n_rows;
  ensure_work(8, n);
  double *r = work.p, *rt = r + work_n, *p = rt + work_n, *ph = p + work_n, *s = ph + work_n,
         *sh = s + work_n, *t = sh + work_n, *v = t + work_n;
  double rho_2 = 1.0, alpha = 1.0, omega = 1.0;
  csr_apply(c, M, EPI_DEFECT, sol, r, rhs, 1.0);
  vcopy(c, n, r, rt);
  double normb = std::sqrt(dot_host(c, n, rhs, rhs));
  if (normb == 0.0) normb = 1.0;
  double resid = std::sqrt(dot_host(c, n, r, r)) / normb;
  if (converged(resid, 0)) return;
  for (unsigned i = 1; i <= (unsigned long)max_it; ++i) {
    const double rho_1 = dot_host(c, n, rt, r);
    if (rho_1 == 0.0) {
      last_it = int(i);
      last_res = std::sqrt(dot_host(c, n, r, r)) / normb;
      return;
    }
    if (i == 1) vcopy(c, n, r, p);
    else {
      const double beta = (rho_1 / rho_2) * (alpha / omega);
      vaxpy(c, n, -omega, v, p);
      vaxpby(c, n, 1.0, r, beta, p);  // p = beta p + r
    }
    precondition(p, ph);
    csr_apply(c, M, EPI_SET, ph, v, nullptr, 1.0);
    alpha = rho_1 / dot_host(c, n, rt, v);
    vcopy(c, n, r, s);
    vaxpy(c, n, -alpha, v, s);
    resid = std::sqrt(dot_host(c, n, s, s)) / normb;
    if (converged(resid, i)) {
      vaxpy(c, n, alpha, ph, sol);
      return;
    }
    precondition(s, sh);
    csr_apply(c, M, EPI_SET, sh, t, nullptr, 1.0);
    omega = dot_host(c, n, t, s) / dot_host(c, n, t, t);
    vaxpy(c, n, alpha, ph, sol);
    vaxpy(c, n, omega, sh, sol);
    vcopy(c, n, s, r);
    vaxpy(c, n, -omega, t, r);
    rho_2 = rho_1;
    resid = std::sqrt(dot_host(c, n, r, r)) / normb;
    if (converged(resid, i)) return;
    if (omega == 0.0)
      throw Error(PM_E_BREAKDOWN, "unhappy breakdown in Bi-CGStab. iteration " + std::to_string(i));
  }
}

// Iteration_jacobi::iterate (src/Solver/Iteration_jacobi.C:31-90)
void pm_solver::jacobi_iter(const double* rhs, double* sol) {
  pm_ctx* c = ctx;
  const DevCsr& M = A->csr;
  const int n = M.n_rows;
  if (!M.diag.p) A->csr.make_diag(c);
  ensure_work(2, n);
  double *r = work.p, *xn = r + work_n;
  csr_apply(c, M, EPI_DEFECT, sol, r, rhs, 1.0);
  double normb = std::sqrt(dot_host(c, n, rhs, rhs));
  if (normb == 0.0) normb = 1.0;
  double resid = std::sqrt(dot_host(c, n, r, r)) / normb;
  if (converged(resid, 0)) return;
  for (unsigned i = 1; i <= (unsigned long)max_it; ++i) {
    // x_new = x + w D^{-1}(b - A x); the fused sweep computes the defect itself
    csr_apply(c, M, EPI_JACOBI, sol, xn, rhs, damping);
    vcopy(c, n, xn, sol);
    csr_apply(c, M, EPI_DEFECT, sol, r, rhs, 1.0);
    resid = std::sqrt(dot_host(c, n, r, r)) / normb;
    if (converged(resid, i)) return;
  }
}

// Iteration_sor::iterate (src/Solver/Iteration_sor.C:24-60): one (S)SOR sweep
// per iteration in the colour order, then the defect for the stopping test
void pm_solver::sor_iter(const double* rhs, double* sol, bool symmetric) {
  pm_ctx* c = ctx;
  const DevCsr& M = A->csr;
  const int n = M.n_rows;
  ensure_work(1, n);
  double* r = work.p;
  csr_apply(c, M, EPI_DEFECT, sol, r, rhs, 1.0);
  double normb = std::sqrt(dot_host(c, n, rhs, rhs));
  if (normb == 0.0) normb = 1.0;
  double resid = std::sqrt(dot_host(c, n, r, r)) / normb;
  if (converged(resid, 0)) return;
  for (unsigned i = 1; i <= (unsigned long)max_it; ++i) {
    sor_sweep(c, M, sor, rhs, sol, sor_omega, false);
    if (symmetric) sor_sweep(c, M, sor, rhs, sol, sor_omega, true);
    csr_apply(c, M, EPI_DEFECT, sol, r, rhs, 1.0);
    resid = std::sqrt(dot_host(c, n, r, r)) / normb;
    if (converged(resid, i)) return;
  }
}

// Iteration_richardson::iterate (src/Solver/Iteration_richardson.C:24-110):
// x += damping * P^{-1}(b - A x) with the configured preconditioner
void pm_solver::richardson(const double* rhs, double* sol) {
  pm_ctx* c = ctx;
  const DevCsr& M = A->csr;
  const int n = M.n_rows;
  ensure_work(2, n);
  double *r = work.p, *z = r + work_n;
  double normb = std::sqrt(dot_host(c, n, rhs, rhs));
  if (normb == 0.0) normb = 1.0;
  csr_apply(c, M, EPI_DEFECT, sol, r, rhs, 1.0);
  double resid = std::sqrt(dot_host(c, n, r, r)) / normb;
  if (converged(resid, 0)) return;
  for (unsigned i = 1; i <= (unsigned long)max_it; ++i) {
    precondition(r, z, false);
    vaxpy(c, n, damping, z, sol);
    csr_apply(c, M, EPI_DEFECT, sol, r, rhs, 1.0);
    resid = std::sqrt(dot_host(c, n, r, r)) / normb;
    if (converged(resid, i)) return;
  }
}

// Iteration_cgs::iterate (src/Solver/Iteration_cgs.C:22-110): conjugate
// gradient squared with right preconditioning
void pm_solver::cgs(const double* rhs, double* sol) {
  pm_ctx* c = ctx;
  const DevCsr& M = A->csr;
  const int n = M.n_rows;
  ensure_work(9, n);
  double* r = work.p;
  double* rt = r + work_n;
  double* p = rt + work_n;
  double* ph = p + work_n;
  double* q = ph + work_n;
  double* u = q + work_n;
  double* uh = u + work_n;
  double* qh = uh + work_n;
  double* vh = qh + work_n;
  csr_apply(c, M, EPI_DEFECT, sol, r, rhs, 1.0);
  vcopy(c, n, r, rt);
  double normb = std::sqrt(dot_host(c, n, rhs, rhs));
  if (normb == 0.0) normb = 1.0;
  double resid = std::sqrt(dot_host(c, n, r, r)) / normb;
  if (converged(resid, 0)) return;
  double rho_2 = 0.0;
  for (unsigned i = 1; i <= (unsigned long)max_it; ++i) {
    const double rho_1 = dot_host(c, n, rt, r);
    if (rho_1 == 0.0) {
      last_it = int(i);
      last_res = std::sqrt(dot_host(c, n, r, r)) / normb;
      return;
    }
    if (i == 1) {
      vcopy(c, n, r, u);
      vcopy(c, n, u, p);
    } else {
      const double beta = rho_1 / rho_2;
      vcopy(c, n, q, u);
      vscale(c, n, u, beta);
      vaxpy(c, n, 1.0, r, u);     // u = beta q + r
      vscale(c, n, p, beta);
      vaxpy(c, n, 1.0, q, p);
      vscale(c, n, p, beta);
      vaxpy(c, n, 1.0, u, p);     // p = beta (beta p + q) + u
    }
    precondition(p, ph);
    csr_apply(c, M, EPI_SET, ph, vh, nullptr, 1.0);
    const double alpha = rho_1 / dot_host(c, n, rt, vh);
    vcopy(c, n, u, q);
    vaxpy(c, n, -alpha, vh, q);   // q = u - alpha vhat
    vaxpy(c, n, 1.0, q, u);       // u = u + q
    precondition(u, uh);
    vaxpy(c, n, alpha, uh, sol);
    csr_apply(c, M, EPI_SET, uh, qh, nullptr, 1.0);
    vaxpy(c, n, -alpha, qh, r);   // r += -alpha qhat
    rho_2 = rho_1;
    resid = std::sqrt(dot_host(c, n, r, r)) / normb;
    if (converged(resid, i)) return;
  }
}

// Iteration_gmres::left_gmres (src/Solver/Iteration_gmres.C:173-268): GMRES on
// P^{-1} A with the preconditioned residual as the stopping quantity; the
// Arnoldi step is the reference's modified Gram-Schmidt (v_k scaled by h,
// subtracted, scaled back), host Givens rotations
void pm_solver::left_gmres(const double* rhs, double* sol) {
  pm_ctx* c = ctx;
  const DevCsr& M = A->csr;
  const int n = M.n_rows;
  const int m = int(restart);
  ensure_work(size_t(m) + 4, n);
  double* a = work.p;
  double* w = a + work_n;
  double* r = w + work_n;
  auto V = [&](int k) { return r + size_t(k + 1) * work_n; };
  std::vector<double> Hm(size_t(m + 1) * size_t(m + 1), 0.0), s(size_t(m) + 1), cs(size_t(m) + 1),
      sn(size_t(m) + 1);
  auto Hij = [&](int i, int j) -> double& { return Hm[size_t(i) * size_t(m + 1) + size_t(j)]; };
  auto gen = [](double dx, double dy, double& c_, double& s_) {
    if (dy == 0.0) { c_ = 1.0; s_ = 0.0; }
    else if (std::fabs(dy) > std::fabs(dx)) { const double t = dx / dy; s_ = 1.0 / std::sqrt(1.0 + t * t); c_ = t * s_; }
    else { const double t = dy / dx; c_ = 1.0 / std::sqrt(1.0 + t * t); s_ = t * c_; }
  };
  auto app = [](double& dx, double& dy, double c_, double s_) {
    const double t = c_ * dx + s_ * dy;
    dy = -s_ * dx + c_ * dy;
    dx = t;
  };
  // x += sum_k y_k v_k with H y = s (upper triangular, rows 0..k)
  auto update = [&](int k) {
    std::vector<double> y(s.begin(), s.end());
    for (int i = k; i >= 0; --i) {
      y[size_t(i)] /= Hij(i, i);
      for (int j = i - 1; j >= 0; --j) y[size_t(j)] -= Hij(j, i) * y[size_t(i)];
    }
    for (int j = 0; j <= k; ++j) vaxpy(c, n, y[size_t(j)], V(j), sol);
  };
  csr_apply(c, M, EPI_DEFECT, sol, a, rhs, 1.0);
  precondition(a, r);
  double resid = std::sqrt(dot_host(c, n, r, r));
  double beta = resid;
  if (converged(resid, 0)) return;
  unsigned j = 1;
  while (j <= (unsigned long)max_it) {
    vcopy(c, n, r, V(0));
    vscale(c, n, V(0), 1.0 / beta);
    std::fill(s.begin(), s.end(), 0.0);
    s[0] = beta;
    for (int i = 0; i < m && j <= (unsigned long)max_it; ++i, ++j) {
      csr_apply(c, M, EPI_SET, V(i), a, nullptr, 1.0);
      precondition(a, w);
      for (int k = 0; k <= i; ++k) {
        const double h = dot_host(c, n, w, V(k));
        Hij(k, i) = h;
        if (h != 0.0) {
          vscale(c, n, V(k), h);
          vaxpy(c, n, -1.0, V(k), w);
          vscale(c, n, V(k), 1.0 / h);
        }
      }
      Hij(i + 1, i) = std::sqrt(dot_host(c, n, w, w));
      vcopy(c, n, w, V(i + 1));
      vscale(c, n, V(i + 1), 1.0 / Hij(i + 1, i));
      for (int k = 0; k < i; ++k) app(Hij(k, i), Hij(k + 1, i), cs[size_t(k)], sn[size_t(k)]);
      gen(Hij(i, i), Hij(i + 1, i), cs[size_t(i)], sn[size_t(i)]);
      app(Hij(i, i), Hij(i + 1, i), cs[size_t(i)], sn[size_t(i)]);
      app(s[size_t(i)], s[size_t(i) + 1], cs[size_t(i)], sn[size_t(i)]);
      resid = std::fabs(s[size_t(i) + 1]);
      if (converged(resid, j)) {
        update(i);
        return;
      }
    }
    update(m - 1);
    csr_apply(c, M, EPI_DEFECT, sol, a, rhs, 1.0);
    precondition(a, r);
    beta = std::sqrt(dot_host(c, n, r, r));
    if (converged(resid, j)) return;
  }
}

void pm_solver::solve(const double* rhs, double* sol) {
  if (!A) throw Error(PM_E_INVALID, "Solver::solve called before update_matrix");
  history.clear();
  if (solver_type == "direct") {
    if (!direct_ready) {
      direct.build(ctx, A->csr);
      direct_ready = true;
    }
    direct.solve(ctx, A->csr, rhs, sol);
    last_it = 1;
    last_res = 0.0;
    return;
  }
  if (method == "fgmres" || method == "right_gmres") fgmres(rhs, sol);
  else if (method == "cg") cg(rhs, sol);
  else if (method == "bi_cgstab") bicgstab(rhs, sol);
  else if (method == "jacobi") jacobi_iter(rhs, sol);
  else if (method == "sor" || method == "ssor") sor_iter(rhs, sol, method == "ssor");
  else if (method == "richardson") richardson(rhs, sol);
  else if (method == "cgs") cgs(rhs, sol);
  else if (method == "left_gmres") left_gmres(rhs, sol);
  else throw Error(PM_E_UNSUPPORTED, "iterative_solver_type '" + method + "' is not implemented on the GPU");
}
