// BatchEngine (pm_batch.h): FGMRES with a geometric multigrid preconditioner
// for up to kMaxBatch convection-diffusion problems of one set-up, advanced
// in lockstep so that every kernel of an Arnoldi step serves all slots in one
// launch (blockIdx.y = slot).
//
// The algorithm per slot is pm_solver::fgmres with the fused CGS2
// orthogonalisation and Multigrid::apply with damped Jacobi smoothing and the
// direct coarse solve (src/Solver/Iteration_gmres.C:376-532,
// src/Multigrid/Multigrid.C:200-420, src/Multigrid/JacobiSmoother.C:22), with
// the same kernels bodies, launch shapes and reduction trees: a slot's
// iterates are the bits a lone solve of its problem produces.
//
// Memory: the matrices, diagonals and coarse inverses stay in each slot's
// problem (pm_problem, assembled and updated by the caller); the engine owns
// one block per slot with the slot's FGMRES state (residual, m+1 basis
// vectors, m preconditioned vectors, Hessenberg matrix, rotations, partial
// sums), its solution and right-hand side, and its multigrid vectors, so every
// vector argument of a batched launch is slot 0's pointer plus blockIdx.y
// times the block size. Per-slot matrix pointers come from small device
// tables, refreshed when a slot gets another problem.
//
// Lockstep: the slots run the same Arnoldi index i. A problem joins at a
// restart-cycle boundary (its first cycle starts with the others' next one)
// and leaves as soon as its residual test passes; launches skip slots that are
// not in the current phase (per-slot masks in device memory). Each Arnoldi
// step of the batch is one CUDA graph, captured once per index and precision
// and valid for any slot composition (masks and tables are read at run time).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "pm_batch.h"
#include "pm_problem.h"

namespace pm {

namespace {

enum MaskKind { MASK_STEP = 0, MASK_CYCLE = 1, MASK_FINAL = 2, N_MASKS = 3 };

struct SlotState {
  pm_problem* p = nullptr;
  bool in_cycle = false;   // takes part in the current restart cycle
  bool is_new = false;     // joined at this boundary
  unsigned j = 1;          // Iteration_gmres loop index of the next Arnoldi step
  double init_res = 0.0, prev_res = 0.0, last_res = 0.0;
  int last_it = 0;
  bool na_zero = true;     // the initial residual has exact-zero non-actives
};

}  // namespace

class BatchEngine {
 public:
  pm_ctx* c = nullptr;
  int B = 0;               // slots
  int L = 0;               // multigrid levels
  int m = 30;              // restart
  bool mixed = false;
  int n_pre = 2, n_post = 2;
  double jacobi_damp = 1.0, correction_damp = 1.0;
  std::vector<int> control;
  double tol = 1e-8, reduction = 0.0, divergence = 1e10, stagnation = 1e10;
  long max_it = 100, min_it = 0;
  pm_problem* templ = nullptr;   // structure, shapes and transfer operators of the set-up
  std::vector<int> n_lvl;        // rows per level
  // slot block layout (byte offsets)
  size_t S = 0;
  size_t off_r = 0, off_V = 0, off_Z = 0, off_x = 0, off_b = 0, off_gm = 0, off_flags = 0;
  size_t ld = 0;                 // doubles between basis vectors
  size_t off_H = 0, off_s = 0, off_cs = 0, off_sn = 0, off_y = 0, off_dres = 0, off_cgs = 0, off_h1 = 0,
         off_h2 = 0, off_pA = 0, off_pB = 0;
  std::vector<size_t> off_rhs, off_sol, off_alt, off_def;  // per level (FP32 or FP64 by the form)
  DBuf<char> block;
  // device tables: per level [2B] matrix values (sliced, CSR) and [B]
  // diagonals, in FP32 (mixed cycle) and FP64 (FGMRES SpMV, FP64 cycle);
  // [B] coarse inverses
  DBuf<const void*> tab;
  std::vector<const void*> htab;
  std::vector<size_t> t_v32, t_d32, t_v64, t_d64;
  size_t t_inv = 0;
  DBuf<int> masks;         // [N_MASKS][B]
  // host copy of the masks; upload_masks() copies it into one of kStage
  // pinned staging buffers whose previous copy has completed, so the host
  // may change the masks again while an upload is still queued
  std::vector<int> hmask;
  static constexpr int kStage = 8;
  int* stage = nullptr;    // pinned, kStage x N_MASKS x B
  cudaEvent_t stage_done[kStage] = {};
  int stage_next = 0;
  double* hres = nullptr;  // pinned: per slot residual and flags read-back
  int* hflag = nullptr;
  std::vector<SlotState> slots;
  std::vector<cudaGraphExec_t> graphs;  // [na_zero][i]
  uint64_t graph_launches[2][64] = {};

  ~BatchEngine() {
    for (auto g : graphs)
      if (g) cudaGraphExecDestroy(g);
    for (auto e : stage_done)
      if (e) cudaEventDestroy(e);
    if (stage) cudaFreeHost(stage);
    if (hres) cudaFreeHost(hres);
    if (hflag) cudaFreeHost(hflag);
  }

  template <class T>
  T* at(size_t off) const { return reinterpret_cast<T*>(block.p + off); }
  Batch bt(MaskKind k, size_t vals_tab = SIZE_MAX, size_t aux_tab = SIZE_MAX) const {
    Batch b;
    b.on = masks.p + size_t(k) * B;
    b.stride = (long long)S;
    b.vals = vals_tab == SIZE_MAX ? nullptr : tab.p + vals_tab;
    b.aux = aux_tab == SIZE_MAX ? nullptr : tab.p + aux_tab;
    return b;
  }
  const DevCsr& A(int l) const { return templ->mats[size_t(l)]->csr; }
  const MGLevel& lvl(int l) const { return templ->solver->mg.levels[size_t(l)]; }

  void layout();
  void set_tables(int s, pm_problem* p);
  void upload_masks() {
    const size_t cnt = size_t(N_MASKS) * B;
    const int k = stage_next;
    stage_next = (stage_next + 1) % kStage;
    PM_CUDA(cudaEventSynchronize(stage_done[k]));  // the buffer's previous copy has run
    int* buf = stage + size_t(k) * cnt;
    std::copy(hmask.begin(), hmask.end(), buf);
    PM_CUDA(cudaMemcpyAsync(masks.p, buf, sizeof(int) * cnt, cudaMemcpyHostToDevice, c->stream));
    PM_CUDA(cudaEventRecord(stage_done[k], c->stream));
  }
  // the batched pieces of the Arnoldi step
  void smooth(int l, std::vector<char>& cur_sol);
  void mg_apply(const double* z_in, double* r_out, bool na_zero);
  void arnoldi_step(int i, bool na_zero);
  bool slot_converged(SlotState& st, double r, unsigned it, int& status);
  std::vector<BatchDone> cycle(const std::vector<pm_problem*>& join);
};

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

void BatchEngine::layout() {
  const int n = n_lvl.back();
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o = align_up(o + bytes, 256);
    return at;
  };
  ld = align_up(size_t(n), 32);  // doubles between the basis vectors of a slot
  off_r = take(sizeof(double) * ld);
  off_V = take(sizeof(double) * ld * size_t(m + 1));
  off_Z = take(sizeof(double) * ld * size_t(m));
  off_x = take(sizeof(double) * ld);
  off_b = take(sizeof(double) * ld);
  const int ldh = m + 1;
  off_H = take(sizeof(double) * size_t(ldh) * m);
  off_s = take(sizeof(double) * size_t(m + 1));
  off_cs = take(sizeof(double) * size_t(m + 1));
  off_sn = take(sizeof(double) * size_t(m + 1));
  off_y = take(sizeof(double) * size_t(m + 1));
  off_dres = take(sizeof(double) * 8);
  off_cgs = take(sizeof(double) * 64 * size_t(kRedBlocks));
  off_h1 = take(sizeof(double) * 64);
  off_h2 = take(sizeof(double) * 64);
  off_pA = take(sizeof(double) * size_t(kRedBlocks));
  off_pB = take(sizeof(double) * size_t(kRedBlocks));
  off_flags = take(sizeof(int) * 4);
  const size_t eb = mixed ? sizeof(float) : sizeof(double);
  off_rhs.resize(size_t(L));
  off_sol.resize(size_t(L));
  off_alt.resize(size_t(L));
  off_def.resize(size_t(L));
  for (int l = 0; l < L; ++l) {
    const size_t nl = size_t(n_lvl[size_t(l)]);
    off_rhs[size_t(l)] = take(eb * nl);
    off_sol[size_t(l)] = take(eb * nl);
    off_alt[size_t(l)] = take(eb * nl);
    off_def[size_t(l)] = take(eb * nl);
  }
  S = align_up(o, 4096);
  block.alloc(S * size_t(B));
  PM_CUDA(cudaMemsetAsync(block.p, 0, S * size_t(B), c->stream));
  // tables
  size_t t = 0;
  t_v32.resize(size_t(L));
  t_d32.resize(size_t(L));
  t_v64.resize(size_t(L));
  t_d64.resize(size_t(L));
  for (int l = 0; l < L; ++l) {
    t_v32[size_t(l)] = t; t += 2 * size_t(B);
    t_d32[size_t(l)] = t; t += size_t(B);
    t_v64[size_t(l)] = t; t += 2 * size_t(B);
    t_d64[size_t(l)] = t; t += size_t(B);
  }
  t_inv = t; t += size_t(B);
  htab.assign(t, nullptr);
  tab.alloc(t);
  masks.alloc(size_t(N_MASKS) * B);
  hmask.assign(size_t(N_MASKS) * B, 0);
  PM_CUDA(cudaMallocHost(&stage, sizeof(int) * size_t(N_MASKS) * B * kStage));
  for (auto& e : stage_done) {
    PM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    PM_CUDA(cudaEventRecord(e, c->stream));
  }
  PM_CUDA(cudaMallocHost(&hres, sizeof(double) * size_t(B)));
  PM_CUDA(cudaMallocHost(&hflag, sizeof(int) * size_t(B) * 4));
  upload_masks();
}

// the slot's matrix values, diagonals and coarse inverse
void BatchEngine::set_tables(int s, pm_problem* p) {
  const auto& mg = p->solver->mg;
  for (int l = 0; l < L; ++l) {
    const DevCsr& M = p->mats[size_t(l)]->csr;
    htab[t_v32[size_t(l)] + 2 * size_t(s)] = M.sell_vals.p;
    htab[t_v32[size_t(l)] + 2 * size_t(s) + 1] = M.vals32.p;
    htab[t_d32[size_t(l)] + size_t(s)] = M.diag32.p;
    htab[t_v64[size_t(l)] + 2 * size_t(s)] = M.sell_vals64.p;
    htab[t_v64[size_t(l)] + 2 * size_t(s) + 1] = M.vals.p;
    htab[t_d64[size_t(l)] + size_t(s)] = M.diag.p;
  }
  const DenseInverse& inv = mg.levels[0].coarse;
  htab[t_inv + size_t(s)] = mixed ? static_cast<const void*>(inv.inv32.p) : static_cast<const void*>(inv.inv.p);
}

// one damped Jacobi sweep of level l on every slot of the step
void BatchEngine::smooth(int l, std::vector<char>& cur_sol) {
  const size_t cur = cur_sol[size_t(l)] ? off_sol[size_t(l)] : off_alt[size_t(l)];
  const size_t oth = cur_sol[size_t(l)] ? off_alt[size_t(l)] : off_sol[size_t(l)];
  if (mixed)
    csr_apply32_batch(c, A(l), B, bt(MASK_STEP, t_v32[size_t(l)], t_d32[size_t(l)]), EPI_JACOBI, at<float>(cur),
                      at<float>(oth), at<float>(off_rhs[size_t(l)]), float(jacobi_damp));
  else
    csr_apply_batch(c, A(l), B, bt(MASK_STEP, t_v64[size_t(l)], t_d64[size_t(l)]), EPI_JACOBI, at<double>(cur),
                    at<double>(oth), at<double>(off_rhs[size_t(l)]), jacobi_damp);
  cur_sol[size_t(l)] = !cur_sol[size_t(l)];
}

// Multigrid::apply for the slots of the step (damped Jacobi, direct coarse
// solve, the cycle's control sequence); z_in and r_out are slot 0's vectors
void BatchEngine::mg_apply(const double* z_in, double* r_out, bool na_zero) {
  const int finest = L - 1;
  const int nf = n_lvl.back();
  std::vector<char> cur_sol(size_t(L), 1);  // the iterate is in sol (1) or alt (0)
  auto cur = [&](int l) { return cur_sol[size_t(l)] ? off_sol[size_t(l)] : off_alt[size_t(l)]; };
  const Batch shared = bt(MASK_STEP);
  if (mixed) {
    vcvt_d2f_batch(c, B, shared, nf, z_in, at<float>(off_rhs[size_t(finest)]));
    init_solution_batch<float>(c, B, shared, nf, A(finest).mask, at<float>(off_rhs[size_t(finest)]),
                               at<float>(cur(finest)));
  } else {
    vcopy_batch(c, B, shared, nf, z_in, at<double>(off_rhs[size_t(finest)]));
    init_solution_batch<double>(c, B, shared, nf, A(finest).mask, at<double>(off_rhs[size_t(finest)]),
                                at<double>(cur(finest)));
  }
  std::vector<char> zero(size_t(L), 0);
  zero[size_t(finest)] = na_zero ? 1 : 0;
  const int n_steps = int(control.size()) - 1;
  int level = finest;
  for (int step = 1; step <= n_steps && level >= 0; ++step) {
    if (level == 0) {
      // direct coarse solve of the restricted defect, then up
      if (mixed)
        coarse_solve32_batch(c, B, bt(MASK_STEP, SIZE_MAX, t_inv), lvl(0).coarse, at<float>(off_rhs[0]),
                             at<float>(cur(0)));
      else
        coarse_solve_batch(c, B, bt(MASK_STEP, SIZE_MAX, t_inv), lvl(0).coarse, at<double>(off_rhs[0]),
                           at<double>(cur(0)));
      zero[0] = 0;
      // prolongate_from(0): shared transfer values
      if (mixed)
        csr_apply32_batch(c, lvl(0).P, B, shared, EPI_PROLONG, at<float>(cur(0)), at<float>(cur(1)), nullptr,
                          float(correction_damp));
      else
        csr_apply_batch(c, lvl(0).P, B, shared, EPI_PROLONG, at<double>(cur(0)), at<double>(cur(1)), nullptr,
                        correction_damp);
      zero[1] = 0;
      level = 1;
      continue;
    }
    const bool from_below = control[size_t(step) - 1] == DIR_UP;
    const bool up = control[size_t(step)] == DIR_UP;
    const bool down = control[size_t(step)] == DIR_DOWN;
    if (from_below)
      for (int i = 0; i < n_post; ++i) smooth(level, cur_sol);
    if (down) {
      for (int i = 0; i < n_pre; ++i) {
        if (i == 0 && zero[size_t(level)] && c->jacobi_zero_start) {
          // the first sweep from an exactly zero iterate: x = w b / d
          if (mixed)
            jacobi_from_zero_batch<float>(c, B, bt(MASK_STEP, SIZE_MAX, t_d32[size_t(level)]), n_lvl[size_t(level)],
                                          at<float>(off_rhs[size_t(level)]), float(jacobi_damp),
                                          at<float>(cur(level)));
          else
            jacobi_from_zero_batch<double>(c, B, bt(MASK_STEP, SIZE_MAX, t_d64[size_t(level)]),
                                           n_lvl[size_t(level)], at<double>(off_rhs[size_t(level)]), jacobi_damp,
                                           at<double>(cur(level)));
        } else {
          smooth(level, cur_sol);
        }
        zero[size_t(level)] = 0;
      }
      // defect
      if (mixed)
        csr_apply32_batch(c, A(level), B, bt(MASK_STEP, t_v32[size_t(level)]), EPI_DEFECT, at<float>(cur(level)),
                          at<float>(off_def[size_t(level)]), at<float>(off_rhs[size_t(level)]), 1.0f);
      else
        csr_apply_batch(c, A(level), B, bt(MASK_STEP, t_v64[size_t(level)]), EPI_DEFECT, at<double>(cur(level)),
                        at<double>(off_def[size_t(level)]), at<double>(off_rhs[size_t(level)]), 1.0);
      // the coarse iterate starts at zero: its first step writes every entry
      // (a Jacobi sweep from zero, the direct coarse solve), so no reset
      const int lc = level - 1;
      const bool written = (lc > 0 && n_pre >= 1 && c->jacobi_zero_start) || lc == 0;
      if (!written) {
        const size_t eb = mixed ? sizeof(float) : sizeof(double);
        PM_CUDA(cudaMemset2DAsync(block.p + cur(lc), S, 0, eb * size_t(n_lvl[size_t(lc)]), size_t(B), c->stream));
      }
      zero[size_t(lc)] = 1;
      // DefectRestriction + ResetNonActive: shared transfer values
      if (mixed)
        csr_apply32_batch(c, lvl(lc).R, B, shared, EPI_RESTRICT, at<float>(off_def[size_t(level)]),
                          at<float>(off_rhs[size_t(lc)]), nullptr, 1.0f);
      else
        csr_apply_batch(c, lvl(lc).R, B, shared, EPI_RESTRICT, at<double>(off_def[size_t(level)]),
                        at<double>(off_rhs[size_t(lc)]), nullptr, 1.0);
      level -= 1;
    } else if (up) {
      if (mixed)
        csr_apply32_batch(c, lvl(level).P, B, shared, EPI_PROLONG, at<float>(cur(level)), at<float>(cur(level + 1)),
                          nullptr, float(correction_damp));
      else
        csr_apply_batch(c, lvl(level).P, B, shared, EPI_PROLONG, at<double>(cur(level)),
                        at<double>(cur(level + 1)), nullptr, correction_damp);
      zero[size_t(level) + 1] = 0;
      level += 1;
    } else {
      level = -1;
    }
  }
  if (mixed) vcvt_f2d_batch(c, B, shared, nf, at<float>(cur(finest)), r_out);
  else vcopy_batch(c, B, shared, nf, at<double>(cur(finest)), r_out);
}

// z_i = M^-1 v_i, r = A z_i, CGS2, H(i+1,i), v_{i+1}, Givens rotation, and the
// slots' residuals and breakdown flags copied to pinned host memory
void BatchEngine::arnoldi_step(int i, bool na_zero) {
  const int n = n_lvl.back();
  const int ldh = m + 1;
  double* V = at<double>(off_V);
  double* Z = at<double>(off_Z);
  double* r = at<double>(off_r);
  const Batch step = bt(MASK_STEP);
  mg_apply(V + ld * size_t(i), Z + ld * size_t(i), na_zero);
  csr_apply_batch(c, A(L - 1), B, bt(MASK_STEP, t_v64[size_t(L) - 1]), EPI_SET, Z + ld * size_t(i), r, nullptr, 1.0);
  fg_cgs2_batch(c, B, step, n, i, ldh, r, V, ld, at<double>(off_cgs), at<double>(off_h1), at<double>(off_h2),
                at<double>(off_H), at<double>(off_pA));
  fg_normalize_batch(c, B, step, n, ldh, i, r, V + ld * size_t(i + 1), at<double>(off_pA), at<double>(off_H),
                     at<int>(off_flags));
  fg_givens_batch(c, B, step, ldh, i, at<double>(off_H), at<double>(off_cs), at<double>(off_sn), at<double>(off_s),
                  at<double>(off_dres));
  PM_CUDA(cudaMemcpy2DAsync(hres, sizeof(double), block.p + off_dres, S, sizeof(double), size_t(B),
                            cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaMemcpy2DAsync(hflag, sizeof(int), block.p + off_flags, S, sizeof(int), size_t(B),
                            cudaMemcpyDeviceToHost, c->stream));
}

// IterativeMethod::converged (include/Solver/IterativeMethod.h:81-140), per
// slot; status: PM_OK to go on or finish, PM_E_DIVERGED
bool BatchEngine::slot_converged(SlotState& st, double r, unsigned it, int& status) {
  status = PM_OK;
  if (it == 0) {
    st.init_res = r;
    st.prev_res = r;
    st.p->solver->history.clear();
  }
  st.p->solver->history.push_back(r);  // as pm_solver::converged keeps it
  const bool small = r < tol;
  const bool red = r < reduction * st.init_res;
  const bool enough = it > (unsigned long)min_it || min_it == 0;
  const bool stag = r > stagnation * st.prev_res;
  const bool div = r > divergence * st.init_res;
  bool conv = (small || red || stag || div) && enough;
  if (it == (unsigned long)max_it) conv = true;
  st.prev_res = r;
  st.last_it = int(it);
  st.last_res = r;
  if (div || !std::isfinite(r)) {
    status = PM_E_DIVERGED;
    return true;
  }
  return conv;
}

std::vector<BatchDone> BatchEngine::cycle(const std::vector<pm_problem*>& join) {
  std::vector<BatchDone> out;
  const int n = n_lvl.back();
  const int ldh = m + 1;
  double* r = at<double>(off_r);
  double* x = at<double>(off_x);
  double* b = at<double>(off_b);
  // admission: free slots take the joining problems
  size_t next = 0;
  bool tables_changed = false;
  for (int s = 0; s < B && next < join.size(); ++s) {
    SlotState& st = slots[size_t(s)];
    if (st.p) continue;
    pm_problem* p = join[next++];
    if (p->mats.back()->csr.n_rows != n || p->mats.size() != size_t(L))
      throw Error(PM_E_INVALID, "a batch takes problems of one set-up only");
    st = SlotState();
    st.p = p;
    st.is_new = true;
    st.in_cycle = true;
    set_tables(s, p);
    tables_changed = true;
    // the problem's right-hand side and initial iterate into the slot
    PM_CUDA(cudaMemcpyAsync(b + size_t(s) * S / sizeof(double), p->rhs.p, sizeof(double) * size_t(n),
                            cudaMemcpyDeviceToDevice, c->stream));
    PM_CUDA(cudaMemcpyAsync(x + size_t(s) * S / sizeof(double), p->sol.p, sizeof(double) * size_t(n),
                            cudaMemcpyDeviceToDevice, c->stream));
  }
  if (next < join.size()) throw Error(PM_E_INVALID, "more joining problems than free slots");
  if (tables_changed) PM_CUDA(cudaMemcpyAsync(tab.p, htab.data(), sizeof(const void*) * htab.size(),
                                              cudaMemcpyHostToDevice, c->stream));
  // every slot in the cycle: r = b - A x, <r, r>; new slots: the non-active
  // test and the initial residual
  for (int s = 0; s < B; ++s) {
    hmask[MASK_CYCLE * B + s] = slots[size_t(s)].in_cycle ? 1 : 0;
    hmask[MASK_FINAL * B + s] = slots[size_t(s)].is_new ? 1 : 0;  // the new slots, for the tests below
  }
  upload_masks();
  const Batch cyc = bt(MASK_CYCLE);
  csr_apply_batch(c, A(L - 1), B, bt(MASK_CYCLE, t_v64[size_t(L) - 1]), EPI_DEFECT, x, r, b, 1.0);
  {
    const Batch nw = bt(MASK_FINAL);
    PM_CUDA(cudaMemset2DAsync(block.p + off_flags, S, 0, sizeof(int) * 4, size_t(B), c->stream));
    nonactive_nonzero_batch(c, B, nw, A(L - 1).mask, r, at<int>(off_flags) + 2);
  }
  dot_partials_batch(c, B, cyc, n, r, r, at<double>(off_pA));
  finish_sum_batch(c, B, cyc, at<double>(off_pA), at<double>(off_dres), true);
  PM_CUDA(cudaMemcpy2DAsync(hres, sizeof(double), block.p + off_dres, S, sizeof(double), size_t(B),
                            cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaMemcpy2DAsync(hflag, sizeof(int) * 4, block.p + off_flags, S, sizeof(int) * 4, size_t(B),
                            cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));
  auto finish = [&](int s, int status) {
    SlotState& st = slots[size_t(s)];
    BatchDone d;
    d.p = st.p;
    d.r.status = status;
    d.r.iterations = st.last_it;
    d.r.residual = st.last_res;
    d.r.initial_residual = st.init_res;
    if (status == PM_OK && !(st.last_res <= std::max(tol, reduction * st.init_res))) d.r.status = PM_E_MAXIT;
    // the solution back into the problem
    PM_CUDA(cudaMemcpyAsync(st.p->sol.p, x + size_t(s) * S / sizeof(double), sizeof(double) * size_t(n),
                            cudaMemcpyDeviceToDevice, c->stream));
    st.p->solver->last_it = st.last_it;
    st.p->solver->last_res = st.last_res;
    st.p->solver->init_res = st.init_res;
    out.push_back(d);
    st = SlotState();
  };
  for (int s = 0; s < B; ++s) {
    SlotState& st = slots[size_t(s)];
    if (!st.is_new) continue;
    st.na_zero = hflag[4 * s + 2] == 0;
    int status = PM_OK;
    if (slot_converged(st, hres[s], 0, status)) finish(s, status);
    else st.is_new = false;
  }
  bool na_zero = true;
  int n_in = 0;
  for (int s = 0; s < B; ++s) {
    SlotState& st = slots[size_t(s)];
    st.in_cycle = st.p != nullptr;
    if (st.in_cycle) {
      na_zero = na_zero && st.na_zero;
      ++n_in;
    }
    hmask[MASK_CYCLE * B + s] = st.in_cycle ? 1 : 0;
    hmask[MASK_STEP * B + s] = st.in_cycle ? 1 : 0;
    hmask[MASK_FINAL * B + s] = 0;
  }
  if (n_in == 0) {
    PM_CUDA(cudaStreamSynchronize(c->stream));
    return out;
  }
  upload_masks();
  // v_0 = r / beta, s = (beta, 0, ...)
  fg_start_batch(c, B, bt(MASK_CYCLE), n, m, r, at<double>(off_V), at<double>(off_pA), at<double>(off_s),
                 at<double>(off_dres) + 1);
  PM_CUDA(cudaMemset2DAsync(block.p + off_H, S, 0, sizeof(double) * size_t(ldh) * m, size_t(B), c->stream));
  int i = 0;
  for (; i < m && n_in > 0; ++i) {
    // one graph per Arnoldi index and non-active variant
    const int gi = (na_zero ? m : 0) + i;
    if (graphs.empty()) graphs.assign(size_t(2 * m), nullptr);
    if (!graphs[size_t(gi)]) {
      const uint64_t before = c->kernel_launches;
      cudaGraph_t g = nullptr;
      PM_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      try {
        arnoldi_step(i, na_zero);
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
      graphs[size_t(gi)] = ex;
      graph_launches[na_zero ? 1 : 0][i] = c->kernel_launches - before;
      c->kernel_launches = before;
    }
    PM_CUDA(cudaGraphLaunch(graphs[size_t(gi)], c->stream));
    c->kernel_launches += graph_launches[na_zero ? 1 : 0][i];
    PM_CUDA(cudaStreamSynchronize(c->stream));
    bool any_final = false;
    for (int s = 0; s < B; ++s) {
      SlotState& st = slots[size_t(s)];
      hmask[MASK_FINAL * B + s] = 0;
      if (!st.in_cycle) continue;
      int status = PM_OK;
      bool stop;
      if (hflag[s]) {
        status = PM_E_BREAKDOWN;  // Unhappy breakdown (Iteration_gmres.C:476)
        stop = true;
      } else {
        stop = slot_converged(st, hres[s], st.j, status);
      }
      ++st.j;
      if (stop) {
        st.in_cycle = false;
        hmask[MASK_STEP * B + s] = 0;
        if (status == PM_OK) {
          hmask[MASK_FINAL * B + s] = 1;  // its solution update below
          any_final = true;
        } else {
          finish(s, status);  // no update, as where the reference throws
        }
      } else if (st.j > (unsigned long)max_it) {
        // cannot happen: converged() forces the stop at max_it
        st.in_cycle = false;
      }
    }
    if (any_final) {
      upload_masks();
      fg_update_batch(c, B, bt(MASK_FINAL), n, ldh, i, at<double>(off_H), at<double>(off_s), at<double>(off_y),
                      at<double>(off_Z), ld, x);
      for (int s = 0; s < B; ++s)
        if (hmask[MASK_FINAL * B + s]) finish(s, PM_OK);
    } else {
      upload_masks();
    }
    n_in = 0;
    for (int s = 0; s < B; ++s) n_in += slots[size_t(s)].in_cycle ? 1 : 0;
  }
  if (n_in > 0) {
    // the end of a restart cycle: x += Z y for the slots still in it; their
    // next cycle starts with the true residual (the next call)
    for (int s = 0; s < B; ++s) hmask[MASK_FINAL * B + s] = slots[size_t(s)].in_cycle ? 1 : 0;
    upload_masks();
    fg_update_batch(c, B, bt(MASK_FINAL), n, ldh, m - 1, at<double>(off_H), at<double>(off_s), at<double>(off_y),
                    at<double>(off_Z), ld, x);
    // the reference tests the last residual once more after the restart
    // update (Iteration_gmres.C:526-531)
    for (int s = 0; s < B; ++s) {
      SlotState& st = slots[size_t(s)];
      if (!st.in_cycle) continue;
      int status = PM_OK;
      if (slot_converged(st, st.last_res, st.j, status)) finish(s, status);
    }
  }
  for (int s = 0; s < B; ++s) {
    hmask[MASK_FINAL * B + s] = 0;
    hmask[MASK_STEP * B + s] = 0;
  }
  PM_CUDA(cudaStreamSynchronize(c->stream));
  return out;
}

BatchEngine* batch_create(pm_ctx* c, int capacity, pm_problem* templ) {
  if (capacity < 1 || capacity > kMaxBatch) throw Error(PM_E_INVALID, "batch capacity is 1 to 16");
  if (!templ || templ->kind != 0) throw Error(PM_E_UNSUPPORTED, "batched solves of convection-diffusion problems only");
  pm_solver* sv = templ->solver;
  if (!sv || sv->solver_type != "iterative" || (sv->method != "fgmres" && sv->method != "right_gmres") || !sv->use_mg)
    throw Error(PM_E_UNSUPPORTED, "batched solves need fgmres with the multigrid preconditioner");
  if (sv->restart > kBatchMaxRestart) throw Error(PM_E_UNSUPPORTED, "batched solves need gmres_restart <= 32");
  if (sv->gram_schmidt != "cgs2")
    throw Error(PM_E_UNSUPPORTED, "batched solves orthogonalise by CGS2 (gpu_gram_schmidt: cgs2)");
  const Multigrid& mg = sv->mg;
  if (!mg.ready) throw Error(PM_E_INVALID, "batch template: the solver's multigrid is not updated");
  for (size_t l = 1; l < mg.levels.size(); ++l)
    if (mg.levels[l].smoother != SM_JACOBI)
      throw Error(PM_E_UNSUPPORTED, "batched solves need damped Jacobi smoothing");
  if (mg.levels[0].smoother != SM_DIRECT) throw Error(PM_E_UNSUPPORTED, "batched solves need a direct coarse solve");
  auto* e = new BatchEngine();
  try {
    e->c = c;
    e->B = capacity;
    e->templ = templ;
    e->L = int(mg.levels.size());
    e->m = int(sv->restart);
    e->mixed = mg.mixed_cfg;
    e->n_pre = mg.n_pre;
    e->n_post = mg.n_post;
    e->jacobi_damp = mg.jacobi_damp;
    e->correction_damp = mg.correction_damp;
    e->control = mg.control;
    e->tol = sv->tol;
    e->reduction = sv->reduction;
    e->divergence = sv->divergence;
    e->stagnation = sv->stagnation;
    e->max_it = sv->max_it;
    e->min_it = sv->min_it;
    for (const auto& lv : mg.levels) e->n_lvl.push_back(lv.A->csr.n_rows);
    e->slots.assign(size_t(capacity), SlotState());
    e->layout();
  } catch (...) {
    delete e;
    throw;
  }
  return e;
}

void batch_destroy(BatchEngine* e) { delete e; }
size_t batch_bytes(const BatchEngine* e) { return e ? e->block.bytes() + e->tab.bytes() : 0; }
int batch_capacity(const BatchEngine* e) { return e ? e->B : 0; }
int batch_active(const BatchEngine* e) {
  int n = 0;
  for (const auto& s : e->slots) n += s.p ? 1 : 0;
  return n;
}
std::vector<BatchDone> batch_cycle(BatchEngine* e, const std::vector<pm_problem*>& join) { return e->cycle(join); }

}  // namespace pm

// ---------------------------------------------------------------------------
// C ABI: batched solve of convection-diffusion problems of one set-up
extern "C" int pm_problem_solve_batched(pm_problem* const* probs, int n_problems, int slots, int* status_out) {
  if (!probs || n_problems < 1 || slots < 1) return PM_E_INVALID;
  for (int k = 0; k < n_problems; ++k)
    if (!probs[k]) return PM_E_INVALID;
  pm_ctx* c = probs[0]->ctx;
  pm::BatchEngine* e = nullptr;
  try {
    for (int k = 0; k < n_problems; ++k) {
      pm_problem* p = probs[k];
      if (p->ctx != c) throw pm::Error(PM_E_INVALID, "batched problems must share one context");
      if (p->kind != 0) throw pm::Error(PM_E_UNSUPPORTED, "batched solves of convection-diffusion problems only");
      if (p->disc != probs[0]->disc) throw pm::Error(PM_E_INVALID, "batched problems must share one set-up");
      if (!p->solver_ready) {
        const int rc = pm_solver_update_matrix(p->solver, p->mats.back());
        if (rc != PM_OK) return rc;
        p->solver_ready = true;
      }
    }
    e = pm::batch_create(c, std::min(slots, std::min(n_problems, pm::kMaxBatch)), probs[0]);
    std::vector<int> status(size_t(n_problems), PM_OK);
    std::vector<pm_problem*> queue(probs, probs + n_problems);
    size_t next = 0;
    int done = 0;
    while (done < n_problems) {
      const int free_slots = pm::batch_capacity(e) - pm::batch_active(e);
      std::vector<pm_problem*> join;
      while (int(join.size()) < free_slots && next < queue.size()) join.push_back(queue[next++]);
      for (const auto& d : pm::batch_cycle(e, join)) {
        for (int k = 0; k < n_problems; ++k)
          if (probs[k] == d.p) status[size_t(k)] = d.r.status;
        ++done;
      }
    }
    pm::batch_destroy(e);
    e = nullptr;
    if (status_out)
      for (int k = 0; k < n_problems; ++k) status_out[k] = status[size_t(k)];
    return PM_OK;
  } catch (const pm::Error& err) {
    pm::batch_destroy(e);
    c->last_error = err.what();
    return err.code;
  } catch (const std::exception& err) {
    pm::batch_destroy(e);
    c->last_error = err.what();
    return PM_E_INVALID;
  }
}
