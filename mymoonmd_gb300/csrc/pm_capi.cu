// extern "C" entry points (include/pmgpu.h). Every call catches the library's
// exceptions and turns them into status codes plus a per-context message.
#include <algorithm>
#include <deque>
#include <cstring>
#include <iterator>
#include <new>
#include <string>

#include "pm_assemble.h"
#include "pm_disc.h"
#include "pm_problem.h"
#include "pm_devsetup.h"
#include "pm_solver.h"

using namespace pm;

static thread_local std::string g_last_error;

static int fail(pm_ctx* c, int code, const char* msg) {
  if (c) c->last_error = msg;
  g_last_error = msg;
  return code;
}

#define PM_TRY try {
#define PM_CATCH(ctxp)                                                 \
  }                                                                    \
  catch (const pm::Error& e) { return fail((ctxp), e.code, e.what()); } \
  catch (const std::invalid_argument& e) { return fail((ctxp), PM_E_INVALID, e.what()); } \
  catch (const std::out_of_range& e) { return fail((ctxp), PM_E_INVALID, e.what()); } \
  catch (const std::bad_alloc&) { return fail((ctxp), PM_E_OOM, "host allocation failed"); } \
  catch (const std::exception& e) { return fail((ctxp), PM_E_INVALID, e.what()); }

extern "C" {

int pm_version(void) { return 1; }

int pm_ctx_create(int device, pm_ctx** out) {
  if (!out) return fail(nullptr, PM_E_INVALID, "null output pointer");
  pm_ctx* c = new (std::nothrow) pm_ctx();
  if (!c) return fail(nullptr, PM_E_OOM, "host allocation failed");
  PM_TRY
  ctx_init(c, device);
  *out = c;
  return PM_OK;
  }
  catch (const pm::Error& e) {
    ctx_destroy(c);
    delete c;
    return fail(nullptr, e.code, e.what());
  }
}

void pm_ctx_destroy(pm_ctx* c) {
  if (!c) return;
  ctx_destroy(c);
  delete c;
}

const char* pm_last_error(const pm_ctx* c) {
  return c ? c->last_error.c_str() : g_last_error.c_str();
}

int pm_ctx_synchronize(pm_ctx* c) {
  PM_TRY
  PM_CUDA(cudaStreamSynchronize(c->stream));
  return PM_OK;
  PM_CATCH(c)
}

int pm_ctx_set_option(pm_ctx* c, const char* key, int value) {
  if (!c || !key) return PM_E_INVALID;
  if (std::string(key) == "assembly_quadrature_loop") {
    c->assembly_quadrature_loop = value != 0;
    return PM_OK;
  }
  if (std::string(key) == "fp32_sliced_spmv") {
    static const int shapes[] = {0, 140, 141, 180, 240, 241, 280, 440, 441, 480, 481, 840, 841, 881};
    if (std::find(std::begin(shapes), std::end(shapes), value) == std::end(shapes))
      return fail(c, PM_E_INVALID,
                  "fp32_sliced_spmv is 0 or one of 140 141 180 240 241 280 440 441 480 481 840 841 881");
    c->sell_shape = value;
    return PM_OK;
  }
  if (std::string(key) == "fp64_sliced_spmv") {
    if (value != 0 && value != 441 && value != 481 && value != 841)
      return fail(c, PM_E_INVALID, "fp64_sliced_spmv is 0, 441, 481 or 841");
    c->sell_shape64 = value;
    return PM_OK;
  }
  if (std::string(key) == "coarse_cluster") {
    if (value != 1 && value != 2 && value != 4 && value != 8)
      return fail(c, PM_E_INVALID, "coarse_cluster is 1, 2, 4 or 8");
    c->coarse_cluster = value;
    return PM_OK;
  }
  if (std::string(key) == "sliced_min_entries") {
    if (value < 0) return fail(c, PM_E_INVALID, "sliced_min_entries is >= 0");
    c->sell_min_avg = value;
    return PM_OK;
  }
  if (std::string(key) == "coarse_threads") {
    if (value != 0 && value != 256 && value != 512 && value != 1024)
      return fail(c, PM_E_INVALID, "coarse_threads is 0, 256, 512 or 1024");
    c->coarse_threads = value;
    return PM_OK;
  }
  if (std::string(key) == "jacobi_zero_start") {
    c->jacobi_zero_start = value != 0;
    return PM_OK;
  }
  if (std::string(key) == "pdl") {
    if (value < 0 || value > 1) return fail(c, PM_E_INVALID, "pdl is 0 or 1");
    c->pdl = value;
    return PM_OK;
  }
  if (std::string(key) == "probe_epilogue") {
    c->probe_epilogue = value;
    return PM_OK;
  }
  if (std::string(key) == "probe_nodal") {
    c->probe_nodal = value != 0;
    return PM_OK;
  }
  if (std::string(key) == "nodal_sliced") {
    if (value != 0 && value != 1 && value != 4 && value != 8)
      return fail(c, PM_E_INVALID, "nodal_sliced is 0, 1, 4 or 8");
    if (value == 1) value = 4;
    c->nodal_sliced = value;
    return PM_OK;
  }
  if (std::string(key) == "probe_precision") {
    if (value != 0 && value != 4 && value != 8) return fail(c, PM_E_INVALID, "probe_precision is 0, 4 or 8");
    c->probe_precision = value;
    return PM_OK;
  }
  return fail(c, PM_E_INVALID, (std::string("unknown context option ") + key).c_str());
}

int pm_ctx_kernel_launches(const pm_ctx* c, uint64_t* out) {
  if (!c || !out) return PM_E_INVALID;
  *out = c->kernel_launches;
  return PM_OK;
}

static thread_local cudaEvent_t g_ev0 = nullptr, g_ev1 = nullptr;

int pm_ctx_time_begin(pm_ctx* c) {
  PM_TRY
  if (!g_ev0) {
    PM_CUDA(cudaEventCreate(&g_ev0));
    PM_CUDA(cudaEventCreate(&g_ev1));
  }
  PM_CUDA(cudaEventRecord(g_ev0, c->stream));
  return PM_OK;
  PM_CATCH(c)
}

int pm_ctx_time_end(pm_ctx* c, float* ms) {
  PM_TRY
  PM_CUDA(cudaEventRecord(g_ev1, c->stream));
  PM_CUDA(cudaEventSynchronize(g_ev1));
  PM_CUDA(cudaEventElapsedTime(ms, g_ev0, g_ev1));
  return PM_OK;
  PM_CATCH(c)
}

int pm_dev_alloc(pm_ctx* c, size_t bytes, void** out) {
  PM_TRY
  PM_CUDA(cudaSetDevice(c->device));
  cudaError_t e = cudaMalloc(out, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(c, PM_E_OOM, "cudaMalloc failed");
  }
  return PM_OK;
  PM_CATCH(c)
}

int pm_dev_free(pm_ctx* c, void* p) {
  PM_TRY
  PM_CUDA(cudaStreamSynchronize(c->stream));
  PM_CUDA(cudaFree(p));
  return PM_OK;
  PM_CATCH(c)
}

int pm_memcpy_h2d(pm_ctx* c, void* dst, const void* src, size_t bytes) {
  PM_TRY
  PM_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));
  return PM_OK;
  PM_CATCH(c)
}

int pm_memcpy_d2h(pm_ctx* c, void* dst, const void* src, size_t bytes) {
  PM_TRY
  PM_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));
  return PM_OK;
  PM_CATCH(c)
}

int pm_memset_dev(pm_ctx* c, void* dst, int value, size_t bytes) {
  PM_TRY
  PM_CUDA(cudaMemsetAsync(dst, value, bytes, c->stream));
  return PM_OK;
  PM_CATCH(c)
}

int pm_host_alloc(pm_ctx* c, size_t bytes, void** out) {
  if (!c || !out) return PM_E_INVALID;
  PM_TRY
  cudaError_t e = cudaMallocHost(out, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(c, PM_E_OOM, "cudaMallocHost failed");
  }
  return PM_OK;
  PM_CATCH(c)
}

int pm_host_free(pm_ctx* c, void* p) {
  if (!c) return PM_E_INVALID;
  PM_TRY
  PM_CUDA(cudaStreamSynchronize(c->stream));
  PM_CUDA(cudaFreeHost(p));
  return PM_OK;
  PM_CATCH(c)
}

// ------------------------------------------------------------- matrices ----
static int check_csr(int n_rows, int n_cols, int n_active, const int* rp, const int* ci) {
  if (n_rows < 0 || n_cols < 0 || n_active < 0 || n_active > n_rows || !rp) return 0;
  if (rp[0] != 0) return 0;
  for (int i = 0; i < n_rows; ++i) {
    if (rp[i + 1] < rp[i]) return 0;
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      if (ci[k] < 0 || ci[k] >= n_cols) return 0;
      if (k > rp[i] && ci[k] <= ci[k - 1]) return 0;
    }
  }
  return 1;
}

int pm_matrix_create_csr(pm_ctx* c, int n_rows, int n_cols, int n_active, const int* row_ptr,
                         const int* cols, const double* vals, pm_matrix** out) {
  if (!c || !out) return fail(c, PM_E_INVALID, "null argument");
  if (!check_csr(n_rows, n_cols, n_active, row_ptr, cols))
    return fail(c, PM_E_INVALID, "invalid CSR: row pointers must ascend from 0, columns must be in range and ascending within each row");
  PM_TRY
  auto* A = new pm_matrix();
  A->ctx = c;
  try {
    A->csr.upload(c, n_rows, n_cols, n_active, row_ptr, cols, vals);
    PM_CUDA(cudaStreamSynchronize(c->stream));
  } catch (...) {
    delete A;
    throw;
  }
  *out = A;
  return PM_OK;
  PM_CATCH(c)
}

void pm_matrix_destroy(pm_matrix* A) {
  if (!A) return;
  if (A->ctx && A->ctx->stream) cudaStreamSynchronize(A->ctx->stream);
  delete A;
}

int pm_matrix_set_blocks(pm_matrix* A, int nb, const int* lengths, const int* actives) {
  if (!A || !lengths || !actives) return fail(A ? A->ctx : nullptr, PM_E_INVALID, "null argument");
  PM_TRY
  A->csr.set_blocks(nb, lengths, actives);
  return PM_OK;
  PM_CATCH(A->ctx)
}

int pm_matrix_info(const pm_matrix* A, int* n_rows, int* n_cols, int* n_active, int64_t* nnz) {
  if (!A) return PM_E_INVALID;
  if (n_rows) *n_rows = A->csr.n_rows;
  if (n_cols) *n_cols = A->csr.n_cols;
  if (n_active) *n_active = A->csr.n_active;
  if (nnz) *nnz = A->csr.nnz;
  return PM_OK;
}

int pm_matrix_set_values(pm_matrix* A, const double* vals) {
  if (!A || !vals) return PM_E_INVALID;
  PM_TRY
  A->csr.vals.upload(vals, size_t(A->csr.nnz), A->ctx->stream);
  A->csr.values_changed(A->ctx);
  if (A->csr.vals32.p) A->csr.make_fp32(A->ctx);
  if (A->csr.diag.p) A->csr.make_diag(A->ctx);
  PM_CUDA(cudaStreamSynchronize(A->ctx->stream));
  return PM_OK;
  PM_CATCH(A->ctx)
}

int pm_matrix_get_values(const pm_matrix* A, double* vals) {
  if (!A || !vals) return PM_E_INVALID;
  PM_TRY
  A->csr.vals.download(vals, A->ctx->stream);
  PM_CUDA(cudaStreamSynchronize(A->ctx->stream));
  return PM_OK;
  PM_CATCH(A->ctx)
}

int pm_matrix_get_structure(const pm_matrix* A, int* rp, int* ci) {
  if (!A) return PM_E_INVALID;
  PM_TRY
  if (rp) A->csr.row_ptr.download(rp, A->ctx->stream);
  if (ci) A->csr.cols.download(ci, A->ctx->stream);
  PM_CUDA(cudaStreamSynchronize(A->ctx->stream));
  return PM_OK;
  PM_CATCH(A->ctx)
}

int pm_matrix_apply_scaled_add(pm_matrix* A, const double* x, double* y, double a) {
  if (!A || !x || !y) return PM_E_INVALID;
  PM_TRY
  if (a == 0.0) return PM_OK;  // TMatrix::multiply returns at once for a == 0
  csr_apply(A->ctx, A->csr, EPI_AXPY, x, y, nullptr, a);
  return PM_OK;
  PM_CATCH(A->ctx)
}

int pm_matrix_apply(pm_matrix* A, const double* x, double* y) {
  if (!A || !x || !y) return PM_E_INVALID;
  PM_TRY
  csr_apply(A->ctx, A->csr, EPI_SET, x, y, nullptr, 1.0);
  return PM_OK;
  PM_CATCH(A->ctx)
}

int pm_matrix_get_diagonal(pm_matrix* A, double* d) {
  if (!A || !d) return PM_E_INVALID;
  PM_TRY
  A->csr.make_diag(A->ctx);
  vcopy(A->ctx, A->csr.n_rows, A->csr.diag.p, d);
  return PM_OK;
  PM_CATCH(A->ctx)
}

int pm_matrix_make_fp32(pm_matrix* A) {
  if (!A) return PM_E_INVALID;
  PM_TRY
  A->csr.make_fp32(A->ctx);
  return PM_OK;
  PM_CATCH(A->ctx)
}

int pm_matrix_make_sliced64(pm_matrix* A) {
  if (!A) return PM_E_INVALID;
  PM_TRY
  A->csr.make_sliced64(A->ctx);
  return PM_OK;
  PM_CATCH(A->ctx)
}

int pm_matrix_apply_f32(pm_matrix* A, const float* x, float* y) {
  if (!A || !x || !y) return PM_E_INVALID;
  PM_TRY
  csr_apply32(A->ctx, A->csr, EPI_SET, x, y, nullptr, 1.0f);
  return PM_OK;
  PM_CATCH(A->ctx)
}

int pm_matrix_set_kernel(pm_matrix* A, int lanes, int unroll) {
  if (!A) return PM_E_INVALID;
  if (lanes && lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32)
    return fail(A->ctx, PM_E_INVALID, "lanes per row must be 1, 2, 4, 8, 16 or 32");
  if (unroll && unroll != 2 && unroll != 4 && unroll != 8 && unroll != 16)
    return fail(A->ctx, PM_E_INVALID, "entries per lane must be 2, 4, 8 or 16");
  if (lanes) A->csr.lanes = A->csr.lanes32 = lanes;
  if (unroll) A->csr.unroll = A->csr.unroll32 = unroll;
  // an explicit group shape selects the per-row-group kernel; (0, 0) goes back
  // to the row-block streaming kernel
  A->csr.stream = (lanes == 0 && unroll == 0);
  return PM_OK;
}

int pm_matrix_bench_apply(pm_matrix* A, int fp32, const void* x, void* y, int reps, float* ms,
                          double* bytes) {
  if (!A || !x || !y || reps < 1) return PM_E_INVALID;
  PM_TRY
  pm_ctx* c = A->ctx;
  cudaEvent_t e0, e1;
  PM_CUDA(cudaEventCreate(&e0));
  PM_CUDA(cudaEventCreate(&e1));
  PM_CUDA(cudaEventRecord(e0, c->stream));
  for (int r = 0; r < reps; ++r) {
    if (fp32) csr_apply32(c, A->csr, EPI_SET, (const float*)x, (float*)y, nullptr, 1.0f);
    else csr_apply(c, A->csr, EPI_SET, (const double*)x, (double*)y, nullptr, 1.0);
  }
  PM_CUDA(cudaEventRecord(e1, c->stream));
  PM_CUDA(cudaEventSynchronize(e1));
  float total = 0.0f;
  PM_CUDA(cudaEventElapsedTime(&total, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ms) *ms = total / reps;
  if (bytes) *bytes = double(A->csr.spmv_bytes(fp32 ? 4 : 8, false));
  return PM_OK;
  PM_CATCH(A->ctx)
}

// ---------------------------------------------------------------- BLAS -----
int pm_dot(pm_ctx* c, int n, const double* x, const double* y, double* out) {
  if (!c || !out) return PM_E_INVALID;
  PM_TRY
  *out = dot_host(c, n, x, y);
  return PM_OK;
  PM_CATCH(c)
}

int pm_norm(pm_ctx* c, int n, const double* x, double* out) {
  if (!c || !out) return PM_E_INVALID;
  PM_TRY
  *out = std::sqrt(dot_host(c, n, x, x));
  return PM_OK;
  PM_CATCH(c)
}

int pm_axpy(pm_ctx* c, int n, double a, const double* x, double* y) {
  if (!c) return PM_E_INVALID;
  PM_TRY
  vaxpy(c, n, a, x, y);
  return PM_OK;
  PM_CATCH(c)
}

int pm_scal(pm_ctx* c, int n, double a, double* x) {
  if (!c) return PM_E_INVALID;
  PM_TRY
  vscale(c, n, x, a);
  return PM_OK;
  PM_CATCH(c)
}

// ---------------------------------------------------------------- solver ---
int pm_solver_create(pm_ctx* c, const char* params, pm_solver** out) {
  if (!c || !out) return fail(c, PM_E_INVALID, "null argument");
  PM_TRY
  auto* s = new pm_solver();
  s->ctx = c;
  try {
    s->params = Params::parse(params);
    const Params& p = s->params;
    s->solver_type = p.str("solver_type", "direct");
    if (s->solver_type != "direct" && s->solver_type != "iterative")
      throw Error(PM_E_UNSUPPORTED, "solver_type must be direct or iterative");
    s->method = p.str("iterative_solver_type", "fgmres");
    s->prec = p.str("preconditioner", "no_preconditioner");
    s->tol = p.num("residual_tolerance", 1e-8);
    s->reduction = p.num("residual_reduction", 0.0);
    s->divergence = p.num("divergence_factor", 1e10);
    s->max_it = p.integer("max_n_iterations", 100);
    s->min_it = p.integer("min_n_iterations", 0);
    s->restart = p.integer("gmres_restart", 20);
    s->damping = p.num("damping_factor", 1.0);
    s->mixed = p.str("gpu_precision", "fp64") == "mixed";
    s->use_graphs = p.integer("gpu_cuda_graphs", 1) != 0;
    s->mixed_fallback = p.integer("gpu_mixed_fallback", 1) != 0;
    s->gram_schmidt = p.str("gpu_gram_schmidt", s->mixed ? "cgs2" : "mgs");
    if (s->gram_schmidt != "mgs" && s->gram_schmidt != "cgs2" && s->gram_schmidt != "cgs2_cond")
      throw Error(PM_E_INVALID, "gpu_gram_schmidt is mgs, cgs2 or cgs2_cond");
    if (s->prec != "no_preconditioner" && s->prec != "jacobi" && s->prec != "multigrid" && s->prec != "sor" &&
        s->prec != "ssor")
      throw Error(PM_E_UNSUPPORTED, "preconditioner '" + s->prec + "' is not implemented on the GPU");
    s->sor_omega = p.num("sor_omega", 1.5);
    s->use_mg = s->solver_type == "iterative" && s->prec == "multigrid";
    if (s->use_mg) {
      s->mg.configure(p);
      const int nl = int(p.integer("multigrid_n_levels", 2));
      if (nl < 2) throw Error(PM_E_INVALID, "for multigrid you need at least two multigrid levels");
      s->mg.levels.resize(nl);
    }
    if (s->mixed && !s->use_mg)
      throw Error(PM_E_INVALID, "gpu_precision mixed needs the multigrid preconditioner");
  } catch (...) {
    delete s;
    throw;
  }
  *out = s;
  return PM_OK;
  PM_CATCH(c)
}

void pm_solver_destroy(pm_solver* s) {
  if (!s) return;
  if (s->ctx && s->ctx->stream) cudaStreamSynchronize(s->ctx->stream);
  delete s;
}

static void transpose_csr(int nr, int nc, const int* rp, const int* ci, const double* v,
                          std::vector<int>& trp, std::vector<int>& tci, std::vector<double>& tv) {
  trp.assign(size_t(nc) + 1, 0);
  const int nnz = rp[nr];
  for (int k = 0; k < nnz; ++k) trp[ci[k] + 1]++;
  for (int j = 0; j < nc; ++j) trp[j + 1] += trp[j];
  tci.resize(nnz);
  tv.resize(nnz);
  std::vector<int> fill(trp.begin(), trp.end() - 1);
  for (int i = 0; i < nr; ++i)
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      tci[fill[ci[k]]] = i;
      tv[fill[ci[k]]++] = v[k];
    }
}

int pm_solver_set_multigrid_level(pm_solver* s, int level, int n_levels, pm_matrix* A, int p_rows,
                                  int p_cols, const int* p_rp, const int* p_ci, const double* p_v) {
  if (!s || !A) return fail(s ? s->ctx : nullptr, PM_E_INVALID, "null argument");
  PM_TRY
  if (!s->use_mg) throw Error(PM_E_INVALID, "solver does not use the multigrid preconditioner");
  if (n_levels != int(s->mg.levels.size()))
    throw Error(PM_E_INVALID, "multigrid_n_levels does not match the number of levels given");
  if (level < 0 || level >= n_levels) throw Error(PM_E_INVALID, "multigrid level out of range");
  MGLevel& lv = s->mg.levels[level];
  s->drop_graphs();
  lv.A = A;
  if (level < n_levels - 1) {
    if (!p_rp || !p_ci || !p_v) throw Error(PM_E_INVALID, "coarse levels need a prolongation");
    if (p_cols != A->csr.n_rows) throw Error(PM_E_INVALID, "prolongation columns must match the level size");
    if (!check_csr(p_rows, p_cols, p_rows, p_rp, p_ci)) throw Error(PM_E_INVALID, "invalid prolongation CSR");
    lv.P.upload(s->ctx, p_rows, p_cols, p_rows, p_rp, p_ci, p_v);
    std::vector<int> trp, tci;
    std::vector<double> tv;
    transpose_csr(p_rows, p_cols, p_rp, p_ci, p_v, trp, tci, tv);
    lv.R.upload(s->ctx, p_cols, p_rows, p_cols, trp.data(), tci.data(), tv.data());
  }
  s->mg.ready = false;
  return PM_OK;
  PM_CATCH(s->ctx)
}

int pm_solver_update_matrix(pm_solver* s, pm_matrix* A) {
  if (!s || !A) return fail(s ? s->ctx : nullptr, PM_E_INVALID, "null argument");
  PM_TRY
  s->A = A;
  s->direct_ready = false;
  if (s->use_mg) {
    auto& top = s->mg.levels.back();
    if (top.A && top.A != A) throw Error(PM_E_INVALID, "finest multigrid level must be the solver's matrix");
    top.A = A;
    s->mg.update(s->ctx);
  } else {
    A->csr.make_sliced64(s->ctx);
  }
  const bool sor = s->solver_type == "iterative" &&
                   (s->prec == "sor" || s->prec == "ssor" || s->method == "sor" || s->method == "ssor");
  if ((!s->use_mg && (s->prec == "jacobi" || s->method == "jacobi")) || sor) A->csr.make_diag(s->ctx);
  if (sor) {
    // the colour order of the sweeps (Iteration_sor as a solver or as the
    // preconditioner)
    s->sor.build(s->ctx, A->csr);
    pm::sor_check_diagonal(s->ctx, A->csr);
  }
  PM_CUDA(cudaStreamSynchronize(s->ctx->stream));
  return PM_OK;
  PM_CATCH(s->ctx)
}

int pm_solver_solve(pm_solver* s, const double* rhs, double* sol) {
  if (!s || !rhs || !sol) return fail(s ? s->ctx : nullptr, PM_E_INVALID, "null argument");
  PM_TRY
  s->solve(rhs, sol);
  return PM_OK;
  PM_CATCH(s->ctx)
}

int pm_solver_solve_host(pm_solver* s, const double* rhs_h, double* sol_h, int n) {
  if (!s || !rhs_h || !sol_h) return fail(s ? s->ctx : nullptr, PM_E_INVALID, "null argument");
  PM_TRY
  if (!s->A || n != s->A->csr.n_rows) throw Error(PM_E_INVALID, "vector length does not match the matrix");
  pm_ctx* c = s->ctx;
  DBuf<double> r(n), x(n);
  r.upload(rhs_h, n, c->stream);
  x.upload(sol_h, n, c->stream);
  s->solve(r.p, x.p);
  x.download(sol_h, c->stream);
  return PM_OK;
  PM_CATCH(s->ctx)
}

int pm_solver_last_info(const pm_solver* s, int* it, double* res, double* init) {
  if (!s) return PM_E_INVALID;
  if (it) *it = s->last_it;
  if (res) *res = s->last_res;
  if (init) *init = s->init_res;
  return PM_OK;
}

int pm_solver_residual_history(const pm_solver* s, double* out, int cap, int* count) {
  if (!s) return PM_E_INVALID;
  const int n = int(s->history.size());
  for (int i = 0; i < n && i < cap; ++i) out[i] = s->history[i];
  if (count) *count = n;
  return PM_OK;
}

int pm_solver_apply_preconditioner(pm_solver* s, const double* z, double* r) {
  if (!s || !z || !r) return PM_E_INVALID;
  PM_TRY
  if (!s->A) throw Error(PM_E_INVALID, "preconditioner used before update_matrix");
  s->precondition(z, r);
  return PM_OK;
  PM_CATCH(s->ctx)
}

// ------------------------------------------------------------------ disc ---
int pm_disc_create(int geometry, int root_n, int n_refine, int n_levels, int kind, int elem,
                   pm_disc** out) {
  if (!out) return fail(nullptr, PM_E_INVALID, "null argument");
  PM_TRY
  auto* d = new pm_disc();
  d->d = build_disc(geometry, root_n, n_refine, n_levels, kind, elem);
  *out = d;
  return PM_OK;
  PM_CATCH(nullptr)
}

int pm_disc_create_bc(int geometry, int root_n, int n_refine, int n_levels, int kind, int elem,
                      int neumann_sides, pm_disc** out) {
  if (!out) return fail(nullptr, PM_E_INVALID, "null argument");
  PM_TRY
  auto* d = new pm_disc();
  try {
    d->d = build_disc(geometry, root_n, n_refine, n_levels, kind, elem, neumann_sides);
  } catch (...) {
    delete d;
    throw;
  }
  *out = d;
  return PM_OK;
  PM_CATCH(nullptr)
}

int pm_disc_create_device(pm_ctx* c, int geometry, int root_n, int n_refine, int n_levels, int kind, int elem,
                          int neumann_sides, pm_disc** out) {
  if (!c || !out) return fail(c, PM_E_INVALID, "null argument");
  PM_TRY
  auto* d = new pm_disc();
  try {
    SetupParts parts;
    parts.hierarchy = [c](int g, int r, int n) { return device_hierarchy(c, g, r, n); };
    parts.space = [c](const pmsetup::Hierarchy& h, int level, int elem_, int bnd, int ns) {
      return device_space(c, h, level, elem_, bnd, ns);
    };
    parts.structure = [c](DiscLevel& L) { device_level_structure(c, L); };
    parts.stokes_structure = [c](DiscLevel& L, const std::vector<char>& act) { device_stokes_structure(c, L, act); };
    d->d = build_disc(geometry, root_n, n_refine, n_levels, kind, elem, neumann_sides, &parts);
  } catch (...) {
    delete d;
    throw;
  }
  *out = d;
  return PM_OK;
  PM_CATCH(c)
}

void pm_disc_destroy(pm_disc* d) { delete d; }

static const DiscLevel* disc_level(const pm_disc* d, int level) {
  if (!d || level < 0 || level >= int(d->d->levels.size())) return nullptr;
  return &d->d->levels[level];
}

int pm_disc_level_info(const pm_disc* d, int level, int space, int* n_cells, int* nloc,
                       int* n_dofs, int* n_active, int64_t* nnz) {
  const DiscLevel* L = disc_level(d, level);
  if (!L) return fail(nullptr, PM_E_INVALID, "level out of range");
  const pmsetup::Space& s = space == 1 ? L->pspace : L->space;
  if (n_cells) *n_cells = L->n_cells;
  if (nloc) *nloc = s.nloc;
  if (n_dofs) *n_dofs = s.n_dofs;
  if (n_active) *n_active = s.n_active;
  if (nnz) *nnz = L->sys.row_ptr.empty() ? 0 : L->sys.row_ptr.back();
  return PM_OK;
}

int pm_disc_dofmap(const pm_disc* d, int level, int space, int* out) {
  const DiscLevel* L = disc_level(d, level);
  if (!L || !out) return fail(nullptr, PM_E_INVALID, "bad argument");
  const pmsetup::Space& s = space == 1 ? L->pspace : L->space;
  std::memcpy(out, s.dofmap.data(), s.dofmap.size() * sizeof(int));
  return PM_OK;
}

int pm_disc_cell_vertices(const pm_disc* d, int level, double* out) {
  const DiscLevel* L = disc_level(d, level);
  if (!L || !out) return fail(nullptr, PM_E_INVALID, "bad argument");
  std::memcpy(out, L->verts.data(), L->verts.size() * sizeof(double));
  return PM_OK;
}

int pm_disc_structure(const pm_disc* d, int level, int* rp, int* ci) {
  const DiscLevel* L = disc_level(d, level);
  if (!L) return fail(nullptr, PM_E_INVALID, "level out of range");
  if (rp) std::memcpy(rp, L->sys.row_ptr.data(), L->sys.row_ptr.size() * sizeof(int));
  if (ci) std::memcpy(ci, L->sys.cols.data(), L->sys.cols.size() * sizeof(int));
  return PM_OK;
}

int pm_disc_prolongation_info(const pm_disc* d, int level, int* rows, int* cols, int64_t* nnz) {
  const DiscLevel* L = disc_level(d, level);
  if (!L || level + 1 >= int(d->d->levels.size())) return fail(nullptr, PM_E_INVALID, "no prolongation above the finest level");
  if (rows) *rows = L->P.n_rows;
  if (cols) *cols = L->P.n_cols;
  if (nnz) *nnz = L->P.row_ptr.back();
  return PM_OK;
}

int pm_disc_prolongation(const pm_disc* d, int level, int* rp, int* ci, double* v) {
  const DiscLevel* L = disc_level(d, level);
  if (!L || level + 1 >= int(d->d->levels.size())) return fail(nullptr, PM_E_INVALID, "no prolongation above the finest level");
  if (rp) std::memcpy(rp, L->P.row_ptr.data(), L->P.row_ptr.size() * sizeof(int));
  if (ci) std::memcpy(ci, L->P.cols.data(), L->P.cols.size() * sizeof(int));
  if (v) std::memcpy(v, L->P.vals.data(), L->P.vals.size() * sizeof(double));
  return PM_OK;
}

// --------------------------------------------------------------- assembly --
static int default_quad_points(const Disc& D) {
  // ParMooN picks degree N_terms * polynomial degree (FEDatabase3D.C:1153-1207);
  // for convection-diffusion (N_terms = 3): Q1 -> Gauss3, Q2 -> Gauss4; on
  // tetrahedra P1 (degree 3) -> P4Tetra (11 points), P2 (degree 6) ->
  // P5Tetra (15 points)
  if (D.elem == pmsetup::EL_P1) return 11;
  if (D.elem == pmsetup::EL_P2) return 15;
  if (D.elem == 1) return 3;
  return 4;
}

int pm_assemble_cd(pm_ctx* c, const pm_disc* d, int level, const pm_cd_coeffs* cf, int qn,
                   pm_matrix* A, double* rhs) {
  if (!c || !d || !cf || !A || !rhs) return fail(c, PM_E_INVALID, "null argument");
  PM_TRY
  const DiscLevel* L = disc_level(d, level);
  if (!L) throw Error(PM_E_INVALID, "level out of range");
  if (A->csr.nnz != L->sys.row_ptr.back() || A->csr.n_rows != L->sys.n_rows)
    throw Error(PM_E_INVALID, "matrix does not have the level's CSR pattern");
  if (qn == 0) qn = default_quad_points(*d->d);
  RefTables t;
  build_element_tables(d->d->dim(), d->d->elem, qn, t);
  DevRefTables rt;
  rt.upload(c, t);
  DevAssemblyLevel dl;
  dl.upload(c, *L, d->d->dim(), d->d->nvc());
  size_t kn, fn;
  dl.scratch_sizes(kn, fn);
  DBuf<double> K(kn), F(fn);
  assemble_cd_level(c, dl, d->d->dim(), d->d->elem, qn, *cf, rt, A->csr, rhs, K.p, F.p);
  if (A->csr.diag.p) A->csr.make_diag(c);
  if (A->csr.vals32.p) A->csr.make_fp32(c);
  PM_CUDA(cudaStreamSynchronize(c->stream));
  return PM_OK;
  PM_CATCH(c)
}

// --------------------------------------------------------------- problem ---
int pm_problem_create_cd(pm_ctx* c, const pm_disc* d, const pm_cd_coeffs* cf, int qn,
                         const char* params, pm_problem** out) {
  if (!c || !d || !cf || !out) return fail(c, PM_E_INVALID, "null argument");
  PM_TRY
  auto* p = new pm_problem();
  try {
    p->ctx = c;
    p->disc = d;
    p->coeffs = *cf;
    const Disc& D = *d->d;
    p->qn = qn ? qn : default_quad_points(D);
    RefTables t;
    build_element_tables(D.dim(), D.elem, p->qn, t);
    p->ref.upload(c, t);
    size_t kmax = 0, fmax = 0;
    const int nl = int(D.levels.size());
    p->alev.resize(nl);
    for (int l = 0; l < nl; ++l) {
      const DiscLevel& L = D.levels[l];
      pm_matrix* A = new pm_matrix();
      A->ctx = c;
      A->owned_by_problem = true;
      p->mats.push_back(A);
      A->csr.upload(c, L.sys.n_rows, L.sys.n_cols, L.space.n_active, L.sys.row_ptr.data(),
                    L.sys.cols.data(), nullptr);
      p->alev[l].upload(c, L, D.dim(), D.nvc());
      size_t kn, fn;
      p->alev[l].scratch_sizes(kn, fn);
      kmax = std::max(kmax, kn);
      fmax = std::max(fmax, fn);
    }
    p->K.alloc(kmax);
    p->F.alloc(fmax);
    const int n = D.levels.back().sys.n_rows;
    p->rhs.alloc(n);
    p->sol.alloc(n);
    p->rhs_coarse.alloc(n);
    PM_CUDA(cudaMemsetAsync(p->sol.p, 0, sizeof(double) * n, c->stream));
    // solver from the parameter text; multigrid levels follow the disc levels
    std::string text = params ? params : "";
    Params prm = Params::parse(text.c_str());
    if (prm.str("preconditioner", "") == "multigrid" && !prm.has("multigrid_n_levels"))
      text += "\nmultigrid_n_levels: " + std::to_string(nl) + "\n";
    int rc = pm_solver_create(c, text.c_str(), &p->solver);
    if (rc != PM_OK) throw Error(rc, c->last_error);
    if (p->solver->use_mg) {
      const int ml = int(p->solver->mg.levels.size());
      if (ml > nl) throw Error(PM_E_INVALID, "more multigrid levels requested than the discretisation keeps");
      for (int l = 0; l < ml; ++l) {
        const int dl = nl - ml + l;
        const DiscLevel& L = D.levels[dl];
        if (l < ml - 1) {
          rc = pm_solver_set_multigrid_level(p->solver, l, ml, p->mats[dl], L.P.n_rows, L.P.n_cols,
                                             L.P.row_ptr.data(), L.P.cols.data(), L.P.vals.data());
        } else {
          rc = pm_solver_set_multigrid_level(p->solver, l, ml, p->mats[dl], 0, 0, nullptr, nullptr, nullptr);
        }
        if (rc != PM_OK) throw Error(rc, c->last_error);
      }
    }
  } catch (...) {
    delete p;
    throw;
  }
  *out = p;
  return PM_OK;
  PM_CATCH(c)
}

void pm_problem_destroy(pm_problem* p) { delete p; }

int pm_problem_create_stokes(pm_ctx* c, const pm_disc* d, double nu, const char* params, pm_problem** out) {
  if (!c || !d || !out) return fail(c, PM_E_INVALID, "null argument");
  PM_TRY
  if (d->d->kind != KIND_STOKES) throw Error(PM_E_INVALID, "the discretisation is not a Stokes set-up");
  auto* p = new pm_problem();
  try {
    p->ctx = c;
    p->disc = d;
    p->kind = KIND_STOKES;
    p->nu = nu;
    // Example_NSE3D's "example" key: -3 is the polynomial solution in P2 / P1
    p->stokes_example = int(Params::parse(params ? params : "").integer("example", 0));
    if (p->stokes_example != 0 && p->stokes_example != -3)
      throw Error(PM_E_UNSUPPORTED, "Stokes example must be 0 (manufactured) or -3 (test_u_2_p_1)");
    // problem_type 3 Stokes, 5 Navier-Stokes (ParameterDatabase "problem_type")
    p->problem_type = int(Params::parse(params ? params : "").integer("problem_type", 3));
    if (p->problem_type != 3 && p->problem_type != 5)
      throw Error(PM_E_UNSUPPORTED, "problem_type must be 3 (Stokes) or 5 (Navier-Stokes)");
    if (p->problem_type == 5 && p->stokes_example != -3)
      throw Error(PM_E_UNSUPPORTED, "the Navier-Stokes problem is implemented for example -3 (test_u_2_p_1)");
    p->params_text = params ? params : "";
    // nse_nonlinear_form (LocalAssembling.C:593): the convective and the
    // skew-symmetric forms act on the diagonal velocity blocks; rotational,
    // divergence and emac couple the velocity components (blocks A12 ...)
    const std::string form = Params::parse(params ? params : "").str("nse_nonlinear_form", "convective");
    if (form != "convective" && form != "skew_symmetric")
      throw Error(PM_E_UNSUPPORTED, "nse_nonlinear_form '" + form + "': convective or skew_symmetric");
    const Disc& D = *d->d;
    const int nl = int(D.levels.size());
    // the rule of the assembly: degree 2 x 2 for the linear (Stokes) problem,
    // 3 x 2 for the nonlinear one (FEDatabase3D.C:1153-1219)
    p->stab.upload(c, p->problem_type == 5 ? 15 : 11, form == "skew_symmetric");
    size_t kmax = 0, fmax = 0;
    p->slev.resize(nl);
    const Params pre = Params::parse(params ? params : "");
    const bool want_nodal = pre.str("multigrid_smoother", "").rfind("nodal_vanka", 0) == 0 ||
                            pre.str("multigrid_smoother_coarse", "").rfind("nodal_vanka", 0) == 0;
    for (int l = 0; l < nl; ++l) {
      const DiscLevel& L = D.levels[l];
      pm_matrix* A = new pm_matrix();
      A->ctx = c;
      A->owned_by_problem = true;
      p->mats.push_back(A);
      A->csr.upload(c, L.sys.n_rows, L.sys.n_cols, L.sys.n_active, L.sys.row_ptr.data(), L.sys.cols.data(),
                    nullptr);
      A->csr.set_blocks(L.n_blocks, L.block_len, L.block_active);
      p->slev[l].upload(c, L);
      auto pr = std::make_unique<ProjectedMatrix>();
      pr->build(c, L.sys, L.pressure_row0, A->csr.mask);
      p->proj.push_back(std::move(pr));
      auto vk = std::make_unique<DevVanka>();
      vk->setup(c, L);
      p->vanka.push_back(std::move(vk));
      if (want_nodal) {
        auto nv = std::make_unique<DevNodalVanka>();
        nv->setup(c, L);
        p->nodal.push_back(std::move(nv));
      }
      kmax = std::max(kmax, size_t(L.n_cells) * L.elem_stride);
      fmax = std::max(fmax, size_t(L.n_cells) * L.rhs_stride);
    }
    p->K.alloc(kmax);
    p->F.alloc(fmax);
    const int n = D.levels.back().sys.n_rows;
    p->rhs.alloc(n);
    p->sol.alloc(n);
    p->rhs_coarse.alloc(n);
    PM_CUDA(cudaMemsetAsync(p->sol.p, 0, sizeof(double) * n, c->stream));
    p->defect.alloc(n);
    p->res2.alloc(kResidualScratch);
    if (p->problem_type == 5) {
      // velocities of the coarser levels (zero until the first restriction)
      size_t cmax = 0;
      p->ulev.resize(nl);
      for (int l = 0; l + 1 < nl; ++l) {
        p->slev[l].set_children(c, D.h.levels[D.levels[l + 1].level_in_hierarchy], D.levels[l]);
        p->ulev[l].alloc(size_t(3) * p->slev[l].nvel);
        PM_CUDA(cudaMemsetAsync(p->ulev[l].p, 0, p->ulev[l].bytes(), c->stream));
        cmax = std::max(cmax, size_t(p->slev[l].n_cells) * 30);
      }
      if (nl > 1) {
        std::vector<double> q;
        build_p2_restriction(D.h, q);
        p->rq.upload(q, c->stream);
        p->cellval.alloc(cmax);
      }
    }
    std::string text = params ? params : "";
    Params prm = Params::parse(text.c_str());
    if (prm.str("preconditioner", "") == "multigrid" && !prm.has("multigrid_n_levels"))
      text += "\nmultigrid_n_levels: " + std::to_string(nl) + "\n";
    int rc = pm_solver_create(c, text.c_str(), &p->solver);
    if (rc != PM_OK) throw Error(rc, c->last_error);
    if (p->solver->use_mg) {
      const int ml = int(p->solver->mg.levels.size());
      if (ml > nl) throw Error(PM_E_INVALID, "more multigrid levels requested than the discretisation keeps");
      for (int l = 0; l < ml; ++l) {
        const int dl = nl - ml + l;
        const DiscLevel& L = D.levels[dl];
        if (l < ml - 1)
          rc = pm_solver_set_multigrid_level(p->solver, l, ml, p->mats[dl], L.P.n_rows, L.P.n_cols,
                                             L.P.row_ptr.data(), L.P.cols.data(), L.P.vals.data());
        else
          rc = pm_solver_set_multigrid_level(p->solver, l, ml, p->mats[dl], 0, 0, nullptr, nullptr, nullptr);
        if (rc != PM_OK) throw Error(rc, c->last_error);
        p->solver->mg.levels[l].proj = p->proj[dl].get();
        p->solver->mg.levels[l].vanka = p->vanka[dl].get();
        if (want_nodal) p->solver->mg.levels[l].nodal = p->nodal[dl].get();
      }
    }
  } catch (...) {
    delete p;
    throw;
  }
  *out = p;
  return PM_OK;
  PM_CATCH(c)
}

int pm_problem_assemble(pm_problem* p) {
  if (!p) return PM_E_INVALID;
  PM_TRY
  pm_ctx* c = p->ctx;
  const Disc& D = *p->disc->d;
  const int nl = int(D.levels.size());
  if (p->kind == KIND_STOKES) {
    // NavierStokes<3>::assemble_linear_terms (NavierStokes.C:407-570); for the
    // Navier-Stokes problem NavierStokesAll holds the convective term of each
    // level's current velocity (zero before the first solve)
    for (int l = 0; l < nl; ++l) {
      double* r = (l == nl - 1) ? p->rhs.p : p->rhs_coarse.p;
      if (p->problem_type == 5)
        assemble_nse_level(c, p->slev[l], p->stab, p->nu, p->mats[l]->csr, l == nl - 1 ? p->sol.p : p->ulev[l].p,
                           r, p->K.p, p->F.p);
      else
        assemble_stokes_level(c, p->slev[l], p->stab, p->nu, p->mats[l]->csr, r, p->K.p, p->F.p,
                              p->stokes_example);
    }
    const DevCsr& top = p->mats.back()->csr;
    copy_nonactive(c, top.n_rows, top.mask, p->rhs.p, p->sol.p);
    p->solver_ready = false;
    return PM_OK;
  }
  for (int l = 0; l < nl; ++l) {
    double* r = (l == nl - 1) ? p->rhs.p : p->rhs_coarse.p;
    assemble_cd_level(c, p->alev[l], D.dim(), D.elem, p->qn, p->coeffs, p->ref, p->mats[l]->csr, r,
                      p->K.p, p->F.p);
    // the coarse factorisation overlaps the assembly of the finer levels; the
    // multigrid's coarsest level is disc level nl - (multigrid levels)
    if (p->solver->use_mg && l == nl - int(p->solver->mg.levels.size()) && l + 1 < nl)
      p->solver->mg.start_coarse(c);
  }
  // copy_nonactive(rhs -> solution) (ConvectionDiffusion.C:343)
  const DevCsr& top = p->mats.back()->csr;
  const int n = top.n_rows, na = top.n_active;
  if (n > na)
    PM_CUDA(cudaMemcpyAsync(p->sol.p + na, p->rhs.p + na, sizeof(double) * (n - na),
                            cudaMemcpyDeviceToDevice, c->stream));
  // matrices changed: the solver's update_matrix runs again before the solve
  p->solver_ready = false;
  return PM_OK;
  PM_CATCH(p->ctx)
}

int pm_problem_solve(pm_problem* p) {
  if (!p) return PM_E_INVALID;
  PM_TRY
  if (!p->solver_ready) {
    int rc = pm_solver_update_matrix(p->solver, p->mats.back());
    if (rc != PM_OK) return rc;
    p->solver_ready = true;
  }
  p->solver->solve(p->rhs.p, p->sol.p);
  // NavierStokes::solve (NavierStokes.C:910-912): with the pressure projection
  // (all-Dirichlet velocity) the pressure is moved into L2_0
  if (p->kind == KIND_STOKES) project_pressure_l20(p->ctx, p->slev.back(), p->sol.p + 3 * size_t(p->slev.back().nvel));
  return PM_OK;
  PM_CATCH(p->ctx)
}

int pm_problem_assemble_nonlinear(pm_problem* p) {
  if (!p) return PM_E_INVALID;
  PM_TRY
  if (p->kind != KIND_STOKES || p->problem_type != 5)
    throw Error(PM_E_INVALID, "assemble_nonlinear_term needs a Navier-Stokes problem (problem_type 5)");
  pm_ctx* c = p->ctx;
  const int nl = int(p->slev.size());
  // RestrictFunctionRepeatedly: finest -> coarsest, each from the one above
  for (int l = nl - 2; l >= 0; --l) {
    const double* uf = (l == nl - 2) ? p->sol.p : p->ulev[l + 1].p;
    restrict_velocity(c, p->slev[l], p->slev[l + 1], p->rq.p, uf, p->ulev[l].p, p->cellval.p);
  }
  for (int l = 0; l < nl; ++l)
    assemble_nse_level(c, p->slev[l], p->stab, p->nu, p->mats[l]->csr, l == nl - 1 ? p->sol.p : p->ulev[l].p,
                       nullptr, p->K.p, p->F.p);
  p->solver_ready = false;
  return PM_OK;
  PM_CATCH(p->ctx)
}

int pm_problem_residuals(pm_problem* p, double* out) {
  if (!p || !out) return PM_E_INVALID;
  PM_TRY
  if (p->kind != KIND_STOKES) throw Error(PM_E_INVALID, "residuals of a convection-diffusion problem");
  pm_ctx* c = p->ctx;
  nse_residuals(c, p->slev.back(), p->mats.back()->csr, p->rhs.p, p->sol.p, p->defect.p, p->res2.p);
  double h[4];
  PM_CUDA(cudaMemcpyAsync(h, p->res2.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));
  // BlockVector::norm(blocks) (src/Matrix/BlockVector.C:293) sums the blocks'
  // 2-norms; Residuals(imR, maR) takes the squares of the two sums
  out[0] = std::sqrt(h[0]) + std::sqrt(h[1]) + std::sqrt(h[2]);
  out[1] = std::sqrt(h[3]);
  out[2] = std::sqrt(out[0] * out[0] + out[1] * out[1]);
  return PM_OK;
  PM_CATCH(p->ctx)
}

int pm_problem_solve_nonlinear(pm_problem* p, int max_records, double* residuals, int* n_steps) {
  if (!p) return PM_E_INVALID;
  PM_TRY
  if (p->kind != KIND_STOKES || p->problem_type != 5)
    throw Error(PM_E_INVALID, "the nonlinear loop needs a Navier-Stokes problem (problem_type 5)");
  pm_ctx* c = p->ctx;
  const Params prm = Params::parse(p->params_text.c_str());
  const long max_it = prm.integer("nonlinloop_maxit", 100);
  const long min_it = prm.integer("nonlinloop_minit", 1);
  double limit = prm.num("nonlinloop_epsilon", 1e-10);
  const double damping = prm.num("nonlinloop_damping_factor", 1.0);
  const double slow = prm.num("nonlinloop_slowfactor", 1e10);
  auto flag = [&](const char* k) {
    const std::string v = prm.str(k, "false");
    return v == "true" || v == "1";
  };
  const int n = p->mats.back()->csr.n_rows;
  if (flag("nonlinloop_scale_epsilon_with_size")) limit *= std::sqrt(double(n));
  // old_residuals: FixedSizeQueue<10, Residuals>, filled with 1e10 at the start
  std::deque<double> old(10, 1e10);
  double initial_rhs_norm = 0.0;
  pm::DBuf<double> prev;
  if (damping != 1.0) prev.alloc(n);
  int k = 0;
  auto record = [&](const double* r) {
    if (residuals && k < max_records)
      for (int i = 0; i < 3; ++i) residuals[3 * k + i] = r[i];
  };
  // NavierStokes::stop_it (NavierStokes.C:753-816)
  auto stop_it = [&](int it) {
    double r[3];
    int rc = pm_problem_residuals(p, r);
    if (rc != PM_OK) throw Error(rc, c->last_error);
    record(r);
    old.push_back(r[2]);
    old.pop_front();
    if (it == 0) initial_rhs_norm = std::sqrt(dot_host(c, n, p->rhs.p, p->rhs.p));
    if (it < min_it) return false;
    const bool slow_conv = r[2] >= slow * old.front();
    double lim = limit;
    if (flag("nonlinloop_residual_relative_to_rhs")) lim *= initial_rhs_norm;
    return r[2] <= lim || it == max_it || slow_conv;
  };
  stop_it(0);
  for (k = 1;; ++k) {
    if (damping != 1.0) vcopy(c, n, p->sol.p, prev.p);
    int rc = pm_problem_solve(p);
    if (rc != PM_OK) return rc;
    if (damping != 1.0) {
      // x = w x_new + (1 - w) x_old, then the pressure back into L2_0
      vaxpby(c, n, 1.0 - damping, prev.p, damping, p->sol.p);
      project_pressure_l20(c, p->slev.back(), p->sol.p + 3 * size_t(p->slev.back().nvel));
    }
    rc = pm_problem_assemble_nonlinear(p);
    if (rc != PM_OK) return rc;
    if (stop_it(k)) break;
  }
  if (n_steps) *n_steps = k;
  return PM_OK;
  PM_CATCH(p->ctx)
}

int pm_problem_reset_solution(pm_problem* p) {
  if (!p) return PM_E_INVALID;
  PM_TRY
  PM_CUDA(cudaMemsetAsync(p->sol.p, 0, p->sol.bytes(), p->ctx->stream));
  return PM_OK;
  PM_CATCH(p->ctx)
}

int pm_problem_size(const pm_problem* p, int* n, int* na) {
  if (!p) return PM_E_INVALID;
  if (n) *n = p->mats.back()->csr.n_rows;
  if (na) *na = p->mats.back()->csr.n_active;
  return PM_OK;
}

int pm_problem_get_solution(const pm_problem* p, double* out) {
  if (!p || !out) return PM_E_INVALID;
  PM_TRY
  p->sol.download(out, p->ctx->stream);
  PM_CUDA(cudaStreamSynchronize(p->ctx->stream));
  return PM_OK;
  PM_CATCH(p->ctx)
}

int pm_problem_set_solution(pm_problem* p, const double* in) {
  if (!p || !in) return PM_E_INVALID;
  PM_TRY
  PM_CUDA(cudaMemcpyAsync(p->sol.p, in, p->sol.bytes(), cudaMemcpyHostToDevice, p->ctx->stream));
  PM_CUDA(cudaStreamSynchronize(p->ctx->stream));
  return PM_OK;
  PM_CATCH(p->ctx)
}

int pm_problem_get_rhs(const pm_problem* p, double* out) {
  if (!p || !out) return PM_E_INVALID;
  PM_TRY
  p->rhs.download(out, p->ctx->stream);
  PM_CUDA(cudaStreamSynchronize(p->ctx->stream));
  return PM_OK;
  PM_CATCH(p->ctx)
}

int pm_problem_matrix(pm_problem* p, int level, pm_matrix** out) {
  if (!p || !out || level < 0 || level >= int(p->mats.size())) return PM_E_INVALID;
  *out = p->mats[level];
  return PM_OK;
}

int pm_problem_solver(pm_problem* p, pm_solver** out) {
  if (!p || !out) return PM_E_INVALID;
  *out = p->solver;
  return PM_OK;
}

int pm_problem_solution_dev(pm_problem* p, double** sol, double** rhs) {
  if (!p) return PM_E_INVALID;
  if (sol) *sol = p->sol.p;
  if (rhs) *rhs = p->rhs.p;
  return PM_OK;
}

int pm_problem_run_host(pm_problem* p, const pm_cd_coeffs* cf, const double* const* level_verts,
                        double* sol_host) {
  if (!p || !sol_host) return PM_E_INVALID;
  PM_TRY
  pm_ctx* c = p->ctx;
  if (cf) p->coeffs = *cf;
  if (level_verts)
    for (size_t l = 0; l < p->mats.size(); ++l) {
      DBuf<double>& verts = p->kind == KIND_STOKES ? p->slev[l].verts : p->alev[l].verts;
      if (level_verts[l])
        PM_CUDA(cudaMemcpyAsync(verts.p, level_verts[l], verts.bytes(), cudaMemcpyHostToDevice, c->stream));
    }
  // a new request starts from the zero initial guess
  PM_CUDA(cudaMemsetAsync(p->sol.p, 0, p->sol.bytes(), c->stream));
  int rc = pm_problem_assemble(p);
  if (rc != PM_OK) return rc;
  // a Navier-Stokes request runs the nonlinear loop
  rc = (p->kind == KIND_STOKES && p->problem_type == 5) ? pm_problem_solve_nonlinear(p, 0, nullptr, nullptr)
                                                        : pm_problem_solve(p);
  if (rc != PM_OK) return rc;
  p->sol.download(sol_host, c->stream);
  PM_CUDA(cudaStreamSynchronize(c->stream));
  return PM_OK;
  PM_CATCH(p->ctx)
}

int pm_problem_errors(pm_problem* p, double* errors) {
  if (!p || !errors) return PM_E_INVALID;
  PM_TRY
  if (p->kind != KIND_CD) throw Error(PM_E_UNSUPPORTED, "pm_problem_errors: convection-diffusion problems only");
  pm_ctx* c = p->ctx;
  const Disc& D = *p->disc->d;
  const DiscLevel& top = D.levels.back();
  // TFEFunction{2,3}D::GetErrors evaluate on the rule TFEDatabase{2,3}D::GetOrig
  // picks, the assembly's (degree N_terms x k, FEDatabase2D.C:1718-1790,
  // FEDatabase3D.C:1129-1163)
  const int qn = p->qn;
  if (p->err_qn != qn) {
    RefTables t;
    build_element_tables(D.dim(), D.elem, qn, t);
    p->err_ref.upload(c, t);
    p->err_dofmap.upload(top.space.dofmap, c->stream);
    p->err_out.alloc(4);
    p->err_qn = qn;
  }
  if (size_t(error_blocks(top.n_cells)) * 4 > p->F.n) throw Error(PM_E_INVALID, "error partials exceed the scratch");
  launch_cd_errors(c, D.dim(), D.elem, qn, top.n_cells, p->alev.back().verts.p, p->err_dofmap.p, p->sol.p,
                   p->err_ref, p->coeffs, p->F.p, p->err_out.p);
  p->err_out.download(errors, c->stream);
  PM_CUDA(cudaStreamSynchronize(c->stream));
  return PM_OK;
  PM_CATCH(p->ctx)
}

int pm_problem_last_info(const pm_problem* p, int* it, double* res, double* init) {
  if (!p) return PM_E_INVALID;
  return pm_solver_last_info(p->solver, it, res, init);
}

int pm_ctx_probe(pm_ctx* c, int64_t nnz) {
  if (!c) return PM_E_INVALID;
  PM_TRY
  probe_reset(c, nnz);
  return PM_OK;
  PM_CATCH(c)
}

int pm_ctx_probe_result(pm_ctx* c, int* launches, double* ms, double* bytes) {
  if (!c || !launches || !ms || !bytes) return PM_E_INVALID;
  PM_TRY
  probe_result(c, launches, ms, bytes);
  return PM_OK;
  PM_CATCH(c)
}

}  // extern "C"

pm_problem::~pm_problem() {
  if (ctx && ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (solver) pm_solver_destroy(solver);
  for (auto* m : mats) delete m;
}
