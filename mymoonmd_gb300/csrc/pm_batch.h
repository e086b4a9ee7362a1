// Batched launches: one kernel launch carries the same operation of up to
// kMaxBatch convection-diffusion problems of one set-up (one mesh hierarchy,
// one FE space, hence one CSR structure per level). blockIdx.y selects the
// problem ("slot"), except in the SpMV family, where blockIdx.x is the slot
// and blockIdx.y the row block: consecutive blocks then read the same part of
// the shared structure (column indices, slice layout) for the different slots,
// so it comes from L2 after the first slot. The kernels run the bodies of the
// single-problem kernels
// with the slot's pointers, so every slot computes exactly what a lone solve
// computes (same rows, same summation orders, same bits).
//
// Per launch, a Batch value tells each kernel where its slot's operands are:
//   on      per slot: 1 = the slot takes part in this launch (others return)
//   stride  bytes between the slots' copies of every vector argument: the
//           vectors of all slots live in one allocation, one block per slot
//   vals    per slot: the matrix values of this launch (the slot's own
//           assembled matrix), or null when all slots share the values
//           (the grid transfer operators depend on the mesh only)
//   aux     per slot: a second per-slot operand (the Jacobi diagonal, the
//           coarse-grid inverse), or null
#pragma once
#include "pm_linalg.cuh"

namespace pm {

constexpr int kMaxBatch = 16;
// the fused CGS2 sweeps of a batch hold at most 32 basis vectors
constexpr int kBatchMaxRestart = 32;

struct Batch {
  const int* on = nullptr;
  long long stride = 0;
  const void* const* vals = nullptr;
  const void* const* aux = nullptr;
};

// p moved to slot s (default: the slot of blockIdx.y)
template <class T>
__device__ __forceinline__ T* slot_ptr(T* p, const Batch& bt, int s) {
  return p ? reinterpret_cast<T*>(reinterpret_cast<char*>(const_cast<void*>(static_cast<const void*>(p))) +
                                  (long long)s * bt.stride)
           : p;
}
template <class T>
__device__ __forceinline__ T* slot_ptr(T* p, const Batch& bt) {
  return slot_ptr(p, bt, int(blockIdx.y));
}

// ---- SpMV family on the matrices of a slot (pm_linalg.cu) ----------------
// y = epilogue(A_s x_s) for every slot s with bt.on[s]; A is slot 0's matrix
// (structure and launch shape shared by all slots); vectors and the diagonal
// follow bt. Same kernel choice as csr_apply / csr_apply32.
void csr_apply_batch(pm_ctx* c, const DevCsr& A, int n_slots, const Batch& bt, int epi, const double* x,
                     double* y, const double* b, double alpha);
void csr_apply32_batch(pm_ctx* c, const DevCsr& A, int n_slots, const Batch& bt, int epi, const float* x,
                       float* y, const float* b, float alpha);

// ---- vector kernels (pm_linalg.cu) ----------------------------------------
void vcopy_batch(pm_ctx* c, int n_slots, const Batch& bt, int n, const double* x, double* y);
void vcvt_d2f_batch(pm_ctx* c, int n_slots, const Batch& bt, int n, const double* x, float* y);
void vcvt_f2d_batch(pm_ctx* c, int n_slots, const Batch& bt, int n, const float* x, double* y);
template <class T>
void init_solution_batch(pm_ctx* c, int n_slots, const Batch& bt, int n, const BlockMask& m, const T* rhs, T* sol);
// x = w (b / d) with d from bt.aux (per slot)
template <class T>
void jacobi_from_zero_batch(pm_ctx* c, int n_slots, const Batch& bt, int n, const T* b, T w, T* x);
// coarse direct solve x = Inv b on the active rows (Inv from bt.aux, act/pos shared)
void coarse_solve_batch(pm_ctx* c, int n_slots, const Batch& bt, const DenseInverse& inv0, const double* b,
                        double* x);
void coarse_solve32_batch(pm_ctx* c, int n_slots, const Batch& bt, const DenseInverse& inv0, const float* b,
                          float* x);
// partial sums of <x, y> per slot (kRedBlocks per slot at `part`), then
// out = sum (sqrt if asked)
void dot_partials_batch(pm_ctx* c, int n_slots, const Batch& bt, int n, const double* x, const double* y,
                        double* part);
void finish_sum_batch(pm_ctx* c, int n_slots, const Batch& bt, const double* part, double* out, bool take_sqrt);
void nonactive_nonzero_batch(pm_ctx* c, int n_slots, const Batch& bt, const BlockMask& m, const double* x,
                             int* flag);

// ---- FGMRES kernels (pm_solver.cu) -----------------------------------------
// all pointers are slot 0's; bt.stride moves them to the other slots
void fg_start_batch(pm_ctx* c, int n_slots, const Batch& bt, int n, int m, const double* r, double* v0,
                    const double* part, double* s, double* beta_out);
void fg_cgs2_batch(pm_ctx* c, int n_slots, const Batch& bt, int n, int i, int ldh, double* r, const double* V,
                   size_t ld, double* cgs_part, double* h1, double* h2, double* H, double* part_norm);
void fg_normalize_batch(pm_ctx* c, int n_slots, const Batch& bt, int n, int ldh, int i, const double* r,
                        double* v, const double* part, double* H, int* flag);
void fg_givens_batch(pm_ctx* c, int n_slots, const Batch& bt, int ldh, int i, double* H, double* cs, double* sn,
                     double* s, double* resid);
void fg_update_batch(pm_ctx* c, int n_slots, const Batch& bt, int n, int ldh, int k, const double* H,
                     const double* s, double* y, const double* Z, size_t ldz, double* x);

}  // namespace pm

// ---------------------------------------------------------------------------
// BatchEngine: FGMRES + geometric multigrid (damped Jacobi smoothing, direct
// coarse solve, V/W/F cycle; FP32 cycle inside FP64 FGMRES or FP64
// throughout) for up to kMaxBatch problems of one set-up, advanced in
// lockstep. Problems join at restart-cycle boundaries and leave as soon as
// they converge. Each Arnoldi step of all slots is one CUDA graph.
struct pm_problem;
namespace pm {

struct BatchSlotResult {
  int status = 0;  // PM_OK, PM_E_MAXIT, PM_E_DIVERGED, PM_E_BREAKDOWN
  int iterations = 0;
  double residual = 0.0, initial_residual = 0.0;
};

class BatchEngine;
// capacity: slots (1..kMaxBatch); template: a problem of the set-up (its
// solver's parameters and level shapes are used for all slots)
BatchEngine* batch_create(pm_ctx* c, int capacity, pm_problem* templ);
void batch_destroy(BatchEngine* e);
// slot layout bytes (device memory the engine holds besides the problems)
size_t batch_bytes(const BatchEngine* e);
int batch_capacity(const BatchEngine* e);

// One cohort step of the engine's host loop. join: problems to start now
// (assembled and updated; their solution vectors hold the initial iterates),
// at most the number of free slots. Runs one restart cycle of every slot (or
// less when all slots finish earlier) and returns the problems that finished
// in it with their results (their solution vectors hold the solutions).
struct BatchDone {
  pm_problem* p;
  BatchSlotResult r;
};
std::vector<BatchDone> batch_cycle(BatchEngine* e, const std::vector<pm_problem*>& join);
int batch_active(const BatchEngine* e);

}  // namespace pm
