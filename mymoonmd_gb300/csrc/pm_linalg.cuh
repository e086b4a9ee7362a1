// Internal device linear algebra: CSR matrices, deterministic BLAS-1, dense
// coarse-grid inverse. Shared by the multigrid, Krylov, assembly and serving
// layers; the C ABI in pm_capi.cpp wraps these.
#pragma once
#include "pm_core.h"
#include "pm_spmv.cuh"

namespace pm {

// Plain launch on the context's stream, counted. The vector and Krylov
// kernels launched this way begin with pdl_enter(): its trigger lets a
// following sliced-ELL sweep (launched with programmatic stream
// serialization) load its slice layout while they run.
template <class... KArgs, class... Args>
inline void launch_k(pm_ctx* c, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, Args... args) {
  kern<<<grid, block, smem, c->stream>>>(static_cast<KArgs>(args)...);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

// device CSR with optional FP32 copy of the values
struct DevCsr {
  int n_rows = 0, n_cols = 0, n_active = 0;
  int64_t nnz = 0;
  int lanes = 8;   // lanes per row in the SpMV kernels (FP64 values)
  int unroll = 4;  // entries per lane per chunk (FP64 values)
  int lanes32 = 8;   // the same for the FP32 copy of the values
  int unroll32 = 16;
  // row blocks of the streaming kernel (consecutive rows with at most
  // kStreamNnz entries); empty when a row is longer than that
  DBuf<int> rblock;
  int n_rblocks = 0;
  bool stream = true;  // use the streaming kernel when row blocks exist
  int64_t nnz4() const { return (nnz + 3) & ~int64_t(3); }
  // sliced-ELL copy of the FP32 values (sell_kernel): built by make_fp32 for
  // matrices with more than 16 entries per row when the context asks for it;
  // sell_lanes = lanes per row of the layout (0: none)
  int sell_lanes = 0;
  int n_slices = 0;
  int64_t sell_entries = 0;
  DBuf<int> sell_perm, sell_off, sell_cols, sell_src;  // sell_src: CSR entry of each slot, -1 = padding
  DBuf<float> sell_vals;
  // FP64 values in the sliced layout (make_sliced64); sell64_ok: they are the
  // current values (every writer of vals calls values_changed)
  DBuf<double> sell_vals64;
  bool sell64_ok = false;
  BlockMask mask{};
  DBuf<int> row_ptr, cols;
  DBuf<double> vals;
  DBuf<float> vals32;
  DBuf<double> diag;
  DBuf<float> diag32;

  void upload(pm_ctx* c, int nr, int nc, int na, const int* rp, const int* ci, const double* v);
  void set_single_block();
  void set_blocks(int nb, const int* lengths, const int* actives);
  void make_fp32(pm_ctx* c);  // FP32 values (and the sliced copy, see sell_lanes)
  void build_sell(pm_ctx* c, int lanes);
  void drop_sell();
  // FP64 sliced copy for the context's fp64 shape (lays out the slices if the
  // matrix has none yet)
  void make_sliced64(pm_ctx* c);
  // to be called after every write of vals: refreshes the FP64 sliced copy
  void values_changed(pm_ctx* c);
  void make_diag(pm_ctx* c);  // FP64 diagonal (and FP32 copy if vals32 exists)
  size_t spmv_bytes(int elem_bytes, bool read_y) const;
};

int choose_lanes(double avg_nnz_per_row);
constexpr int kStreamNnz = 2048;  // entries per row block of the streaming kernel
// greedy row blocks over a host row-pointer array; empty if a row is too long
std::vector<int> build_row_blocks(int n_rows, const int* rp, int max_nnz, int max_rows);
// sliced-ELL layout (see sell_kernel) of a host CSR structure with `lanes`
// lanes per row and sorting windows of `window` rows; false if the padded
// layout would exceed 2^31 - 1 entries
bool build_sell_layout(int n_rows, const int* rp, const int* ci, int lanes, int window, std::vector<int>& perm,
                       std::vector<int>& off, std::vector<int>& cols, std::vector<int>& src);

// an event for the launch probe (from the context's pool)
cudaEvent_t probe_event(pm_ctx* c);

// y := epilogue(A x); see pm_spmv.cuh for the epilogue meanings
void csr_apply(pm_ctx* c, const DevCsr& A, int epi, const double* x, double* y, const double* b,
               double alpha, int n_rows_override = -1);
void csr_apply32(pm_ctx* c, const DevCsr& A, int epi, const float* x, float* y, const float* b,
                 float alpha, int n_rows_override = -1);

// launch probe of SpMV-family kernels on matrices with `nnz` nonzeros
void probe_reset(pm_ctx* c, int64_t nnz);
void probe_result(pm_ctx* c, int* count, double* total_ms, double* total_bytes);

// BLAS-1 (deterministic fixed-tree reductions)
void dot_partials(pm_ctx* c, int n, const double* x, const double* y, double* partials);
double dot_host(pm_ctx* c, int n, const double* x, const double* y);  // synchronising
void finish_sum(pm_ctx* c, const double* partials, double* out, bool take_sqrt);
void vcopy(pm_ctx* c, int n, const double* x, double* y);
void vset(pm_ctx* c, int n, double* y, double v);
void vscale(pm_ctx* c, int n, double* y, double a);
void vaxpy(pm_ctx* c, int n, double a, const double* x, double* y);  // y += a x
void vaxpby(pm_ctx* c, int n, double a, const double* x, double b, double* y);  // y = a x + b y
void vcvt_d2f(pm_ctx* c, int n, const double* x, float* y);
void vcvt_f2d(pm_ctx* c, int n, const float* x, double* y);
void vcopy32(pm_ctx* c, int n, const float* x, float* y);
// sol := 0 on active rows, rhs on non-active rows (Multigrid::cycle start)
void init_solution(pm_ctx* c, int n, const BlockMask& m, const double* rhs, double* sol);
void init_solution32(pm_ctx* c, int n, const BlockMask& m, const float* rhs, float* sol);
// x := w (b / d), the damped Jacobi sweep from x = 0
void jacobi_from_zero(pm_ctx* c, int n, const double* b, const double* d, double w, double* x);
void jacobi_from_zero32(pm_ctx* c, int n, const float* b, const float* d, float w, float* x);
void vdiv(pm_ctx* c, int n, const double* d, double* y);  // y /= d
// BlockVector::copy_nonactive: dst := src on the non-active rows
void copy_nonactive(pm_ctx* c, int n, const BlockMask& m, const double* src, double* dst);
// *flag := 1 if some non-active entry of x is not zero (the caller clears it)
void nonactive_nonzero(pm_ctx* c, const BlockMask& m, const double* x, int* flag);

// Multicolour order of the SOR / SSOR sweeps (TMatrix::sor_sweep,
// src/Matrix/Matrix.C:943-1031, visits the rows in order): a greedy colouring
// of the matrix graph (rows i and j adjacent when a_ij or a_ji is stored), in
// row order, each row taking the smallest colour none of its already coloured
// neighbours has. Rows of one colour do not couple, so a colour is updated in
// parallel and the sweep equals the sequential one over the rows ordered by
// colour.
struct SorColours {
  DBuf<int> rows;        // rows grouped by colour, increasing within a colour
  std::vector<int> ptr;  // colour k: rows[ptr[k], ptr[k+1])
  const int* key = nullptr;  // the structure (row pointer array) it was built for
  int64_t key_nnz = -1;
  void build(pm_ctx* c, const DevCsr& A);  // once per structure
};
// one SOR sweep x += omega D^-1 (b - A x), row by row in colour order
// (backward: colours in reverse), FP64 or on the FP32 copy
// TMatrix::sor_sweep refuses a zero on the diagonal (src/Matrix/Matrix.C:956-961);
// reads the diagonal made by make_diag
void sor_check_diagonal(pm_ctx* c, const DevCsr& A);
void sor_sweep(pm_ctx* c, const DevCsr& A, const SorColours& col, const double* b, double* x, double omega,
               bool backward);
void sor_sweep32(pm_ctx* c, const DevCsr& A, const SorColours& col, const float* b, float* x, float omega,
                 bool backward);

// dense inverse of the active block of a small CSR matrix (Gauss-Jordan with
// partial pivoting on the device); used by the coarse-grid direct solve
struct DenseInverse {
  int n = 0;         // rows of the full matrix
  int na = 0;        // active rows (the inverted block)
  DBuf<double> inv;  // na x na row-major
  DBuf<int> act;     // active row indices (na)
  DBuf<int> pos;     // row -> position among the active rows, -1 if non-active
  DBuf<double> tmp;  // na
  DBuf<int> perm;    // pivot rows (na)
  DBuf<int> flag;    // singular pivot flag
  DBuf<double> rowk, oldk, part_v;  // cooperative elimination: pivot row, old row k, block arg-max
  DBuf<int> part_i;
  // row-resident elimination: per step, every block's candidate pivot row and
  // the old row k, double-buffered ([2][blocks + 1][na]), and the candidates'
  // arg-max values and positions ([2][blocks])
  DBuf<double> pub_rows, pub_v;
  DBuf<int> pub_i;
  // FP32 inverse for the mixed-precision cycle (build32); has64/has32: which
  // inverse holds the current matrix
  DBuf<float> inv32;
  bool has64 = false, has32 = false;
  void build(pm_ctx* c, const DevCsr& A);
  // act, pos and the dense active block (FP64) in inv
  void prepare(pm_ctx* c, const DevCsr& A);
  // the FP32 inverse: Gauss-Jordan in FP32 on one thread-block cluster when
  // the active block fits its distributed shared memory, else the FP64
  // inverse rounded to FP32
  void build32(pm_ctx* c, const DevCsr& A);
  // build32 in two halves: launch32 queues the factorisation on the stream s
  // (no host synchronisation; the large-matrix path runs build() at once),
  // complete32 waits for it, checks the pivot flag and falls back to the FP64
  // inverse if needed
  void launch32(pm_ctx* c, const DevCsr& A, cudaStream_t s);
  void complete32(pm_ctx* c, const DevCsr& A);
  bool pending32 = false;   // launch32 queued, complete32 not yet run
  // build in two halves, the same way (FP64 inverse)
  void launch64(pm_ctx* c, const DevCsr& A, cudaStream_t s);
  void complete64(pm_ctx* c);
  bool pending64 = false;
  cudaEvent_t done_event = nullptr;  // recorded after the queued factorisation
  // x_a = inv32 b_a, x_n = b_n for a right-hand side with zero non-actives
  void solve32(pm_ctx* c, const float* b, float* x);
  // the same with the FP64 inverse: FP32 vectors, FP64 products and sums
  void solve_mixed(pm_ctx* c, const float* b, float* x);
  // x_a = inv (b_a - A_{a,n} b_n), x_n = b_n  (a: active rows, n: non-active);
  // rhs_nonactive_zero skips the b_n correction (the multigrid coarse rhs has
  // its non-actives reset to zero)
  void solve(pm_ctx* c, const DevCsr& A, const double* b, double* x, bool rhs_nonactive_zero = false);
};

}  // namespace pm
