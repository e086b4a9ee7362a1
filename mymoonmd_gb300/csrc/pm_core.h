// Core device plumbing of the GB300 solve path: context (one CUDA stream per
// context), error state, device buffers and the kernel entry points shared by
// the matrix, multigrid and Krylov layers.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pmgpu.h"

namespace pm {

// Error raised inside the library; the C ABI turns it into a status code.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define PM_CUDA(call)                                                          \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess)                                                     \
      throw ::pm::Error(PM_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define PM_CHECK_LAUNCH() PM_CUDA(cudaGetLastError())

// device buffer owned by the library
// device bytes held by DBufs allocated on this host thread (the request
// executor's footprint estimate of its cached problems)
inline thread_local int64_t g_thread_dev_bytes = 0;

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  explicit DBuf(size_t count) { alloc(count); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DBuf() { release(); }
  void alloc(size_t count) {
    release();
    if (count) {
      cudaError_t e = cudaMalloc(&p, count * sizeof(T));
      if (e != cudaSuccess) {
        p = nullptr;
        cudaGetLastError();
        throw Error(PM_E_OOM, "cudaMalloc of " + std::to_string(count * sizeof(T)) + " bytes failed");
      }
      g_thread_dev_bytes += int64_t(count * sizeof(T));
    }
    n = count;
  }
  // keep the allocation (and its address) when the size already matches
  void ensure(size_t count) {
    if (count != n || (count && !p)) alloc(count);
  }
  void release() {
    if (p) {
      cudaFree(p);
      g_thread_dev_bytes -= int64_t(n * sizeof(T));
    }
    p = nullptr;
    n = 0;
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    if (count != n) alloc(count);
    if (count) PM_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void upload(const std::vector<T>& v, cudaStream_t s) { upload(v.data(), v.size(), s); }
  void download(T* h, cudaStream_t s) const {
    if (n) PM_CUDA(cudaMemcpyAsync(h, p, n * sizeof(T), cudaMemcpyDeviceToHost, s));
  }
  size_t bytes() const { return n * sizeof(T); }
};

}  // namespace pm

// The context behind the opaque pm_ctx handle.
struct pm_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  // second stream for work that overlaps the main stream (the coarse-grid
  // factorisation during the assembly of the finer levels)
  cudaStream_t side = nullptr;
  cudaEvent_t side_event = nullptr;
  int num_sms = 0;
  std::string last_error;
  int verbosity = 1;
  // pinned host scratch for small device->host reads (residuals, flags)
  double* host_scalars = nullptr;
  pm::DBuf<double> dev_scalars;  // device-side scalars (dot results, Givens state)
  pm::DBuf<double> partials;     // per-block partial sums of reductions
  int n_partials = 0;
  uint64_t kernel_launches = 0;  // kernels this library launched on the stream
  // element matrices by the per-quadrature-point loop instead of the
  // reference-tensor contraction (option "assembly_quadrature_loop")
  int assembly_quadrature_loop = 0;
  // launch probe: CUDA events around every SpMV-family launch on matrices
  // with probe_nnz nonzeros (0 = off); resolved by pm_ctx_probe_result
  // device flag passed to the SpMV-family and Vanka launches of this context
  // while set (nullptr = none): a set flag turns those launches into no-ops
  const int* guard = nullptr;
  // FP32 SpMV by the sliced-ELL kernel: 0 = off, else 100 L + 10 U + P (L lanes
  // per row, U steps in flight, P = 1: next steps' loads issued before the
  // current gathers); the matrix copies are laid out for L in make_fp32
  int sell_shape = 481;
  // FP64 SpMV-family launches by the sliced-ELL kernel (same encoding; the
  // layout's lanes must equal those of the FP32 shape when both are used)
  int sell_shape64 = 441;
  // matrices with more entries per row than this on average get sliced copies
  // (option "sliced_min_entries")
  int sell_min_avg = 16;
  // launches of the sliced-ELL sweeps with programmatic stream serialization
  // (option "pdl": 0 off, 1 on)
  int pdl = 1;
  // first Jacobi sweep from an exactly zero iterate as a diagonal scaling
  // (option "jacobi_zero_start"; same bits as the full sweep)
  bool jacobi_zero_start = true;
  // thread blocks of the FP32 coarse Gauss-Jordan cluster (option
  // "coarse_cluster": 1, 2, 4 or 8; more when the matrix does not fit)
  int coarse_cluster = 8;
  int coarse_threads = 0;  // threads per block of it (option "coarse_threads"; 0 = by cluster size)
  int64_t probe_nnz = 0;
  int probe_epilogue = -1;  // only launches with this epilogue (-1 = all)
  int probe_precision = 0;  // only launches with values of this size in bytes (0 = all)
  // launch probe of the multiplicative nodal Vanka sweeps: events around the
  // residual + local-solve pair of every colour (option "probe_nodal")
  int probe_nodal = 0;
  // local residuals of the multiplicative nodal Vanka sweep from the
  // per-colour sliced copy of the patch rows with 4 or 8 lanes per row, or
  // from the CSR rows, one block per patch (0) (option "nodal_sliced"; read
  // when a problem lays out its smoothers)
  int nodal_sliced = 8;
  std::vector<cudaEvent_t> probe_events;  // start/end pairs
  std::vector<double> probe_bytes;        // algorithmic bytes of each probed launch
  std::vector<cudaEvent_t> probe_pool;
};

namespace pm {
// the number of thread blocks used by every deterministic reduction
constexpr int kRedBlocks = 304;  // 2 per SM on GB300
constexpr int kRedThreads = 256;

void ctx_init(pm_ctx* c, int device);
void ctx_destroy(pm_ctx* c);
}  // namespace pm
