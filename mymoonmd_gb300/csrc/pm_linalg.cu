// Device linear algebra: CSR SpMV launchers, deterministic BLAS-1 reductions and
// the dense coarse-grid inverse.
#include <algorithm>
#include <cmath>
#include <mutex>

#include <cooperative_groups.h>

#include "pm_linalg.cuh"

namespace pm {

// ---------------------------------------------------------------- context ---
void ctx_init(pm_ctx* c, int device) {
  c->device = device;
  PM_CUDA(cudaSetDevice(device));
  PM_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  PM_CUDA(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
  PM_CUDA(cudaEventCreateWithFlags(&c->side_event, cudaEventDisableTiming));
  PM_CUDA(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
  PM_CUDA(cudaMallocHost(&c->host_scalars, 64 * sizeof(double)));
  c->dev_scalars.alloc(256);
  c->partials.alloc(4 * kRedBlocks);
  c->n_partials = kRedBlocks;
}

void ctx_destroy(pm_ctx* c) {
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->dev_scalars.release();
  c->partials.release();
  if (c->host_scalars) cudaFreeHost(c->host_scalars);
  c->host_scalars = nullptr;
  if (c->side) cudaStreamSynchronize(c->side);
  if (c->side_event) cudaEventDestroy(c->side_event);
  if (c->side) cudaStreamDestroy(c->side);
  c->side_event = nullptr;
  c->side = nullptr;
  if (c->stream) cudaStreamDestroy(c->stream);
  c->stream = nullptr;
}

static inline int nblocks(long long n, int t) { return int((n + t - 1) / t); }

// -------------------------------------------------------------------- CSR ---
int choose_lanes(double avg) {
  if (avg <= 6.0) return 4;
  if (avg <= 12.0) return 8;
  if (avg <= 28.0) return 16;
  return 32;
}

void DevCsr::upload(pm_ctx* c, int nr, int nc, int na, const int* rp, const int* ci,
                    const double* v) {
  n_rows = nr;
  n_cols = nc;
  n_active = na;
  nnz = rp[nr];
  row_ptr.upload(rp, size_t(nr) + 1, c->stream);
  // column indices readable up to nnz rounded up to 4 entries; the tail holds
  // zeros
  cols.alloc(size_t(nnz4()));
  if (nnz) PM_CUDA(cudaMemcpyAsync(cols.p, ci, size_t(nnz) * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  if (nnz4() > nnz)
    PM_CUDA(cudaMemsetAsync(cols.p + nnz, 0, size_t(nnz4() - nnz) * sizeof(int), c->stream));
  if (v) vals.upload(v, size_t(nnz), c->stream);
  else {
    vals.alloc(size_t(nnz));
    if (nnz) PM_CUDA(cudaMemsetAsync(vals.p, 0, vals.bytes(), c->stream));
  }
  drop_sell();  // a new structure: no sliced layout yet
  // measured on GB300 (3D Q2, 15.8 M and 54.5 M nonzeros): four lanes per row
  // with eight loads in flight per lane is the fastest launch shape for both
  // FP64 and FP32 values; short rows take four loads per lane
  // FP64: four lanes x eight loads (the FP64 pipe is the limit); FP32: eight
  // lanes x sixteen loads in flight (3.9 TB/s vs 3.4 TB/s at four x eight)
  const double avg = nr ? double(nnz) / nr : 1.0;
  lanes = 4;
  unroll = avg > 16.0 ? 8 : 4;
  lanes32 = avg > 16.0 ? 8 : 4;
  unroll32 = avg > 16.0 ? 16 : 4;
  stream = false;
  std::vector<int> rb = build_row_blocks(nr, rp, kStreamNnz, 1024);
  n_rblocks = rb.empty() ? 0 : int(rb.size()) - 1;
  if (n_rblocks) rblock.upload(rb, c->stream);
  else rblock.release();
  set_single_block();
}

std::vector<int> build_row_blocks(int n_rows, const int* rp, int max_nnz, int max_rows) {
  std::vector<int> rb;
  if (n_rows <= 0) return rb;
  rb.push_back(0);
  int r0 = 0;
  for (int i = 0; i < n_rows; ++i) {
    if (rp[i + 1] - rp[i] > max_nnz) return std::vector<int>();
    if (rp[i + 1] - rp[r0] > max_nnz || i - r0 >= max_rows) {
      rb.push_back(i);
      r0 = i;
    }
  }
  rb.push_back(n_rows);
  return rb;
}

bool build_sell_layout(int n_rows, const int* rp, const int* ci, int L, int window, std::vector<int>& perm,
                       std::vector<int>& off, std::vector<int>& cols, std::vector<int>& src) {
  const int C = 32 / L;
  if (L < 1 || 32 % L != 0 || window % C != 0) throw Error(PM_E_INVALID, "sliced layout: bad lanes or window");
  const int n_sl = (n_rows + C - 1) / C;
  perm.assign(size_t(n_sl) * C, -1);
  // rows sorted by length, longest first, ties in row order, per window
  std::vector<int> idx;
  for (int w0 = 0; w0 < n_rows; w0 += window) {
    const int w1 = std::min(n_rows, w0 + window);
    idx.resize(size_t(w1 - w0));
    for (int i = w0; i < w1; ++i) idx[size_t(i - w0)] = i;
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int a, int b) { return rp[a + 1] - rp[a] > rp[b + 1] - rp[b]; });
    std::copy(idx.begin(), idx.end(), perm.begin() + w0);
  }
  off.assign(size_t(n_sl) + 1, 0);
  int64_t total = 0;
  for (int sl = 0; sl < n_sl; ++sl) {
    int width = 0;
    for (int q = 0; q < C; ++q) {
      const int r = perm[size_t(sl) * C + q];
      if (r >= 0) width = std::max(width, rp[r + 1] - rp[r]);
    }
    total += int64_t(32) * ((width + L - 1) / L);
    if (total > int64_t(0x7fffffff)) return false;
    off[size_t(sl) + 1] = int(total);
  }
  cols.assign(size_t(total), 0);
  src.assign(size_t(total), -1);
  for (int sl = 0; sl < n_sl; ++sl) {
    const int T = (off[size_t(sl) + 1] - off[size_t(sl)]) / 32;
    for (int q = 0; q < C; ++q) {
      const int r = perm[size_t(sl) * C + q];
      const int len = r >= 0 ? rp[r + 1] - rp[r] : 0;
      // padding repeats the row's last column (its x is already cached)
      const int pad_col = len > 0 ? ci[rp[r] + len - 1] : 0;
      for (int t = 0; t < T; ++t)
        for (int sub = 0; sub < L; ++sub) {
          const int j = t * L + sub;
          const size_t slot = size_t(off[size_t(sl)]) + size_t(t) * 32 + size_t(sub) * C + q;
          if (j < len) {
            cols[slot] = ci[rp[r] + j];
            src[slot] = rp[r] + j;
          } else {
            cols[slot] = pad_col;
          }
        }
    }
  }
  return true;
}

void DevCsr::drop_sell() {
  sell_lanes = 0;
  n_slices = 0;
  sell_entries = 0;
  sell64_ok = false;
  sell_perm.release();
  sell_off.release();
  sell_cols.release();
  sell_src.release();
  sell_vals.release();
  sell_vals64.release();
}

void DevCsr::build_sell(pm_ctx* c, int L) {
  const bool had64 = sell_vals64.p != nullptr;
  sell_lanes = 0;
  n_slices = 0;
  sell_entries = 0;
  sell64_ok = false;
  std::vector<int> rp(static_cast<size_t>(n_rows) + 1), ci(static_cast<size_t>(nnz));
  PM_CUDA(cudaMemcpyAsync(rp.data(), row_ptr.p, rp.size() * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if (nnz) PM_CUDA(cudaMemcpyAsync(ci.data(), cols.p, ci.size() * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));
  std::vector<int> perm, off, sc, src;
  if (!build_sell_layout(n_rows, rp.data(), ci.data(), L, kSellWindow, perm, off, sc, src)) {
    drop_sell();
    return;
  }
  sell_perm.upload(perm, c->stream);
  sell_off.upload(off, c->stream);
  sell_cols.upload(sc, c->stream);
  sell_src.upload(src, c->stream);
  sell_vals.ensure(sc.size());
  PM_CUDA(cudaStreamSynchronize(c->stream));  // the host vectors go out of scope
  sell_lanes = L;
  n_slices = int(off.size()) - 1;
  sell_entries = int64_t(sc.size());
  if (had64) {  // the FP64 copy follows the new layout
    sell_vals64.ensure(sc.size());
    values_changed(c);
  }
}

void DevCsr::set_single_block() {
  mask = BlockMask{};
  mask.nb = 1;
  mask.start[0] = 0;
  mask.active_end[0] = n_active;
  mask.end[0] = n_rows;
}

void DevCsr::set_blocks(int nb, const int* lengths, const int* actives) {
  if (nb < 1 || nb > 4) throw Error(PM_E_INVALID, "block vectors hold 1..4 blocks");
  mask = BlockMask{};
  mask.nb = nb;
  int off = 0;
  for (int b = 0; b < nb; ++b) {
    mask.start[b] = off;
    mask.active_end[b] = off + actives[b];
    off += lengths[b];
    mask.end[b] = off;
  }
  if (off != n_rows) throw Error(PM_E_INVALID, "block lengths do not add up to the matrix rows");
  n_active = 0;
  for (int b = 0; b < nb; ++b) n_active += actives[b];
}

__global__ void k_d2f(long long n, const double* __restrict__ x, float* __restrict__ y) {
  pdl_enter();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = float(x[i]);
}
__global__ void k_f2d(long long n, const float* __restrict__ x, double* __restrict__ y) {
  pdl_enter();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = double(x[i]);
}

static int grid_for(pm_ctx* c, long long n) {
  long long b = (n + 255) / 256;
  long long cap = (long long)c->num_sms * 8;
  return int(std::max<long long>(1, std::min(b, cap)));
}

template <class TO>
__global__ void k_sell_fill(long long n, const int* __restrict__ src, const double* __restrict__ v,
                            TO* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int k = src[i];
    out[i] = k >= 0 ? TO(v[k]) : TO(0);
  }
}

void DevCsr::values_changed(pm_ctx* c) {
  sell64_ok = false;
  if (sell_lanes && sell_entries && sell_vals64.p) {
    k_sell_fill<double><<<grid_for(c, sell_entries), 256, 0, c->stream>>>(sell_entries, sell_src.p, vals.p,
                                                                         sell_vals64.p);
    PM_CHECK_LAUNCH();
    c->kernel_launches++;
    sell64_ok = true;
  }
}

void DevCsr::make_sliced64(pm_ctx* c) {
  const int want = c->sell_shape64 / 100;
  if (want <= 0 || nnz <= c->sell_min_avg * int64_t(n_rows)) return;
  if (sell_lanes == 0) build_sell(c, want);
  if (sell_lanes != want || !sell_entries) return;
  if (!sell_vals64.p) sell_vals64.ensure(size_t(sell_entries));
  if (!sell64_ok) values_changed(c);
}

void DevCsr::make_fp32(pm_ctx* c) {
  // the sliced copy: matrices with more than sell_min_avg entries per row on
  // average; laid out once per lane count
  const int want = c->sell_shape / 100;
  if (want > 0 && want != sell_lanes && nnz > c->sell_min_avg * int64_t(n_rows)) build_sell(c, want);
  if (sell_lanes && sell_entries) {
    k_sell_fill<float><<<grid_for(c, sell_entries), 256, 0, c->stream>>>(sell_entries, sell_src.p, vals.p,
                                                                       sell_vals.p);
    PM_CHECK_LAUNCH();
    c->kernel_launches++;
  }
  vals32.ensure(size_t(nnz4()));
  if (nnz4() > nnz)
    PM_CUDA(cudaMemsetAsync(vals32.p + nnz, 0, size_t(nnz4() - nnz) * sizeof(float), c->stream));
  if (nnz) {
    k_d2f<<<grid_for(c, nnz), 256, 0, c->stream>>>(nnz, vals.p, vals32.p);
    PM_CHECK_LAUNCH();
    c->kernel_launches++;
  }
  if (diag.p) {
    diag32.ensure(size_t(n_rows));
    k_d2f<<<grid_for(c, n_rows), 256, 0, c->stream>>>(n_rows, diag.p, diag32.p);
    PM_CHECK_LAUNCH();
    c->kernel_launches++;
  }
}

// diagonal entries (Iteration_jacobi: extract_diagonal_entries); a missing
// diagonal entry is recorded as 0 and reported by the caller
__global__ void k_diag(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                       const double* __restrict__ v, double* __restrict__ d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double r = 0.0;
  for (int k = rp[i]; k < rp[i + 1]; ++k)
    if (ci[k] == i) { r = v[k]; break; }
  d[i] = r;
}

void DevCsr::make_diag(pm_ctx* c) {
  diag.ensure(size_t(n_rows));
  if (n_rows) {
    k_diag<<<nblocks(n_rows, 256), 256, 0, c->stream>>>(n_rows, row_ptr.p, cols.p, vals.p, diag.p);
    PM_CHECK_LAUNCH();
    c->kernel_launches++;
  }
  if (vals32.p) {
    diag32.ensure(size_t(n_rows));
    if (n_rows) {
      k_d2f<<<grid_for(c, n_rows), 256, 0, c->stream>>>(n_rows, diag.p, diag32.p);
      PM_CHECK_LAUNCH();
      c->kernel_launches++;
    }
  }
}

size_t DevCsr::spmv_bytes(int eb, bool read_y) const {
  // values + column indices + row pointers + x gathered once + y written (+read)
  return size_t(nnz) * (eb + 4) + size_t(n_rows + 1) * 4 + size_t(n_cols) * eb +
         size_t(n_rows) * eb * (read_y ? 2 : 1);
}

template <class TV, class TX, class TA, int G, int EPI>
static void launch_gu(pm_ctx* c, int U, int grid, int n, const int* rp, const int* ci, const TV* v,
                      const TX* x, TX* y, const TX* b, const TX* d, TA alpha, const BlockMask& m) {
  const dim3 gr(grid), bl(256);
  switch (U) {
    case 2: launch_k(c, csr_kernel<TV, TX, TA, G, 2, EPI>, gr, bl, 0, n, rp, ci, v, x, y, b, d, x, alpha, m); break;
    case 4: launch_k(c, csr_kernel<TV, TX, TA, G, 4, EPI>, gr, bl, 0, n, rp, ci, v, x, y, b, d, x, alpha, m); break;
    case 16: launch_k(c, csr_kernel<TV, TX, TA, G, 16, EPI>, gr, bl, 0, n, rp, ci, v, x, y, b, d, x, alpha, m); break;
    default: launch_k(c, csr_kernel<TV, TX, TA, G, 8, EPI>, gr, bl, 0, n, rp, ci, v, x, y, b, d, x, alpha, m); break;
  }
}

template <class TV, class TX, class TA, int EPI>
static void launch_epi(pm_ctx* c, int G, int U, int n, const int* rp, const int* ci, const TV* v,
                       const TX* x, TX* y, const TX* b, const TX* d, TA alpha, const BlockMask& m,
                       const int* rblock = nullptr, int n_rblocks = 0) {
  if (n <= 0) return;
  BlockMask mg = m;
  mg.guard = c->guard;
  if (rblock && n_rblocks > 0) {
    csr_stream_kernel<TV, TX, TA, kStreamNnz, EPI><<<n_rblocks, 256, 0, c->stream>>>(
        rblock, rp, ci, v, x, y, b, d, alpha, mg);
    PM_CHECK_LAUNCH();
    c->kernel_launches++;
    return;
  }
  const int grid = nblocks((long long)n * G, 256);
  switch (G) {
    case 1: launch_gu<TV, TX, TA, 1, EPI>(c, U, grid, n, rp, ci, v, x, y, b, d, alpha, mg); break;
    case 2: launch_gu<TV, TX, TA, 2, EPI>(c, U, grid, n, rp, ci, v, x, y, b, d, alpha, mg); break;
    case 4: launch_gu<TV, TX, TA, 4, EPI>(c, U, grid, n, rp, ci, v, x, y, b, d, alpha, mg); break;
    case 8: launch_gu<TV, TX, TA, 8, EPI>(c, U, grid, n, rp, ci, v, x, y, b, d, alpha, mg); break;
    case 16: launch_gu<TV, TX, TA, 16, EPI>(c, U, grid, n, rp, ci, v, x, y, b, d, alpha, mg); break;
    default: launch_gu<TV, TX, TA, 32, EPI>(c, U, grid, n, rp, ci, v, x, y, b, d, alpha, mg); break;
  }
}

cudaEvent_t probe_event(pm_ctx* c) {
  if (!c->probe_pool.empty()) {
    cudaEvent_t e = c->probe_pool.back();
    c->probe_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  PM_CUDA(cudaEventCreate(&e));
  return e;
}

// algorithmic bytes of one SpMV-family launch: values, column indices, row
// pointers, the gathered vector once, and the per-row vectors the epilogue
// reads and writes
static double epi_bytes(const DevCsr& A, int epi, int eb, int n) {
  double rows_vec = 1.0;  // y written
  if (epi == EPI_AXPY || epi == EPI_PROLONG) rows_vec += 1.0;  // y read
  if (epi == EPI_DEFECT) rows_vec += 1.0;                      // b read
  if (epi == EPI_JACOBI) rows_vec += 2.0;                      // b and diag read
  return double(A.nnz) * (eb + 4) + double(n + 1) * 4 + double(A.n_cols) * eb + double(n) * eb * rows_vec;
}

template <class T>
static const T* sell_values(const DevCsr& A);
template <>
const float* sell_values<float>(const DevCsr& A) { return A.sell_vals.p; }
template <>
const double* sell_values<double>(const DevCsr& A) { return A.sell_vals64.p; }

template <class T, int L, int U, bool P, int EPI>
static void launch_sell_epi(pm_ctx* c, const DevCsr& A, const T* x, T* y, const T* b, const T* d, T alpha,
                            const BlockMask& m) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(unsigned(nblocks(A.n_slices, 4)));  // four warps (slices) per block
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = c->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = c->pdl >= 1 ? 1 : 0;
  PM_CUDA(cudaLaunchKernelEx(&cfg, sell_kernel<T, L, U, P, EPI>, A.n_slices, (const int*)A.sell_perm.p,
                             (const int*)A.sell_off.p, (const int*)A.sell_cols.p, sell_values<T>(A), x, y, b, d,
                             alpha, m));
}

template <class T, int L, int U, bool P>
static void launch_sell_shape(pm_ctx* c, const DevCsr& A, int epi, const T* x, T* y, const T* b, const T* d,
                              T alpha, const BlockMask& m) {
  switch (epi) {
    case EPI_AXPY: launch_sell_epi<T, L, U, P, EPI_AXPY>(c, A, x, y, b, d, alpha, m); break;
    case EPI_SET: launch_sell_epi<T, L, U, P, EPI_SET>(c, A, x, y, b, d, alpha, m); break;
    case EPI_DEFECT: launch_sell_epi<T, L, U, P, EPI_DEFECT>(c, A, x, y, b, d, alpha, m); break;
    case EPI_JACOBI: launch_sell_epi<T, L, U, P, EPI_JACOBI>(c, A, x, y, b, d, alpha, m); break;
    case EPI_RESTRICT: launch_sell_epi<T, L, U, P, EPI_RESTRICT>(c, A, x, y, b, d, alpha, m); break;
    case EPI_PROLONG: launch_sell_epi<T, L, U, P, EPI_PROLONG>(c, A, x, y, b, d, alpha, m); break;
    default: throw Error(PM_E_INVALID, "unknown SpMV epilogue");
  }
}

static void launch_sell(pm_ctx* c, const DevCsr& A, int epi, const float* x, float* y, const float* b,
                        const float* d, float alpha) {
  BlockMask mg = A.mask;
  mg.guard = c->guard;
  switch (c->sell_shape) {
    case 140: launch_sell_shape<float, 1, 4, false>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 141: launch_sell_shape<float, 1, 4, true>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 180: launch_sell_shape<float, 1, 8, false>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 240: launch_sell_shape<float, 2, 4, false>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 241: launch_sell_shape<float, 2, 4, true>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 280: launch_sell_shape<float, 2, 8, false>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 440: launch_sell_shape<float, 4, 4, false>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 441: launch_sell_shape<float, 4, 4, true>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 480: launch_sell_shape<float, 4, 8, false>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 481: launch_sell_shape<float, 4, 8, true>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 840: launch_sell_shape<float, 8, 4, false>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 841: launch_sell_shape<float, 8, 4, true>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 881: launch_sell_shape<float, 8, 8, true>(c, A, epi, x, y, b, d, alpha, mg); break;
    default: throw Error(PM_E_INVALID, "unknown sliced SpMV shape " + std::to_string(c->sell_shape));
  }
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

static void launch_sell64(pm_ctx* c, const DevCsr& A, int epi, const double* x, double* y, const double* b,
                          const double* d, double alpha) {
  BlockMask mg = A.mask;
  mg.guard = c->guard;
  switch (c->sell_shape64) {
    case 441: launch_sell_shape<double, 4, 4, true>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 481: launch_sell_shape<double, 4, 8, true>(c, A, epi, x, y, b, d, alpha, mg); break;
    case 841: launch_sell_shape<double, 8, 4, true>(c, A, epi, x, y, b, d, alpha, mg); break;
    default: throw Error(PM_E_INVALID, "unknown FP64 sliced SpMV shape " + std::to_string(c->sell_shape64));
  }
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

template <class TV, class TX, class TA>
static void csr_dispatch(pm_ctx* c, const DevCsr& A, const TV* vals, const TX* diag, int epi,
                         const TX* x, TX* y, const TX* b, TA alpha, int n) {
  const bool fp32 = sizeof(TV) == 4;
  const int G = fp32 ? A.lanes32 : A.lanes;
  const int U = fp32 ? A.unroll32 : A.unroll;
  const bool use_stream = A.stream && A.n_rblocks > 0 && n == A.n_rows;
  const int* rb = use_stream ? A.rblock.p : nullptr;
  const int nrb = use_stream ? A.n_rblocks : 0;
  const int* rp = A.row_ptr.p;
  const int* ci = A.cols.p;
  const bool probe = c->probe_nnz != 0 && A.nnz == c->probe_nnz &&
                     (c->probe_epilogue < 0 || c->probe_epilogue == epi) &&
                     (c->probe_precision == 0 || c->probe_precision == int(sizeof(TV)));
  if (probe) {
    cudaEvent_t e0 = probe_event(c);
    PM_CUDA(cudaEventRecord(e0, c->stream));
    c->probe_events.push_back(e0);
    c->probe_bytes.push_back(epi_bytes(A, epi, int(sizeof(TV)), n));
  }
  if constexpr (sizeof(TV) == 8) {
    if (c->sell_shape64 > 0 && A.sell64_ok && A.sell_lanes == c->sell_shape64 / 100 && A.n_slices > 0 &&
        n == A.n_rows) {
      launch_sell64(c, A, epi, reinterpret_cast<const double*>(x), reinterpret_cast<double*>(y),
                    reinterpret_cast<const double*>(b), reinterpret_cast<const double*>(diag), double(alpha));
      if (probe) {
        cudaEvent_t e1 = probe_event(c);
        PM_CUDA(cudaEventRecord(e1, c->stream));
        c->probe_events.push_back(e1);
      }
      return;
    }
  }
  if constexpr (sizeof(TV) == 4) {
    if (c->sell_shape > 0 && A.sell_lanes == c->sell_shape / 100 &&
        A.n_slices > 0 && n == A.n_rows) {
      launch_sell(c, A, epi, reinterpret_cast<const float*>(x), reinterpret_cast<float*>(y),
                  reinterpret_cast<const float*>(b), reinterpret_cast<const float*>(diag), float(alpha));
      if (probe) {
        cudaEvent_t e1 = probe_event(c);
        PM_CUDA(cudaEventRecord(e1, c->stream));
        c->probe_events.push_back(e1);
      }
      return;
    }
  }
  switch (epi) {
    case EPI_AXPY: launch_epi<TV, TX, TA, EPI_AXPY>(c, G, U, n, rp, ci, vals, x, y, b, diag, alpha, A.mask, rb, nrb); break;
    case EPI_SET: launch_epi<TV, TX, TA, EPI_SET>(c, G, U, n, rp, ci, vals, x, y, b, diag, alpha, A.mask, rb, nrb); break;
    case EPI_DEFECT: launch_epi<TV, TX, TA, EPI_DEFECT>(c, G, U, n, rp, ci, vals, x, y, b, diag, alpha, A.mask, rb, nrb); break;
    case EPI_JACOBI: launch_epi<TV, TX, TA, EPI_JACOBI>(c, G, U, n, rp, ci, vals, x, y, b, diag, alpha, A.mask, rb, nrb); break;
    case EPI_RESTRICT: launch_epi<TV, TX, TA, EPI_RESTRICT>(c, G, U, n, rp, ci, vals, x, y, b, diag, alpha, A.mask, rb, nrb); break;
    case EPI_PROLONG: launch_epi<TV, TX, TA, EPI_PROLONG>(c, G, U, n, rp, ci, vals, x, y, b, diag, alpha, A.mask, rb, nrb); break;
    default: throw Error(PM_E_INVALID, "unknown SpMV epilogue");
  }
  if (probe) {
    cudaEvent_t e1 = probe_event(c);
    PM_CUDA(cudaEventRecord(e1, c->stream));
    c->probe_events.push_back(e1);
  }
}

void probe_reset(pm_ctx* c, int64_t nnz) {
  for (auto e : c->probe_events) c->probe_pool.push_back(e);
  c->probe_events.clear();
  c->probe_bytes.clear();
  c->probe_nnz = nnz;
}

void probe_result(pm_ctx* c, int* count, double* total_ms, double* total_bytes) {
  PM_CUDA(cudaStreamSynchronize(c->stream));
  const int pairs = int(c->probe_events.size() / 2);
  double ms = 0.0, bytes = 0.0;
  for (int i = 0; i < pairs; ++i) {
    float t = 0.0f;
    PM_CUDA(cudaEventElapsedTime(&t, c->probe_events[2 * i], c->probe_events[2 * i + 1]));
    ms += t;
    bytes += c->probe_bytes[i];
  }
  *count = pairs;
  *total_ms = ms;
  *total_bytes = bytes;
}

void csr_apply(pm_ctx* c, const DevCsr& A, int epi, const double* x, double* y, const double* b,
               double alpha, int n_rows_override) {
  if (epi == EPI_JACOBI && !A.diag.p) throw Error(PM_E_INVALID, "Jacobi sweep without diagonal");
  csr_dispatch<double, double, double>(c, A, A.vals.p, A.diag.p, epi, x, y, b, alpha,
                                       n_rows_override >= 0 ? n_rows_override : A.n_rows);
}

void csr_apply32(pm_ctx* c, const DevCsr& A, int epi, const float* x, float* y, const float* b,
                 float alpha, int n_rows_override) {
  if (!A.vals32.p && A.nnz) throw Error(PM_E_INVALID, "matrix has no FP32 copy");
  if (epi == EPI_JACOBI && !A.diag32.p) throw Error(PM_E_INVALID, "Jacobi sweep without FP32 diagonal");
  csr_dispatch<float, float, float>(c, A, A.vals32.p, A.diag32.p, epi, x, y, b, alpha,
                                    n_rows_override >= 0 ? n_rows_override : A.n_rows);
}

// ------------------------------------------------------------------ BLAS-1 ---
// block-level sum with a fixed tree (deterministic)
__device__ __forceinline__ double block_sum(double v, double* sh) {
  const int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (t < s) sh[t] += sh[t + s];
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

template <class T>
__global__ void __launch_bounds__(256) k_dot_partials(int n, const T* __restrict__ x,
                                                      const T* __restrict__ y,
                                                      double* __restrict__ part) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    s += double(x[i]) * double(y[i]);
  double r = block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = r;
}

__global__ void k_finish_sum(const double* __restrict__ part, int np, double* out, int take_sqrt) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
  double r = block_sum(s, sh);
  if (threadIdx.x == 0) *out = take_sqrt ? sqrt(r) : r;
}

void dot_partials(pm_ctx* c, int n, const double* x, const double* y, double* partials) {
  k_dot_partials<double><<<kRedBlocks, kRedThreads, 0, c->stream>>>(n, x, y, partials);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

void finish_sum(pm_ctx* c, const double* partials, double* out, bool take_sqrt) {
  k_finish_sum<<<1, 256, 0, c->stream>>>(partials, kRedBlocks, out, take_sqrt ? 1 : 0);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

double dot_host(pm_ctx* c, int n, const double* x, const double* y) {
  dot_partials(c, n, x, y, c->partials.p);
  finish_sum(c, c->partials.p, c->dev_scalars.p, false);
  PM_CUDA(cudaMemcpyAsync(c->host_scalars, c->dev_scalars.p, sizeof(double),
                          cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));
  return c->host_scalars[0];
}

template <class T>
__global__ void k_copy(long long n, const T* __restrict__ x, T* __restrict__ y) {
  pdl_enter();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = x[i];
}
__global__ void k_set(long long n, double* __restrict__ y, double v) {
  pdl_enter();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = v;
}
__global__ void k_scale(long long n, double* __restrict__ y, double a) {
  pdl_enter();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] *= a;
}
__global__ void k_axpy(long long n, double a, const double* __restrict__ x, double* __restrict__ y) {
  pdl_enter();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}
__global__ void k_axpby(long long n, double a, const double* __restrict__ x, double b,
                        double* __restrict__ y) {
  pdl_enter();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}
__global__ void k_div(long long n, const double* __restrict__ d, double* __restrict__ y) {
  pdl_enter();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] /= d[i];
}
template <class T>
__global__ void k_init_sol(int n, BlockMask m, const T* __restrict__ rhs, T* __restrict__ sol) {
  pdl_enter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    sol[i] = row_is_active(m, i) ? T(0) : rhs[i];
}

#define PM_LAUNCH1D(kern, n, ...)                                                     \
  do {                                                                                \
    if ((n) > 0) launch_k(c, kern, dim3(grid_for(c, (n))), dim3(256), 0, __VA_ARGS__); \
  } while (0)

void vcopy(pm_ctx* c, int n, const double* x, double* y) { PM_LAUNCH1D(k_copy<double>, n, n, x, y); }
void vcopy32(pm_ctx* c, int n, const float* x, float* y) { PM_LAUNCH1D(k_copy<float>, n, n, x, y); }
void vset(pm_ctx* c, int n, double* y, double v) { PM_LAUNCH1D(k_set, n, n, y, v); }
void vscale(pm_ctx* c, int n, double* y, double a) { PM_LAUNCH1D(k_scale, n, n, y, a); }
void vaxpy(pm_ctx* c, int n, double a, const double* x, double* y) { PM_LAUNCH1D(k_axpy, n, n, a, x, y); }
void vaxpby(pm_ctx* c, int n, double a, const double* x, double b, double* y) {
  PM_LAUNCH1D(k_axpby, n, n, a, x, b, y);
}
void vdiv(pm_ctx* c, int n, const double* d, double* y) { PM_LAUNCH1D(k_div, n, n, d, y); }
void vcvt_d2f(pm_ctx* c, int n, const double* x, float* y) { PM_LAUNCH1D(k_d2f, n, n, x, y); }
void vcvt_f2d(pm_ctx* c, int n, const float* x, double* y) { PM_LAUNCH1D(k_f2d, n, n, x, y); }
__global__ void k_copy_nonactive(int n, BlockMask m, const double* __restrict__ src, double* __restrict__ dst) {
  pdl_enter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (!row_is_active(m, i)) dst[i] = src[i];
}
void copy_nonactive(pm_ctx* c, int n, const BlockMask& m, const double* src, double* dst) {
  PM_LAUNCH1D(k_copy_nonactive, n, n, m, src, dst);
}

// flag := 1 if a non-active entry of x is not zero
__global__ void k_nonactive_nonzero(BlockMask m, const double* __restrict__ x, int* __restrict__ flag) {
  for (int b = 0; b < m.nb; ++b)
    for (int i = m.active_end[b] + blockIdx.x * blockDim.x + threadIdx.x; i < m.end[b];
         i += gridDim.x * blockDim.x)
      if (x[i] != 0.0) *flag = 1;
}
void nonactive_nonzero(pm_ctx* c, const BlockMask& m, const double* x, int* flag) {
  k_nonactive_nonzero<<<kRedBlocks, 256, 0, c->stream>>>(m, x, flag);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

void init_solution(pm_ctx* c, int n, const BlockMask& m, const double* rhs, double* sol) {
  PM_LAUNCH1D(k_init_sol<double>, n, n, m, rhs, sol);
}
void init_solution32(pm_ctx* c, int n, const BlockMask& m, const float* rhs, float* sol) {
  PM_LAUNCH1D(k_init_sol<float>, n, n, m, rhs, sol);
}

// x = 0 + w ((b - 0) / d): the damped Jacobi sweep of an exactly zero iterate
// (the sweep's row sums of a_ij * 0 are +0; fma(w, q, +0) rounds like its
// x + w q with x = +0)
template <class T>
__global__ void k_jacobi_zero(int n, const T* __restrict__ b, const T* __restrict__ d, T w, T* __restrict__ x) {
  pdl_enter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] = fmadd(w, (b[i] - T(0)) / d[i], T(0));
}
void jacobi_from_zero(pm_ctx* c, int n, const double* b, const double* d, double w, double* x) {
  PM_LAUNCH1D(k_jacobi_zero<double>, n, n, b, d, w, x);
}
void jacobi_from_zero32(pm_ctx* c, int n, const float* b, const float* d, float w, float* x) {
  PM_LAUNCH1D(k_jacobi_zero<float>, n, n, b, d, w, x);
}

// ------------------------------------------------------------ SOR ----------
void SorColours::build(pm_ctx* c, const DevCsr& A) {
  if (key == A.row_ptr.p && key_nnz == A.nnz) return;
  const int n = A.n_rows;
  if (A.n_cols != n) throw Error(PM_E_INVALID, "SOR needs a square matrix");
  std::vector<int> rp(static_cast<size_t>(n) + 1), ci(static_cast<size_t>(A.nnz));
  PM_CUDA(cudaMemcpyAsync(rp.data(), A.row_ptr.p, rp.size() * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if (A.nnz)
    PM_CUDA(cudaMemcpyAsync(ci.data(), A.cols.p, ci.size() * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));
  // the transposed pattern: rows k that store column i
  std::vector<int> tp(static_cast<size_t>(n) + 1, 0), tc(ci.size());
  for (int k : ci) tp[size_t(k) + 1]++;
  for (int i = 0; i < n; ++i) tp[size_t(i) + 1] += tp[size_t(i)];
  std::vector<int> fill(tp.begin(), tp.end() - 1);
  for (int i = 0; i < n; ++i)
    for (int k = rp[size_t(i)]; k < rp[size_t(i) + 1]; ++k) tc[size_t(fill[size_t(ci[size_t(k)])]++)] = i;
  std::vector<int> colour(static_cast<size_t>(n), -1), stamp;
  int n_col = 0;
  for (int i = 0; i < n; ++i) {
    auto mark = [&](int j) {
      if (j < i && j != i) {
        const int cj = colour[size_t(j)];
        if (cj >= int(stamp.size())) stamp.resize(size_t(cj) + 1, -1);
        stamp[size_t(cj)] = i;
      }
    };
    for (int k = rp[size_t(i)]; k < rp[size_t(i) + 1]; ++k) mark(ci[size_t(k)]);
    for (int k = tp[size_t(i)]; k < tp[size_t(i) + 1]; ++k) mark(tc[size_t(k)]);
    int cc = 0;
    while (cc < int(stamp.size()) && stamp[size_t(cc)] == i) ++cc;
    colour[size_t(i)] = cc;
    n_col = std::max(n_col, cc + 1);
  }
  ptr.assign(size_t(n_col) + 1, 0);
  for (int i = 0; i < n; ++i) ptr[size_t(colour[size_t(i)]) + 1]++;
  for (int k = 0; k < n_col; ++k) ptr[size_t(k) + 1] += ptr[size_t(k)];
  std::vector<int> order(static_cast<size_t>(n)), pos(ptr.begin(), ptr.end() - 1);
  for (int i = 0; i < n; ++i) order[size_t(pos[size_t(colour[size_t(i)])]++)] = i;
  rows.upload(order, c->stream);
  PM_CUDA(cudaStreamSynchronize(c->stream));
  key = A.row_ptr.p;
  key_nnz = A.nnz;
}

void sor_check_diagonal(pm_ctx* c, const DevCsr& A) {
  if (!A.diag.p) throw Error(PM_E_INVALID, "SOR check without diagonal");
  std::vector<double> d(static_cast<size_t>(A.n_rows));
  if (!d.empty())
    PM_CUDA(cudaMemcpyAsync(d.data(), A.diag.p, d.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));
  for (double v : d)
    if (v == 0.0) throw Error(PM_E_INVALID, "There is a zero on the diagonal. You can not use `sor` in this case");
}

// x_row += omega (b_row - sum_k a_row,k x_k) / d_row for the rows of one
// colour, G lanes per row (they do not couple, so x is updated in place)
template <class T, int G>
__global__ void __launch_bounds__(256) k_sor_rows(int cnt, const int* __restrict__ rows, const int* __restrict__ rp,
                                                  const int* __restrict__ ci, const T* __restrict__ v,
                                                  const T* __restrict__ d, const T* __restrict__ b, T* x, T omega,
                                                  const int* __restrict__ guard) {
  if (guarded(guard)) return;  // uniform for the whole grid
  const int lane = threadIdx.x & (G - 1);
  const int q = (blockIdx.x * blockDim.x + threadIdx.x) / G;
  const bool valid = q < cnt;
  const int row = valid ? __ldg(rows + q) : 0;
  const int beg = valid ? __ldg(rp + row) : 0;
  const int end = valid ? __ldg(rp + row + 1) : 0;
  T s = T(0);
  for (int k = beg + lane; k < end; k += G) s += __ldg(v + k) * x[__ldg(ci + k)];
#pragma unroll
  for (int off = G / 2; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off, G);
  if (valid && lane == 0) x[row] = x[row] + omega * (b[row] - s) / d[row];
}

template <class T>
static void sor_sweep_t(pm_ctx* c, const DevCsr& A, const T* vals, const T* diag, const SorColours& col, const T* b,
                        T* x, T omega, bool backward) {
  if (!diag) throw Error(PM_E_INVALID, "SOR sweep without diagonal");
  if (col.ptr.empty() || col.key != A.row_ptr.p) throw Error(PM_E_INVALID, "SOR sweep without the matrix's colours");
  const int nc = int(col.ptr.size()) - 1;
  const bool wide = A.nnz > 16 * int64_t(A.n_rows);
  for (int q = 0; q < nc; ++q) {
    const int k = backward ? nc - 1 - q : q;
    const int cnt = col.ptr[size_t(k) + 1] - col.ptr[size_t(k)];
    if (!cnt) continue;
    const int* rows = col.rows.p + col.ptr[size_t(k)];
    if (wide)
      k_sor_rows<T, 8><<<nblocks((long long)cnt * 8, 256), 256, 0, c->stream>>>(
          cnt, rows, A.row_ptr.p, A.cols.p, vals, diag, b, x, omega, c->guard);
    else
      k_sor_rows<T, 4><<<nblocks((long long)cnt * 4, 256), 256, 0, c->stream>>>(
          cnt, rows, A.row_ptr.p, A.cols.p, vals, diag, b, x, omega, c->guard);
    PM_CHECK_LAUNCH();
    c->kernel_launches++;
  }
}

void sor_sweep(pm_ctx* c, const DevCsr& A, const SorColours& col, const double* b, double* x, double omega,
               bool backward) {
  sor_sweep_t<double>(c, A, A.vals.p, A.diag.p, col, b, x, omega, backward);
}
void sor_sweep32(pm_ctx* c, const DevCsr& A, const SorColours& col, const float* b, float* x, float omega,
                 bool backward) {
  if (!A.vals32.p) throw Error(PM_E_INVALID, "matrix has no FP32 copy");
  sor_sweep_t<float>(c, A, A.vals32.p, A.diag32.p, col, b, x, omega, backward);
}

// ------------------------------------------------------- dense inverse ------
__global__ void k_dense_fill(int na, const int* __restrict__ act, const int* __restrict__ pos,
                             const int* __restrict__ rp, const int* __restrict__ ci,
                             const double* __restrict__ v, double* __restrict__ M) {
  int ia = blockIdx.x * blockDim.x + threadIdx.x;
  if (ia >= na) return;
  const int i = act[ia];
  double* row = M + (size_t)ia * na;
  for (int j = 0; j < na; ++j) row[j] = 0.0;
  for (int k = rp[i]; k < rp[i + 1]; ++k) {
    const int jp = pos[ci[k]];
    if (jp >= 0) row[jp] = v[k];
  }
}

// pivot search, row swap and pivot-row scaling of Gauss-Jordan step k
__global__ void __launch_bounds__(256) k_gj_pivot(int na, int k, double* __restrict__ M,
                                                  int* __restrict__ perm, double* __restrict__ colk,
                                                  int* __restrict__ flag) {
  __shared__ double sv[256];
  __shared__ int si[256];
  const int t = threadIdx.x;
  double best = -1.0;
  int bi = na;
  for (int i = k + t; i < na; i += blockDim.x) {
    const double a = fabs(M[(size_t)i * na + k]);
    if (a > best) { best = a; bi = i; }
  }
  sv[t] = best;
  si[t] = bi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (t < s) {
      if (sv[t + s] > sv[t] || (sv[t + s] == sv[t] && si[t + s] < si[t])) {
        sv[t] = sv[t + s];
        si[t] = si[t + s];
      }
    }
    __syncthreads();
  }
  const int p = si[0];
  const bool singular = !(sv[0] > 0.0);
  if (t == 0) {
    perm[k] = singular ? k : p;
    if (singular) *flag = 1;
  }
  if (!singular && p != k)
    for (int j = t; j < na; j += blockDim.x) {
      double a = M[(size_t)k * na + j];
      M[(size_t)k * na + j] = M[(size_t)p * na + j];
      M[(size_t)p * na + j] = a;
    }
  __syncthreads();
  const double piv = singular ? 1.0 : M[(size_t)k * na + k];
  for (int i = t; i < na; i += blockDim.x) {
    colk[i] = (i == k) ? 0.0 : M[(size_t)i * na + k];
  }
  __syncthreads();
  for (int i = t; i < na; i += blockDim.x)
    if (i != k) M[(size_t)i * na + k] = 0.0;
  __syncthreads();
  if (t == 0) M[(size_t)k * na + k] = 1.0;
  __syncthreads();
  for (int j = t; j < na; j += blockDim.x) M[(size_t)k * na + j] /= piv;
}

__global__ void k_gj_update(int na, int k, double* __restrict__ M, const double* __restrict__ colk) {
  const long long total = (long long)na * na;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = int(e / na), j = int(e % na);
    if (i == k) continue;
    const double f = colk[i];
    if (f != 0.0) M[e] -= f * M[(size_t)k * na + j];
  }
}

__global__ void k_gj_unswap(int na, double* __restrict__ M, const int* __restrict__ perm) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= na) return;
  double* row = M + (size_t)i * na;
  for (int k = na - 1; k >= 0; --k) {
    const int p = perm[k];
    if (p != k) {
      double a = row[k];
      row[k] = row[p];
      row[p] = a;
    }
  }
}

// The whole Gauss-Jordan elimination in one cooperative launch (all blocks
// resident; cooperative_groups grid barriers, two per column). Every block owns
// a contiguous range of rows. Step k: every block reduces the per-block
// partial arg-max of column k in the same fixed order (largest magnitude, the
// smallest row on ties: the pivot rule of k_gj_pivot), then writes its share of
// the scaled pivot row, the old row k and the column multipliers; after the
// barrier each block eliminates its own rows and records the partial arg-max
// of column k+1. The values are those of k_gj_pivot + k_gj_update (same
// operations per entry), without 2 launches per column.
__global__ void __launch_bounds__(256) k_gj_coop(int na, double* __restrict__ M, int* __restrict__ perm,
                                                 double* __restrict__ rowk, double* __restrict__ oldk,
                                                 double* __restrict__ colk, double* __restrict__ part_v,
                                                 int* __restrict__ part_i, int* __restrict__ flag) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  __shared__ double sv[256];
  __shared__ int si[256];
  __shared__ int s_p;
  __shared__ double s_pv;
  const int t = threadIdx.x, nb = gridDim.x, b = blockIdx.x;
  const int per = (na + nb - 1) / nb;
  const int r0 = min(na, b * per), r1 = min(na, r0 + per);
  auto block_argmax = [&](int col, int from) {
    double best = -1.0;
    int bi = na;
    for (int i = max(r0, from) + t; i < r1; i += blockDim.x) {
      const double a = fabs(M[(size_t)i * na + col]);
      if (a > best) { best = a; bi = i; }
    }
    sv[t] = best;
    si[t] = bi;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (t < s && (sv[t + s] > sv[t] || (sv[t + s] == sv[t] && si[t + s] < si[t]))) {
        sv[t] = sv[t + s];
        si[t] = si[t + s];
      }
      __syncthreads();
    }
    if (t == 0) {
      part_v[b] = sv[0];
      part_i[b] = si[0];
    }
  };
  block_argmax(0, 0);
  for (int k = 0; k < na; ++k) {
    grid.sync();
    // pivot of column k: the same reduction in every block
    if (t == 0) {
      double best = -1.0;
      int bi = na;
      for (int q = 0; q < nb; ++q)
        if (part_v[q] > best || (part_v[q] == best && part_i[q] < bi)) {
          best = part_v[q];
          bi = part_i[q];
        }
      const bool singular = !(best > 0.0);
      s_p = singular ? k : bi;
      s_pv = singular ? 1.0 : M[(size_t)bi * na + k];
      if (b == 0) {
        perm[k] = s_p;
        if (singular) *flag = 1;
      }
    }
    __syncthreads();
    const int p = s_p;
    const double pv = s_pv;
    // scaled pivot row, old row k and the multipliers (rows after the swap)
    for (int e = b * blockDim.x + t; e < na; e += nb * blockDim.x) {
      rowk[e] = (e == k ? 1.0 : M[(size_t)p * na + e]) / pv;
      oldk[e] = M[(size_t)k * na + e];
      colk[e] = (e == p && p != k) ? M[(size_t)k * na + k] : M[(size_t)e * na + k];
    }
    grid.sync();
    // elimination of this block's rows
    const long long cnt = (long long)(r1 - r0) * na;
    for (long long e = t; e < cnt; e += blockDim.x) {
      const int i = r0 + int(e / na), j = int(e % na);
      double* Mi = M + (size_t)i * na;
      if (i == k) {
        Mi[j] = rowk[j];
      } else {
        const double base = (i == p && p != k) ? oldk[j] : Mi[j];
        const double f = colk[i];
        Mi[j] = (j == k ? 0.0 : base) - f * rowk[j];
      }
    }
    __syncthreads();
    if (k + 1 < na) block_argmax(k + 1, k + 1);
  }
}

// (value, position) arg-max with the pivot rule of k_gj_pivot: the largest
// |a|, the smallest position on ties; NaN never wins
__device__ __forceinline__ void gj_merge(double& v, int& i, double v2, int i2) {
  if (v2 > v || (v2 == v && i2 < i)) {
    v = v2;
    i = i2;
  }
}

__device__ __forceinline__ void gj_warp_argmax(double& v, int& i) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
    const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
    gj_merge(v, i, v2, i2);
  }
}

// Gauss-Jordan inverse with the rows resident in shared memory: block b owns
// positions [b R, b R + R). One grid barrier per column: after step k every
// block publishes its best pivot candidate for column k+1 (the arg-max value,
// the position and the whole row) and the owner of position k+1 publishes that
// row; at step k+1 every block picks the same pivot from the published
// candidates, reads the pivot row and the old row k+1 from the published
// copies and eliminates its own rows in shared memory. The operations per
// entry are those of k_gj_pivot + k_gj_update, so the inverse is identical.
__global__ void __launch_bounds__(256) k_gj_rows(int na, int R, double* __restrict__ M, int* __restrict__ perm,
                                                 double* __restrict__ pub_rows, double* __restrict__ pub_v,
                                                 int* __restrict__ pub_i, int* __restrict__ flag) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  extern __shared__ double gj_smem[];
  __shared__ double s_f[32];  // multipliers of the own rows (R <= 32)
  __shared__ double wv[8];
  __shared__ int wi[8];
  __shared__ int s_p, s_src, s_cand;
  __shared__ double s_pv;
  const int t = threadIdx.x, nb = gridDim.x, b = blockIdx.x;
  const int lane = t & 31, warp = t >> 5;
  const int r0 = min(na, b * R), r1 = min(na, r0 + R), nr = r1 - r0;
  double* own = gj_smem;                 // [R][na]
  double* prow = own + (size_t)R * na;   // scaled pivot row of the step
  double* orow = prow + na;              // row k before the step
  const size_t slot = (size_t)(nb + 1) * na;
  for (int e = t; e < nr * na; e += blockDim.x) own[e] = M[(size_t)r0 * na + e];
  __syncthreads();
  // candidates of column col (positions >= col) into buffer buf
  auto publish = [&](int col, int buf) {
    if (warp == 0) {
      double v = -1.0;
      int i = na;
      if (lane < nr && r0 + lane >= col) {
        const double a = fabs(own[(size_t)lane * na + col]);
        if (a > v) {
          v = a;
          i = r0 + lane;
        }
      }
      gj_warp_argmax(v, i);
      if (lane == 0) {
        pub_v[buf * nb + b] = v;
        pub_i[buf * nb + b] = i;
        s_cand = i < na ? i - r0 : -1;
      }
    }
    __syncthreads();
    double* out = pub_rows + buf * slot;
    if (s_cand >= 0)
      for (int j = t; j < na; j += blockDim.x) out[(size_t)b * na + j] = own[(size_t)s_cand * na + j];
    if (col >= r0 && col < r1)
      for (int j = t; j < na; j += blockDim.x) out[(size_t)nb * na + j] = own[(size_t)(col - r0) * na + j];
  };
  publish(0, 0);
  grid.sync();
  for (int k = 0; k < na; ++k) {
    const int buf = k & 1;
    const double* pub = pub_rows + buf * slot;
    {  // the pivot: the same reduction in every block
      double v = -1.0;
      int i = na;
      for (int q = t; q < nb; q += blockDim.x) gj_merge(v, i, pub_v[buf * nb + q], pub_i[buf * nb + q]);
      gj_warp_argmax(v, i);
      if (lane == 0) {
        wv[warp] = v;
        wi[warp] = i;
      }
      __syncthreads();
      if (t == 0) {
        double best = wv[0];
        int bi = wi[0];
        for (int w = 1; w < int(blockDim.x >> 5); ++w) gj_merge(best, bi, wv[w], wi[w]);
        const bool singular = !(best > 0.0);
        s_p = singular ? k : bi;
        s_src = singular ? nb : bi / R;
        s_pv = singular ? 1.0 : pub[(size_t)(bi / R) * na + k];
        if (b == 0) {
          perm[k] = s_p;
          if (singular) *flag = 1;
        }
      }
      __syncthreads();
    }
    const int p = s_p;
    const double pv = s_pv;
    const double* src = pub + (size_t)s_src * na;
    const double* old = pub + (size_t)nb * na;
    for (int j = t; j < na; j += blockDim.x) {
      prow[j] = (j == k ? 1.0 : src[j]) / pv;
      orow[j] = old[j];
    }
    if (t < nr) {
      const int i = r0 + t;
      s_f[t] = (i == p && p != k) ? old[k] : own[(size_t)t * na + k];
    }
    __syncthreads();
    for (int e = t; e < nr * na; e += blockDim.x) {
      const int ii = e / na, j = e - ii * na;
      const int i = r0 + ii;
      double* Mi = own + (size_t)ii * na;
      if (i == k) {
        Mi[j] = prow[j];
      } else {
        const double base = (i == p && p != k) ? orow[j] : Mi[j];
        Mi[j] = (j == k ? 0.0 : base) - s_f[ii] * prow[j];
      }
    }
    __syncthreads();
    if (k + 1 < na) publish(k + 1, buf ^ 1);
    grid.sync();
  }
  for (int e = t; e < nr * na; e += blockDim.x) M[(size_t)r0 * na + e] = own[e];
}

constexpr size_t kGjRowsSmem = 160 * 1024;  // dynamic shared memory cap of k_gj_rows

// Gauss-Jordan inverse in FP32 on one cluster of CS thread blocks (CS = 1: a
// single block): block r keeps positions [r R, r R + R) in its shared memory.
// Per column one cluster barrier. Before it, every block pushes its pivot
// candidate for the next column (arg-max value and position) into every
// block's candidate table, keeps the candidate row in its own double-buffered
// publication slot, and the owner of the next position pushes that row into
// every block's old-row buffer. After it, every block picks the pivot from its
// local table (the rule of k_gj_pivot: largest |a|, smallest position on
// ties), reads the pivot row from the winner's slot (the one remote read of
// the step) and eliminates its own rows, thread tx on column tx for the rows
// ty, ty + G, ... . The column swaps are undone on the rows in shared memory
// before they are written out.
constexpr int kGjCluster = 8;
constexpr size_t kGjClusterSmem = 220 * 1024;

template <class T>
__device__ __forceinline__ void gj_merge(T& v, int& i, T v2, int i2) {
  if (v2 > v || (v2 == v && i2 < i)) {
    v = v2;
    i = i2;
  }
}

// T = float: the mixed cycle's inverse; T = double: the FP64 inverse, written
// in place over the dense block M (every block reads its rows of M before the
// first cluster barrier and writes them after the last one)
template <class T, int NT>
__global__ void __launch_bounds__(NT)
k_gj_cluster(int na, int R, const double* M, T* out, int* __restrict__ flag) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char gjc_raw[];
  T* gjc_smem = reinterpret_cast<T*>(gjc_raw);
  __shared__ T cand_v[2][kGjCluster];
  __shared__ int cand_i[2][kGjCluster];
  __shared__ T s_f[256];  // multipliers of the own rows (R <= 256)
  __shared__ int s_p, s_src, s_cand, s_sing;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int CS = int(cluster.num_blocks());
  const int rank = int(cluster.block_rank());
  const int r0 = min(na, rank * R), r1 = min(na, r0 + R), nr = r1 - r0;
  // column-major thread layout of the elimination: CW threads per row pass
  const int na32 = (na + 31) & ~31;
  const int G = max(1, NT / na32), CW = NT / G;
  const int tx = t % CW, ty = t / CW;
  T* own = gjc_smem;                    // [R][na]
  T* pubrow = own + (size_t)R * na;     // [2][na] pivot candidate for the next column
  T* oldrow = pubrow + 2 * (size_t)na;  // [2][na] the row at the next position (pushed by its owner)
  T* prow = oldrow + 2 * (size_t)na;    // scaled pivot row of the step
  int* perm_s = reinterpret_cast<int*>(prow + na);  // pivot positions
  for (int e = t; e < nr * na; e += NT) own[e] = T(M[(size_t)r0 * na + e]);
  if (t == 0) s_sing = 0;
  __syncthreads();
  auto publish = [&](int col, int buf) {
    if (warp == 0) {
      T v = -T(1.0);
      int i = na;
      for (int q = lane; q < nr; q += 32)
        if (r0 + q >= col) gj_merge<T>(v, i, fabs(own[(size_t)q * na + col]), r0 + q);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const T v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
        gj_merge<T>(v, i, v2, i2);
      }
      if (lane < CS) {  // into every block's candidate table
        cluster.map_shared_rank(&cand_v[buf][0], lane)[rank] = v;
        cluster.map_shared_rank(&cand_i[buf][0], lane)[rank] = i;
      }
      if (lane == 0) s_cand = i < na ? i - r0 : -1;
    }
    __syncthreads();
    if (s_cand >= 0)
      for (int j = t; j < na; j += NT) pubrow[(size_t)buf * na + j] = own[(size_t)s_cand * na + j];
    if (col >= r0 && col < r1)  // the old row of the next step, into every block
      for (int q = 0; q < CS; ++q) {
        T* dst = cluster.map_shared_rank(oldrow, q) + (size_t)buf * na;
        for (int j = t; j < na; j += NT) dst[j] = own[(size_t)(col - r0) * na + j];
      }
  };
  publish(0, 0);
  cluster.sync();
  for (int k = 0; k < na; ++k) {
    const int buf = k & 1;
    if (warp == 0) {  // the pivot: the same reduction in every block
      T v = -T(1.0);
      int i = na;
      if (lane < CS) {
        v = cand_v[buf][lane];
        i = cand_i[buf][lane];
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const T v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
        gj_merge<T>(v, i, v2, i2);
      }
      if (lane == 0) {
        const bool singular = !(v > T(0.0));
        s_p = singular ? k : i;
        s_src = singular ? -1 : i / R;  // -1: the pivot row is the old row k
        perm_s[k] = s_p;
        if (singular) s_sing = 1;
      }
    }
    __syncthreads();
    const int p = s_p;
    const T* old = oldrow + (size_t)buf * na;
    const T* src = s_src < 0 ? old : cluster.map_shared_rank(pubrow, s_src) + (size_t)buf * na;
    const T pv = s_src < 0 ? T(1.0) : src[k];
    for (int j = t; j < na; j += NT) prow[j] = (j == k ? T(1.0) : src[j]) / pv;
    if (t < nr) {
      const int i = r0 + t;
      s_f[t] = (i == p && p != k) ? old[k] : own[(size_t)t * na + k];
    }
    __syncthreads();
    for (int j = tx; j < na; j += CW) {
      const T pj = prow[j], oj = old[j];
      const bool jk = j == k;
      for (int ii = ty; ii < nr; ii += G) {  // the row index is the same across a warp
        const int i = r0 + ii;
        T* Mij = own + (size_t)ii * na + j;
        if (i != k && i != p) {
          *Mij = (jk ? T(0.0) : *Mij) - s_f[ii] * pj;
        } else if (i == k) {
          *Mij = pj;
        } else {  // i == p != k: the old row k moves here
          *Mij = (jk ? T(0.0) : oj) - s_f[ii] * pj;
        }
      }
    }
    __syncthreads();
    if (k + 1 < na) publish(k + 1, buf ^ 1);
    cluster.sync();  // publications visible; every block is done reading this step's
  }
  // undo the column swaps (k_gj_unswap) on the own rows, write them out
  for (int q = t; q < nr; q += NT) {
    T* row = own + (size_t)q * na;
    for (int k = na - 1; k >= 0; --k) {
      const int pk = perm_s[k];
      if (pk != k) {
        const T a = row[k];
        row[k] = row[pk];
        row[pk] = a;
      }
    }
  }
  __syncthreads();
  for (int e = t; e < nr * na; e += NT) out[(size_t)r0 * na + e] = own[e];
  if (t == 0 && s_sing) *flag = 1;
}

__global__ void k_coarse_gemv32(int n, int na, const int* __restrict__ act, const int* __restrict__ pos,
                                const float* __restrict__ inv, const float* __restrict__ b,
                                float* __restrict__ x) {
  pdl_enter();
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp < na) {
    const float* row = inv + (size_t)warp * na;
    float s = 0.0f;
    for (int j = lane; j < na; j += 32) s += row[j] * b[act[j]];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) x[act[warp]] = s;
  } else {
    const int t = (warp - na) * 32 + lane;
    if (t < n && pos[t] < 0) x[t] = b[t];
  }
}

// the mixed cycle's coarse solve with the FP64 inverse: FP32 right-hand
// side and iterate, FP64 inverse entries and FP64 accumulation (the split
// of the outer solve: FP64 for the coarse-grid direct solve)
__global__ void k_coarse_gemv_mixed(int n, int na, const int* __restrict__ act, const int* __restrict__ pos,
                                    const double* __restrict__ inv, const float* __restrict__ b,
                                    float* __restrict__ x) {
  pdl_enter();
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp < na) {
    const double* row = inv + (size_t)warp * na;
    double s = 0.0;
    for (int j = lane; j < na; j += 32) s = fma(row[j], double(b[act[j]]), s);
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) x[act[warp]] = float(s);
  } else {
    const int t = (warp - na) * 32 + lane;
    if (t < n && pos[t] < 0) x[t] = b[t];
  }
}

void DenseInverse::solve_mixed(pm_ctx* c, const float* b, float* x) {
  if (!has64) throw Error(PM_E_INVALID, "coarse solve before the FP64 inverse was built");
  const long long threads = (long long)na * 32 + n;
  launch_k(c, k_coarse_gemv_mixed, dim3(nblocks(threads, 256)), dim3(256), 0, n, na, (const int*)act.p,
           (const int*)pos.p, (const double*)inv.p, b, x);
}

void DenseInverse::build32(pm_ctx* c, const DevCsr& A) {
  launch32(c, A, c->stream);
  complete32(c, A);
}

void DenseInverse::launch32(pm_ctx* c, const DevCsr& A, cudaStream_t s) {
  pending32 = false;
  n = A.n_rows;
  int na_ = 0;
  for (int i = 0; i < n; ++i)
    for (int b = 0; b < A.mask.nb; ++b)
      if (i >= A.mask.start[b] && i < A.mask.end[b] && i < A.mask.active_end[b]) ++na_;
  // one block when the whole active block fits its shared memory, else a
  // cluster of kGjCluster blocks
  auto smem_for = [&](int R) { return (size_t(R) + 5) * na_ * sizeof(float) + size_t(na_) * sizeof(int); };
  int cs = std::max(1, std::min(kGjCluster, c->coarse_cluster)), R = (na_ + cs - 1) / cs;
  while (cs < kGjCluster && smem_for(R) > kGjClusterSmem) {
    cs *= 2;
    R = (na_ + cs - 1) / cs;
  }
  const size_t smem = smem_for(R);
  if (na_ == 0 || R > 256 || smem > kGjClusterSmem) {
    build(c, A);  // large: the FP64 inverse, rounded
    inv32.ensure(size_t(na) * na);
    if (na) {
      k_d2f<<<grid_for(c, (long long)na * na), 256, 0, c->stream>>>((long long)na * na, inv.p, inv32.p);
      PM_CHECK_LAUNCH();
      c->kernel_launches++;
    }
    has32 = true;
    return;
  }
  // the preparation and the kernel on stream s (restored on every exit)
  struct StreamSwap {
    pm_ctx* c;
    cudaStream_t saved;
    StreamSwap(pm_ctx* c_, cudaStream_t s_) : c(c_), saved(c_->stream) { c->stream = s_; }
    ~StreamSwap() { c->stream = saved; }
  } swap(c, s);
  prepare(c, A);  // act, pos, the dense active block in inv (FP64)
  inv32.ensure(size_t(na) * na);
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(k_gj_cluster<float, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    int(kGjClusterSmem));
    if (attr_err == cudaSuccess)
      attr_err = cudaFuncSetAttribute(k_gj_cluster<float, 512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      int(kGjClusterSmem));
    if (attr_err == cudaSuccess)
      attr_err = cudaFuncSetAttribute(k_gj_cluster<float, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      int(kGjClusterSmem));
  });
  PM_CUDA(attr_err);
  // measured on GB300 (225 and 343 active rows): 8 blocks of 1024 threads
  const int nt = c->coarse_threads > 0 ? c->coarse_threads : 1024;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(unsigned(cs));
  cfg.blockDim = dim3(unsigned(nt));
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = unsigned(cs);
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const double* Mp = inv.p;
  float* outp = inv32.p;
  int* fl = flag.p;
  int na_arg = na, R_arg = R;
  if (nt == 1024) PM_CUDA(cudaLaunchKernelEx(&cfg, k_gj_cluster<float, 1024>, na_arg, R_arg, Mp, outp, fl));
  else if (nt == 512) PM_CUDA(cudaLaunchKernelEx(&cfg, k_gj_cluster<float, 512>, na_arg, R_arg, Mp, outp, fl));
  else PM_CUDA(cudaLaunchKernelEx(&cfg, k_gj_cluster<float, 256>, na_arg, R_arg, Mp, outp, fl));
  c->kernel_launches++;
  if (!done_event) PM_CUDA(cudaEventCreateWithFlags(&done_event, cudaEventDisableTiming));
  PM_CUDA(cudaEventRecord(done_event, s));
  pending32 = true;
}

void DenseInverse::complete32(pm_ctx* c, const DevCsr& A) {
  if (!pending32) return;  // done at launch (large matrices) or nothing queued
  pending32 = false;
  int h_flag = 0;
  PM_CUDA(cudaStreamWaitEvent(c->stream, done_event, 0));
  PM_CUDA(cudaMemcpyAsync(&h_flag, flag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));
  if (h_flag) {
    // no FP32 pivot (a singular matrix, or values beyond the FP32 range): the
    // FP64 inverse decides (and throws if the matrix is singular), rounded
    build(c, A);
    if (na) {
      k_d2f<<<grid_for(c, (long long)na * na), 256, 0, c->stream>>>((long long)na * na, inv.p, inv32.p);
      PM_CHECK_LAUNCH();
      c->kernel_launches++;
    }
    has32 = true;
    return;
  }
  has64 = false;  // inv holds the active block, not its inverse
  has32 = true;
}

void DenseInverse::solve32(pm_ctx* c, const float* b, float* x) {
  if (!has32) throw Error(PM_E_INVALID, "coarse FP32 inverse used before build32");
  const long long threads = (long long)(na + (n + 31) / 32) * 32;
  launch_k(c, k_coarse_gemv32, dim3(nblocks(threads, 256)), dim3(256), 0, n, na, (const int*)act.p,
             (const int*)pos.p, (const float*)inv32.p, b, x);
}

void DenseInverse::prepare(pm_ctx* c, const DevCsr& A) {
  n = A.n_rows;
  std::vector<int> h_act, h_pos(n, -1);
  for (int i = 0; i < n; ++i) {
    bool active = false;
    for (int b = 0; b < A.mask.nb; ++b)
      if (i >= A.mask.start[b] && i < A.mask.end[b]) active = i < A.mask.active_end[b];
    if (active) {
      h_pos[i] = int(h_act.size());
      h_act.push_back(i);
    }
  }
  na = int(h_act.size());
  if (na > 20000) throw Error(PM_E_UNSUPPORTED, "coarse direct solve limited to 20000 active rows");
  act.upload(h_act, c->stream);
  pos.upload(h_pos, c->stream);
  inv.ensure(size_t(na) * na);
  tmp.ensure(std::max(na, 1));
  perm.ensure(std::max(na, 1));
  flag.ensure(1);
  PM_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), c->stream));
  has64 = has32 = false;
  if (na == 0) return;
  k_dense_fill<<<nblocks(na, 128), 128, 0, c->stream>>>(na, act.p, pos.p, A.row_ptr.p, A.cols.p,
                                                        A.vals.p, inv.p);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

void DenseInverse::build(pm_ctx* c, const DevCsr& A) {
  launch64(c, A, c->stream);
  complete64(c);
}

void DenseInverse::complete64(pm_ctx* c) {
  if (!pending64) return;
  pending64 = false;
  int h_flag = 0;
  PM_CUDA(cudaStreamWaitEvent(c->stream, done_event, 0));
  PM_CUDA(cudaMemcpyAsync(&h_flag, flag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));
  if (h_flag) throw Error(PM_E_BREAKDOWN, "coarse matrix is singular (zero pivot)");
  has64 = true;
}

void DenseInverse::launch64(pm_ctx* c, const DevCsr& A, cudaStream_t s) {
  pending64 = false;
  struct StreamSwap {
    pm_ctx* c;
    cudaStream_t saved;
    StreamSwap(pm_ctx* c_, cudaStream_t s_) : c(c_), saved(c_->stream) { c->stream = s_; }
    ~StreamSwap() { c->stream = saved; }
  } swap(c, s);
  prepare(c, A);
  if (na == 0) {
    has64 = true;
    return;
  }
  // Gauss-Jordan on one thread-block cluster when the active block fits its
  // distributed shared memory (cluster barriers per column instead of grid
  // barriers; the same pivot rule), in place
  {
    auto smem_for = [&](int R) { return (size_t(R) + 5) * na * sizeof(double) + size_t(na) * sizeof(int); };
    int cs = std::max(1, std::min(kGjCluster, c->coarse_cluster)), R = (na + cs - 1) / cs;
    while (cs < kGjCluster && smem_for(R) > kGjClusterSmem) {
      cs *= 2;
      R = (na + cs - 1) / cs;
    }
    const size_t smem = smem_for(R);
    if (R <= 256 && smem <= kGjClusterSmem) {
      static std::once_flag once;
      static cudaError_t attr_err = cudaSuccess;
      std::call_once(once, [] {
        attr_err = cudaFuncSetAttribute(k_gj_cluster<double, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        int(kGjClusterSmem));
        if (attr_err == cudaSuccess)
          attr_err = cudaFuncSetAttribute(k_gj_cluster<double, 512>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, int(kGjClusterSmem));
        if (attr_err == cudaSuccess)
          attr_err = cudaFuncSetAttribute(k_gj_cluster<double, 256>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, int(kGjClusterSmem));
      });
      PM_CUDA(attr_err);
      const int nt = c->coarse_threads > 0 ? c->coarse_threads : 1024;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(unsigned(cs));
      cfg.blockDim = dim3(unsigned(nt));
      cfg.dynamicSmemBytes = smem;
      cfg.stream = s;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = unsigned(cs);
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      const double* Mp = inv.p;
      double* outp = inv.p;
      int* fl = flag.p;
      int na_arg = na, R_arg = R;
      if (nt == 1024) PM_CUDA(cudaLaunchKernelEx(&cfg, k_gj_cluster<double, 1024>, na_arg, R_arg, Mp, outp, fl));
      else if (nt == 512) PM_CUDA(cudaLaunchKernelEx(&cfg, k_gj_cluster<double, 512>, na_arg, R_arg, Mp, outp, fl));
      else PM_CUDA(cudaLaunchKernelEx(&cfg, k_gj_cluster<double, 256>, na_arg, R_arg, Mp, outp, fl));
      c->kernel_launches++;
      if (!done_event) PM_CUDA(cudaEventCreateWithFlags(&done_event, cudaEventDisableTiming));
      PM_CUDA(cudaEventRecord(done_event, s));
      pending64 = true;
      return;
    }
  }
  int coop = 0, per_sm = 0;
  PM_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device));
  PM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gj_coop, 256, 0));
  // row-resident variant: R rows per block (at most 32), rows and two row
  // buffers in shared memory
  const int R = std::max(2, (na + c->num_sms - 1) / c->num_sms);
  const size_t rsmem = size_t(R + 2) * na * sizeof(double);
  const int rblocks = (na + R - 1) / R;
  int rows_per_sm = 0;
  if (coop && R <= 32 && rsmem <= kGjRowsSmem) {
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
      attr_err = cudaFuncSetAttribute(k_gj_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kGjRowsSmem));
    });
    PM_CUDA(attr_err);
    PM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rows_per_sm, k_gj_rows, 256, rsmem));
  }
  if (rows_per_sm > 0 && rows_per_sm * c->num_sms >= rblocks) {
    pub_rows.ensure(2 * size_t(rblocks + 1) * na);
    pub_v.ensure(2 * size_t(rblocks));
    pub_i.ensure(2 * size_t(rblocks));
    double* M = inv.p;
    int* pp = perm.p;
    double* pr = pub_rows.p;
    double* pv = pub_v.p;
    int* pi = pub_i.p;
    int* fl = flag.p;
    int nan_ = na, R_ = R;
    void* args[] = {&nan_, &R_, &M, &pp, &pr, &pv, &pi, &fl};
    PM_CUDA(cudaLaunchCooperativeKernel((const void*)k_gj_rows, dim3(rblocks), dim3(256), args, rsmem, c->stream));
    c->kernel_launches++;
  } else if (coop && per_sm > 0) {
    // one cooperative launch; at most one block per SM and about 8 rows per block
    int nb = std::min(c->num_sms, std::max(1, (na + 7) / 8));
    rowk.ensure(na);
    oldk.ensure(na);
    part_v.ensure(nb);
    part_i.ensure(nb);
    double* M = inv.p;
    int* pp = perm.p;
    double* rk = rowk.p;
    double* ok = oldk.p;
    double* ck = tmp.p;
    double* pv = part_v.p;
    int* pi = part_i.p;
    int* fl = flag.p;
    int nan_ = na;
    void* args[] = {&nan_, &M, &pp, &rk, &ok, &ck, &pv, &pi, &fl};
    PM_CUDA(cudaLaunchCooperativeKernel((const void*)k_gj_coop, dim3(nb), dim3(256), args, 0, c->stream));
    c->kernel_launches++;
  } else {
    const int ugrid = std::max(1, std::min(nblocks((long long)na * na, 256), c->num_sms * 8));
    for (int k = 0; k < na; ++k) {
      k_gj_pivot<<<1, 256, 0, c->stream>>>(na, k, inv.p, perm.p, tmp.p, flag.p);
      k_gj_update<<<ugrid, 256, 0, c->stream>>>(na, k, inv.p, tmp.p);
      c->kernel_launches += 2;
    }
  }
  PM_CHECK_LAUNCH();
  k_gj_unswap<<<nblocks(na, 128), 128, 0, c->stream>>>(na, inv.p, perm.p);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
  if (!done_event) PM_CUDA(cudaEventCreateWithFlags(&done_event, cudaEventDisableTiming));
  PM_CUDA(cudaEventRecord(done_event, s));
  pending64 = true;
}

// tmp_a = b_a - sum over non-active columns of A_{a,j} b_j
__global__ void k_coarse_rhs(int na, const int* __restrict__ act, const int* __restrict__ pos,
                             const int* __restrict__ rp, const int* __restrict__ ci,
                             const double* __restrict__ v, const double* __restrict__ b,
                             double* __restrict__ tmp) {
  int ia = blockIdx.x * blockDim.x + threadIdx.x;
  if (ia >= na) return;
  const int i = act[ia];
  double r = b[i];
  for (int k = rp[i]; k < rp[i + 1]; ++k)
    if (pos[ci[k]] < 0) r -= v[k] * b[ci[k]];
  tmp[ia] = r;
}

// x_a = inv * tmp (one warp per row), x_n = b_n
__global__ void k_coarse_gemv(int n, int na, const int* __restrict__ act, const int* __restrict__ pos,
                              const double* __restrict__ inv, const double* __restrict__ tmp,
                              const double* __restrict__ b, double* __restrict__ x,
                              const int* __restrict__ gather) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp < na) {
    const double* row = inv + (size_t)warp * na;
    double s = 0.0;
    // gather != null: the right-hand side's non-actives are zero, read b directly
    for (int j = lane; j < na; j += 32) s += row[j] * (gather ? b[gather[j]] : tmp[j]);
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) x[act[warp]] = s;
  } else {
    // remaining threads copy the non-active entries
    const int t = (warp - na) * 32 + lane;
    if (t < n && pos[t] < 0) x[t] = b[t];
  }
}

void DenseInverse::solve(pm_ctx* c, const DevCsr& A, const double* b, double* x, bool rhs_nonactive_zero) {
  if (na > 0 && !rhs_nonactive_zero) {
    k_coarse_rhs<<<nblocks(na, 128), 128, 0, c->stream>>>(na, act.p, pos.p, A.row_ptr.p, A.cols.p,
                                                          A.vals.p, b, tmp.p);
    PM_CHECK_LAUNCH();
    c->kernel_launches++;
  }
  const long long threads = (long long)(na + (n + 31) / 32) * 32;
  k_coarse_gemv<<<nblocks(threads, 256), 256, 0, c->stream>>>(n, na, act.p, pos.p, inv.p, tmp.p, b, x,
                                                              rhs_nonactive_zero ? act.p : nullptr);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

}  // namespace pm

// ---------------------------------------------------------------------------
// Batched launches (pm_batch.h): the same operation for the slots of a batch
// in one launch (the slot is blockIdx.x in the SpMV family, blockIdx.y
// elsewhere). The SpMV family runs csr_body / sell_body,
// the other kernels restate the single-problem loops line for line, so each
// slot gets the bits a lone launch gives.
#include "pm_batch.h"

namespace pm {

// SpMV-family launches: bt.vals holds two pointers per slot, the sliced-ELL
// values [2 s] and the CSR values [2 s + 1]; bt.aux the slot's diagonal
template <class TV, class TX, class TA, int G, int U, int EPI>
__global__ void __launch_bounds__(256)
csr_batch_kernel(int n_rows, const int* __restrict__ row_ptr, const int* __restrict__ cols,
                 const TV* __restrict__ vals, const TX* __restrict__ x, TX* __restrict__ y,
                 const TX* __restrict__ b, const TX* __restrict__ diag, TA alpha, BlockMask mask, Batch bt) {
  const int s = blockIdx.x;
  if (!bt.on[s]) return;
  const TV* v = bt.vals ? static_cast<const TV*>(bt.vals[2 * s + 1]) : vals;
  const TX* d = bt.aux ? static_cast<const TX*>(bt.aux[s]) : diag;
  const TX* xs = slot_ptr(x, bt, s);
  csr_body<TV, TX, TA, G, U, EPI>(n_rows, row_ptr, cols, v, xs, slot_ptr(y, bt, s), slot_ptr(b, bt, s), d, xs,
                                  alpha, mask, blockIdx.y, gridDim.y);
}

template <class T, int L, int U, bool PIPE, int EPI>
__global__ void __launch_bounds__(128)
sell_batch_kernel(int n_slices, const int* __restrict__ perm, const int* __restrict__ soff,
                  const int* __restrict__ scols, const T* __restrict__ svals, const T* __restrict__ x,
                  T* __restrict__ y, const T* __restrict__ b, const T* __restrict__ diag, T alpha, BlockMask mask,
                  Batch bt) {
  const int s = blockIdx.x;
  if (!bt.on[s]) return;
  const T* v = bt.vals ? static_cast<const T*>(bt.vals[2 * s]) : svals;
  const T* d = bt.aux ? static_cast<const T*>(bt.aux[s]) : diag;
  sell_body<T, L, U, PIPE, EPI>(n_slices, perm, soff, scols, v, slot_ptr(x, bt, s), slot_ptr(y, bt, s),
                                slot_ptr(b, bt, s), d, alpha, mask, blockIdx.y);
}

template <class T, int L, int U, bool P, int EPI>
static void launch_sell_batch_epi(pm_ctx* c, const DevCsr& A, int ns, const Batch& bt, const T* x, T* y, const T* b,
                                  const T* d, T alpha, const BlockMask& m) {
  cudaLaunchConfig_t cfg = {};
  if (nblocks(A.n_slices, 4) > 65535) throw Error(PM_E_UNSUPPORTED, "batched launch: too many row blocks");
  cfg.gridDim = dim3(unsigned(ns), unsigned(nblocks(A.n_slices, 4)));
  cfg.blockDim = dim3(128);
  cfg.stream = c->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = c->pdl >= 1 ? 1 : 0;
  PM_CUDA(cudaLaunchKernelEx(&cfg, sell_batch_kernel<T, L, U, P, EPI>, A.n_slices, (const int*)A.sell_perm.p,
                             (const int*)A.sell_off.p, (const int*)A.sell_cols.p, sell_values<T>(A), x, y, b, d,
                             alpha, m, bt));
  c->kernel_launches++;
}

template <class T, int L, int U, bool P>
static void launch_sell_batch(pm_ctx* c, const DevCsr& A, int ns, const Batch& bt, int epi, const T* x, T* y,
                              const T* b, const T* d, T alpha, const BlockMask& m) {
  switch (epi) {
    case EPI_AXPY: launch_sell_batch_epi<T, L, U, P, EPI_AXPY>(c, A, ns, bt, x, y, b, d, alpha, m); break;
    case EPI_SET: launch_sell_batch_epi<T, L, U, P, EPI_SET>(c, A, ns, bt, x, y, b, d, alpha, m); break;
    case EPI_DEFECT: launch_sell_batch_epi<T, L, U, P, EPI_DEFECT>(c, A, ns, bt, x, y, b, d, alpha, m); break;
    case EPI_JACOBI: launch_sell_batch_epi<T, L, U, P, EPI_JACOBI>(c, A, ns, bt, x, y, b, d, alpha, m); break;
    case EPI_RESTRICT: launch_sell_batch_epi<T, L, U, P, EPI_RESTRICT>(c, A, ns, bt, x, y, b, d, alpha, m); break;
    case EPI_PROLONG: launch_sell_batch_epi<T, L, U, P, EPI_PROLONG>(c, A, ns, bt, x, y, b, d, alpha, m); break;
    default: throw Error(PM_E_INVALID, "unknown SpMV epilogue");
  }
}

template <class TV, class TX, class TA, int G, int U>
static void launch_csr_batch_gu(pm_ctx* c, int ns, const Batch& bt, int epi, int n, const DevCsr& A, const TV* v,
                                const TX* x, TX* y, const TX* b, const TX* d, TA alpha, const BlockMask& m) {
  if (nblocks((long long)n * G, 256) > 65535) throw Error(PM_E_UNSUPPORTED, "batched launch: too many row blocks");
  const dim3 gr = dim3(unsigned(ns), unsigned(nblocks((long long)n * G, 256))), bl = dim3(256);
  const int* rp = A.row_ptr.p;
  const int* ci = A.cols.p;
  switch (epi) {
    case EPI_AXPY: csr_batch_kernel<TV, TX, TA, G, U, EPI_AXPY><<<gr, bl, 0, c->stream>>>(n, rp, ci, v, x, y, b, d, alpha, m, bt); break;
    case EPI_SET: csr_batch_kernel<TV, TX, TA, G, U, EPI_SET><<<gr, bl, 0, c->stream>>>(n, rp, ci, v, x, y, b, d, alpha, m, bt); break;
    case EPI_DEFECT: csr_batch_kernel<TV, TX, TA, G, U, EPI_DEFECT><<<gr, bl, 0, c->stream>>>(n, rp, ci, v, x, y, b, d, alpha, m, bt); break;
    case EPI_JACOBI: csr_batch_kernel<TV, TX, TA, G, U, EPI_JACOBI><<<gr, bl, 0, c->stream>>>(n, rp, ci, v, x, y, b, d, alpha, m, bt); break;
    case EPI_RESTRICT: csr_batch_kernel<TV, TX, TA, G, U, EPI_RESTRICT><<<gr, bl, 0, c->stream>>>(n, rp, ci, v, x, y, b, d, alpha, m, bt); break;
    case EPI_PROLONG: csr_batch_kernel<TV, TX, TA, G, U, EPI_PROLONG><<<gr, bl, 0, c->stream>>>(n, rp, ci, v, x, y, b, d, alpha, m, bt); break;
    default: throw Error(PM_E_INVALID, "unknown SpMV epilogue");
  }
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

// the launch shapes DevCsr::upload picks: FP64 four lanes x four or eight
// loads, FP32 four x four or eight x sixteen
template <class TV, class TX, class TA>
static void launch_csr_batch(pm_ctx* c, int ns, const Batch& bt, int epi, int n, const DevCsr& A, const TV* v,
                             const TX* x, TX* y, const TX* b, const TX* d, TA alpha, const BlockMask& m) {
  const bool fp32 = sizeof(TV) == 4;
  const int G = fp32 ? A.lanes32 : A.lanes;
  const int U = fp32 ? A.unroll32 : A.unroll;
  if (G == 4 && U == 4) launch_csr_batch_gu<TV, TX, TA, 4, 4>(c, ns, bt, epi, n, A, v, x, y, b, d, alpha, m);
  else if (G == 4 && U == 8) launch_csr_batch_gu<TV, TX, TA, 4, 8>(c, ns, bt, epi, n, A, v, x, y, b, d, alpha, m);
  else if (G == 8 && U == 16) launch_csr_batch_gu<TV, TX, TA, 8, 16>(c, ns, bt, epi, n, A, v, x, y, b, d, alpha, m);
  else throw Error(PM_E_UNSUPPORTED, "batched CSR launch shape " + std::to_string(G) + "x" + std::to_string(U));
}

void csr_apply_batch(pm_ctx* c, const DevCsr& A, int ns, const Batch& bt, int epi, const double* x, double* y,
                     const double* b, double alpha) {
  const int n = A.n_rows;
  if (n <= 0) return;
  if (A.stream && A.n_rblocks > 0) throw Error(PM_E_UNSUPPORTED, "batched launch of the streaming CSR kernel");
  if (c->sell_shape64 > 0 && A.sell64_ok && A.sell_lanes == c->sell_shape64 / 100 && A.n_slices > 0) {
    switch (c->sell_shape64) {
      case 441: launch_sell_batch<double, 4, 4, true>(c, A, ns, bt, epi, x, y, b, A.diag.p, alpha, A.mask); break;
      case 481: launch_sell_batch<double, 4, 8, true>(c, A, ns, bt, epi, x, y, b, A.diag.p, alpha, A.mask); break;
      case 841: launch_sell_batch<double, 8, 4, true>(c, A, ns, bt, epi, x, y, b, A.diag.p, alpha, A.mask); break;
      default: throw Error(PM_E_INVALID, "unknown FP64 sliced SpMV shape");
    }
    PM_CHECK_LAUNCH();
    return;
  }
  launch_csr_batch<double, double, double>(c, ns, bt, epi, n, A, A.vals.p, x, y, b, A.diag.p, alpha, A.mask);
}

void csr_apply32_batch(pm_ctx* c, const DevCsr& A, int ns, const Batch& bt, int epi, const float* x, float* y,
                       const float* b, float alpha) {
  const int n = A.n_rows;
  if (n <= 0) return;
  if (A.stream && A.n_rblocks > 0) throw Error(PM_E_UNSUPPORTED, "batched launch of the streaming CSR kernel");
  if (c->sell_shape > 0 && A.sell_lanes == c->sell_shape / 100 && A.n_slices > 0) {
    switch (c->sell_shape) {
      case 441: launch_sell_batch<float, 4, 4, true>(c, A, ns, bt, epi, x, y, b, A.diag32.p, alpha, A.mask); break;
      case 481: launch_sell_batch<float, 4, 8, true>(c, A, ns, bt, epi, x, y, b, A.diag32.p, alpha, A.mask); break;
      case 841: launch_sell_batch<float, 8, 4, true>(c, A, ns, bt, epi, x, y, b, A.diag32.p, alpha, A.mask); break;
      case 881: launch_sell_batch<float, 8, 8, true>(c, A, ns, bt, epi, x, y, b, A.diag32.p, alpha, A.mask); break;
      default: throw Error(PM_E_UNSUPPORTED, "batched launch of sliced shape " + std::to_string(c->sell_shape));
    }
    PM_CHECK_LAUNCH();
    return;
  }
  launch_csr_batch<float, float, float>(c, ns, bt, epi, n, A, A.vals32.p, x, y, b, A.diag32.p, alpha, A.mask);
}

__global__ void kb_copy(long long n, const double* __restrict__ x, double* __restrict__ y, Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  x = slot_ptr(x, bt);
  y = slot_ptr(y, bt);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = x[i];
}
__global__ void kb_d2f(long long n, const double* __restrict__ x, float* __restrict__ y, Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  x = slot_ptr(x, bt);
  y = slot_ptr(y, bt);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = float(x[i]);
}
__global__ void kb_f2d(long long n, const float* __restrict__ x, double* __restrict__ y, Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  x = slot_ptr(x, bt);
  y = slot_ptr(y, bt);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = double(x[i]);
}
template <class T>
__global__ void kb_init_sol(int n, BlockMask m, const T* __restrict__ rhs, T* __restrict__ sol, Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  rhs = slot_ptr(rhs, bt);
  sol = slot_ptr(sol, bt);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    sol[i] = row_is_active(m, i) ? T(0) : rhs[i];
}
template <class T>
__global__ void kb_jacobi_zero(int n, const T* __restrict__ b, T w, T* __restrict__ x, Batch bt) {
  const int s = blockIdx.y;
  if (!bt.on[s]) return;
  const T* d = static_cast<const T*>(bt.aux[s]);
  b = slot_ptr(b, bt);
  x = slot_ptr(x, bt);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] = fmadd(w, (b[i] - T(0)) / d[i], T(0));
}

#define PM_LAUNCH_BATCH(kern, ns, n, ...)                                                       \
  do {                                                                                          \
    if ((n) > 0) {                                                                              \
      kern<<<dim3(unsigned(grid_for(c, (n))), unsigned(ns)), 256, 0, c->stream>>>(__VA_ARGS__); \
      PM_CHECK_LAUNCH();                                                                        \
      c->kernel_launches++;                                                                     \
    }                                                                                           \
  } while (0)

void vcopy_batch(pm_ctx* c, int ns, const Batch& bt, int n, const double* x, double* y) {
  PM_LAUNCH_BATCH(kb_copy, ns, n, n, x, y, bt);
}
void vcvt_d2f_batch(pm_ctx* c, int ns, const Batch& bt, int n, const double* x, float* y) {
  PM_LAUNCH_BATCH(kb_d2f, ns, n, n, x, y, bt);
}
void vcvt_f2d_batch(pm_ctx* c, int ns, const Batch& bt, int n, const float* x, double* y) {
  PM_LAUNCH_BATCH(kb_f2d, ns, n, n, x, y, bt);
}
template <class T>
void init_solution_batch(pm_ctx* c, int ns, const Batch& bt, int n, const BlockMask& m, const T* rhs, T* sol) {
  PM_LAUNCH_BATCH(kb_init_sol<T>, ns, n, n, m, rhs, sol, bt);
}
template void init_solution_batch<float>(pm_ctx*, int, const Batch&, int, const BlockMask&, const float*, float*);
template void init_solution_batch<double>(pm_ctx*, int, const Batch&, int, const BlockMask&, const double*, double*);
template <class T>
void jacobi_from_zero_batch(pm_ctx* c, int ns, const Batch& bt, int n, const T* b, T w, T* x) {
  PM_LAUNCH_BATCH(kb_jacobi_zero<T>, ns, n, n, b, w, x, bt);
}
template void jacobi_from_zero_batch<float>(pm_ctx*, int, const Batch&, int, const float*, float, float*);
template void jacobi_from_zero_batch<double>(pm_ctx*, int, const Batch&, int, const double*, double, double*);

// the coarse-grid inverse of slot s is bt.aux[s]; act / pos are the same for
// every slot (one set-up)
__global__ void kb_coarse_gemv32(int n, int na, const int* __restrict__ act, const int* __restrict__ pos,
                                 const float* __restrict__ b, float* __restrict__ x, Batch bt) {
  const int s = blockIdx.y;
  if (!bt.on[s]) return;
  const float* inv = static_cast<const float*>(bt.aux[s]);
  b = slot_ptr(b, bt);
  x = slot_ptr(x, bt);
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp < na) {
    const float* row = inv + (size_t)warp * na;
    float sum = 0.0f;
    for (int j = lane; j < na; j += 32) sum += row[j] * b[act[j]];
    for (int off = 16; off > 0; off >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, off);
    if (lane == 0) x[act[warp]] = sum;
  } else {
    const int t = (warp - na) * 32 + lane;
    if (t < n && pos[t] < 0) x[t] = b[t];
  }
}
// the FP64 coarse solve of a right-hand side with zero non-actives (the
// gather form of k_coarse_gemv)
__global__ void kb_coarse_gemv(int n, int na, const int* __restrict__ act, const int* __restrict__ pos,
                               const double* __restrict__ b, double* __restrict__ x, Batch bt) {
  const int s = blockIdx.y;
  if (!bt.on[s]) return;
  const double* inv = static_cast<const double*>(bt.aux[s]);
  b = slot_ptr(b, bt);
  x = slot_ptr(x, bt);
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp < na) {
    const double* row = inv + (size_t)warp * na;
    double sum = 0.0;
    for (int j = lane; j < na; j += 32) sum += row[j] * b[act[j]];
    for (int off = 16; off > 0; off >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, off);
    if (lane == 0) x[act[warp]] = sum;
  } else {
    const int t = (warp - na) * 32 + lane;
    if (t < n && pos[t] < 0) x[t] = b[t];
  }
}

void coarse_solve32_batch(pm_ctx* c, int ns, const Batch& bt, const DenseInverse& inv0, const float* b, float* x) {
  const long long threads = (long long)(inv0.na + (inv0.n + 31) / 32) * 32;
  kb_coarse_gemv32<<<dim3(unsigned(nblocks(threads, 256)), unsigned(ns)), 256, 0, c->stream>>>(
      inv0.n, inv0.na, inv0.act.p, inv0.pos.p, b, x, bt);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

void coarse_solve_batch(pm_ctx* c, int ns, const Batch& bt, const DenseInverse& inv0, const double* b, double* x) {
  const long long threads = (long long)(inv0.na + (inv0.n + 31) / 32) * 32;
  kb_coarse_gemv<<<dim3(unsigned(nblocks(threads, 256)), unsigned(ns)), 256, 0, c->stream>>>(
      inv0.n, inv0.na, inv0.act.p, inv0.pos.p, b, x, bt);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

__global__ void __launch_bounds__(256) kb_dot_partials(int n, const double* __restrict__ x,
                                                       const double* __restrict__ y, double* __restrict__ part,
                                                       Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  x = slot_ptr(x, bt);
  y = slot_ptr(y, bt);
  part = slot_ptr(part, bt);
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s += x[i] * y[i];
  double r = block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = r;
}
__global__ void kb_finish_sum(const double* __restrict__ part, int np, double* out, int take_sqrt, Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  part = slot_ptr(part, bt);
  out = slot_ptr(out, bt);
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
  double r = block_sum(s, sh);
  if (threadIdx.x == 0) *out = take_sqrt ? sqrt(r) : r;
}
void dot_partials_batch(pm_ctx* c, int ns, const Batch& bt, int n, const double* x, const double* y, double* part) {
  kb_dot_partials<<<dim3(kRedBlocks, unsigned(ns)), kRedThreads, 0, c->stream>>>(n, x, y, part, bt);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}
void finish_sum_batch(pm_ctx* c, int ns, const Batch& bt, const double* part, double* out, bool take_sqrt) {
  kb_finish_sum<<<dim3(1, unsigned(ns)), 256, 0, c->stream>>>(part, kRedBlocks, out, take_sqrt ? 1 : 0, bt);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}
__global__ void kb_nonactive_nonzero(BlockMask m, const double* __restrict__ x, int* __restrict__ flag, Batch bt) {
  if (!bt.on[blockIdx.y]) return;
  x = slot_ptr(x, bt);
  flag = slot_ptr(flag, bt);
  for (int b = 0; b < m.nb; ++b)
    for (int i = m.active_end[b] + blockIdx.x * blockDim.x + threadIdx.x; i < m.end[b]; i += gridDim.x * blockDim.x)
      if (x[i] != 0.0) *flag = 1;
}
void nonactive_nonzero_batch(pm_ctx* c, int ns, const Batch& bt, const BlockMask& m, const double* x, int* flag) {
  kb_nonactive_nonzero<<<dim3(kRedBlocks, unsigned(ns)), 256, 0, c->stream>>>(m, x, flag, bt);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

}  // namespace pm
