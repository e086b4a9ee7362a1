// CSR sparse matrix-vector kernels with fused epilogues.
//
// One group of G lanes (G = 4..32, a power of two) walks one CSR row: each lane
// streams every G-th entry (values and column indices with evict-first loads so
// that the gathered vector x stays resident in L2), the group reduces with
// shuffles, and the group's first lane applies the epilogue. The epilogues give
// the operations the reference builds from TMatrix::multiply
// (src/Matrix/Matrix.C:430-451) and BlockFEMatrix::apply_scaled_add
// (src/Matrix/BlockFEMatrix.C:863-925):
//   AXPY    y_i += a * (A x)_i                      apply_scaled_add
//   SET     y_i  = (A x)_i                          apply
//   DEFECT  y_i  = b_i - (A x)_i                    MultigridLevel::calculate_defect
//   JACOBI  y_i  = x_i + w * ((b_i - (A x)_i)/d_i)  JacobiSmoother::smooth
//   RESTRICT y_i = active(i) ? (A x)_i : 0           DefectRestriction + ResetNonActive
//   PROLONG y_i += active(i) ? w * (A x)_i : 0       update_solution_in_finer_grid
// Non-active (Dirichlet) rows of FE matrices hold a single unit diagonal, so the
// uniform row sum reproduces BlockVector::addScaledNonActive exactly.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace pm {

enum Epi { EPI_AXPY = 0, EPI_SET = 1, EPI_DEFECT = 2, EPI_JACOBI = 3, EPI_RESTRICT = 4, EPI_PROLONG = 5 };

// Up to four contiguous blocks [start, end) of a block vector; rows in
// [active_end, end) of each block are non-active.
struct BlockMask {
  int nb;
  int start[4];
  int active_end[4];
  int end[4];
  // device flag: when set, the launch does nothing (the coarse-level smoothing
  // loop stops once its residual is small enough, without a host round trip)
  const int* guard = nullptr;
};

__device__ __forceinline__ bool guarded(const int* g) { return g != nullptr && *(volatile const int*)g != 0; }

__device__ __forceinline__ bool row_is_active(const BlockMask& m, int i) {
#pragma unroll
  for (int b = 0; b < 4; ++b)
    if (b < m.nb && i >= m.start[b] && i < m.end[b]) return i < m.active_end[b];
  return false;
}

template <class T>
__device__ __forceinline__ T ld_stream(const T* p) { return __ldcs(p); }

// Programmatic dependent launch: pdl_trigger lets the next kernel on the
// stream (if launched with programmatic stream serialization) start once all
// blocks of this one have started; pdl_wait blocks until the previous kernel
// has completed and its writes are visible (a no-op without the attribute).
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// the start of a kernel launched by launch_k that reads nothing before the
// previous kernel has completed
__device__ __forceinline__ void pdl_enter() {
  pdl_trigger();
  pdl_wait();
}

// G lanes per row, U entries per lane per chunk: a lane first issues its U
// value and U column loads, then its U gathers of x, then the U products, so
// that every lane keeps U independent DRAM requests in flight.
template <class TV, class TX, class TA, int G, int U, int EPI>
__device__ __forceinline__ void
csr_body(int n_rows, const int* __restrict__ row_ptr, const int* __restrict__ cols,
         const TV* __restrict__ vals, const TX* __restrict__ x, TX* __restrict__ y,
         const TX* __restrict__ b, const TX* __restrict__ diag, const TX* __restrict__ xold,
         TA alpha, const BlockMask& mask, int bx, int gx) {
  pdl_enter();
  if (guarded(mask.guard)) {  // uniform for the whole grid
    // a skipped Jacobi sweep leaves the iterate as it is (the caller swaps
    // the two iterate buffers after every sweep)
    if (EPI == EPI_JACOBI)
      for (int i = bx * blockDim.x + threadIdx.x; i < n_rows; i += gx * blockDim.x) y[i] = xold[i];
    return;
  }
  const int lane = threadIdx.x & (G - 1);
  const int row = (bx * blockDim.x + threadIdx.x) / G;
  const bool valid = row < n_rows;  // whole groups share a row: no early exit before the shuffles
  const int beg = valid ? __ldg(row_ptr + row) : 0;
  const int end = valid ? __ldg(row_ptr + row + 1) : 0;
  // the epilogue's per-row operands are loaded before the row walk, so their
  // latency overlaps with it instead of following the reduction
  TX pre_b = TX(0), pre_d = TX(1), pre_x = TX(0), pre_y = TX(0);
  if (valid && lane == 0) {
    if constexpr (EPI == EPI_AXPY || EPI == EPI_PROLONG) pre_y = y[row];
    if constexpr (EPI == EPI_DEFECT || EPI == EPI_JACOBI) pre_b = __ldg(b + row);
    if constexpr (EPI == EPI_JACOBI) {
      pre_d = __ldg(diag + row);
      pre_x = __ldg(xold + row);
    }
  }
  TA s = TA(0);
  for (int base = beg; base < end; base += G * U) {
    TV v[U];
    int c[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int k = base + u * G + lane;
      if (k < end) {
        v[u] = ld_stream(vals + k);
        c[u] = ld_stream(cols + k);
      } else {
        v[u] = TV(0);
        c[u] = 0;  // x[0] exists whenever the row has entries
      }
    }
    TX xv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) xv[u] = __ldg(x + c[u]);
#pragma unroll
    for (int u = 0; u < U; ++u) s += TA(v[u]) * TA(xv[u]);
  }
#pragma unroll
  for (int off = G / 2; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off, G);
  if (!valid) return;
  if (lane != 0) return;
  if constexpr (EPI == EPI_AXPY) {
    y[row] = TX(TA(pre_y) + alpha * s);
  } else if constexpr (EPI == EPI_SET) {
    y[row] = TX(s);
  } else if constexpr (EPI == EPI_DEFECT) {
    y[row] = TX(TA(pre_b) - s);
  } else if constexpr (EPI == EPI_JACOBI) {
    const TA d = (TA(pre_b) - s) / TA(pre_d);
    y[row] = TX(TA(pre_x) + alpha * d);
  } else if constexpr (EPI == EPI_RESTRICT) {
    y[row] = row_is_active(mask, row) ? TX(s) : TX(0);
  } else if constexpr (EPI == EPI_PROLONG) {
    if (row_is_active(mask, row)) y[row] = TX(TA(pre_y) + alpha * s);
  }
}

template <class TV, class TX, class TA, int G, int U, int EPI>
__global__ void __launch_bounds__(256)
csr_kernel(int n_rows, const int* __restrict__ row_ptr, const int* __restrict__ cols,
           const TV* __restrict__ vals, const TX* __restrict__ x, TX* __restrict__ y,
           const TX* __restrict__ b, const TX* __restrict__ diag, const TX* __restrict__ xold,
           TA alpha, BlockMask mask) {
  csr_body<TV, TX, TA, G, U, EPI>(n_rows, row_ptr, cols, vals, x, y, b, diag, xold, alpha, mask, blockIdx.x,
                                  gridDim.x);
}

// Row-block streaming variant. Block b owns the consecutive rows
// [rblock[b], rblock[b+1]) whose entries, at most NNZB, form one contiguous
// slice of the CSR arrays. Phase 1: the block streams that slice with
// warp-contiguous loads (every thread keeps NNZB/256 independent loads in
// flight), gathers x and stages (value, x) pairs in shared memory. Phase 2:
// four lanes per row accumulate the row's pairs with one fused multiply-add
// per entry and combine with two shuffle steps (a fixed order, so results are
// deterministic), then apply the epilogue. One FMA per entry matters on GB300,
// whose FP64 pipe is narrow enough for extra FP64 adds to become the limit.
template <class TV, class TX, class TA, int NNZB, int EPI>
__global__ void __launch_bounds__(256)
csr_stream_kernel(const int* __restrict__ rblock, const int* __restrict__ row_ptr,
                  const int* __restrict__ cols, const TV* __restrict__ vals, const TX* __restrict__ x,
                  TX* __restrict__ y, const TX* __restrict__ b, const TX* __restrict__ diag,
                  TA alpha, BlockMask mask) {
  constexpr int PER = NNZB / 256;
  __shared__ TV sv[NNZB];
  __shared__ TX sx[NNZB];
  if (guarded(mask.guard)) {  // uniform for the whole grid
    if (EPI == EPI_JACOBI) {
      const int g0 = __ldg(rblock + blockIdx.x), g1 = __ldg(rblock + blockIdx.x + 1);
      for (int i = g0 + int(threadIdx.x); i < g1; i += blockDim.x) y[i] = x[i];
    }
    return;
  }
  const int r0 = __ldg(rblock + blockIdx.x), r1 = __ldg(rblock + blockIdx.x + 1);
  const int s = __ldg(row_ptr + r0), e = __ldg(row_ptr + r1);
  const int t = threadIdx.x;
  TV v[PER];
  int c[PER];
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int k = s + u * 256 + t;
    if (k < e) {
      v[u] = ld_stream(vals + k);
      c[u] = ld_stream(cols + k);
    } else {
      v[u] = TV(0);
      c[u] = -1;
    }
  }
  TX xv[PER];
#pragma unroll
  for (int u = 0; u < PER; ++u) xv[u] = c[u] >= 0 ? __ldg(x + c[u]) : TX(0);
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    sv[u * 256 + t] = v[u];
    sx[u * 256 + t] = xv[u];
  }
  __syncthreads();
  const int slot = t >> 2, lane = t & 3;
  // every thread runs the same number of row rounds so the shuffles see full warps
  for (int base = r0; base < r1; base += 64) {
    const int row = base + slot;
    const bool has_row = row < r1;
    const int a = has_row ? __ldg(row_ptr + row) - s : 0;
    const int z = has_row ? __ldg(row_ptr + row + 1) - s : 0;
    TA sum = TA(0);
    for (int k = a + lane; k < z; k += 4) sum = fma(TA(sv[k]), TA(sx[k]), sum);
    sum += __shfl_down_sync(0xffffffffu, sum, 2, 4);
    sum += __shfl_down_sync(0xffffffffu, sum, 1, 4);
    if (has_row && lane == 0) {
      if constexpr (EPI == EPI_AXPY) {
        y[row] = TX(TA(y[row]) + alpha * sum);
      } else if constexpr (EPI == EPI_SET) {
        y[row] = TX(sum);
      } else if constexpr (EPI == EPI_DEFECT) {
        y[row] = TX(TA(b[row]) - sum);
      } else if constexpr (EPI == EPI_JACOBI) {
        const TA d = (TA(b[row]) - sum) / TA(diag[row]);
        y[row] = TX(TA(x[row]) + alpha * d);
      } else if constexpr (EPI == EPI_RESTRICT) {
        y[row] = row_is_active(mask, row) ? TX(sum) : TX(0);
      } else if constexpr (EPI == EPI_PROLONG) {
        if (row_is_active(mask, row)) y[row] = TX(TA(y[row]) + alpha * sum);
      }
    }
  }
}


// Sliced-ELL copy of an FP32 matrix (SELL-C-sigma, C = 32/L rows per slice).
// Rows are sorted by length, longest first (ties in row order), inside windows
// of kSellWindow consecutive rows; slice s holds C consecutive sorted rows,
// padded to the slice's longest row and stored step-major: step t of the
// slice is 32 consecutive entries at soff[s] + 32 t, lane sub*C + p holding
// entry t*L + sub of the slice's p-th row. One warp walks one slice, so every
// value and index load of a warp is one aligned 128-byte line, and with L = 1
// a thread owns a whole row (no shuffles). Padding entries hold value 0 and a
// column index of their own row. Each lane sums its entries in row order; the
// L partial sums of a row combine in a fixed order, so results are
// deterministic (but rounded differently from csr_kernel's row groups).
// PIPE issues the value and index loads of the next U steps before the
// gathers of the current ones. Launched with programmatic stream
// serialization, a sweep loads its permutation, slice offsets and (PIPE) first
// U steps while the previous kernel finishes.
constexpr int kSellWindow = 1024;

template <class T>
__device__ __forceinline__ T fmadd(T a, T b, T c);
template <>
__device__ __forceinline__ float fmadd<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <>
__device__ __forceinline__ double fmadd<double>(double a, double b, double c) { return __fma_rn(a, b, c); }

template <class T, int L, int U, bool PIPE, int EPI>
__device__ __forceinline__ void
sell_body(int n_slices, const int* __restrict__ perm, const int* __restrict__ soff,
          const int* __restrict__ scols, const T* __restrict__ svals, const T* __restrict__ x,
          T* __restrict__ y, const T* __restrict__ b, const T* __restrict__ diag, T alpha,
          const BlockMask& mask, int bx) {
  constexpr int C = 32 / L;
  pdl_trigger();
  const int s = bx * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (s >= n_slices) return;  // whole warps leave: the shuffles below stay full-warp
  const int lane = threadIdx.x & 31;
  const int p = lane % C, sub = lane / C;
  // the matrix arrays are not written by the kernels that precede a sweep:
  // their loads start before the wait for the previous kernel
  const int row = __ldg(perm + s * C + p);  // -1: padding row of the last window
  const int beg = __ldg(soff + s);
  const int NT = (__ldg(soff + s + 1) - beg) >> 5;
  const T* vp = svals + beg + lane;
  const int* cp = scols + beg + lane;
  T v[U];
  int c[U];
  if constexpr (PIPE) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const bool in = u < NT;
      v[u] = in ? ld_stream(vp + u * 32) : T(0);
      c[u] = in ? ld_stream(cp + u * 32) : 0;
    }
  }
  pdl_wait();  // x, b, y and the guard flag come from earlier kernels
  if (guarded(mask.guard)) {  // uniform for the whole grid
    if (EPI == EPI_JACOBI && row >= 0 && sub == 0) y[row] = x[row];
    return;
  }
  T pre_b = T(0), pre_d = T(1), pre_x = T(0), pre_y = T(0);
  if (row >= 0 && sub == 0) {
    if constexpr (EPI == EPI_AXPY || EPI == EPI_PROLONG) pre_y = y[row];
    if constexpr (EPI == EPI_DEFECT || EPI == EPI_JACOBI) pre_b = __ldg(b + row);
    if constexpr (EPI == EPI_JACOBI) {
      pre_d = __ldg(diag + row);
      pre_x = __ldg(x + row);
    }
  }
  T acc = T(0);
  if constexpr (!PIPE) {
    for (int t0 = 0; t0 < NT; t0 += U) {
      T xv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const bool in = t0 + u < NT;
        v[u] = in ? ld_stream(vp + (t0 + u) * 32) : T(0);
        c[u] = in ? ld_stream(cp + (t0 + u) * 32) : 0;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) xv[u] = __ldg(x + c[u]);
#pragma unroll
      for (int u = 0; u < U; ++u) acc = fmadd(v[u], xv[u], acc);
    }
  } else {
    for (int t0 = 0; t0 < NT; t0 += U) {
      T vn[U], xv[U];
      int cn[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const bool in = t0 + U + u < NT;
        vn[u] = in ? ld_stream(vp + (t0 + U + u) * 32) : T(0);
        cn[u] = in ? ld_stream(cp + (t0 + U + u) * 32) : 0;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) xv[u] = __ldg(x + c[u]);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        acc = fmadd(v[u], xv[u], acc);
        v[u] = vn[u];
        c[u] = cn[u];
      }
    }
  }
#pragma unroll
  for (int off = 16; off >= C; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if (row < 0 || sub != 0) return;
  if constexpr (EPI == EPI_AXPY) {
    y[row] = pre_y + alpha * acc;
  } else if constexpr (EPI == EPI_SET) {
    y[row] = acc;
  } else if constexpr (EPI == EPI_DEFECT) {
    y[row] = pre_b - acc;
  } else if constexpr (EPI == EPI_JACOBI) {
    const T d = (pre_b - acc) / pre_d;
    y[row] = pre_x + alpha * d;
  } else if constexpr (EPI == EPI_RESTRICT) {
    y[row] = row_is_active(mask, row) ? acc : T(0);
  } else if constexpr (EPI == EPI_PROLONG) {
    if (row_is_active(mask, row)) y[row] = pre_y + alpha * acc;
  }
}

template <class T, int L, int U, bool PIPE, int EPI>
__global__ void __launch_bounds__(128)
sell_kernel(int n_slices, const int* __restrict__ perm, const int* __restrict__ soff,
            const int* __restrict__ scols, const T* __restrict__ svals, const T* __restrict__ x,
            T* __restrict__ y, const T* __restrict__ b, const T* __restrict__ diag, T alpha,
            BlockMask mask) {
  sell_body<T, L, U, PIPE, EPI>(n_slices, perm, soff, scols, svals, x, y, b, diag, alpha, mask, blockIdx.x);
}

}  // namespace pm
