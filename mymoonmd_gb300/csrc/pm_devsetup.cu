// Device-side construction of a scalar level's CSR structure and assembly
// gather plans (the set-up that TStructure(space) and the element loop's
// scatter imply, src/Matrix/Structure.C:829-1283, Structure.C:2681 Sort(),
// src/AssembleRoutines/Assemble3D.C:346-370), from the level's GlobalNumbers.
//
// One stable radix sort does both. Every element-matrix entry e of an active
// row (e = (cell * nloc + m) * nloc + k, increasing in cell order) becomes the
// pair (key = row * n + column, value = e); every non-active row adds its
// diagonal (value -1). After a stable sort by key:
//   * the first item of each key run is one CSR entry: the columns of a row
//     come out ascending (the reference's sorted structure), a row's entries
//     are the union of its cells' DOFs;
//   * the items of a run, in order, are the element entries that add to that
//     CSR entry in cell order - the gather plan of the assembly;
//   * the -1 items are the unit diagonals of the non-active rows.
// The right-hand side plan is the same with keys = row and values = the
// positions cell * nloc + m. The results equal the host construction
// (pm_disc.cpp) entry for entry.
#include <cub/cub.cuh>

#include "pm_devsetup.h"

namespace pm {

namespace {

// element-entry pairs, then one pair per non-active row
__global__ void k_entry_pairs(int n_cells, int nloc, int n, int n_active, const int* __restrict__ dm,
                              unsigned long long* __restrict__ key, int* __restrict__ val) {
  const long long ne = (long long)n_cells * nloc * nloc;
  const long long total = ne + (n - n_active);
  const unsigned long long invalid = (unsigned long long)n * n;  // past every valid key
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    if (e < ne) {
      const long long cm = e / nloc;
      const int k = int(e % nloc);
      const long long c = cm / nloc;
      const int row = dm[cm];
      if (row < n_active) {
        key[e] = (unsigned long long)row * n + (unsigned long long)dm[c * nloc + k];
        val[e] = int(e);
      } else {
        key[e] = invalid;
        val[e] = -1;
      }
    } else {
      const int i = n_active + int(e - ne);
      key[e] = (unsigned long long)i * n + i;
      val[e] = -1;
    }
  }
}

// run heads (first item of each valid key) and contributing items (value >= 0)
__global__ void k_heads(long long total, int n, const unsigned long long* __restrict__ key,
                        const int* __restrict__ val, int* __restrict__ head, int* __restrict__ contrib) {
  const unsigned long long invalid = (unsigned long long)n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const bool valid = key[i] < invalid;
    head[i] = valid && (i == 0 || key[i] != key[i - 1]) ? 1 : 0;
    contrib[i] = valid && val[i] >= 0 ? 1 : 0;
  }
}

// CSR columns, row starts, gather plan and the non-active diagonals
__global__ void k_fill_structure(long long total, int n, int n_active, const unsigned long long* __restrict__ key,
                                 const int* __restrict__ val, const int* __restrict__ head,
                                 const int* __restrict__ hpos, const int* __restrict__ cpos,
                                 int* __restrict__ row_ptr, int* __restrict__ cols, int* __restrict__ gat_ptr,
                                 int* __restrict__ gat_idx, int* __restrict__ diag_pos) {
  const unsigned long long invalid = (unsigned long long)n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long k = key[i];
    if (k >= invalid) continue;
    const int row = int(k / n);
    if (head[i]) {
      const int p = hpos[i];
      cols[p] = int(k % n);
      gat_ptr[p] = cpos[i];
      if (i == 0 || int(key[i - 1] / n) != row) row_ptr[row] = p;
      if (val[i] < 0) diag_pos[row - n_active] = p;
    }
    if (val[i] >= 0) gat_idx[cpos[i]] = val[i];
  }
}

__global__ void k_dof_pairs(long long total, int n, int n_active, const int* __restrict__ dm,
                            unsigned int* __restrict__ key, int* __restrict__ val) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int d = dm[t];
    key[t] = d < n_active ? unsigned(d) : unsigned(n);
    val[t] = int(t);
  }
}

// right-hand side plan: rgat_ptr[d] = first item of active DOF d
__global__ void k_fill_rhs(long long total, int n, const unsigned int* __restrict__ key, const int* __restrict__ val,
                           int* __restrict__ rgat_ptr, int* __restrict__ rgat_idx) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned k = key[i];
    if (k >= unsigned(n)) continue;
    if (i == 0 || key[i - 1] != k) rgat_ptr[k] = int(i);
    rgat_idx[i] = val[i];
  }
}

__global__ void k_set_tail(int* __restrict__ p, int from, int to, int value) {
  for (int i = from + blockIdx.x * blockDim.x + threadIdx.x; i < to; i += gridDim.x * blockDim.x) p[i] = value;
}

int bits_for(unsigned long long v) {
  int b = 0;
  while (b < 64 && (v >> b) != 0) ++b;
  return b;
}

template <class T>
void download(pm_ctx* c, std::vector<int>& out, const T& buf, size_t count) {
  out.resize(count);
  if (count) PM_CUDA(cudaMemcpyAsync(out.data(), buf.p, count * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
}

}  // namespace

void device_level_structure(pm_ctx* c, DiscLevel& L) {
  const pmsetup::Space& s = L.space;
  const int n = s.n_dofs, na = s.n_active, nloc = s.nloc, nc = L.n_cells;
  const long long ne = (long long)nc * nloc * nloc, total = ne + (n - na);
  const long long nt = (long long)nc * nloc;
  if (total >= (1LL << 31) || (unsigned long long)n * n >= (1ULL << 63))
    throw Error(PM_E_INVALID, "level too large for the device structure build");
  const int grid = std::max(1, std::min(int((total + 255) / 256), c->num_sms * 8));
  cudaStream_t st = c->stream;
  DBuf<int> dm;
  dm.upload(s.dofmap, st);
  // --- system structure and the matrix gather plan
  DBuf<unsigned long long> key_in(static_cast<size_t>(total)), key_out(static_cast<size_t>(total));
  DBuf<int> val_in(static_cast<size_t>(total)), val_out(static_cast<size_t>(total));
  k_entry_pairs<<<grid, 256, 0, st>>>(nc, nloc, n, na, dm.p, key_in.p, val_in.p);
  PM_CHECK_LAUNCH();
  const int end_bit = bits_for((unsigned long long)n * n);
  size_t tmp_bytes = 0;
  PM_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, key_in.p, key_out.p, val_in.p, val_out.p,
                                          int(total), 0, end_bit, st));
  size_t scan_bytes = 0;
  PM_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, val_in.p, val_out.p, int(total), st));
  DBuf<unsigned char> tmp(std::max(tmp_bytes, scan_bytes));
  PM_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, key_in.p, key_out.p, val_in.p, val_out.p,
                                          int(total), 0, end_bit, st));
  key_in.release();
  // heads and contributions, and their exclusive sums
  const size_t tn = static_cast<size_t>(total);
  DBuf<int> head(tn), contrib(tn), hpos(tn), cpos(tn);
  k_heads<<<grid, 256, 0, st>>>(total, n, key_out.p, val_out.p, head.p, contrib.p);
  PM_CHECK_LAUNCH();
  size_t sb = tmp.n;
  PM_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, sb, head.p, hpos.p, int(total), st));
  sb = tmp.n;
  PM_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, sb, contrib.p, cpos.p, int(total), st));
  int last[4] = {0, 0, 0, 0};  // hpos, head, cpos, contrib of the last item
  PM_CUDA(cudaMemcpyAsync(&last[0], hpos.p + total - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  PM_CUDA(cudaMemcpyAsync(&last[1], head.p + total - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  PM_CUDA(cudaMemcpyAsync(&last[2], cpos.p + total - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  PM_CUDA(cudaMemcpyAsync(&last[3], contrib.p + total - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  PM_CUDA(cudaStreamSynchronize(st));
  const int nnz = last[0] + last[1], ncontrib = last[2] + last[3];
  DBuf<int> row_ptr(static_cast<size_t>(n) + 1), cols(static_cast<size_t>(nnz));
  DBuf<int> gat_ptr(static_cast<size_t>(nnz) + 1), gat_idx(static_cast<size_t>(ncontrib));
  DBuf<int> diag_pos(static_cast<size_t>(std::max(1, n - na)));
  k_fill_structure<<<grid, 256, 0, st>>>(total, n, na, key_out.p, val_out.p, head.p, hpos.p, cpos.p, row_ptr.p,
                                         cols.p, gat_ptr.p, gat_idx.p, diag_pos.p);
  PM_CHECK_LAUNCH();
  k_set_tail<<<1, 32, 0, st>>>(row_ptr.p, n, n + 1, nnz);
  k_set_tail<<<1, 32, 0, st>>>(gat_ptr.p, nnz, nnz + 1, ncontrib);
  PM_CHECK_LAUNCH();
  c->kernel_launches += 5;
  // --- right-hand side plan
  DBuf<unsigned int> rkey_in(static_cast<size_t>(nt)), rkey_out(static_cast<size_t>(nt));
  DBuf<int> rval_in(static_cast<size_t>(nt)), rval_out(static_cast<size_t>(nt));
  DBuf<int> rgat_ptr(static_cast<size_t>(n) + 1);
  k_dof_pairs<<<grid, 256, 0, st>>>(nt, n, na, dm.p, rkey_in.p, rval_in.p);
  PM_CHECK_LAUNCH();
  size_t rb = 0;
  const int rend = bits_for((unsigned long long)n);
  PM_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, rb, rkey_in.p, rkey_out.p, rval_in.p, rval_out.p, int(nt), 0,
                                          rend, st));
  if (rb > tmp.n) tmp.alloc(rb);
  rb = tmp.n;
  PM_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, rb, rkey_in.p, rkey_out.p, rval_in.p, rval_out.p, int(nt), 0,
                                          rend, st));
  // the active DOFs' items come first (keys below n), in DOF order and, for
  // one DOF, in the order of t; every active DOF has at least one item
  DBuf<int> rgat_idx(static_cast<size_t>(nt));
  k_fill_rhs<<<grid, 256, 0, st>>>(nt, n, rkey_out.p, rval_out.p, rgat_ptr.p, rgat_idx.p);
  PM_CHECK_LAUNCH();
  c->kernel_launches += 2;
  // --- results into the host level (the host containers the rest of the
  // set-up reads)
  L.sys = pmsetup::Csr();
  L.sys.n_rows = n;
  L.sys.n_cols = n;
  L.sys.n_active = na;
  download(c, L.sys.row_ptr, row_ptr, size_t(n) + 1);
  download(c, L.sys.cols, cols, size_t(nnz));
  download(c, L.gat_ptr, gat_ptr, size_t(nnz) + 1);
  download(c, L.gat_idx, gat_idx, size_t(ncontrib));
  download(c, L.diag_pos, diag_pos, size_t(n - na));
  // the items of non-active DOFs sort last: the valid count is the number of
  // positions t whose DOF is active
  long long valid = 0;
  for (int d : s.dofmap) valid += d < na ? 1 : 0;
  std::vector<int> rp, ri;
  download(c, rp, rgat_ptr, size_t(n) + 1);
  download(c, ri, rgat_idx, size_t(valid));
  PM_CUDA(cudaStreamSynchronize(st));
  for (int i = na; i <= n; ++i) rp[size_t(i)] = int(valid);
  L.rgat_ptr = std::move(rp);
  L.rgat_idx = std::move(ri);
}

}  // namespace pm
