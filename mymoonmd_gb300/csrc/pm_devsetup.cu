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
//
// The mesh hierarchy and the DOF numbering come from the GPU as well: regular
// refinement one thread per child cell with the refinement tables of the host
// set-up (pm_refine_tables.h), and the first-touch numbering (inner DOFs,
// then Neumann, then Dirichlet, each in order of first touch over the cells
// in collection order and their local DOFs in local order,
// TFESpace{2,3}D::ConstructSpace) by two stable radix sorts: the local DOF
// positions t = cell * nloc + m by the lattice key of their node (the first
// item of each key run is the node's first touch), then the distinct nodes by
// (class, first touch), whose order is the numbering.
#include <cub/cub.cuh>

#include "pm_devsetup.h"
#include "pm_refine_tables.h"

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

// ------------------------------------------------------------ refinement --
struct RefineTables {
  int quad_child[4][4], quad_new[5][4];
  int hex_child[8][8], hex_new[19][8];
  int tet_child[8][4], tet_new[6][2];
};

RefineTables refine_tables() {
  RefineTables t{};
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) t.quad_child[a][b] = pmsetup::kQuadChild[a][b];
  for (int a = 0; a < 5; ++a)
    for (int b = 0; b < 4; ++b) t.quad_new[a][b] = pmsetup::kQuadNew[a][b];
  for (int a = 0; a < 8; ++a)
    for (int b = 0; b < 8; ++b) t.hex_child[a][b] = pmsetup::kHexChild[a][b];
  for (int a = 0; a < 19; ++a)
    for (int b = 0; b < 8; ++b) t.hex_new[a][b] = pmsetup::kHexNew[a][b];
  for (int a = 0; a < 8; ++a)
    for (int b = 0; b < 4; ++b) t.tet_child[a][b] = pmsetup::kTetChild[a][b];
  for (int a = 0; a < 6; ++a)
    for (int b = 0; b < 2; ++b) t.tet_new[a][b] = pmsetup::kTetNew[a][b];
  return t;
}

// one thread per child cell: its vertices from the parent's (a parent vertex,
// or the mean of the parent vertices a new vertex averages), in the child's
// vertex order; children of a cell are consecutive (cell order, child order)
__global__ void k_refine(int geometry, int n_coarse, int nvc, int dim, const long long* __restrict__ cv,
                         long long* __restrict__ fv, int* __restrict__ parent, int* __restrict__ child_no,
                         RefineTables T) {
  const int nchild = dim == 2 ? 4 : 8;
  const long long total = (long long)n_coarse * nchild;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int c = int(t / nchild), ch = int(t % nchild);
    const long long* pv = cv + (long long)c * nvc * dim;
    long long* out = fv + t * nvc * dim;
    for (int v = 0; v < nvc; ++v) {
      const int idx = geometry == pmsetup::GEO_SQUARE_QUAD ? T.quad_child[ch][v]
                      : geometry == pmsetup::GEO_CUBE_HEXA ? T.hex_child[ch][v]
                                                           : T.tet_child[ch][v];
      for (int d = 0; d < dim; ++d) {
        long long val;
        if (idx < nvc) {
          val = pv[idx * dim + d];
        } else {
          const int n = idx - nvc;
          if (geometry == pmsetup::GEO_SQUARE_QUAD) {
            long long sum = 0;
            int cnt = 0;
            for (int q = 0; q < 4 && T.quad_new[n][q] >= 0; ++q, ++cnt) sum += pv[T.quad_new[n][q] * 2 + d];
            val = sum / cnt;
          } else if (geometry == pmsetup::GEO_CUBE_HEXA) {
            long long sum = 0;
            int cnt = 0;
            for (; cnt < 8 && T.hex_new[n][cnt] >= 0; ++cnt) sum += pv[T.hex_new[n][cnt] * 3 + d];
            val = sum / cnt;
          } else {
            val = (pv[T.tet_new[n][0] * 3 + d] + pv[T.tet_new[n][1] * 3 + d]) / 2;
          }
        }
        out[v * dim + d] = val;
      }
    }
    parent[t] = c;
    child_no[t] = ch;
  }
}

// ------------------------------------------------------------- numbering --
// lattice coordinates of local DOF m of a cell (cell_nodes of the host set-up)
__device__ void node_of(int geometry, int elem, const long long* v, int m, long long* x) {
  if (geometry == pmsetup::GEO_SQUARE_QUAD) {
    const int k = elem == pmsetup::EL_Q2 ? 2 : 1;
    const int a = m % (k + 1), b = m / (k + 1);
    for (int d = 0; d < 2; ++d) x[d] = v[d] + (v[2 + d] - v[d]) * a / k + (v[6 + d] - v[d]) * b / k;
  } else if (geometry == pmsetup::GEO_CUBE_HEXA) {
    const int k = elem == pmsetup::EL_Q2 ? 2 : 1;
    const int a = m % (k + 1), b = (m / (k + 1)) % (k + 1), cc = m / ((k + 1) * (k + 1));
    for (int d = 0; d < 3; ++d)
      x[d] = v[d] + (v[3 + d] - v[d]) * a / k + (v[9 + d] - v[d]) * b / k + (v[12 + d] - v[d]) * cc / k;
  } else if (elem == pmsetup::EL_P1) {
    for (int d = 0; d < 3; ++d) x[d] = v[m * 3 + d];
  } else {
    // v0, m01, v1, m02, m12, v2, m03, m13, m23, v3
    const int pa[10] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3}, pb[10] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3};
    for (int d = 0; d < 3; ++d) x[d] = (v[pa[m] * 3 + d] + v[pb[m] * 3 + d]) / 2;
  }
}

// class of a node: 0 inner, 1 Neumann (every side it lies on is a Neumann
// side, 2D), 2 other boundary
__device__ int node_class(int dim, long long S, int neumann_sides, const long long* x) {
  bool on_bnd = false;
  for (int d = 0; d < dim; ++d) on_bnd |= (x[d] == 0 || x[d] == S);
  if (!on_bnd) return 0;
  if (neumann_sides) {
    int sides = 0;
    if (x[1] == 0) sides |= pmsetup::SIDE_Y0;
    if (x[0] == S) sides |= pmsetup::SIDE_X1;
    if (x[1] == S) sides |= pmsetup::SIDE_Y1;
    if (x[0] == 0) sides |= pmsetup::SIDE_X0;
    if ((sides & neumann_sides) == sides) return 1;
  }
  return 2;
}

__global__ void k_node_keys(int geometry, int elem, int nvc, int dim, int nloc, long long nt, long long W,
                            const long long* __restrict__ vtx, unsigned long long* __restrict__ key,
                            int* __restrict__ val) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nt;
       t += (long long)gridDim.x * blockDim.x) {
    const long long c = t / nloc;
    const int m = int(t % nloc);
    long long x[3] = {0, 0, 0};
    node_of(geometry, elem, vtx + c * nvc * dim, m, x);
    key[t] = (unsigned long long)(x[0] + W * (x[1] + (dim == 3 ? W * x[2] : 0)));
    val[t] = int(t);
  }
}

__global__ void k_key_heads(long long nt, const unsigned long long* __restrict__ key, int* __restrict__ head) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nt;
       i += (long long)gridDim.x * blockDim.x)
    head[i] = (i == 0 || key[i] != key[i - 1]) ? 1 : 0;
}

// per distinct node g (run head i, gid[i] = g + 1): (class, first touch)
__global__ void k_distinct(long long nt, int dim, long long W, long long S, int neumann_sides,
                           const unsigned long long* __restrict__ key, const int* __restrict__ val,
                           const int* __restrict__ head, const int* __restrict__ gid,
                           unsigned long long* __restrict__ ukey, unsigned long long* __restrict__ order_key,
                           int* __restrict__ order_val) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nt;
       i += (long long)gridDim.x * blockDim.x) {
    if (!head[i]) continue;
    const int g = gid[i] - 1;
    const unsigned long long k = key[i];
    long long x[3];
    x[0] = (long long)(k % (unsigned long long)W);
    x[1] = (long long)((k / (unsigned long long)W) % (unsigned long long)W);
    x[2] = dim == 3 ? (long long)(k / ((unsigned long long)W * W)) : 0;
    ukey[g] = k;
    order_key[g] = ((unsigned long long)node_class(dim, S, neumann_sides, x) << 32) | (unsigned)val[i];
    order_val[g] = g;
  }
}

// number[g] = position of node g in (class, first touch) order; its
// coordinates at that position; the first position of each class
__global__ void k_number(int U, int dim, long long W, const unsigned long long* __restrict__ order_key,
                         const int* __restrict__ order_g, const unsigned long long* __restrict__ ukey,
                         int* __restrict__ number, long long* __restrict__ node, int* __restrict__ class_first) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < U; p += gridDim.x * blockDim.x) {
    const int g = order_g[p];
    number[g] = p;
    const unsigned long long k = ukey[g];
    node[(long long)p * dim + 0] = (long long)(k % (unsigned long long)W);
    node[(long long)p * dim + 1] = (long long)((k / (unsigned long long)W) % (unsigned long long)W);
    if (dim == 3) node[(long long)p * dim + 2] = (long long)(k / ((unsigned long long)W * W));
    const int cls = int(order_key[p] >> 32);
    if (p == 0 || int(order_key[p - 1] >> 32) != cls) class_first[cls] = p;
  }
}

__global__ void k_dofmap(long long nt, const int* __restrict__ val, const int* __restrict__ gid,
                         const int* __restrict__ number, int* __restrict__ dofmap) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nt;
       i += (long long)gridDim.x * blockDim.x)
    dofmap[val[i]] = number[gid[i] - 1];
}

// ------------------------------------------------------- Stokes structure --
// the local coupling of the Stokes element (pm_disc.cpp stokes_local()) on
// the device: item j of a cell is the pair (lm[j], lk[j]) with storage lpos[j]
struct StokesItems {
  short lm[540], lk[540], lpos[540];
  int n;
};

// items t = c * n + j: key row * N + column for active rows (invalid key
// otherwise), value = element storage position c * 220 + lpos; then one
// unit-diagonal item per non-active row (value -1)
__global__ void k_stokes_pairs(int n_cells, int N, int n_inactive, const int* __restrict__ cdof,
                               const unsigned char* __restrict__ act, const int* __restrict__ inactive_rows,
                               StokesItems S, unsigned long long* __restrict__ key, int* __restrict__ val) {
  const long long ne = (long long)n_cells * S.n;
  const long long total = ne + n_inactive;
  const unsigned long long invalid = (unsigned long long)N * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    if (e < ne) {
      const long long c = e / S.n;
      const int j = int(e % S.n);
      const int row = cdof[c * 34 + S.lm[j]];
      if (act[row]) {
        key[e] = (unsigned long long)row * N + (unsigned long long)cdof[c * 34 + S.lk[j]];
        val[e] = int(c * 220 + S.lpos[j]);
      } else {
        key[e] = invalid;
        val[e] = -1;
      }
    } else {
      const int i = inactive_rows[e - ne];
      key[e] = (unsigned long long)i * N + i;
      val[e] = -1;
    }
  }
}

// as k_fill_structure, with the non-active rows' diagonal positions indexed
// by their rank among the non-active rows
__global__ void k_fill_structure_ranked(long long total, int n, const unsigned long long* __restrict__ key,
                                        const int* __restrict__ val, const int* __restrict__ head,
                                        const int* __restrict__ hpos, const int* __restrict__ cpos,
                                        const int* __restrict__ inactive_rank, int* __restrict__ row_ptr,
                                        int* __restrict__ cols, int* __restrict__ gat_ptr, int* __restrict__ gat_idx,
                                        int* __restrict__ diag_pos) {
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
      if (val[i] < 0) diag_pos[inactive_rank[row]] = p;
    }
    if (val[i] >= 0) gat_idx[cpos[i]] = val[i];
  }
}

// right-hand side items t = c * 34 + m: key = row for active rows, N otherwise
__global__ void k_stokes_rhs_pairs(long long nt, int N, const int* __restrict__ cdof,
                                   const unsigned char* __restrict__ act, unsigned int* __restrict__ key,
                                   int* __restrict__ val) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nt;
       t += (long long)gridDim.x * blockDim.x) {
    const int d = cdof[t];
    key[t] = act[d] ? unsigned(d) : unsigned(N);
    val[t] = int(t);
  }
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

pmsetup::Hierarchy device_hierarchy(pm_ctx* c, int geometry, int root_n, int n_refine) {
  pmsetup::Hierarchy h = pmsetup::root_hierarchy(geometry, root_n, n_refine);
  const int dim = h.dim, nvc = h.nvc, nchild = dim == 2 ? 4 : 8;
  cudaStream_t st = c->stream;
  const RefineTables T = refine_tables();
  static_assert(sizeof(long long) == sizeof(int64_t), "lattice coordinates are 64-bit");
  DBuf<long long> cur;
  cur.upload(reinterpret_cast<const long long*>(h.levels[0].vtx.data()), h.levels[0].vtx.size(), st);
  for (int r = 0; r < n_refine; ++r) {
    const int nc = h.levels.back().n_cells;
    if ((long long)nc * nchild >= (1LL << 31)) throw Error(PM_E_INVALID, "mesh too large for the device refinement");
    pmsetup::Level fine;
    fine.n_cells = nc * nchild;
    const size_t nv = size_t(fine.n_cells) * nvc * dim;
    DBuf<long long> fv(nv);
    DBuf<int> parent(size_t(fine.n_cells)), child(size_t(fine.n_cells));
    const int grid = std::max(1, std::min((fine.n_cells + 255) / 256, c->num_sms * 8));
    k_refine<<<grid, 256, 0, st>>>(geometry, nc, nvc, dim, cur.p, fv.p, parent.p, child.p, T);
    PM_CHECK_LAUNCH();
    c->kernel_launches++;
    fine.vtx.resize(nv);
    fine.parent.resize(size_t(fine.n_cells));
    fine.child_no.resize(size_t(fine.n_cells));
    PM_CUDA(cudaMemcpyAsync(fine.vtx.data(), fv.p, nv * sizeof(long long), cudaMemcpyDeviceToHost, st));
    PM_CUDA(cudaMemcpyAsync(fine.parent.data(), parent.p, fine.parent.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
    PM_CUDA(cudaMemcpyAsync(fine.child_no.data(), child.p, fine.child_no.size() * sizeof(int), cudaMemcpyDeviceToHost,
                            st));
    PM_CUDA(cudaStreamSynchronize(st));
    h.levels.push_back(std::move(fine));
    cur = std::move(fv);
  }
  return h;
}

pmsetup::Space device_space(pm_ctx* c, const pmsetup::Hierarchy& h, int level, int elem, int boundary,
                            int neumann_sides) {
  const pmsetup::Level& L = h.levels.at(size_t(level));
  const int dim = h.dim, nvc = h.nvc;
  if (neumann_sides && (dim != 2 || boundary != pmsetup::BND_DIRICHLET))
    throw Error(PM_E_INVALID, "Neumann sides are supported on the unit square with Dirichlet elsewhere");
  pmsetup::Space s;
  s.elem = elem;
  s.boundary = boundary;
  s.neumann_sides = neumann_sides;
  s.nloc = pmsetup::space_nloc(h.geometry, elem);
  const long long S = h.scale, W = S + 1;
  const long long nt = (long long)L.n_cells * s.nloc;
  if (nt >= (1LL << 31)) throw Error(PM_E_INVALID, "level too large for the device numbering");
  cudaStream_t st = c->stream;
  const int grid = std::max(1, std::min(int((nt + 255) / 256), c->num_sms * 8));
  DBuf<long long> vtx;
  vtx.upload(reinterpret_cast<const long long*>(L.vtx.data()), L.vtx.size(), st);
  // local DOF positions sorted by the lattice key of their node (stable: a
  // run's first item is the node's first touch)
  DBuf<unsigned long long> key_in(static_cast<size_t>(nt)), key_out(static_cast<size_t>(nt));
  DBuf<int> val_in(static_cast<size_t>(nt)), val_out(static_cast<size_t>(nt));
  k_node_keys<<<grid, 256, 0, st>>>(h.geometry, elem, nvc, dim, s.nloc, nt, W, vtx.p, key_in.p, val_in.p);
  PM_CHECK_LAUNCH();
  const unsigned long long kmax = (unsigned long long)W * W * (dim == 3 ? (unsigned long long)W : 1ULL);
  const int end_bit = bits_for(kmax);
  size_t tb = 0, sb = 0;
  PM_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, key_in.p, key_out.p, val_in.p, val_out.p, int(nt), 0, end_bit,
                                          st));
  DBuf<int> head(static_cast<size_t>(nt)), gid(static_cast<size_t>(nt));
  PM_CUDA(cub::DeviceScan::InclusiveSum(nullptr, sb, head.p, gid.p, int(nt), st));
  DBuf<unsigned char> tmp(std::max(tb, sb));
  tb = tmp.n;
  PM_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tb, key_in.p, key_out.p, val_in.p, val_out.p, int(nt), 0, end_bit,
                                          st));
  k_key_heads<<<grid, 256, 0, st>>>(nt, key_out.p, head.p);
  PM_CHECK_LAUNCH();
  sb = tmp.n;
  PM_CUDA(cub::DeviceScan::InclusiveSum(tmp.p, sb, head.p, gid.p, int(nt), st));
  int U = 0;
  PM_CUDA(cudaMemcpyAsync(&U, gid.p + nt - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  PM_CUDA(cudaStreamSynchronize(st));
  // the distinct nodes in (class, first touch) order
  DBuf<unsigned long long> ukey(static_cast<size_t>(U)), okey_in(static_cast<size_t>(U)),
      okey_out(static_cast<size_t>(U));
  DBuf<int> oval_in(static_cast<size_t>(U)), oval_out(static_cast<size_t>(U));
  k_distinct<<<grid, 256, 0, st>>>(nt, dim, W, S, neumann_sides, key_out.p, val_out.p, head.p, gid.p, ukey.p,
                                   okey_in.p, oval_in.p);
  PM_CHECK_LAUNCH();
  size_t ob = 0;
  PM_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, ob, okey_in.p, okey_out.p, oval_in.p, oval_out.p, U, 0, 34, st));
  if (ob > tmp.n) tmp.alloc(ob);
  ob = tmp.n;
  PM_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, ob, okey_in.p, okey_out.p, oval_in.p, oval_out.p, U, 0, 34, st));
  DBuf<int> number(static_cast<size_t>(U)), class_first(3), dofmap(static_cast<size_t>(nt));
  DBuf<long long> node(static_cast<size_t>(U) * dim);
  const int init[3] = {-1, -1, -1};
  PM_CUDA(cudaMemcpyAsync(class_first.p, init, sizeof(init), cudaMemcpyHostToDevice, st));
  const int ugrid = std::max(1, std::min((U + 255) / 256, c->num_sms * 8));
  k_number<<<ugrid, 256, 0, st>>>(U, dim, W, okey_out.p, oval_out.p, ukey.p, number.p, node.p, class_first.p);
  PM_CHECK_LAUNCH();
  k_dofmap<<<grid, 256, 0, st>>>(nt, val_out.p, gid.p, number.p, dofmap.p);
  PM_CHECK_LAUNCH();
  c->kernel_launches += 5;
  int first[3];
  s.dofmap.resize(static_cast<size_t>(nt));
  s.node.resize(static_cast<size_t>(U) * dim);
  PM_CUDA(cudaMemcpyAsync(first, class_first.p, sizeof(first), cudaMemcpyDeviceToHost, st));
  PM_CUDA(cudaMemcpyAsync(s.dofmap.data(), dofmap.p, s.dofmap.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
  PM_CUDA(cudaMemcpyAsync(s.node.data(), node.p, s.node.size() * sizeof(long long), cudaMemcpyDeviceToHost, st));
  PM_CUDA(cudaStreamSynchronize(st));
  // class sizes from the first position of each class (absent classes: -1)
  int count[3];
  for (int k = 0; k < 3; ++k) {
    int next = U;
    for (int j = k + 1; j < 3; ++j)
      if (first[j] >= 0) {
        next = first[j];
        break;
      }
    count[k] = first[k] >= 0 ? next - first[k] : 0;
  }
  s.n_dofs = U;
  s.n_neumann = count[1];
  s.n_active = boundary == pmsetup::BND_DIRICHLET ? count[0] + count[1] : U;
  return s;
}

void device_stokes_structure(pm_ctx* c, DiscLevel& L, const std::vector<char>& active) {
  const int N = int(active.size()), nc = L.n_cells;
  const StokesLocal& loc = stokes_local();
  StokesItems S{};
  S.n = loc.n;
  for (int j = 0; j < loc.n; ++j) {
    S.lm[j] = short(loc.m[j]);
    S.lk[j] = short(loc.k[j]);
    S.lpos[j] = short(loc.pos[j]);
  }
  std::vector<int> inactive, rank(N, -1);
  for (int i = 0; i < N; ++i)
    if (!active[i]) {
      rank[i] = int(inactive.size());
      inactive.push_back(i);
    }
  const int ni = int(inactive.size()), na = N - ni;
  const long long ne = (long long)nc * S.n, total = ne + ni;
  const long long nt = (long long)nc * 34;
  if (total >= (1LL << 31) || (unsigned long long)N * N >= (1ULL << 63))
    throw Error(PM_E_INVALID, "level too large for the device structure build");
  const int grid = std::max(1, std::min(int((total + 255) / 256), c->num_sms * 8));
  cudaStream_t st = c->stream;
  DBuf<int> cdof, inact, irank;
  DBuf<unsigned char> act;
  cdof.upload(L.cdof, st);
  std::vector<unsigned char> a8(active.begin(), active.end());
  act.upload(a8, st);
  inact.upload(inactive.empty() ? std::vector<int>{0} : inactive, st);
  irank.upload(rank, st);
  DBuf<unsigned long long> key_in(static_cast<size_t>(total)), key_out(static_cast<size_t>(total));
  DBuf<int> val_in(static_cast<size_t>(total)), val_out(static_cast<size_t>(total));
  k_stokes_pairs<<<grid, 256, 0, st>>>(nc, N, ni, cdof.p, act.p, inact.p, S, key_in.p, val_in.p);
  PM_CHECK_LAUNCH();
  const int end_bit = bits_for((unsigned long long)N * N);
  size_t tmp_bytes = 0, scan_bytes = 0;
  PM_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, key_in.p, key_out.p, val_in.p, val_out.p,
                                          int(total), 0, end_bit, st));
  PM_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, val_in.p, val_out.p, int(total), st));
  DBuf<unsigned char> tmp(std::max(tmp_bytes, scan_bytes));
  PM_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, key_in.p, key_out.p, val_in.p, val_out.p,
                                          int(total), 0, end_bit, st));
  key_in.release();
  const size_t tn = static_cast<size_t>(total);
  DBuf<int> head(tn), contrib(tn), hpos(tn), cpos(tn);
  k_heads<<<grid, 256, 0, st>>>(total, N, key_out.p, val_out.p, head.p, contrib.p);
  PM_CHECK_LAUNCH();
  size_t sb = tmp.n;
  PM_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, sb, head.p, hpos.p, int(total), st));
  sb = tmp.n;
  PM_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, sb, contrib.p, cpos.p, int(total), st));
  int last[4] = {0, 0, 0, 0};
  PM_CUDA(cudaMemcpyAsync(&last[0], hpos.p + total - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  PM_CUDA(cudaMemcpyAsync(&last[1], head.p + total - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  PM_CUDA(cudaMemcpyAsync(&last[2], cpos.p + total - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  PM_CUDA(cudaMemcpyAsync(&last[3], contrib.p + total - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  PM_CUDA(cudaStreamSynchronize(st));
  const int nnz = last[0] + last[1], ncontrib = last[2] + last[3];
  DBuf<int> row_ptr(static_cast<size_t>(N) + 1), cols(static_cast<size_t>(nnz));
  DBuf<int> gat_ptr(static_cast<size_t>(nnz) + 1), gat_idx(static_cast<size_t>(std::max(1, ncontrib)));
  DBuf<int> diag_pos(static_cast<size_t>(std::max(1, ni)));
  k_fill_structure_ranked<<<grid, 256, 0, st>>>(total, N, key_out.p, val_out.p, head.p, hpos.p, cpos.p, irank.p,
                                                row_ptr.p, cols.p, gat_ptr.p, gat_idx.p, diag_pos.p);
  PM_CHECK_LAUNCH();
  k_set_tail<<<1, 32, 0, st>>>(row_ptr.p, N, N + 1, nnz);
  k_set_tail<<<1, 32, 0, st>>>(gat_ptr.p, nnz, nnz + 1, ncontrib);
  PM_CHECK_LAUNCH();
  c->kernel_launches += 5;
  // right-hand side plan
  DBuf<unsigned int> rkey_in(static_cast<size_t>(nt)), rkey_out(static_cast<size_t>(nt));
  DBuf<int> rval_in(static_cast<size_t>(nt)), rval_out(static_cast<size_t>(nt));
  const int rgrid = std::max(1, std::min(int((nt + 255) / 256), c->num_sms * 8));
  k_stokes_rhs_pairs<<<rgrid, 256, 0, st>>>(nt, N, cdof.p, act.p, rkey_in.p, rval_in.p);
  PM_CHECK_LAUNCH();
  size_t rb = 0;
  const int rend = bits_for((unsigned long long)N);
  PM_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, rb, rkey_in.p, rkey_out.p, rval_in.p, rval_out.p, int(nt), 0,
                                          rend, st));
  if (rb > tmp.n) tmp.alloc(rb);
  rb = tmp.n;
  PM_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, rb, rkey_in.p, rkey_out.p, rval_in.p, rval_out.p, int(nt), 0,
                                          rend, st));
  c->kernel_launches++;
  // results into the host level
  L.sys = pmsetup::Csr();
  L.sys.n_rows = N;
  L.sys.n_cols = N;
  L.sys.n_active = na;
  download(c, L.sys.row_ptr, row_ptr, size_t(N) + 1);
  download(c, L.sys.cols, cols, size_t(nnz));
  download(c, L.gat_ptr, gat_ptr, size_t(nnz) + 1);
  download(c, L.gat_idx, gat_idx, size_t(ncontrib));
  download(c, L.diag_pos, diag_pos, size_t(ni));
  std::vector<unsigned> rk(static_cast<size_t>(nt));
  std::vector<int> rv;
  download(c, rv, rval_out, size_t(nt));
  PM_CUDA(cudaMemcpyAsync(rk.data(), rkey_out.p, rk.size() * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  PM_CUDA(cudaStreamSynchronize(st));
  L.sys.vals.assign(L.sys.cols.size(), 0.0);
  // the rhs items of active rows come first, in row order and, per row, in
  // the order of t; rows without items (non-active) get empty ranges
  std::vector<int> rp(size_t(N) + 1, 0);
  size_t valid = 0;
  while (valid < rk.size() && rk[valid] < unsigned(N)) {
    rp[rk[valid] + 1]++;
    ++valid;
  }
  for (int i = 0; i < N; ++i) rp[size_t(i) + 1] += rp[size_t(i)];
  rv.resize(valid);
  L.rgat_ptr = std::move(rp);
  L.rgat_idx = std::move(rv);
}

}  // namespace pm
