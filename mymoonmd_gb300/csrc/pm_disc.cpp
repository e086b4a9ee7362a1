// Discretisation hierarchy set-up (host): spaces, CSR patterns, gather plans,
// prolongations for every kept multigrid level.
#include "pm_disc.h"

#include <algorithm>
#include <stdexcept>

#include "../../include/pmgpu.h"

namespace pm {

using namespace pmsetup;

// gather plan of a square system on one level: element matrices of `nloc` x
// `nloc` per cell, local DOF m of cell c maps to global row/column gdof[c*nloc+m]
static void build_gather(DiscLevel& L, int nloc, const std::vector<int>& gdof,
                         const std::vector<char>& row_active) {
  const Csr& A = L.sys;
  const int nnz = A.row_ptr[A.n_rows];
  std::vector<int> cnt(size_t(nnz) + 1, 0);
  auto find = [&](int row, int col) {
    const int* b = A.cols.data() + A.row_ptr[row];
    const int* e = A.cols.data() + A.row_ptr[row + 1];
    const int* it = std::lower_bound(b, e, col);
    if (it == e || *it != col) throw std::logic_error("element entry outside the CSR pattern");
    return int(it - A.cols.data());
  };
  std::vector<int> pos(size_t(L.n_cells) * nloc * nloc, -1);
  for (int c = 0; c < L.n_cells; ++c) {
    const int* d = &gdof[size_t(c) * nloc];
    for (int m = 0; m < nloc; ++m) {
      if (!row_active[d[m]]) continue;
      for (int k = 0; k < nloc; ++k) {
        const int e = find(d[m], d[k]);
        pos[(size_t(c) * nloc + m) * nloc + k] = e;
        cnt[e + 1]++;
      }
    }
  }
  for (int e = 0; e < nnz; ++e) cnt[e + 1] += cnt[e];
  L.gat_ptr = cnt;
  L.gat_idx.assign(cnt[nnz], 0);
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (size_t t = 0; t < pos.size(); ++t)
    if (pos[t] >= 0) L.gat_idx[fill[pos[t]]++] = int(t);
  // right-hand side plan
  const int n = A.n_rows;
  std::vector<int> rc(size_t(n) + 1, 0);
  for (size_t t = 0; t < gdof.size(); ++t)
    if (row_active[gdof[t]]) rc[gdof[t] + 1]++;
  for (int i = 0; i < n; ++i) rc[i + 1] += rc[i];
  L.rgat_ptr = rc;
  L.rgat_idx.assign(rc[n], 0);
  std::vector<int> rf(rc.begin(), rc.end() - 1);
  for (size_t t = 0; t < gdof.size(); ++t)
    if (row_active[gdof[t]]) L.rgat_idx[rf[gdof[t]]++] = int(t);
  // unit diagonal of non-active rows
  L.diag_pos.clear();
  for (int i = 0; i < n; ++i)
    if (!row_active[i]) L.diag_pos.push_back(find(i, i));
}

std::unique_ptr<Disc> build_disc(int geometry, int root_n, int n_refine, int n_levels, int kind, int elem) {
  if (n_levels < 1 || n_levels > n_refine + 1)
    throw std::invalid_argument("multigrid levels must be between 1 and refinements + 1");
  auto D = std::make_unique<Disc>();
  D->kind = kind;
  D->geometry = geometry;
  D->root_n = root_n;
  D->n_refine = n_refine;
  D->n_levels = n_levels;
  D->elem = elem;
  if (kind == KIND_CD) {
    if (geometry == GEO_CUBE_TETRA) throw std::invalid_argument("convection-diffusion uses quadrilaterals or hexahedra");
    if (elem != EL_Q1 && elem != EL_Q2) throw std::invalid_argument("convection-diffusion elements are Q1 or Q2");
  } else {
    throw std::invalid_argument("Stokes set-up is not available in this build");
  }
  D->h = build_hierarchy(geometry, root_n, n_refine);
  const int first = n_refine + 1 - n_levels;
  D->levels.resize(n_levels);
  for (int l = 0; l < n_levels; ++l) {
    DiscLevel& L = D->levels[l];
    L.level_in_hierarchy = first + l;
    L.n_cells = D->h.levels[first + l].n_cells;
    L.space = build_space(D->h, first + l, elem, BND_DIRICHLET);
    L.sys = build_structure(L.space, L.n_cells);
    L.verts = cell_vertices(D->h, first + l);
    std::vector<char> act(L.space.n_dofs, 0);
    for (int i = 0; i < L.space.n_active; ++i) act[i] = 1;
    build_gather(L, L.space.nloc, L.space.dofmap, act);
    L.n_blocks = 1;
    L.block_len[0] = L.space.n_dofs;
    L.block_active[0] = L.space.n_active;
  }
  for (int l = 0; l + 1 < n_levels; ++l) {
    Csr R;
    build_transfer(D->h, D->levels[l + 1].level_in_hierarchy, D->levels[l].space,
                   D->levels[l + 1].space, D->levels[l].P, R);
  }
  return D;
}

}  // namespace pm
