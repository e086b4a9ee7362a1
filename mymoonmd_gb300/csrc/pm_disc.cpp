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

// --------------------------------------------------------------- Stokes ----
// Combined local DOF m of a P2/P1 cell: 0..29 velocity (component m/10, local
// m%10), 30..33 pressure. Block (bm, bk) is non-zero for the diagonal A
// blocks, B^T (velocity rows, pressure columns) and B (pressure rows, velocity
// columns) - the NSTYPE 4 Stokes blocks with the Laplace form
// (src/Matrix/BlockFEMatrix.C:616-664, NSE_local_assembling_routines.C:82-225).
static inline int stokes_block(int m) { return m < 30 ? m / 10 : 3; }
static inline bool stokes_nonzero(int m, int k) {
  const int bm = stokes_block(m), bk = stokes_block(k);
  if (bm < 3 && bk < 3) return bm == bk;
  return !(bm == 3 && bk == 3);
}
// element storage of a cell: A (10x10) then B_0, B_1, B_2 (4x10 each)
static inline int stokes_pos(int c, int m, int k) {
  const int bm = stokes_block(m), bk = stokes_block(k);
  const size_t base = size_t(c) * 220;
  if (bm < 3 && bk < 3) return bm == bk ? int(base + (m % 10) * 10 + (k % 10)) : -1;
  if (bm < 3) return int(base + 100 + bm * 40 + (k - 30) * 10 + (m % 10));  // B^T = B transposed
  if (bk < 3) return int(base + 100 + bk * 40 + (m - 30) * 10 + (k % 10));
  return -1;
}

const StokesLocal& stokes_local() {
  static const StokesLocal t = [] {
    StokesLocal r;
    for (int m = 0; m < 34; ++m)
      for (int k = 0; k < 34; ++k) {
        const int p = stokes_pos(0, m, k);
        if (p < 0) continue;
        r.m[r.n] = m;
        r.k[r.n] = k;
        r.pos[r.n] = p;
        ++r.n;
      }
    return r;
  }();
  return t;
}

// physical coordinates of the non-active DOFs of L.space (lattice coordinates
// converted the way cell_vertices converts them)
static void fill_bnd_xyz(const Hierarchy& h, DiscLevel& L) {
  const int dim = h.dim;
  const int64_t S = h.scale;
  const double inv = 1.0 / double(S);
  const bool pow2 = (S & (S - 1)) == 0;
  L.bnd_xyz.assign(size_t(L.space.n_dofs - L.space.n_active) * 3, 0.0);
  for (int i = L.space.n_active; i < L.space.n_dofs; ++i)
    for (int d = 0; d < dim; ++d) {
      const double v = double(L.space.node[size_t(i) * dim + d]);
      L.bnd_xyz[size_t(i - L.space.n_active) * 3 + d] = pow2 ? v * inv : v / double(S);
    }
}

static void build_stokes_structure(DiscLevel& L, const std::vector<char>& act);
static void finish_stokes_level(DiscLevel& L, int nu, int np, int nau);

static void build_stokes_level(const Hierarchy& h, int lvl, DiscLevel& L, const SetupParts* parts) {
  const bool dev = parts && parts->space;
  L.space = dev ? parts->space(h, lvl, EL_P2, BND_DIRICHLET, 0) : build_space(h, lvl, EL_P2, BND_DIRICHLET);
  L.pspace = dev ? parts->space(h, lvl, EL_P1, BND_NEUMANN, 0) : build_space(h, lvl, EL_P1, BND_NEUMANN);
  const int nu = L.space.n_dofs, np = L.pspace.n_dofs, nau = L.space.n_active;
  const int N = 3 * nu + np, nc = L.n_cells;
  L.cdof.resize(size_t(nc) * 34);
  for (int c = 0; c < nc; ++c)
    for (int m = 0; m < 34; ++m)
      L.cdof[size_t(c) * 34 + m] = m < 30 ? (m / 10) * nu + L.space.dofmap[size_t(c) * 10 + m % 10]
                                          : 3 * nu + L.pspace.dofmap[size_t(c) * 4 + (m - 30)];
  std::vector<char> act(N, 1);
  for (int b = 0; b < 3; ++b)
    for (int i = nau; i < nu; ++i) act[size_t(b) * nu + i] = 0;
  if (parts && parts->stokes_structure) {
    parts->stokes_structure(L, act);
  } else {
    build_stokes_structure(L, act);
  }
  finish_stokes_level(L, nu, np, nau);
}

// the combined pattern and the gather plans of a Stokes level (host)
static void build_stokes_structure(DiscLevel& L, const std::vector<char>& act) {
  const int N = int(act.size()), nc = L.n_cells;
  int n_inactive = 0;
  for (char a : act) n_inactive += a ? 0 : 1;
  // incidence: combined DOF -> (cell, local index), cells in order
  std::vector<int> iptr(N + 1, 0), inc;
  for (size_t t = 0; t < L.cdof.size(); ++t) iptr[L.cdof[t] + 1]++;
  for (int i = 0; i < N; ++i) iptr[i + 1] += iptr[i];
  inc.resize(iptr[N]);
  {
    std::vector<int> fill(iptr.begin(), iptr.end() - 1);
    for (size_t t = 0; t < L.cdof.size(); ++t) inc[fill[L.cdof[t]]++] = int(t);
  }
  // combined pattern
  Csr& A = L.sys;
  A = Csr();
  A.n_rows = A.n_cols = N;
  A.n_active = N - n_inactive;
  A.row_ptr.assign(N + 1, 0);
  std::vector<int> marker(N, -1), row;
  for (int i = 0; i < N; ++i) {
    row.clear();
    if (act[i]) {
      for (int e = iptr[i]; e < iptr[i + 1]; ++e) {
        const int c = inc[e] / 34, m = inc[e] % 34;
        for (int k = 0; k < 34; ++k) {
          if (!stokes_nonzero(m, k)) continue;
          const int j = L.cdof[size_t(c) * 34 + k];
          if (marker[j] != i) {
            marker[j] = i;
            row.push_back(j);
          }
        }
      }
      std::sort(row.begin(), row.end());
    } else {
      row.push_back(i);
    }
    A.cols.insert(A.cols.end(), row.begin(), row.end());
    A.row_ptr[i + 1] = int(A.cols.size());
  }
  A.vals.assign(A.cols.size(), 0.0);
  // gather plans into the compact element storage
  const int nnz = A.row_ptr[N];
  auto find = [&](int r, int col) {
    const int* b = A.cols.data() + A.row_ptr[r];
    const int* e = A.cols.data() + A.row_ptr[r + 1];
    const int* it = std::lower_bound(b, e, col);
    if (it == e || *it != col) throw std::logic_error("Stokes element entry outside the pattern");
    return int(it - A.cols.data());
  };
  std::vector<int> cnt(size_t(nnz) + 1, 0);
  std::vector<std::pair<int, int>> contrib;  // (entry, element storage position), cell order
  contrib.reserve(size_t(nc) * 34 * 14);
  for (int c = 0; c < nc; ++c)
    for (int m = 0; m < 34; ++m) {
      const int r = L.cdof[size_t(c) * 34 + m];
      if (!act[r]) continue;
      for (int k = 0; k < 34; ++k) {
        const int p = stokes_pos(c, m, k);
        if (p < 0) continue;
        const int e = find(r, L.cdof[size_t(c) * 34 + k]);
        contrib.push_back({e, p});
        cnt[e + 1]++;
      }
    }
  for (int e = 0; e < nnz; ++e) cnt[e + 1] += cnt[e];
  L.gat_ptr = cnt;
  L.gat_idx.assign(cnt[nnz], 0);
  {
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (auto& pr : contrib) L.gat_idx[fill[pr.first]++] = pr.second;
  }
  L.rgat_ptr.assign(N + 1, 0);
  for (size_t t = 0; t < L.cdof.size(); ++t)
    if (act[L.cdof[t]]) L.rgat_ptr[L.cdof[t] + 1]++;
  for (int i = 0; i < N; ++i) L.rgat_ptr[i + 1] += L.rgat_ptr[i];
  L.rgat_idx.assign(L.rgat_ptr[N], 0);
  {
    std::vector<int> fill(L.rgat_ptr.begin(), L.rgat_ptr.end() - 1);
    for (size_t t = 0; t < L.cdof.size(); ++t)
      if (act[L.cdof[t]]) L.rgat_idx[fill[L.cdof[t]]++] = int(t);  // rhs storage: cell*34 + m
  }
  L.diag_pos.clear();
  for (int i = 0; i < N; ++i)
    if (!act[i]) L.diag_pos.push_back(find(i, i));
}

// block layout, Vanka patches and the cell colouring of a Stokes level
static void finish_stokes_level(DiscLevel& L, int nu, int np, int nau) {
  const int N = 3 * nu + np, nc = L.n_cells;
  // incidence: combined DOF -> (cell, local index), cells in order
  std::vector<int> iptr(N + 1, 0), inc;
  for (size_t t = 0; t < L.cdof.size(); ++t) iptr[L.cdof[t] + 1]++;
  for (int i = 0; i < N; ++i) iptr[i + 1] += iptr[i];
  inc.resize(iptr[N]);
  {
    std::vector<int> fill(iptr.begin(), iptr.end() - 1);
    for (size_t t = 0; t < L.cdof.size(); ++t) inc[fill[L.cdof[t]]++] = int(t);
  }
  L.elem_stride = 220;
  L.rhs_stride = 34;
  L.n_blocks = 4;
  for (int b = 0; b < 3; ++b) {
    L.block_len[b] = nu;
    L.block_active[b] = nau;
  }
  L.block_len[3] = np;
  L.block_active[3] = np;
  L.pressure_row0 = 3 * nu;
  // Vanka patches (sorted combined DOFs of each cell) and a greedy colouring
  L.patch_dofs = L.cdof;
  for (int c = 0; c < nc; ++c) std::sort(L.patch_dofs.begin() + size_t(c) * 34, L.patch_dofs.begin() + size_t(c + 1) * 34);
  std::vector<int> color(nc, -1), seen;
  int n_colors = 0;
  for (int c = 0; c < nc; ++c) {
    seen.assign(n_colors + 1, 0);
    for (int m = 0; m < 34; ++m) {
      const int d = L.cdof[size_t(c) * 34 + m];
      for (int e = iptr[d]; e < iptr[d + 1]; ++e) {
        const int oc = inc[e] / 34;
        if (oc < c && color[oc] >= 0) seen[color[oc]] = 1;
      }
    }
    int col = 0;
    while (col < n_colors && seen[col]) ++col;
    color[c] = col;
    if (col == n_colors) ++n_colors;
  }
  L.color_ptr.assign(n_colors + 1, 0);
  for (int c = 0; c < nc; ++c) L.color_ptr[color[c] + 1]++;
  for (int k = 0; k < n_colors; ++k) L.color_ptr[k + 1] += L.color_ptr[k];
  L.color_cells.assign(nc, 0);
  {
    std::vector<int> fill(L.color_ptr.begin(), L.color_ptr.end() - 1);
    for (int c = 0; c < nc; ++c) L.color_cells[fill[color[c]]++] = c;
  }
}

// block-diagonal prolongation of the combined vector between two Stokes levels
static void build_stokes_transfer(const Hierarchy& h, DiscLevel& Lc, const DiscLevel& Lf) {
  Csr Pu, Ru, Pp, Rp;
  build_transfer(h, Lf.level_in_hierarchy, Lc.space, Lf.space, Pu, Ru);
  build_transfer(h, Lf.level_in_hierarchy, Lc.pspace, Lf.pspace, Pp, Rp);
  const int nuf = Lf.space.n_dofs, npf = Lf.pspace.n_dofs, nuc = Lc.space.n_dofs, npc = Lc.pspace.n_dofs;
  Csr& P = Lc.P;
  P = Csr();
  P.n_rows = 3 * nuf + npf;
  P.n_cols = 3 * nuc + npc;
  P.n_active = 3 * Lf.space.n_active + npf;
  P.row_ptr.assign(P.n_rows + 1, 0);
  for (int b = 0; b < 4; ++b) {
    const Csr& S = b < 3 ? Pu : Pp;
    const int roff = b < 3 ? b * nuf : 3 * nuf, coff = b < 3 ? b * nuc : 3 * nuc;
    for (int i = 0; i < S.n_rows; ++i) {
      for (int k = S.row_ptr[i]; k < S.row_ptr[i + 1]; ++k) {
        P.cols.push_back(coff + S.cols[k]);
        P.vals.push_back(S.vals[k]);
      }
      P.row_ptr[roff + i + 1] = int(P.cols.size());
    }
  }
}

// The Neumann plan of one level: for every active DOF on a Neumann edge the
// edges that integrate into its right-hand side entry (only the local DOFs on
// the edge: the others vanish there).
static void build_neumann_plan(const Hierarchy& h, DiscLevel& L, int neumann_sides) {
  L.nm_dof.clear();
  L.nm_ptr.assign(1, 0);
  L.nm_cell.clear();
  L.nm_code.clear();
  const std::vector<NeumannEdge> edges = neumann_edges(h, L.level_in_hierarchy, neumann_sides);
  if (edges.empty()) return;
  const int nloc = L.space.nloc, k = nloc == 9 ? 2 : 1;
  // local DOF (a, b) of a tensor element lies on edge m of [-1,1]^2 when
  // b = 0 (m 0), a = k (m 1), b = k (m 2), a = 0 (m 3)
  auto on_edge = [k](int loc, int m) {
    const int a = loc % (k + 1), b = loc / (k + 1);
    return m == 0 ? b == 0 : m == 1 ? a == k : m == 2 ? b == k : a == 0;
  };
  std::vector<std::vector<std::pair<int, int>>> per(L.space.n_dofs);
  for (const NeumannEdge& e : edges)
    for (int loc = 0; loc < nloc; ++loc) {
      if (!on_edge(loc, e.edge)) continue;
      const int g = L.space.dofmap[size_t(e.cell) * nloc + loc];
      if (g < L.space.n_active) per[g].push_back({e.cell, e.edge | (e.side << 2) | (loc << 4)});
    }
  for (int g = 0; g < L.space.n_dofs; ++g) {
    if (per[g].empty()) continue;
    L.nm_dof.push_back(g);
    for (auto& pc : per[g]) {
      L.nm_cell.push_back(pc.first);
      L.nm_code.push_back(pc.second);
    }
    L.nm_ptr.push_back(int(L.nm_cell.size()));
  }
}

std::unique_ptr<Disc> build_disc(int geometry, int root_n, int n_refine, int n_levels, int kind, int elem,
                                 int neumann_sides, const SetupParts* parts) {
  if (n_levels < 1 || n_levels > n_refine + 1)
    throw std::invalid_argument("multigrid levels must be between 1 and refinements + 1");
  auto D = std::make_unique<Disc>();
  D->kind = kind;
  D->geometry = geometry;
  D->root_n = root_n;
  D->n_refine = n_refine;
  D->n_levels = n_levels;
  D->elem = elem;
  if (neumann_sides < 0 || neumann_sides > 15 || (neumann_sides && (kind != KIND_CD || geometry != GEO_SQUARE_QUAD)))
    throw std::invalid_argument("Neumann sides (a mask of 4 bits) apply to convection-diffusion on the unit square");
  D->neumann_sides = neumann_sides;
  if (kind == KIND_CD) {
    const bool tet = geometry == GEO_CUBE_TETRA;
    if (!tet && elem != EL_Q1 && elem != EL_Q2)
      throw std::invalid_argument("convection-diffusion on quadrilaterals or hexahedra uses Q1 or Q2");
    if (tet && elem != EL_P1 && elem != EL_P2)
      throw std::invalid_argument("convection-diffusion on tetrahedra uses P1 or P2");
  } else {
    if (geometry != GEO_CUBE_TETRA) throw std::invalid_argument("Stokes P2/P1 uses the tetrahedral unit cube");
    D->elem = EL_P2;
    D->h = parts && parts->hierarchy ? parts->hierarchy(geometry, root_n, n_refine)
                                     : build_hierarchy(geometry, root_n, n_refine);
    const int first = n_refine + 1 - n_levels;
    D->levels.resize(n_levels);
    for (int l = 0; l < n_levels; ++l) {
      DiscLevel& L = D->levels[l];
      L.level_in_hierarchy = first + l;
      L.n_cells = D->h.levels[first + l].n_cells;
      L.verts = cell_vertices(D->h, first + l);
      build_stokes_level(D->h, first + l, L, parts);
      fill_bnd_xyz(D->h, L);
    }
    for (int l = 0; l + 1 < n_levels; ++l) build_stokes_transfer(D->h, D->levels[l], D->levels[l + 1]);
    return D;
  }
  D->h = parts && parts->hierarchy ? parts->hierarchy(geometry, root_n, n_refine)
                                   : build_hierarchy(geometry, root_n, n_refine);
  const int first = n_refine + 1 - n_levels;
  D->levels.resize(n_levels);
  for (int l = 0; l < n_levels; ++l) {
    DiscLevel& L = D->levels[l];
    L.level_in_hierarchy = first + l;
    L.n_cells = D->h.levels[first + l].n_cells;
    L.space = parts && parts->space ? parts->space(D->h, first + l, elem, BND_DIRICHLET, neumann_sides)
                                    : build_space(D->h, first + l, elem, BND_DIRICHLET, neumann_sides);
    L.verts = cell_vertices(D->h, first + l);
    if (parts && parts->structure) {
      parts->structure(L);
    } else {
      L.sys = build_structure(L.space, L.n_cells);
      std::vector<char> act(L.space.n_dofs, 0);
      for (int i = 0; i < L.space.n_active; ++i) act[i] = 1;
      build_gather(L, L.space.nloc, L.space.dofmap, act);
    }
    fill_bnd_xyz(D->h, L);
    build_neumann_plan(D->h, L, neumann_sides);
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
