// Host-side mesh hierarchy, DOF numbering, CSR structure and transfer set-up.
// See pm_setup.h for the reference routines each step restates.
#include "pm_setup.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <stdexcept>

#include "pm_refine_tables.h"

namespace pmsetup {

int element_nloc(int elem) {
  switch (elem) {
    case EL_Q1: return -1;  // depends on dim, see space_nloc
    case EL_Q2: return -1;
    case EL_P1: return 4;
    case EL_P2: return 10;
  }
  return 0;
}

int element_dim(int elem) { return (elem == EL_P1 || elem == EL_P2) ? 3 : 0; }

int space_nloc(int geometry, int elem) {
  if (geometry == GEO_SQUARE_QUAD) {
    if (elem == EL_Q1) return 4;
    if (elem == EL_Q2) return 9;
  } else if (geometry == GEO_CUBE_HEXA) {
    if (elem == EL_Q1) return 8;
    if (elem == EL_Q2) return 27;
  } else if (geometry == GEO_CUBE_TETRA) {
    if (elem == EL_P1) return 4;
    if (elem == EL_P2) return 10;
  }
  throw std::invalid_argument("element does not fit the cell shape");
}

Hierarchy root_hierarchy(int geometry, int root_n, int n_refine) {
  if (root_n < 1 || n_refine < 0 || n_refine > 12)
    throw std::invalid_argument("bad mesh size");
  Hierarchy h;
  h.geometry = geometry;
  h.root_n = root_n;
  h.n_refine = n_refine;
  h.dim = geometry == GEO_SQUARE_QUAD ? 2 : 3;
  h.nvc = geometry == GEO_SQUARE_QUAD ? 4 : (geometry == GEO_CUBE_HEXA ? 8 : 4);
  const int64_t unit = int64_t(2) << n_refine;  // root cell edge in lattice units
  h.scale = unit * root_n;
  const int dim = h.dim, nvc = h.nvc;

  Level root;
  if (geometry == GEO_SQUARE_QUAD) {
    // UnitSquare (Tests.C:449): (0,0) (1,0) (1,1) (0,1); larger root meshes
    // are root_n x root_n copies in lexicographic order.
    static const int corner[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
    for (int j = 0; j < root_n; ++j)
      for (int i = 0; i < root_n; ++i) {
        for (int v = 0; v < 4; ++v) {
          root.vtx.push_back((i + corner[v][0]) * unit);
          root.vtx.push_back((j + corner[v][1]) * unit);
        }
        root.n_cells++;
      }
  } else {
    for (int k = 0; k < root_n; ++k)
      for (int j = 0; j < root_n; ++j)
        for (int i = 0; i < root_n; ++i) {
          if (geometry == GEO_CUBE_HEXA) {
            for (int v = 0; v < 8; ++v) {
              root.vtx.push_back((i + kCubeCorner[v][0]) * unit);
              root.vtx.push_back((j + kCubeCorner[v][1]) * unit);
              root.vtx.push_back((k + kCubeCorner[v][2]) * unit);
            }
            root.n_cells++;
          } else {
            for (int t = 0; t < 6; ++t) {
              for (int v = 0; v < 4; ++v) {
                const int c = kKuhn[t][v];
                root.vtx.push_back((i + kCubeCorner[c][0]) * unit);
                root.vtx.push_back((j + kCubeCorner[c][1]) * unit);
                root.vtx.push_back((k + kCubeCorner[c][2]) * unit);
              }
              root.n_cells++;
            }
          }
        }
  }
  root.parent.assign(root.n_cells, -1);
  root.child_no.assign(root.n_cells, -1);
  h.levels.push_back(std::move(root));
  return h;
}

Hierarchy build_hierarchy(int geometry, int root_n, int n_refine) {
  Hierarchy h = root_hierarchy(geometry, root_n, n_refine);
  const int dim = h.dim, nvc = h.nvc;
  for (int r = 0; r < n_refine; ++r) {
    const Level& coarse = h.levels.back();
    Level fine;
    const int nchild = dim == 2 ? 4 : 8;
    fine.n_cells = coarse.n_cells * nchild;
    fine.vtx.resize(size_t(fine.n_cells) * nvc * dim);
    fine.parent.resize(fine.n_cells);
    fine.child_no.resize(fine.n_cells);
    int64_t rv[27][3];
    for (int c = 0; c < coarse.n_cells; ++c) {
      const int64_t* pv = &coarse.vtx[size_t(c) * nvc * dim];
      int n_ref = 0;
      for (int v = 0; v < nvc; ++v, ++n_ref)
        for (int d = 0; d < dim; ++d) rv[v][d] = pv[v * dim + d];
      if (geometry == GEO_SQUARE_QUAD) {
        for (int n = 0; n < 5; ++n, ++n_ref) {
          int cnt = 0;
          int64_t s[2] = {0, 0};
          for (int q = 0; q < 4 && kQuadNew[n][q] >= 0; ++q, ++cnt)
            for (int d = 0; d < 2; ++d) s[d] += pv[kQuadNew[n][q] * 2 + d];
          for (int d = 0; d < 2; ++d) rv[n_ref][d] = s[d] / cnt;
        }
      } else if (geometry == GEO_CUBE_HEXA) {
        for (int n = 0; n < 19; ++n, ++n_ref) {
          int cnt = 0;
          int64_t s[3] = {0, 0, 0};
          for (; cnt < 8 && kHexNew[n][cnt] >= 0; ++cnt)
            for (int d = 0; d < 3; ++d) s[d] += pv[kHexNew[n][cnt] * 3 + d];
          for (int d = 0; d < 3; ++d) rv[n_ref][d] = s[d] / cnt;
        }
      } else {
        for (int n = 0; n < 6; ++n, ++n_ref)
          for (int d = 0; d < 3; ++d)
            rv[n_ref][d] = (pv[kTetNew[n][0] * 3 + d] + pv[kTetNew[n][1] * 3 + d]) / 2;
      }
      for (int ch = 0; ch < nchild; ++ch) {
        const int fc = c * nchild + ch;
        fine.parent[fc] = c;
        fine.child_no[fc] = ch;
        int64_t* out = &fine.vtx[size_t(fc) * nvc * dim];
        for (int v = 0; v < nvc; ++v) {
          const int idx = geometry == GEO_SQUARE_QUAD ? kQuadChild[ch][v]
                          : geometry == GEO_CUBE_HEXA ? kHexChild[ch][v]
                                                      : kTetChild[ch][v];
          for (int d = 0; d < dim; ++d) out[v * dim + d] = rv[idx][d];
        }
      }
    }
    h.levels.push_back(std::move(fine));
  }
  return h;
}

// lattice coordinates of the local DOF nodes of one cell, in local DOF order
// (tensor-lexicographic for Qk, C_T_P2_3D / C_T_P1_3D order for tetrahedra)
static void cell_nodes(int geometry, int elem, const int64_t* v, int64_t* out) {
  if (geometry == GEO_SQUARE_QUAD) {
    const int k = elem == EL_Q2 ? 2 : 1;
    int m = 0;
    for (int b = 0; b <= k; ++b)
      for (int a = 0; a <= k; ++a, ++m)
        for (int d = 0; d < 2; ++d)
          out[m * 2 + d] = v[d] + (v[2 + d] - v[d]) * a / k + (v[6 + d] - v[d]) * b / k;
  } else if (geometry == GEO_CUBE_HEXA) {
    const int k = elem == EL_Q2 ? 2 : 1;
    int m = 0;
    for (int c = 0; c <= k; ++c)
      for (int b = 0; b <= k; ++b)
        for (int a = 0; a <= k; ++a, ++m)
          for (int d = 0; d < 3; ++d)
            out[m * 3 + d] = v[d] + (v[3 + d] - v[d]) * a / k + (v[9 + d] - v[d]) * b / k +
                             (v[12 + d] - v[d]) * c / k;
  } else {
    if (elem == EL_P1) {
      for (int i = 0; i < 12; ++i) out[i] = v[i];
    } else {
      // v0, m01, v1, m02, m12, v2, m03, m13, m23, v3
      static const int pairs[10][2] = {{0, 0}, {0, 1}, {1, 1}, {0, 2}, {1, 2},
                                       {2, 2}, {0, 3}, {1, 3}, {2, 3}, {3, 3}};
      for (int m = 0; m < 10; ++m)
        for (int d = 0; d < 3; ++d)
          out[m * 3 + d] = (v[pairs[m][0] * 3 + d] + v[pairs[m][1] * 3 + d]) / 2;
    }
  }
}

int square_sides(int64_t S, const int64_t* x) {
  int m = 0;
  if (x[1] == 0) m |= SIDE_Y0;
  if (x[0] == S) m |= SIDE_X1;
  if (x[1] == S) m |= SIDE_Y1;
  if (x[0] == 0) m |= SIDE_X0;
  return m;
}

Space build_space(const Hierarchy& h, int level, int elem, int boundary, int neumann_sides) {
  const Level& L = h.levels.at(level);
  const int dim = h.dim, nvc = h.nvc;
  if (neumann_sides && (dim != 2 || boundary != BND_DIRICHLET))
    throw std::invalid_argument("Neumann sides are supported on the unit square with Dirichlet elsewhere");
  Space s;
  s.elem = elem;
  s.boundary = boundary;
  s.neumann_sides = neumann_sides;
  s.nloc = space_nloc(h.geometry, elem);
  const int64_t S = h.scale, W = S + 1;
  size_t lattice = size_t(W) * W * (dim == 3 ? W : 1);
  // provisional number per lattice point: -1 unseen, >= 0 class-local number
  // (class in cls)
  std::vector<int> mark(lattice, -1);
  std::vector<char> cls(lattice, 0);
  s.dofmap.resize(size_t(L.n_cells) * s.nloc);
  std::vector<int> dof_key(size_t(L.n_cells) * s.nloc);
  int count[3] = {0, 0, 0};  // inner, Neumann, Dirichlet (or all-boundary)
  std::vector<int64_t> cls_nodes[3];
  std::vector<int64_t> nodes(size_t(s.nloc) * dim);
  for (int c = 0; c < L.n_cells; ++c) {
    cell_nodes(h.geometry, elem, &L.vtx[size_t(c) * nvc * dim], nodes.data());
    for (int m = 0; m < s.nloc; ++m) {
      const int64_t* x = &nodes[size_t(m) * dim];
      size_t key = size_t(x[0]) + size_t(W) * (size_t(x[1]) + (dim == 3 ? size_t(W) * size_t(x[2]) : 0));
      int& mk = mark[key];
      if (mk == -1) {
        bool on_bnd = false;
        for (int d = 0; d < dim; ++d) on_bnd |= (x[d] == 0 || x[d] == S);
        int k = 0;
        if (on_bnd) {
          k = 2;
          if (neumann_sides) {
            const int sides = square_sides(S, x);
            if ((sides & neumann_sides) == sides) k = 1;
          }
        }
        cls[key] = char(k);
        mk = count[k]++;
        cls_nodes[k].insert(cls_nodes[k].end(), x, x + dim);
      }
      s.dofmap[size_t(c) * s.nloc + m] = mk;
      dof_key[size_t(c) * s.nloc + m] = cls[key];
    }
  }
  const int base[3] = {0, count[0], count[0] + count[1]};
  for (size_t i = 0; i < s.dofmap.size(); ++i) s.dofmap[i] += base[dof_key[i]];
  s.n_dofs = count[0] + count[1] + count[2];
  s.n_neumann = count[1];
  s.n_active = boundary == BND_DIRICHLET ? count[0] + count[1] : s.n_dofs;
  s.node = cls_nodes[0];
  for (int k = 1; k < 3; ++k) s.node.insert(s.node.end(), cls_nodes[k].begin(), cls_nodes[k].end());
  return s;
}

std::vector<NeumannEdge> neumann_edges(const Hierarchy& h, int level, int neumann_sides) {
  std::vector<NeumannEdge> out;
  if (!neumann_sides || h.dim != 2) return out;
  const Level& L = h.levels.at(level);
  for (int c = 0; c < L.n_cells; ++c) {
    const int64_t* v = &L.vtx[size_t(c) * 8];
    for (int m = 0; m < 4; ++m) {
      const int common = square_sides(h.scale, v + 2 * m) & square_sides(h.scale, v + 2 * ((m + 1) % 4));
      for (int sd = 0; sd < 4; ++sd)
        if ((common >> sd) & (neumann_sides >> sd) & 1) out.push_back({c, m, sd});
    }
  }
  return out;
}

static void dof_cells(const Space& s, int n_cells, std::vector<int>& ptr, std::vector<int>& cells) {
  ptr.assign(s.n_dofs + 1, 0);
  for (int c = 0; c < n_cells; ++c)
    for (int m = 0; m < s.nloc; ++m) ptr[s.dofmap[size_t(c) * s.nloc + m] + 1]++;
  for (int i = 0; i < s.n_dofs; ++i) ptr[i + 1] += ptr[i];
  cells.resize(ptr[s.n_dofs]);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int c = 0; c < n_cells; ++c)
    for (int m = 0; m < s.nloc; ++m) cells[fill[s.dofmap[size_t(c) * s.nloc + m]]++] = c;
}

Csr build_structure(const Space& s, int n_cells) {
  return build_structure_rect(s, s, n_cells);
}

Csr build_structure_rect(const Space& test, const Space& ansatz, int n_cells) {
  std::vector<int> ptr, cells;
  dof_cells(test, n_cells, ptr, cells);
  const bool square = (&test == &ansatz);
  Csr a;
  a.n_rows = test.n_dofs;
  a.n_cols = ansatz.n_dofs;
  a.n_active = test.n_active;
  a.row_ptr.assign(a.n_rows + 1, 0);
  std::vector<int> marker(ansatz.n_dofs, -1), row;
  a.cols.reserve(size_t(a.n_rows) * ansatz.nloc * 4);
  for (int i = 0; i < a.n_rows; ++i) {
    row.clear();
    if (i < test.n_active) {
      for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
        const int c = cells[k];
        for (int m = 0; m < ansatz.nloc; ++m) {
          const int j = ansatz.dofmap[size_t(c) * ansatz.nloc + m];
          if (marker[j] != i) {
            marker[j] = i;
            row.push_back(j);
          }
        }
      }
      std::sort(row.begin(), row.end());
    } else if (square) {
      row.push_back(i);
    }
    a.cols.insert(a.cols.end(), row.begin(), row.end());
    a.row_ptr[i + 1] = int(a.cols.size());
  }
  a.vals.assign(a.cols.size(), 0.0);
  return a;
}

// reference coordinates of lattice point x inside cell v: Qk cells use
// [-1,1]^d via vertices 0,1,3(,4); tetrahedra use the unit simplex.
static void ref_coords(int geometry, const int64_t* v, const int64_t* x, double* xi) {
  if (geometry == GEO_SQUARE_QUAD) {
    const double a00 = double(v[2] - v[0]), a10 = double(v[3] - v[1]);
    const double a01 = double(v[6] - v[0]), a11 = double(v[7] - v[1]);
    const double r0 = double(x[0] - v[0]), r1 = double(x[1] - v[1]);
    const double det = a00 * a11 - a01 * a10;
    xi[0] = 2.0 * ((r0 * a11 - a01 * r1) / det) - 1.0;
    xi[1] = 2.0 * ((a00 * r1 - r0 * a10) / det) - 1.0;
    return;
  }
  const int c1 = 1, c2 = geometry == GEO_CUBE_HEXA ? 3 : 2, c3 = geometry == GEO_CUBE_HEXA ? 4 : 3;
  double A[3][3], r[3];
  for (int d = 0; d < 3; ++d) {
    A[d][0] = double(v[c1 * 3 + d] - v[d]);
    A[d][1] = double(v[c2 * 3 + d] - v[d]);
    A[d][2] = double(v[c3 * 3 + d] - v[d]);
    r[d] = double(x[d] - v[d]);
  }
  auto det3 = [](double m[3][3]) {
    return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
           m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
           m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
  };
  const double det = det3(A);
  for (int k = 0; k < 3; ++k) {
    double B[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) B[i][j] = (j == k) ? r[i] : A[i][j];
    const double t = det3(B) / det;
    xi[k] = geometry == GEO_CUBE_HEXA ? 2.0 * t - 1.0 : t;
  }
}

static void lagrange1d(int k, double x, double* l) {
  if (k == 1) {
    l[0] = 0.5 * (1.0 - x);
    l[1] = 0.5 * (1.0 + x);
  } else {
    l[0] = 0.5 * x * (x - 1.0);
    l[1] = 1.0 - x * x;
    l[2] = 0.5 * x * (x + 1.0);
  }
}

// values of the local basis of `elem` at reference point xi (local DOF order)
static void basis_values(int geometry, int elem, const double* xi, double* val) {
  if (geometry == GEO_SQUARE_QUAD || geometry == GEO_CUBE_HEXA) {
    const int k = elem == EL_Q2 ? 2 : 1;
    double lx[3], ly[3], lz[3] = {1.0, 1.0, 1.0};
    lagrange1d(k, xi[0], lx);
    lagrange1d(k, xi[1], ly);
    const int dim = geometry == GEO_SQUARE_QUAD ? 2 : 3;
    if (dim == 3) lagrange1d(k, xi[2], lz);
    int m = 0;
    for (int c = 0; c <= (dim == 3 ? k : 0); ++c)
      for (int b = 0; b <= k; ++b)
        for (int a = 0; a <= k; ++a, ++m) val[m] = lx[a] * ly[b] * (dim == 3 ? lz[c] : 1.0);
    return;
  }
  const double x = xi[0], y = xi[1], z = xi[2];
  if (elem == EL_P1) {
    val[0] = 1.0 - x - y - z;
    val[1] = x;
    val[2] = y;
    val[3] = z;
    return;
  }
  // C_T_P2_3D_Funct (include/FE3D/BF_C_T_P2_3D.h)
  val[0] = 1.0 - 3.0 * x - 3.0 * y - 3.0 * z + 2.0 * x * x + 4.0 * x * y + 4.0 * x * z +
           2.0 * y * y + 4.0 * y * z + 2.0 * z * z;
  val[1] = 4.0 * x - 4.0 * x * x - 4.0 * x * y - 4.0 * x * z;
  val[2] = -x + 2.0 * x * x;
  val[3] = 4.0 * y - 4.0 * x * y - 4.0 * y * y - 4.0 * y * z;
  val[4] = 4.0 * x * y;
  val[5] = -y + 2.0 * y * y;
  val[6] = 4.0 * z - 4.0 * x * z - 4.0 * y * z - 4.0 * z * z;
  val[7] = 4.0 * x * z;
  val[8] = 4.0 * y * z;
  val[9] = -z + 2.0 * z * z;
}

void build_transfer(const Hierarchy& h, int fine_level, const Space& coarse, const Space& fine,
                    Csr& P, Csr& R) {
  const Level& Lf = h.levels.at(fine_level);
  const Level& Lc = h.levels.at(fine_level - 1);
  const int dim = h.dim, nvc = h.nvc;
  // full prolongation rows (every fine DOF), first fine cell containing the DOF
  std::vector<int> done(fine.n_dofs, 0);
  std::vector<std::vector<std::pair<int, double>>> rows(fine.n_dofs);
  std::vector<int64_t> nodes(size_t(fine.nloc) * dim);
  std::vector<double> val(coarse.nloc);
  for (int c = 0; c < Lf.n_cells; ++c) {
    const int p = Lf.parent[c];
    const int64_t* pv = &Lc.vtx[size_t(p) * nvc * dim];
    cell_nodes(h.geometry, fine.elem, &Lf.vtx[size_t(c) * nvc * dim], nodes.data());
    for (int m = 0; m < fine.nloc; ++m) {
      const int f = fine.dofmap[size_t(c) * fine.nloc + m];
      if (done[f]) continue;
      done[f] = 1;
      double xi[3];
      ref_coords(h.geometry, pv, &nodes[size_t(m) * dim], xi);
      basis_values(h.geometry, coarse.elem, xi, val.data());
      for (int j = 0; j < coarse.nloc; ++j)
        if (val[j] != 0.0) rows[f].push_back({coarse.dofmap[size_t(p) * coarse.nloc + j], val[j]});
      std::sort(rows[f].begin(), rows[f].end());
    }
  }
  P = Csr();
  P.n_rows = fine.n_dofs;
  P.n_cols = coarse.n_dofs;
  P.n_active = fine.n_active;
  P.row_ptr.assign(P.n_rows + 1, 0);
  for (int f = 0; f < fine.n_dofs; ++f) {
    if (f < fine.n_active)
      for (auto& e : rows[f]) {
        P.cols.push_back(e.first);
        P.vals.push_back(e.second);
      }
    P.row_ptr[f + 1] = int(P.cols.size());
  }
  // restriction = transpose of the full prolongation
  R = Csr();
  R.n_rows = coarse.n_dofs;
  R.n_cols = fine.n_dofs;
  R.n_active = coarse.n_active;
  R.row_ptr.assign(R.n_rows + 1, 0);
  for (int f = 0; f < fine.n_dofs; ++f)
    for (auto& e : rows[f]) R.row_ptr[e.first + 1]++;
  for (int i = 0; i < R.n_rows; ++i) R.row_ptr[i + 1] += R.row_ptr[i];
  R.cols.resize(R.row_ptr[R.n_rows]);
  R.vals.resize(R.row_ptr[R.n_rows]);
  std::vector<int> fill(R.row_ptr.begin(), R.row_ptr.end() - 1);
  for (int f = 0; f < fine.n_dofs; ++f)
    for (auto& e : rows[f]) {
      R.cols[fill[e.first]] = f;
      R.vals[fill[e.first]++] = e.second;
    }
}

std::vector<double> cell_vertices(const Hierarchy& h, int level) {
  const Level& L = h.levels.at(level);
  std::vector<double> out(L.vtx.size());
  const double inv = 1.0 / double(h.scale);
  const bool pow2 = (h.scale & (h.scale - 1)) == 0;
  for (size_t i = 0; i < out.size(); ++i)
    out[i] = pow2 ? double(L.vtx[i]) * inv : double(L.vtx[i]) / double(h.scale);
  return out;
}

}  // namespace pmsetup
