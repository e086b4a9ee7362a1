// Stokes P2/P1 (Taylor-Hood) on tetrahedra: element assembly, projected
// combined matrix and cell Vanka.
//
// Assembly restates NSLaplaceGradGrad, NSDivergenceBlocks and NSGradientBlocks
// (src/AssembleRoutinesSaddle/NSE_local_assembling_routines.C:82-225) for the
// Stokes Galerkin form with the Laplace operator on affine tetrahedra
// (src/FE/TetraAffin.C:886) and the P4Tetra rule (P4Exact,
// src/QuadFormulas/QuadFormulaTetra.C:73): per cell
//   A_ij   =  nu sum_q w |det J| grad phi_i . grad phi_j   (same in A11,A22,A33)
//   B_k,ij = -sum_q w |det J| psi_i d_k phi_j,   B^T_k = B_k transposed
// computed as contractions of reference tensors over the same quadrature.
// The projected matrix is get_combined_submatrix with the pressure projection
// (src/Matrix/BlockFEMatrix.C:1168-1345). Cell Vanka restates
// VankaSmoother::smooth (src/Multigrid/VankaSmoother.C:110-292).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "pm_stokes.h"
#include "pm_tetra.h"

namespace pm {

// ------------------------------------------------------------- tables ------
// the P4Tetra / P5Tetra rules and the P2 basis: pm_tetra.h

// layout: S[6][100] | D[3][40] | phi2[qn][10] | w[qn] | xi[qn][3] | C[3][10][10][10]
static constexpr int kOffS = 0, kOffD = 600, kOffPhi = 720;
__host__ __device__ constexpr int tab_off_w(int qn) { return kOffPhi + 10 * qn; }
__host__ __device__ constexpr int tab_off_xi(int qn) { return tab_off_w(qn) + qn; }
__host__ __device__ constexpr int tab_off_c(int qn) { return tab_off_xi(qn) + 3 * qn; }
__host__ __device__ constexpr int tab_size(int qn) { return tab_off_c(qn) + 3000; }

void DevStokesTables::upload(pm_ctx* c, int nq, bool skew) {
  if (nq != kP4n && nq != kP5n) throw Error(PM_E_UNSUPPORTED, "Stokes tables: 11 or 15 quadrature points");
  qn = nq;
  const double* qw = nq == kP4n ? kP4w : kP5w;
  const double* qx = nq == kP4n ? kP4x : kP5x;
  const double* qy = nq == kP4n ? kP4y : kP5y;
  const double* qz = nq == kP4n ? kP4z : kP5z;
  std::vector<double> t(tab_size(nq), 0.0);
  std::vector<double> phi(nq * 10), d(3 * nq * 10), psi(nq * 4);
  for (int q = 0; q < nq; ++q) {
    p2_eval(qx[q], qy[q], qz[q], &phi[q * 10], &d[(0 * nq + q) * 10], &d[(1 * nq + q) * 10], &d[(2 * nq + q) * 10]);
    psi[q * 4 + 0] = 1 - qx[q] - qy[q] - qz[q];
    psi[q * 4 + 1] = qx[q];
    psi[q * 4 + 2] = qy[q];
    psi[q * 4 + 3] = qz[q];
  }
  auto D = [&](int a, int q, int i) { return d[(a * nq + q) * 10 + i]; };
  int k = 0;
  for (int a = 0; a < 3; ++a)
    for (int b = a; b < 3; ++b, ++k)
      for (int i = 0; i < 10; ++i)
        for (int j = 0; j < 10; ++j) {
          double s = 0.0;
          for (int q = 0; q < nq; ++q) {
            s += qw[q] * D(a, q, i) * D(b, q, j);
            if (a != b) s += qw[q] * D(b, q, i) * D(a, q, j);
          }
          t[kOffS + k * 100 + i * 10 + j] = s;
        }
  for (int a = 0; a < 3; ++a)
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 10; ++j) {
        double s = 0.0;
        for (int q = 0; q < nq; ++q) s += qw[q] * psi[q * 4 + i] * D(a, q, j);
        t[kOffD + a * 40 + i * 10 + j] = s;
      }
  for (int q = 0; q < nq; ++q) {
    for (int i = 0; i < 10; ++i) t[kOffPhi + q * 10 + i] = phi[q * 10 + i];
    t[tab_off_w(nq) + q] = qw[q];
    t[tab_off_xi(nq) + q * 3 + 0] = qx[q];
    t[tab_off_xi(nq) + q * 3 + 1] = qy[q];
    t[tab_off_xi(nq) + q * 3 + 2] = qz[q];
  }
  // C[a][i][j][k]: test function i, ansatz function j (derivative a), velocity
  // basis function k; for the skew-symmetric form (1/2) [((u.grad) phi_j,
  // phi_i) - ((u.grad) phi_i, phi_j)] (NSNonlinearTerm_skew_symmetric) its
  // antisymmetric part in (i, j)
  auto conv = [&](int a, int i, int j, int l) {
    double s = 0.0;
    for (int q = 0; q < nq; ++q) s += qw[q] * phi[q * 10 + i] * D(a, q, j) * phi[q * 10 + l];
    return s;
  };
  for (int a = 0; a < 3; ++a)
    for (int i = 0; i < 10; ++i)
      for (int j = 0; j < 10; ++j)
        for (int l = 0; l < 10; ++l)
          t[tab_off_c(nq) + a * 1000 + i * 100 + j * 10 + l] =
              skew ? 0.5 * (conv(a, i, j, l) - conv(a, j, i, l)) : conv(a, i, j, l);
  data.upload(t, c->stream);
}

void DevStokesLevel::upload(pm_ctx* c, const DiscLevel& L) {
  n_cells = L.n_cells;
  n = L.sys.n_rows;
  verts.upload(L.verts, c->stream);
  gat_ptr.upload(L.gat_ptr, c->stream);
  gat_idx.upload(L.gat_idx, c->stream);
  rgat_ptr.upload(L.rgat_ptr, c->stream);
  rgat_idx.upload(L.rgat_idx, c->stream);
  diag_pos.upload(L.diag_pos, c->stream);
  nvel = L.block_len[0];
  nvel_active = L.block_active[0];
  np = L.block_len[3];
  bnd_xyz.upload(L.bnd_xyz, c->stream);
  udof.upload(L.space.dofmap, c->stream);
  // pressure integral weights: the P1 integral over a cell is |K| / 4 times
  // the sum of its vertex values
  std::vector<double> w(np, 0.0);
  measure = 0.0;
  for (int cell = 0; cell < n_cells; ++cell) {
    const double* v = L.verts.data() + size_t(cell) * 12;
    double J[3][3];
    for (int d = 0; d < 3; ++d)
      for (int a = 0; a < 3; ++a) J[d][a] = v[3 * (a + 1) + d] - v[d];
    const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                       J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                       J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    const double vol = std::fabs(det) / 6.0;
    measure += vol;
    for (int k = 0; k < 4; ++k) w[L.pspace.dofmap[size_t(cell) * 4 + k]] += vol / 4.0;
  }
  pweight.upload(w, c->stream);
}

void DevStokesLevel::set_children(pm_ctx* c, const pmsetup::Level& fine, const DiscLevel& L) {
  std::vector<int> ch(size_t(n_cells) * 8, -1);
  for (int f = 0; f < fine.n_cells; ++f) {
    const int par = fine.parent[f], j = fine.child_no[f];
    if (par < 0 || par >= n_cells || j < 0 || j >= 8) throw Error(PM_E_INVALID, "tetrahedral refinement: bad parent");
    ch[size_t(par) * 8 + j] = f;
  }
  for (int v : ch)
    if (v < 0) throw Error(PM_E_INVALID, "tetrahedral refinement: a cell without 8 children");
  children.upload(ch, c->stream);
  std::vector<int> ip(nvel + 1, 0), ix(size_t(n_cells) * 10);
  for (int e = 0; e < n_cells * 10; ++e) ip[L.space.dofmap[e] + 1]++;
  for (int d = 0; d < nvel; ++d) ip[d + 1] += ip[d];
  std::vector<int> fill(ip.begin(), ip.end() - 1);
  for (int e = 0; e < n_cells * 10; ++e) ix[fill[L.space.dofmap[e]]++] = e;  // cell order
  vinc_ptr.upload(ip, c->stream);
  vinc_idx.upload(ix, c->stream);
}

// right-hand side f = -nu Lap u + grad p of the manufactured Stokes solution
// (example 0 / -3); with `convective` the example -3 body force of the
// Navier-Stokes equations, which adds (u . grad) u
__device__ void stokes_f(double nu, const double* x, double* f, int example, bool convective = false) {
  if (example == -3) {
    // u = (y^2, xz, -y^2): Lap u = (2, 0, -2); grad p = (1, 1, 1);
    // (u . grad) u = (2xyz, y^2 z - x y^2, -2xyz)
    const double X = x[0], Y = x[1], Z = x[2];
    const double c0 = convective ? 2.0 * X * Y * Z : 0.0;
    const double c1 = convective ? Y * Y * Z - X * Y * Y : 0.0;
    f[0] = -nu * 2.0 + c0 + 1.0;
    f[1] = -nu * 0.0 + c1 + 1.0;
    f[2] = -nu * -2.0 - c0 + 1.0;
    return;
  }
  const double p = 3.14159265358979323846;
  double S[3], S1[3], S2[3], S3[3];
  for (int d = 0; d < 3; ++d) {
    double s, c;
    sincospi(x[d], &s, &c);
    double s2, c2;
    sincospi(2.0 * x[d], &s2, &c2);
    S[d] = s * s;                    // sin^2(pi t)
    S1[d] = p * s2;                  // d/dt
    S2[d] = 2 * p * p * c2;          // d2/dt2
    S3[d] = -4 * p * p * p * s2;     // d3/dt3
  }
  // derivatives of Lap psi, psi = S(x) S(y) S(z)
  const double lx = S3[0] * S[1] * S[2] + S1[0] * S2[1] * S[2] + S1[0] * S[1] * S2[2];
  const double ly = S2[0] * S1[1] * S[2] + S[0] * S3[1] * S[2] + S[0] * S1[1] * S2[2];
  const double lz = S2[0] * S[1] * S1[2] + S[0] * S2[1] * S1[2] + S[0] * S[1] * S3[2];
  // Lap u = curl(Lap psi (1,1,1)); grad p = (1,1,1)
  f[0] = -nu * (ly - lz) + 1.0;
  f[1] = -nu * (lz - lx) + 1.0;
  f[2] = -nu * (lx - ly) + 1.0;
}

// one block per CHUNK cells: per-cell geometry factors, then the element
// matrix as contractions of the reference tensors (A part: stiffness and,
// with a velocity u, the convective term; B part) and, with F, the element
// right-hand side on the NQ-point rule
template <int CHUNK, int NQ>
__global__ void __launch_bounds__(256) k_elem_stokes(int n_cells, const double* __restrict__ verts,
                                                     const double* __restrict__ tab, double nu,
                                                     double* __restrict__ K, double* __restrict__ F, int example,
                                                     bool convective_f, const double* __restrict__ u,
                                                     const int* __restrict__ udof, int nvel) {
  constexpr int kW = tab_off_w(NQ), kXi = tab_off_xi(NQ), kC = tab_off_c(NQ);
  __shared__ double cS[CHUNK][6];
  __shared__ double cB[CHUNK][9];
  __shared__ double geo[CHUNK][13];
  __shared__ double cG[CHUNK][9];
  __shared__ double cV[CHUNK][30];  // |det J| sum_d G[d][a] u_d,k
  __shared__ double fq[CHUNK][NQ][3];
  const int c0 = blockIdx.x * CHUNK;
  const int nc = min(CHUNK, n_cells - c0);
  const int t = threadIdx.x;
  if (t < nc) {
    const double* v = verts + (size_t)(c0 + t) * 12;
    double J[3][3];
    for (int d = 0; d < 3; ++d) {
      J[d][0] = v[3 + d] - v[d];
      J[d][1] = v[6 + d] - v[d];
      J[d][2] = v[9 + d] - v[d];
    }
    const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                       J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                       J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    const double r = 1.0 / det;
    double G[3][3];  // J^{-T}: d_k phi = sum_a G[k][a] dhat_a phi
    G[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * r;
    G[0][1] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]) * r;
    G[0][2] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * r;
    G[1][0] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) * r;
    G[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
    G[1][2] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) * r;
    G[2][0] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
    G[2][1] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) * r;
    G[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
    const double adet = fabs(det);
    int k = 0;
    for (int a = 0; a < 3; ++a)
      for (int b = a; b < 3; ++b) {
        double s = 0.0;
        for (int d = 0; d < 3; ++d) s += G[d][a] * G[d][b];
        cS[t][k++] = nu * adet * s;
      }
    for (int kk = 0; kk < 3; ++kk)
      for (int a = 0; a < 3; ++a) {
        cB[t][kk * 3 + a] = -adet * G[kk][a];
        cG[t][kk * 3 + a] = adet * G[kk][a];
      }
    for (int d = 0; d < 3; ++d) {
      geo[t][d] = v[d];
      for (int a = 0; a < 3; ++a) geo[t][3 + d * 3 + a] = J[d][a];
    }
    geo[t][12] = adet;
  }
  __syncthreads();
  if (u) {
    for (int e = t; e < nc * 30; e += blockDim.x) {
      const int cl = e / 30, ak = e % 30, a = ak / 10, k = ak % 10;
      const int g = udof[(size_t)(c0 + cl) * 10 + k];
      double s = 0.0;
      for (int d = 0; d < 3; ++d) s += cG[cl][d * 3 + a] * u[(size_t)d * nvel + g];
      cV[cl][ak] = s;
    }
  }
  if (F) {
    for (int e = t; e < nc * NQ; e += blockDim.x) {
      const int cl = e / NQ, q = e % NQ;
      double x[3];
      for (int d = 0; d < 3; ++d) {
        double s = geo[cl][d];
        for (int a = 0; a < 3; ++a) s += geo[cl][3 + d * 3 + a] * tab[kXi + q * 3 + a];
        x[d] = s;
      }
      double f[3];
      stokes_f(nu, x, f, example, convective_f);
      const double m = tab[kW + q] * geo[cl][12];
      for (int d = 0; d < 3; ++d) fq[cl][q][d] = m * f[d];
    }
  }
  __syncthreads();
  for (int e = t; e < nc * 220; e += blockDim.x) {
    const int cl = e / 220, p = e % 220;
    double s = 0.0;
    if (p < 100) {
#pragma unroll
      for (int k = 0; k < 6; ++k) s = fma(cS[cl][k], __ldg(tab + kOffS + k * 100 + p), s);
      if (u) {
        // N_ij = sum_a sum_k V[a][k] C[a][i][j][k], p = i * 10 + j
        double nsum = 0.0;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const double* Ca = tab + kC + a * 1000 + p * 10;
#pragma unroll
          for (int k = 0; k < 10; ++k) nsum = fma(cV[cl][a * 10 + k], __ldg(Ca + k), nsum);
        }
        s += nsum;
      }
    } else {
      const int kk = (p - 100) / 40, ij = (p - 100) % 40;
#pragma unroll
      for (int a = 0; a < 3; ++a) s = fma(cB[cl][kk * 3 + a], __ldg(tab + kOffD + a * 40 + ij), s);
    }
    K[(size_t)(c0 + cl) * 220 + p] = s;
  }
  if (F) {
    for (int e = t; e < nc * 34; e += blockDim.x) {
      const int cl = e / 34, m = e % 34;
      double s = 0.0;
      if (m < 30) {
        const int comp = m / 10, i = m % 10;
        for (int q = 0; q < NQ; ++q) s += fq[cl][q][comp] * tab[kOffPhi + q * 10 + i];
      }
      F[(size_t)(c0 + cl) * 34 + m] = s;
    }
  }
}

__global__ void k_gather_stokes(int nnz, const int* __restrict__ ptr, const int* __restrict__ idx,
                                const double* __restrict__ K, double* __restrict__ vals) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int t = ptr[e]; t < ptr[e + 1]; ++t) s += K[idx[t]];
    vals[e] = s;
  }
}

__global__ void k_unit_diag(int n, const int* __restrict__ pos, double* __restrict__ vals) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) vals[pos[i]] = 1.0;
}

// Dirichlet values of example -3 at the non-active velocity DOFs of the three
// components ([u1 | u2 | u3 | p] layout)
__global__ void k_stokes_dirichlet(int nb, int nvel, int nact, const double* __restrict__ xyz,
                                   double* __restrict__ rhs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  rhs[nact + i] = y * y;
  rhs[nvel + nact + i] = x * z;
  rhs[2 * nvel + nact + i] = -y * y;
}

static void launch_elem_stokes(pm_ctx* c, const DevStokesLevel& L, const DevStokesTables& t, double nu,
                               double* K, double* F, int example, bool convective_f, const double* u) {
  constexpr int CHUNK = 32;
  const int g = (L.n_cells + CHUNK - 1) / CHUNK;
  if (t.qn == kP4n)
    k_elem_stokes<CHUNK, kP4n><<<g, 256, 0, c->stream>>>(L.n_cells, L.verts.p, t.data.p, nu, K, F, example,
                                                          convective_f, u, L.udof.p, L.nvel);
  else
    k_elem_stokes<CHUNK, kP5n><<<g, 256, 0, c->stream>>>(L.n_cells, L.verts.p, t.data.p, nu, K, F, example,
                                                          convective_f, u, L.udof.p, L.nvel);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

// element storage -> matrix values (and right-hand side)
static void gather_stokes(pm_ctx* c, const DevStokesLevel& L, DevCsr& A, double* rhs, const double* K,
                          const double* F, int example) {
  const int nnz = int(A.nnz);
  const int g = std::max(1, std::min((nnz + 255) / 256, c->num_sms * 16));
  k_gather_stokes<<<g, 256, 0, c->stream>>>(nnz, L.gat_ptr.p, L.gat_idx.p, K, A.vals.p);
  PM_CHECK_LAUNCH();
  const int nd = int(L.diag_pos.n);
  if (nd) {
    k_unit_diag<<<(nd + 255) / 256, 256, 0, c->stream>>>(nd, L.diag_pos.p, A.vals.p);
    PM_CHECK_LAUNCH();
  }
  c->kernel_launches += nd ? 2 : 1;
  if (rhs) {
    const int gr = std::max(1, std::min((L.n + 255) / 256, c->num_sms * 16));
    k_gather_stokes<<<gr, 256, 0, c->stream>>>(L.n, L.rgat_ptr.p, L.rgat_idx.p, F, rhs);
    PM_CHECK_LAUNCH();
    c->kernel_launches++;
    const int nb = L.nvel - L.nvel_active;
    if (example == -3 && nb > 0) {
      k_stokes_dirichlet<<<(nb + 255) / 256, 256, 0, c->stream>>>(nb, L.nvel, L.nvel_active, L.bnd_xyz.p, rhs);
      PM_CHECK_LAUNCH();
      c->kernel_launches++;
    }
  }
  A.values_changed(c);
}

void assemble_stokes_level(pm_ctx* c, const DevStokesLevel& L, const DevStokesTables& t, double nu,
                           DevCsr& A, double* rhs, double* K, double* F, int example) {
  if (example != 0 && example != -3) throw Error(PM_E_UNSUPPORTED, "Stokes example must be 0 or -3");
  launch_elem_stokes(c, L, t, nu, K, F, example, false, nullptr);
  gather_stokes(c, L, A, rhs, K, F, example);
}

void assemble_nse_level(pm_ctx* c, const DevStokesLevel& L, const DevStokesTables& t, double nu, DevCsr& A,
                        const double* u, double* rhs, double* K, double* F) {
  launch_elem_stokes(c, L, t, nu, K, rhs ? F : nullptr, -3, true, u);
  gather_stokes(c, L, A, rhs, K, F, -3);
}

// ------------------------------------------------------ restriction --------
void build_p2_restriction(const pmsetup::Hierarchy& h, std::vector<double>& q) {
  if (h.geometry != pmsetup::GEO_CUBE_TETRA || h.levels.size() < 2)
    throw Error(PM_E_INVALID, "P2 restriction needs a refined tetrahedral hierarchy");
  const pmsetup::Level& L0 = h.levels[0];
  const pmsetup::Level& L1 = h.levels[1];
  const double s = 1.0 / double(h.scale);
  auto vtx = [&](const pmsetup::Level& L, int cell, int v, int d) {
    return double(L.vtx[(size_t(cell) * 4 + v) * 3 + d]) * s;
  };
  // parent 0: x = v0 + J xi
  double J[3][3], Ji[3][3];
  for (int d = 0; d < 3; ++d)
    for (int a = 0; a < 3; ++a) J[d][a] = vtx(L0, 0, a + 1, d) - vtx(L0, 0, 0, d);
  const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                     J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
  Ji[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) / det;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
  Ji[1][0] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]) / det;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
  Ji[1][2] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) / det;
  Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
  Ji[2][1] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) / det;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  // mass matrix of the parent's basis on the reference cell (P4Tetra: exact)
  double G[10][10] = {};
  double phi[10], dx[10], dy[10], dz[10];
  for (int qq = 0; qq < kP4n; ++qq) {
    p2_eval(kP4x[qq], kP4y[qq], kP4z[qq], phi, dx, dy, dz);
    for (int i = 0; i < 10; ++i)
      for (int j = 0; j < 10; ++j) G[i][j] += kP4w[qq] * phi[i] * phi[j];
  }
  q.assign(8 * 100, 0.0);
  int found = 0;
  for (int f = 0; f < L1.n_cells; ++f) {
    if (L1.parent[f] != 0) continue;
    const int ch = L1.child_no[f];
    ++found;
    // child vertices in the parent's reference coordinates
    double xi[4][3];
    for (int v = 0; v < 4; ++v)
      for (int a = 0; a < 3; ++a) {
        double sum = 0.0;
        for (int d = 0; d < 3; ++d) sum += Ji[a][d] * (vtx(L1, f, v, d) - vtx(L0, 0, 0, d));
        xi[v][a] = sum;
      }
    double Jc[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) Jc[a][b] = xi[b + 1][a] - xi[0][a];
    const double dc = std::fabs(Jc[0][0] * (Jc[1][1] * Jc[2][2] - Jc[1][2] * Jc[2][1]) -
                                Jc[0][1] * (Jc[1][0] * Jc[2][2] - Jc[1][2] * Jc[2][0]) +
                                Jc[0][2] * (Jc[1][0] * Jc[2][1] - Jc[1][1] * Jc[2][0]));
    // R[k][l] = (parent k, child l) over the child (P4Tetra on the child)
    double R[10][10] = {};
    double phc[10], php[10];
    for (int qq = 0; qq < kP4n; ++qq) {
      p2_eval(kP4x[qq], kP4y[qq], kP4z[qq], phc, dx, dy, dz);
      double pt[3];
      for (int a = 0; a < 3; ++a)
        pt[a] = xi[0][a] + Jc[a][0] * kP4x[qq] + Jc[a][1] * kP4y[qq] + Jc[a][2] * kP4z[qq];
      p2_eval(pt[0], pt[1], pt[2], php, dx, dy, dz);
      for (int k = 0; k < 10; ++k)
        for (int l = 0; l < 10; ++l) R[k][l] += kP4w[qq] * dc * php[k] * phc[l];
    }
    // Q = G^{-1} R by Gauss-Jordan with partial pivoting
    double M[10][20];
    for (int i = 0; i < 10; ++i)
      for (int j = 0; j < 10; ++j) {
        M[i][j] = G[i][j];
        M[i][10 + j] = R[i][j];
      }
    for (int k = 0; k < 10; ++k) {
      int pr = k;
      for (int i = k + 1; i < 10; ++i)
        if (std::fabs(M[i][k]) > std::fabs(M[pr][k])) pr = i;
      for (int j = 0; j < 20; ++j) std::swap(M[k][j], M[pr][j]);
      const double pv = M[k][k];
      for (int j = 0; j < 20; ++j) M[k][j] /= pv;
      for (int i = 0; i < 10; ++i) {
        if (i == k) continue;
        const double fct = M[i][k];
        for (int j = 0; j < 20; ++j) M[i][j] -= fct * M[k][j];
      }
    }
    for (int k = 0; k < 10; ++k)
      for (int l = 0; l < 10; ++l) q[size_t(ch) * 100 + k * 10 + l] = M[k][10 + l];
  }
  if (found != 8) throw Error(PM_E_INVALID, "P2 restriction: the root cell has no 8 children");
}

// one thread per (coarse cell, component, coarse local DOF): sum over the
// children j (in order) of sum_l Q_j[k][l] u(child j, l)
__global__ void k_restrict_cells(int n_coarse, const int* __restrict__ children, const int* __restrict__ fdof,
                                 const double* __restrict__ q, const double* __restrict__ uf, int nvf,
                                 double* __restrict__ cellval) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_coarse * 30) return;
  const int cell = e / 30, comp = (e % 30) / 10, k = e % 10;
  double acc = 0.0;
  for (int j = 0; j < 8; ++j) {
    const int f = children[(size_t)cell * 8 + j];
    const int* fd = fdof + (size_t)f * 10;
    const double* Q = q + j * 100 + k * 10;
    double s = 0.0;
    for (int l = 0; l < 10; ++l) s += Q[l] * uf[(size_t)comp * nvf + fd[l]];
    acc += s;
  }
  cellval[e] = acc;
}

// coarse DOF d: the cell values at its positions, in cell order, averaged
__global__ void k_restrict_average(int nvc, const int* __restrict__ ip, const int* __restrict__ ix,
                                   const double* __restrict__ cellval, double* __restrict__ uc) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 3 * nvc) return;
  const int comp = e / nvc, d = e % nvc;
  double s = 0.0;
  for (int t = ip[d]; t < ip[d + 1]; ++t) {
    const int pos = ix[t];
    s += cellval[(size_t)(pos / 10) * 30 + comp * 10 + pos % 10];
  }
  const int cnt = ip[d + 1] - ip[d];
  uc[e] = cnt ? s / double(cnt) : 0.0;
}

void restrict_velocity(pm_ctx* c, const DevStokesLevel& coarse, const DevStokesLevel& fine, const double* q,
                       const double* u_fine, double* u_coarse, double* cellval) {
  if (!coarse.children.p) throw Error(PM_E_INVALID, "restriction: the coarse level has no children map");
  const int nw = coarse.n_cells * 30;
  k_restrict_cells<<<(nw + 255) / 256, 256, 0, c->stream>>>(coarse.n_cells, coarse.children.p, fine.udof.p, q,
                                                            u_fine, fine.nvel, cellval);
  PM_CHECK_LAUNCH();
  const int nd = 3 * coarse.nvel;
  k_restrict_average<<<(nd + 255) / 256, 256, 0, c->stream>>>(coarse.nvel, coarse.vinc_ptr.p, coarse.vinc_idx.p,
                                                              cellval, u_coarse);
  PM_CHECK_LAUNCH();
  c->kernel_launches += 2;
}

// ------------------------------------------- pressure projection, residuals --
// one block: the weighted sum in a fixed order, then p -= sum / measure
__global__ void __launch_bounds__(1024) k_project_l20(int np, const double* __restrict__ w, double measure,
                                                       double* __restrict__ p) {
  __shared__ double red[32];
  __shared__ double mean;
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += w[i] * p[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int k = 0; k < int(blockDim.x >> 5); ++k) tot += red[k];
    mean = tot / measure;
  }
  __syncthreads();
  const double m = mean;
  for (int i = threadIdx.x; i < np; i += blockDim.x) p[i] -= m;
}

void project_pressure_l20(pm_ctx* c, const DevStokesLevel& L, double* p) {
  k_project_l20<<<1, 1024, 0, c->stream>>>(L.np, L.pweight.p, L.measure, p);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

// the squared norms of the blocks [0, nv), [nv, 2 nv), [2 nv, 3 nv) and
// [3 nv, n): per thread block four partial sums over a contiguous chunk (in a
// fixed order), then one block adds the partials in block order
constexpr int kNormBlocks = 256;
static_assert(kResidualScratch >= 4 + 4 * kNormBlocks, "the residual scratch holds the partial sums");
__global__ void __launch_bounds__(256) k_block_norm_partials(int nv, int n, const double* __restrict__ d,
                                                             double* __restrict__ part) {
  __shared__ double red[4][8];
  const int chunk = (n + gridDim.x - 1) / gridDim.x;
  const int beg = blockIdx.x * chunk, end = min(n, beg + chunk);
  double a[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = beg + threadIdx.x; i < end; i += blockDim.x) {
    const double v = d[i];
    const int b = min(i / nv, 3);
#pragma unroll
    for (int k = 0; k < 4; ++k) a[k] += (k == b) ? v * v : 0.0;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    for (int o = 16; o > 0; o >>= 1) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
    if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = a[k];
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double sum = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) sum += red[threadIdx.x][w];
    part[blockIdx.x * 4 + threadIdx.x] = sum;
  }
}

__global__ void k_block_norm_finish(int nb, const double* __restrict__ part, double* __restrict__ out4) {
  if (threadIdx.x < 4) {
    double sum = 0.0;
    for (int b = 0; b < nb; ++b) sum += part[b * 4 + threadIdx.x];
    out4[threadIdx.x] = sum;
  }
}

void nse_residuals(pm_ctx* c, const DevStokesLevel& L, const DevCsr& A, const double* rhs, const double* x,
                   double* d, double* out4) {
  csr_apply(c, A, EPI_DEFECT, x, d, rhs, 1.0);
  project_pressure_l20(c, L, d + 3 * size_t(L.nvel));
  // the partials go to out4 + 4 (the caller's buffer holds 4 + 4 kNormBlocks)
  k_block_norm_partials<<<kNormBlocks, 256, 0, c->stream>>>(L.nvel, L.n, d, out4 + 4);
  k_block_norm_finish<<<1, 32, 0, c->stream>>>(kNormBlocks, out4 + 4, out4);
  PM_CHECK_LAUNCH();
  c->kernel_launches += 2;
}

// --------------------------------------------------- projected matrix ------
void ProjectedMatrix::build(pm_ctx* c, const pmsetup::Csr& sys, int p0, const BlockMask& mask) {
  std::vector<int> rp(sys.n_rows + 1, 0), ci, sr;
  for (int i = 0; i < sys.n_rows; ++i) {
    if (i == p0) {
      ci.push_back(p0);
      sr.push_back(-1);
    } else {
      for (int k = sys.row_ptr[i]; k < sys.row_ptr[i + 1]; ++k) {
        ci.push_back(sys.cols[k]);
        sr.push_back(k);
      }
    }
    rp[i + 1] = int(ci.size());
  }
  csr.upload(c, sys.n_rows, sys.n_cols, sys.n_active, rp.data(), ci.data(), nullptr);
  csr.mask = mask;
  src.upload(sr, c->stream);
}

__global__ void k_project_vals(int nnz, const int* __restrict__ src, const double* __restrict__ v,
                               double* __restrict__ out) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += gridDim.x * blockDim.x) {
    const int s = src[e];
    out[e] = s >= 0 ? v[s] : 1.0;
  }
}

void ProjectedMatrix::refresh(pm_ctx* c, const DevCsr& sys, bool fp32) {
  const int nnz = int(csr.nnz);
  k_project_vals<<<std::max(1, std::min((nnz + 255) / 256, c->num_sms * 16)), 256, 0, c->stream>>>(
      nnz, src.p, sys.vals.p, csr.vals.p);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
  csr.values_changed(c);
  csr.make_sliced64(c);
  if (fp32) csr.make_fp32(c);
}

// ------------------------------------------------------------- Vanka -------
void DevVanka::setup(pm_ctx* c, const DiscLevel& L) {
  n_cells = L.n_cells;
  n = L.sys.n_rows;
  patch.upload(L.patch_dofs, c->stream);
  std::vector<int> fz(n_cells, 0);
  n_frozen = 0;
  for (int cell = 0; cell < n_cells; ++cell) {
    // the 3 rows of each active velocity node must control the cell's
    // pressures: 4, or 3 when the cell holds the first pressure DOF, whose row
    // is a unit row of the projected matrix; otherwise the local matrix is
    // singular
    int n_act = 0, need = 4;
    for (int k = 0; k < 10; ++k)
      if (L.space.dofmap[size_t(cell) * 10 + k] < L.space.n_active) ++n_act;
    for (int j = 0; j < 4; ++j)
      if (L.pspace.dofmap[size_t(cell) * 4 + j] == 0) need = 3;
    if (3 * n_act < need) {
      fz[cell] = 4;
      ++n_frozen;
    }
  }
  freeze.upload(fz, c->stream);
  std::vector<int> ip(n + 1, 0), ix, cnt(n, 0);
  for (int d : L.patch_dofs) ip[d + 1]++;
  for (int i = 0; i < n; ++i) {
    cnt[i] = ip[i + 1];
    ip[i + 1] += ip[i];
  }
  ix.resize(ip[n]);
  std::vector<int> fill(ip.begin(), ip.end() - 1);
  for (size_t t = 0; t < L.patch_dofs.size(); ++t) ix[fill[L.patch_dofs[t]]++] = int(t);
  inc_ptr.upload(ip, c->stream);
  inc_idx.upload(ix, c->stream);
  count.upload(cnt, c->stream);
  color_ptr = L.color_ptr;
  color_cells.upload(L.color_cells, c->stream);
  sol.ensure(size_t(n_cells) * 34);
  flag.ensure(1);
}

// local matrix of one cell from the projected CSR, inverted by Gauss-Jordan
// with partial pivoting in shared memory; stored column-major
template <class T>
__global__ void __launch_bounds__(128) k_vanka_factor(int n_cells, const int* __restrict__ patch,
                                                      const int* __restrict__ rp, const int* __restrict__ ci,
                                                      const T* __restrict__ v, const int* __restrict__ freeze,
                                                      T* __restrict__ inv, int* __restrict__ flag) {
  __shared__ T M[34][35];
  __shared__ T Inv[34][35];
  __shared__ int dof[34];
  __shared__ int piv_row;
  __shared__ T colk[34];
  const int cell = blockIdx.x;
  const int t = threadIdx.x;
  if (cell >= n_cells) return;
  if (t < 34) dof[t] = patch[(size_t)cell * 34 + t];
  for (int e = t; e < 34 * 35; e += blockDim.x) {
    (&M[0][0])[e] = T(0);
    (&Inv[0][0])[e] = T(0);
  }
  __syncthreads();
  if (t < 34) {
    Inv[t][t] = T(1);
    // entries of global row dof[t] whose column is in the patch
    const int r = dof[t];
    for (int k = rp[r]; k < rp[r + 1]; ++k) {
      const T a = v[k];
      if (a == T(0)) continue;
      const int col = ci[k];
      int lo = 0, hi = 33;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (dof[mid] < col) lo = mid + 1;
        else hi = mid;
      }
      if (dof[lo] == col) M[t][lo] = a;
    }
  }
  __syncthreads();
  const int nf = freeze[cell];
  if (nf) {
    // frozen trailing pressures: unit rows and columns
    for (int e = t; e < 34 * nf; e += blockDim.x) {
      const int f = 34 - nf + e / 34, k = e % 34;
      M[f][k] = T(0);
      M[k][f] = T(0);
    }
    __syncthreads();
    if (t < nf) M[34 - nf + t][34 - nf + t] = T(1);
    __syncthreads();
  }
  for (int k = 0; k < 34; ++k) {
    if (t == 0) {
      int p = k;
      T best = fabs(M[k][k]);
      for (int i = k + 1; i < 34; ++i)
        if (fabs(M[i][k]) > best) {
          best = fabs(M[i][k]);
          p = i;
        }
      piv_row = p;
      if (!(best > T(0))) atomicExch(flag, 1);
    }
    __syncthreads();
    const int p = piv_row;
    if (p != k)
      for (int j = t; j < 34; j += blockDim.x) {
        T a = M[k][j];
        M[k][j] = M[p][j];
        M[p][j] = a;
        T b = Inv[k][j];
        Inv[k][j] = Inv[p][j];
        Inv[p][j] = b;
      }
    __syncthreads();
    const T pivv = M[k][k] != T(0) ? M[k][k] : T(1);
    if (t < 34) colk[t] = M[t][k];
    __syncthreads();
    for (int j = t; j < 34; j += blockDim.x) {
      M[k][j] /= pivv;
      Inv[k][j] /= pivv;
    }
    __syncthreads();
    for (int e = t; e < 34 * 34; e += blockDim.x) {
      const int i = e / 34, j = e % 34;
      if (i == k) continue;
      const T f = colk[i];
      M[i][j] -= f * M[k][j];
      Inv[i][j] -= f * Inv[k][j];
    }
    __syncthreads();
  }
  T* out = inv + (size_t)cell * 34 * 34;
  for (int e = t; e < 34 * 34; e += blockDim.x) {
    const int j = e / 34, i = e % 34;  // column-major: out[j*34 + i] = Inv[i][j]
    out[e] = (i >= 34 - nf || j >= 34 - nf) ? T(0) : Inv[i][j];  // frozen: no update
  }
}

void DevVanka::factor(pm_ctx* c, const DevCsr& V, bool fp32) {
  PM_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), c->stream));
  if (fp32) {
    inv32.ensure(size_t(n_cells) * 34 * 34);
    sol32.ensure(size_t(n_cells) * 34);
    k_vanka_factor<float><<<n_cells, 128, 0, c->stream>>>(n_cells, patch.p, V.row_ptr.p, V.cols.p,
                                                          V.vals32.p, freeze.p, inv32.p, flag.p);
  } else {
    inv.ensure(size_t(n_cells) * 34 * 34);
    k_vanka_factor<double><<<n_cells, 128, 0, c->stream>>>(n_cells, patch.p, V.row_ptr.p, V.cols.p,
                                                           V.vals.p, freeze.p, inv.p, flag.p);
  }
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
  int h = 0;
  PM_CUDA(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));
  if (h) throw Error(PM_E_BREAKDOWN, "singular local Vanka system");
}

// one warp per cell: s = damp * inv * r[patch]; written per cell (Jacobi) or
// added into x (colour-ordered sweep, after all local right-hand sides of
// the colour are computed)
template <class T>
__global__ void __launch_bounds__(256) k_vanka_local(const int* __restrict__ guard, int n_cells, const int* __restrict__ cells,
                                                     const int* __restrict__ patch, const T* __restrict__ inv,
                                                     const T* __restrict__ r, const T* __restrict__ rloc,
                                                     T* __restrict__ out, T* __restrict__ x, T damp) {
  if (guarded(guard)) return;  // uniform for the whole grid
  __shared__ T rl[8][34];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int idx = blockIdx.x * 8 + w;
  const bool valid = idx < n_cells;
  const int cell = valid ? (cells ? cells[idx] : idx) : 0;
  if (valid) {
    for (int j = lane; j < 34; j += 32)
      rl[w][j] = rloc ? rloc[(size_t)cell * 34 + j] : r[patch[(size_t)cell * 34 + j]];
  }
  __syncwarp();
  if (!valid) return;
  const T* I = inv + (size_t)cell * 1156;
  for (int i = lane; i < 34; i += 32) {
    T s = T(0);
    for (int j = 0; j < 34; ++j) s += I[j * 34 + i] * rl[w][j];
    if (x) x[patch[(size_t)cell * 34 + i]] += damp * s;
    else out[(size_t)cell * 34 + i] = damp * s;
  }
}

// x[d] += (sum over the patches containing d, in cell order) / count[d]
template <class T>
__global__ void k_vanka_average(const int* __restrict__ guard, int n, const int* __restrict__ ip, const int* __restrict__ ix,
                                const int* __restrict__ cnt, const T* __restrict__ sol, T* __restrict__ x) {
  if (guarded(guard)) return;  // uniform for the whole grid
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < n; d += gridDim.x * blockDim.x) {
    if (cnt[d] == 0) continue;
    T s = T(0);
    for (int t = ip[d]; t < ip[d + 1]; ++t) s += sol[ix[t]];
    x[d] += s / T(cnt[d]);
  }
}

// local right-hand sides b - V x of the cells of one colour (one warp per cell)
template <class T>
__global__ void __launch_bounds__(256) k_vanka_rhs(const int* __restrict__ guard, int n_cells, const int* __restrict__ cells,
                                                   const int* __restrict__ patch, const int* __restrict__ rp,
                                                   const int* __restrict__ ci, const T* __restrict__ v,
                                                   const T* __restrict__ b, const T* __restrict__ x,
                                                   T* __restrict__ rloc) {
  if (guarded(guard)) return;  // uniform for the whole grid
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= n_cells) return;
  const int cell = cells[w];
  for (int i = lane; i < 34; i += 32) {
    const int r = patch[(size_t)cell * 34 + i];
    T s = b[r];
    for (int k = rp[r]; k < rp[r + 1]; ++k) s -= v[k] * x[ci[k]];
    rloc[(size_t)cell * 34 + i] = s;
  }
}

template <class T>
static void jacobi_sweep(pm_ctx* c, DevVanka& vk, const DevCsr& V, const T* vals, const T* inv, T* sol,
                         const T* b, T* x, T* r, T damp) {
  // residual with the projected matrix (residual_glo in the reference)
  if constexpr (sizeof(T) == 8) csr_apply(c, V, EPI_DEFECT, x, r, b, 1.0);
  else csr_apply32(c, V, EPI_DEFECT, x, r, b, 1.0f);
  (void)vals;
  k_vanka_local<T><<<(vk.n_cells + 7) / 8, 256, 0, c->stream>>>(c->guard, vk.n_cells, nullptr, vk.patch.p, inv, r,
                                                                nullptr, sol, nullptr, damp);
  const int g = std::max(1, std::min((vk.n + 255) / 256, c->num_sms * 16));
  k_vanka_average<T><<<g, 256, 0, c->stream>>>(c->guard, vk.n, vk.inc_ptr.p, vk.inc_idx.p, vk.count.p, sol, x);
  PM_CHECK_LAUNCH();
  c->kernel_launches += 2;
}

void DevVanka::sweep_jacobi(pm_ctx* c, const DevCsr& V, const double* b, double* x, double* r, double damp) {
  jacobi_sweep<double>(c, *this, V, V.vals.p, inv.p, sol.p, b, x, r, damp);
}
void DevVanka::sweep_jacobi32(pm_ctx* c, const DevCsr& V, const float* b, float* x, float* r, float damp) {
  jacobi_sweep<float>(c, *this, V, V.vals32.p, inv32.p, sol32.p, b, x, r, damp);
}

template <class T>
static void colored_sweep(pm_ctx* c, DevVanka& vk, const DevCsr& V, const T* vals, const T* inv, T* rloc,
                          const T* b, T* x, T damp) {
  const int ncol = int(vk.color_ptr.size()) - 1;
  for (int k = 0; k < ncol; ++k) {
    const int beg = vk.color_ptr[k], cnt = vk.color_ptr[k + 1] - beg;
    if (!cnt) continue;
    const int* cells = vk.color_cells.p + beg;
    k_vanka_rhs<T><<<(cnt * 32 + 255) / 256, 256, 0, c->stream>>>(c->guard, cnt, cells, vk.patch.p, V.row_ptr.p, V.cols.p,
                                                                   vals, b, x, rloc);
    k_vanka_local<T><<<(cnt + 7) / 8, 256, 0, c->stream>>>(c->guard, cnt, cells, vk.patch.p, inv, nullptr, rloc, nullptr,
                                                           x, damp);
    c->kernel_launches += 2;
  }
  PM_CHECK_LAUNCH();
}

void DevVanka::sweep_colored(pm_ctx* c, const DevCsr& V, const double* b, double* x, double damp) {
  colored_sweep<double>(c, *this, V, V.vals.p, inv.p, sol.p, b, x, damp);
}
void DevVanka::sweep_colored32(pm_ctx* c, const DevCsr& V, const float* b, float* x, float damp) {
  colored_sweep<float>(c, *this, V, V.vals32.p, inv32.p, sol32.p, b, x, damp);
}

}  // namespace pm

// ------------------------------------------------------- nodal Vanka -------
namespace pm {

void DevNodalVanka::build_row_slices(pm_ctx* c, const pmsetup::Csr& S, int p0, const std::vector<int>& vp,
                                     const std::vector<int>& vi, const std::vector<int>& cp) {
  rs_ok = false;
  rs_lanes = 0;
  const int Lanes = c->nodal_sliced == 8 ? 8 : 4, C = 32 / Lanes;
  if (c->nodal_sliced == 0) return;
  // the projected structure: row p0 holds only its diagonal
  auto row_len = [&](int g) { return g == p0 ? 1 : S.row_ptr[g + 1] - S.row_ptr[g]; };
  auto proj_start = [&](int g) {  // first entry of row g in the projected arrays
    const int64_t shift = g > p0 ? int64_t(S.row_ptr[p0 + 1] - S.row_ptr[p0]) - 1 : 0;
    return int64_t(S.row_ptr[g]) - shift;
  };
  const size_t n_slots = size_t(3) * vi.size() + size_t(np);
  std::vector<int> slot_row(n_slots);
  for (int i = 0; i < np; ++i) {
    const int m = vp[i + 1] - vp[i];
    const size_t off = 3 * size_t(vp[i]) + i;
    for (int e = 0; e < 3 * m; ++e) slot_row[off + e] = (e / m) * nu + vi[vp[i] + e % m];
    slot_row[off + 3 * m] = 3 * nu + i;
  }
  const int ncol = int(color_ptr.size()) - 1;
  std::vector<int> perm, soff{0}, cols, src;
  color_slice.assign(size_t(ncol) + 1, 0);
  std::vector<int> rows;
  int64_t total = 0;
  for (int k = 0; k < ncol; ++k) {
    rows.clear();
    for (int t = color_ptr[k]; t < color_ptr[k + 1]; ++t) {
      const int i = cp[t], m = vp[i + 1] - vp[i];
      const int off = 3 * vp[i] + i;
      for (int e = 0; e <= 3 * m; ++e) rows.push_back(off + e);
    }
    // longest rows first (ties in slot order): slices of similar rows
    std::stable_sort(rows.begin(), rows.end(),
                     [&](int a, int b) { return row_len(slot_row[a]) > row_len(slot_row[b]); });
    const int nsl = int((rows.size() + C - 1) / C);
    for (int sl = 0; sl < nsl; ++sl) {
      int width = 0;
      for (int q = 0; q < C; ++q) {
        const size_t r = size_t(sl) * C + q;
        perm.push_back(r < rows.size() ? rows[r] : -1);
        if (r < rows.size()) width = std::max(width, row_len(slot_row[rows[r]]));
      }
      const int T = (width + Lanes - 1) / Lanes;
      if (total + int64_t(32) * T > int64_t(0x7fffffff)) return;  // the residual kernel stays
      cols.resize(size_t(total) + size_t(32) * T);
      src.resize(size_t(total) + size_t(32) * T);
      for (int q = 0; q < C; ++q) {
        const size_t r = size_t(sl) * C + q;
        const int g = r < rows.size() ? slot_row[rows[r]] : -1;
        const int len = g >= 0 ? row_len(g) : 0;
        const int64_t base = g >= 0 ? proj_start(g) : 0;
        auto col_of = [&](int j) { return g == p0 ? p0 : S.cols[S.row_ptr[g] + j]; };
        const int pad = len > 0 ? col_of(len - 1) : 0;
        for (int t = 0; t < T; ++t)
          for (int sub = 0; sub < Lanes; ++sub) {
            const int j = t * Lanes + sub;
            const size_t at = size_t(total) + size_t(t) * 32 + size_t(sub) * C + q;
            cols[at] = j < len ? col_of(j) : pad;
            src[at] = j < len ? int(base + j) : -1;
          }
      }
      total += int64_t(32) * T;
      soff.push_back(int(total));
    }
    color_slice[size_t(k) + 1] = color_slice[size_t(k)] + nsl;
  }
  rs_perm.upload(perm, c->stream);
  rs_off.upload(soff, c->stream);
  rs_cols.upload(cols, c->stream);
  rs_src.upload(src, c->stream);
  bslot.upload(slot_row, c->stream);
  PM_CUDA(cudaStreamSynchronize(c->stream));  // the host vectors go out of scope
  rs_entries = total;
  rs_lanes = Lanes;
  rs_ok = true;
}

// the periodic lattice colouring of the nodal patches (see setup); false if
// the pressure nodes are not on a 3D lattice or two patches of one colour
// share a velocity node
static bool lattice_colours(const pmsetup::Space& ps, const std::vector<int>& vp, const std::vector<int>& vi,
                            std::vector<int>& color, int& n_colors) {
  const int np = int(vp.size()) - 1;
  if (np <= 0 || ps.node.size() != size_t(np) * 3) return false;
  int64_t spacing = 0;
  for (int64_t v : ps.node) spacing = std::gcd(spacing, v < 0 ? -v : v);
  if (spacing <= 0) return false;
  std::vector<int> raw(np);
  for (int i = 0; i < np; ++i) {
    int col = 0, mult = 1;
    for (int d = 0; d < 3; ++d) {
      const int64_t k = ps.node[size_t(i) * 3 + d] / spacing;
      col += int(((k % 3) + 3) % 3) * mult;
      mult *= 3;
    }
    raw[i] = col;
  }
  // check: no velocity node in two patches of one colour
  int nmax = 0;
  for (int v : vi) nmax = std::max(nmax, v + 1);
  std::vector<int> mark(size_t(nmax) * 27, 0);
  for (int i = 0; i < np; ++i)
    for (int t = vp[i]; t < vp[i + 1]; ++t) {
      int& m = mark[size_t(vi[t]) * 27 + raw[i]];
      if (m) return false;
      m = 1;
    }
  int remap[27];
  bool used[27] = {};
  for (int i = 0; i < np; ++i) used[raw[i]] = true;
  n_colors = 0;
  for (int k = 0; k < 27; ++k) remap[k] = used[k] ? n_colors++ : -1;
  for (int i = 0; i < np; ++i) color[i] = remap[raw[i]];
  return true;
}

void DevNodalVanka::setup(pm_ctx* c, const DiscLevel& L) {
  nu = L.space.n_dofs;
  np = L.pspace.n_dofs;
  n = L.sys.n_rows;
  const pmsetup::Csr& S = L.sys;
  std::vector<int> vp(np + 1, 0), vi;
  for (int i = 0; i < np; ++i) {
    const int r = 3 * nu + i;
    for (int k = S.row_ptr[r]; k < S.row_ptr[r + 1]; ++k)
      if (S.cols[k] < nu) vi.push_back(S.cols[k]);  // columns of B1 (sorted)
    vp[i + 1] = int(vi.size());
  }
  max_nodes = 0;
  std::vector<int64_t> ao(np + 1, 0);
  for (int i = 0; i < np; ++i) {
    const int m = vp[i + 1] - vp[i];
    max_nodes = std::max(max_nodes, m);
    ao[i + 1] = ao[i] + int64_t(m) * m;
  }
  if (max_nodes > kNodalMaxNodes)
    throw Error(PM_E_UNSUPPORTED, "nodal Vanka patch with " + std::to_string(max_nodes) +
                                      " velocity nodes exceeds the supported " + std::to_string(kNodalMaxNodes));
  ainv_len = ao[np];
  vptr.upload(vp, c->stream);
  vidx.upload(vi, c->stream);
  aoff.upload(ao, c->stream);
  // incidence of the combined DOFs in the local storage
  std::vector<int> cnt(n, 0);
  for (int i = 0; i < np; ++i) {
    for (int k = 0; k < 3; ++k)
      for (int t = vp[i]; t < vp[i + 1]; ++t) cnt[k * nu + vi[t]]++;
    cnt[3 * nu + i]++;
  }
  std::vector<int> ip(n + 1, 0);
  for (int d = 0; d < n; ++d) ip[d + 1] = ip[d] + cnt[d];
  std::vector<int> ix(ip[n]);
  {
    std::vector<int> fill(ip.begin(), ip.end() - 1);
    for (int i = 0; i < np; ++i) {
      const int m = vp[i + 1] - vp[i], off = 3 * vp[i] + i;
      for (int k = 0; k < 3; ++k)
        for (int a = 0; a < m; ++a) ix[fill[k * nu + vi[vp[i] + a]]++] = off + k * m + a;
      ix[fill[3 * nu + i]++] = off + 3 * m;
    }
  }
  inc_ptr.upload(ip, c->stream);
  inc_idx.upload(ix, c->stream);
  count.upload(cnt, c->stream);
  // colouring: patches of one colour share no velocity node (and so no DOF).
  // On the vertex lattice of the unit-cube meshes the patches of two pressure
  // vertices share a node only when the vertices are at most two lattice
  // steps apart in every direction, so (i mod 3) + 3 (j mod 3) + 9 (k mod 3)
  // is a colouring with 27 colours of equal size; it is checked and used where
  // it holds, the greedy colouring in pressure-DOF order otherwise
  std::vector<int> np_ptr(nu + 1, 0), np_idx(vi.size());
  for (int v : vi) np_ptr[v + 1]++;
  for (int v = 0; v < nu; ++v) np_ptr[v + 1] += np_ptr[v];
  {
    std::vector<int> fill(np_ptr.begin(), np_ptr.end() - 1);
    for (int i = 0; i < np; ++i)
      for (int t = vp[i]; t < vp[i + 1]; ++t) np_idx[fill[vi[t]]++] = i;
  }
  std::vector<int> color(np, -1), seen;
  int n_colors = 0;
  if (!lattice_colours(L.pspace, vp, vi, color, n_colors)) {
    for (int i = 0; i < np; ++i) {
      seen.assign(n_colors + 1, 0);
      for (int t = vp[i]; t < vp[i + 1]; ++t) {
        const int v = vi[t];
        for (int e = np_ptr[v]; e < np_ptr[v + 1]; ++e) {
          const int j = np_idx[e];
          if (j < i) seen[color[j]] = 1;
        }
      }
      int col = 0;
      while (col < n_colors && seen[col]) ++col;
      color[i] = col;
      if (col == n_colors) ++n_colors;
    }
  }
  color_ptr.assign(n_colors + 1, 0);
  for (int i = 0; i < np; ++i) color_ptr[color[i] + 1]++;
  for (int k = 0; k < n_colors; ++k) color_ptr[k + 1] += color_ptr[k];
  std::vector<int> cp(np);
  {
    std::vector<int> fill(color_ptr.begin(), color_ptr.end() - 1);
    for (int i = 0; i < np; ++i) cp[fill[color[i]]++] = i;
  }
  color_patches.upload(cp, c->stream);
  build_row_slices(c, S, L.pressure_row0, vp, vi, cp);
  color_entries.assign(n_colors, 0);
  color_rows.assign(n_colors, 0);
  color_nodes.assign(n_colors, 0);
  color_msq.assign(n_colors, 0);
  for (int i = 0; i < np; ++i) {
    const int k = color[i], m = vp[i + 1] - vp[i];
    auto row_len = [&](int g) { return int64_t(S.row_ptr[g + 1] - S.row_ptr[g]); };
    for (int d = 0; d < 3; ++d)
      for (int t = vp[i]; t < vp[i + 1]; ++t) color_entries[k] += row_len(d * nu + vi[t]);
    color_entries[k] += row_len(3 * nu + i);
    color_rows[k] += 3 * m + 1;
    color_nodes[k] += m;
    color_msq[k] += int64_t(m) * m;
  }
  flag.ensure(1);
}

}  // namespace pm

namespace pm {

static __device__ __forceinline__ int find_sorted(const int* a, int n, int key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return (lo < n && a[lo] == key) ? lo : -1;
}

// one block per pressure DOF: the velocity block of the patch from the
// projected matrix (non-zero entries only, as the reference copies them),
// inverted in place by Gauss-Jordan in shared memory; then t_k = A^{-1} bt_k
// and the Schur complement S. No pivoting: the block is the velocity
// stiffness of the patch nodes (symmetric positive definite on the active
// nodes) with unit rows for Dirichlet nodes, so every leading block is
// nonsingular; a zero pivot still raises the flag. The reference's LAPACK LU
// pivots; the two inverses agree to rounding.
template <class T, int TR>
__global__ void __launch_bounds__(256) k_nodal_factor(int np, int nu, const int* __restrict__ vptr,
                                                      const int* __restrict__ vidx,
                                                      const int64_t* __restrict__ aoff,
                                                      const int* __restrict__ rp, const int* __restrict__ ci,
                                                      const T* __restrict__ v, T* __restrict__ ainv,
                                                      T* __restrict__ tb, T* __restrict__ sinv,
                                                      int* __restrict__ flag) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int i = blockIdx.x;
  if (i >= np) return;
  const int m = vptr[i + 1] - vptr[i];
  const int ld = m + 1;
  T* M = reinterpret_cast<T*>(smem_raw);
  T* Inv = M + m * ld;
  T* bt = Inv + m * ld;  // 3 m
  T* bv = bt + 3 * m;    // 3 m
  T* colk = bv + 3 * m;  // m
  T* tk = colk + m;      // 3 m: t_k = A^{-1} bt_k
  T* red = tk + 3 * m;   // 32
  int* nodes = reinterpret_cast<int*>(red + 32);
  __shared__ T cdiag;
  // rows of the patch's nodes (component 0): start, and the prefix of their
  // lengths, so that the block reads all their entries as one flat range;
  // jpos: position of the coupling to the patch pressure in the row (the rows
  // of components 1 and 2 of a node hold it at the same position)
  __shared__ int rstart[kNodalMaxNodes], rofs[kNodalMaxNodes + 1], jpos[kNodalMaxNodes];
  const int t = threadIdx.x;
  for (int a = t; a < m; a += blockDim.x) {
    const int r = vidx[vptr[i] + a];
    nodes[a] = r;
    const int r0 = rp[r], r1 = rp[r + 1];
    rstart[a] = r0;
    rofs[a + 1] = r1 - r0;
    jpos[a] = -1;
  }
  for (int e = t; e < m * ld; e += blockDim.x) M[e] = T(0);
  for (int e = t; e < 6 * m; e += blockDim.x) bt[e] = T(0);
  if (t == 0) {
    cdiag = T(0);
    rofs[0] = 0;
  }
  __syncthreads();
  if (t == 0)
    for (int a = 0; a < m; ++a) rofs[a + 1] += rofs[a];
  __syncthreads();
  const int prow = 3 * nu + i;
  const int total = rofs[m];
  constexpr int UF = 4;  // entries in flight per thread
  for (int f0 = t; f0 < total; f0 += UF * int(blockDim.x)) {
    T val[UF];
    int col[UF], row[UF], pos[UF];
#pragma unroll
    for (int u = 0; u < UF; ++u) {
      const int f = f0 + u * int(blockDim.x);
      row[u] = -1;
      if (f < total) {
        int lo = 0, hi = m;  // the row a with rofs[a] <= f < rofs[a + 1]
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (rofs[mid] <= f) lo = mid;
          else hi = mid;
        }
        row[u] = lo;
        pos[u] = f - rofs[lo];
        const int k = rstart[lo] + pos[u];
        val[u] = v[k];
        col[u] = ci[k];
      }
    }
#pragma unroll
    for (int u = 0; u < UF; ++u) {
      if (row[u] < 0) continue;
      const int a = row[u];
      if (col[u] == prow) {
        jpos[a] = pos[u];
        bt[a] = val[u];
      } else if (val[u] != T(0) && col[u] < nu) {
        const int b = find_sorted(nodes, m, col[u]);
        if (b >= 0) M[a * ld + b] = val[u];
      }
    }
  }
  __syncthreads();
  for (int e = t; e < 2 * m; e += blockDim.x) {
    const int comp = 1 + e / m, a = e % m;
    if (jpos[a] >= 0) bt[comp * m + a] = v[rp[comp * nu + nodes[a]] + jpos[a]];
  }
  for (int k = rp[prow] + t; k < rp[prow + 1]; k += blockDim.x) {
    const T val = v[k];
    if (val == T(0)) continue;
    const int col = ci[k];
    if (col == prow) {
      cdiag = val;
    } else if (col < 3 * nu) {
      const int comp = col / nu, b = find_sorted(nodes, m, col - comp * nu);
      if (b >= 0) bv[comp * m + b] = val;
    }
  }
  __syncthreads();
  // Gauss-Jordan on register tiles: thread (tr, tc) of a 16 x 16 grid holds
  // the entries (tr + 16 i, tc + 16 j), i, j < TR (the launch picks TR for the
  // level's largest patch). Per column k the owners of row k and
  // of column k publish them (double-buffered by the parity of k, so one
  // barrier per column suffices), then every thread scales the pivot row for
  // its columns by the pivot's reciprocal and updates its tile: row k becomes
  // the scaled pivot row, the others lose their column-k multiple of it
  // (column k: -f / pv).
  constexpr int TD = 16;  // TR x TR entries per thread: m <= 16 TR
  __shared__ T rowb[2][kNodalMaxNodes], colb[2][kNodalMaxNodes];
  const int tr = t / TD, tc = t % TD;
  T reg[TR][TR];
#pragma unroll
  for (int ir = 0; ir < TR; ++ir)
#pragma unroll
    for (int jc = 0; jc < TR; ++jc) {
      const int r = tr + TD * ir, j = tc + TD * jc;
      reg[ir][jc] = (r < m && j < m) ? M[r * ld + j] : T(0);
    }
  for (int k = 0; k < m; ++k) {
    T* rk = rowb[k & 1];
    T* ck = colb[k & 1];
    const int kb = k / TD, km = k % TD;
    if (tr == km) {
#pragma unroll
      for (int ir = 0; ir < TR; ++ir)
        if (ir == kb)
#pragma unroll
          for (int jc = 0; jc < TR; ++jc) {
            const int j = tc + TD * jc;
            if (j < m) rk[j] = reg[ir][jc];
          }
    }
    if (tc == km) {
#pragma unroll
      for (int jc = 0; jc < TR; ++jc)
        if (jc == kb)
#pragma unroll
          for (int ir = 0; ir < TR; ++ir) {
            const int r = tr + TD * ir;
            if (r < m) ck[r] = reg[ir][jc];
          }
    }
    __syncthreads();
    const T pv = ck[k];
    if (t == 0 && !(pv != T(0))) atomicExch(flag, 1);
    const T rpiv = T(1) / (pv != T(0) ? pv : T(1));
    T prj[TR];
#pragma unroll
    for (int jc = 0; jc < TR; ++jc) {
      const int j = tc + TD * jc;
      prj[jc] = j < m ? (j == k ? rpiv : rk[j] * rpiv) : T(0);
    }
#pragma unroll
    for (int ir = 0; ir < TR; ++ir) {
      const int r = tr + TD * ir;
      if (r >= m) continue;
      const T f = ck[r];
#pragma unroll
      for (int jc = 0; jc < TR; ++jc) {
        const int j = tc + TD * jc;
        if (r == k) reg[ir][jc] = prj[jc];
        else reg[ir][jc] = (j == k ? T(0) : reg[ir][jc]) - f * prj[jc];
      }
    }
  }
#pragma unroll
  for (int ir = 0; ir < TR; ++ir)
#pragma unroll
    for (int jc = 0; jc < TR; ++jc) {
      const int r = tr + TD * ir, j = tc + TD * jc;
      if (r < m && j < m) M[r * ld + j] = reg[ir][jc];
    }
  __syncthreads();
  Inv = M;  // the inverse, in place
  // t_k = Inv bt_k
  for (int e = t; e < 3 * m; e += blockDim.x) {
    const int comp = e / m, a = e % m;
    T s = T(0);
    for (int b = 0; b < m; ++b) s += Inv[a * ld + b] * bt[comp * m + b];
    tk[e] = s;
  }
  __syncthreads();
  // S = c - sum_k b_k . t_k, reduced in a fixed order
  T part = T(0);
  for (int e = t; e < 3 * m; e += blockDim.x) part += bv[e] * tk[e];
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((t & 31) == 0) red[t >> 5] = part;
  __syncthreads();
  if (t == 0) {
    T s = T(0);
    for (int w = 0; w < int(blockDim.x >> 5); ++w) s += red[w];
    const T S = cdiag - s;
    if (!(S != T(0))) atomicExch(flag, 1);
    sinv[i] = S != T(0) ? T(1) / S : T(0);
  }
  T* out = ainv + aoff[i];
  for (int e = t; e < m * m; e += blockDim.x) {
    const int b = e / m, a = e % m;  // column-major: out[b*m + a] = Inv[a][b]
    out[e] = Inv[a * ld + b];
  }
  T* otb = tb + 6 * size_t(vptr[i]);
  for (int e = t; e < 3 * m; e += blockDim.x) {
    otb[e] = tk[e];
    otb[3 * m + e] = bv[e];
  }
}

template <class T>
__global__ void k_fill_rows(int64_t n, const int* __restrict__ src, const double* __restrict__ v, T* __restrict__ out) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int k = src[i];
    out[i] = k >= 0 ? T(v[k]) : T(0);
  }
}

template <class T>
static size_t nodal_factor_smem(int m) {
  return sizeof(T) * (size_t(2) * m * (m + 1) + 10 * size_t(m) + 32) + sizeof(int) * size_t(m);
}

template <class T, int TR>
static void launch_nodal_factor_tr(pm_ctx* c, DevNodalVanka& nv, const int* rp, const int* ci, const T* v, T* ainv,
                                   T* tb, T* sinv) {
  const size_t sm = nodal_factor_smem<T>(nv.max_nodes);
  PM_CUDA(cudaFuncSetAttribute(k_nodal_factor<T, TR>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)));
  k_nodal_factor<T, TR><<<nv.np, 256, sm, c->stream>>>(nv.np, nv.nu, nv.vptr.p, nv.vidx.p, nv.aoff.p, rp, ci, v, ainv,
                                                        tb, sinv, nv.flag.p);
}

// the register tile of the factor kernel covers 16 TR rows and columns
template <class T>
static void launch_nodal_factor(pm_ctx* c, DevNodalVanka& nv, const int* rp, const int* ci, const T* v, T* ainv,
                                T* tb, T* sinv) {
  static_assert(kNodalMaxNodes <= 96, "register tiles cover at most 96 nodes");
  if (nv.max_nodes <= 64) launch_nodal_factor_tr<T, 4>(c, nv, rp, ci, v, ainv, tb, sinv);
  else if (nv.max_nodes <= 80) launch_nodal_factor_tr<T, 5>(c, nv, rp, ci, v, ainv, tb, sinv);
  else launch_nodal_factor_tr<T, 6>(c, nv, rp, ci, v, ainv, tb, sinv);
}

void DevNodalVanka::factor(pm_ctx* c, const DevCsr& V, bool fp32) {
  PM_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), c->stream));
  if (fp32) {
    ainv32.ensure(size_t(ainv_len));
    tb32.ensure(size_t(6) * vidx.n);
    sinv32.ensure(np);
    sol32.ensure(size_t(3) * vidx.n + np);
    launch_nodal_factor<float>(c, *this, V.row_ptr.p, V.cols.p, V.vals32.p, ainv32.p, tb32.p, sinv32.p);
  } else {
    ainv.ensure(size_t(ainv_len));
    tb.ensure(size_t(6) * vidx.n);
    sinv.ensure(np);
    sol.ensure(size_t(3) * vidx.n + np);
    launch_nodal_factor<double>(c, *this, V.row_ptr.p, V.cols.p, V.vals.p, ainv.p, tb.p, sinv.p);
  }
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
  if (rs_ok) {
    // the sliced rows take the projected matrix's values (FP32: rounded FP64)
    const int g = int(std::max<int64_t>(1, std::min<int64_t>((rs_entries + 255) / 256, int64_t(c->num_sms) * 8)));
    if (fp32) {
      rs_vals32.ensure(size_t(rs_entries));
      bloc32.ensure(sol32.n);
      k_fill_rows<float><<<g, 256, 0, c->stream>>>(rs_entries, rs_src.p, V.vals.p, rs_vals32.p);
    } else {
      rs_vals.ensure(size_t(rs_entries));
      bloc.ensure(sol.n);
      k_fill_rows<double><<<g, 256, 0, c->stream>>>(rs_entries, rs_src.p, V.vals.p, rs_vals.p);
    }
    PM_CHECK_LAUNCH();
    c->kernel_launches++;
  }
  int h = 0;
  PM_CUDA(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  PM_CUDA(cudaStreamSynchronize(c->stream));
  if (h) throw Error(PM_E_BREAKDOWN, "singular local nodal Vanka system");
}

}  // namespace pm

namespace pm {

// one block of 256 threads per patch (four patches resident per SM, so that
// the few hundred patches of a colour run in one wave): local residual
// (gathered from the global residual r or read from rloc), w_k = A^{-1} r_k
// for the three components (four threads per row, each over a quarter of the
// columns of A^{-1}, its loads issued twelve at a time, combined in a fixed
// order), the pressure from the Schur complement, u_k = w_k - t_k p; the
// damped correction is written to the local storage (additive sweep) or
// added into x (colour sweep). Every load that does not depend on the local
// solve (t_k, b_k, 1/S, the node indices and, in the colour sweep, the
// patch's x values, which no other patch of the colour writes) is issued
// before the first barrier.
constexpr int kLocalThreads = 256;
template <class T>
__global__ void __launch_bounds__(kLocalThreads, 4) k_nodal_local(const int* __restrict__ guard, int cnt, const int* __restrict__ patches, int nu,
                                                     const int* __restrict__ vptr, const int* __restrict__ vidx,
                                                     const int64_t* __restrict__ aoff, const T* __restrict__ ainv,
                                                     const T* __restrict__ tb, const T* __restrict__ sinv,
                                                     const T* __restrict__ r, const T* __restrict__ rloc,
                                                     T* __restrict__ out, T* __restrict__ x, T damp) {
  constexpr int NT = kLocalThreads, P = 4, R = NT / P;  // threads per row, rows per pass
  constexpr int CH = 12;  // loads of A^{-1} in flight per thread (two rounds for up to 96 nodes)
  constexpr int E = (3 * kNodalMaxNodes + NT - 1) / NT;  // velocity unknowns per thread
  static_assert(3 * kNodalMaxNodes + 1 <= 2 * NT, "the local residual takes two loads per thread");
  __shared__ T rl[3 * kNodalMaxNodes + 1];
  __shared__ T w[3 * kNodalMaxNodes];
  __shared__ T part[P][3][R];
  __shared__ T red[NT / 32];
  const int idx = blockIdx.x;
  if (idx >= cnt) return;
  const int t = threadIdx.x;
  // the loads run ahead in dependent rounds (patch, then its offsets, then
  // its operands and the first columns of A^{-1}); the guard is tested
  // before the first store (uniform for the whole grid)
  const int gflag = guard ? *(volatile const int*)guard : 0;
  const int i = patches ? patches[idx] : idx;
  const int v0 = vptr[i];
  const int m = vptr[i + 1] - v0;
  const T si = sinv[i];
  const T* A = ainv + aoff[i];
  const int* nodes = vidx + v0;
  const size_t off = 3 * size_t(v0) + i;
  const int rows3 = 3 * m;
  const int q = t / R;   // column quarter
  const int lr = t % R;  // row within the pass
  const int qlen = (m + P - 1) / P;
  const int b0 = q * qlen, b1 = min(m, b0 + qlen);
  T av[CH];  // the first chunk of the first pass
#pragma unroll
  for (int u = 0; u < CH; ++u) av[u] = (lr < m && b0 + u < b1) ? A[size_t(b0 + u) * m + lr] : T(0);
  // operands independent of the solve: thread t owns the velocity unknowns
  // t, t + NT, ... (3m <= 288)
  const T* tt = tb + 6 * size_t(v0);
  T ttv[E], bbv[E], xv[E];
  int g[E];
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int e = t + k * NT;
    ttv[k] = bbv[k] = xv[k] = T(0);
    g[k] = 0;
    if (e < rows3) {
      ttv[k] = tt[e];
      bbv[k] = tt[rows3 + e];
      g[k] = (e / m) * nu + nodes[e % m];
      if (x) xv[k] = x[g[k]];
    }
  }
  T xp = T(0);
  if (x && t == 0) xp = x[3 * nu + i];
  T rv[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int e = t + k * NT;
    rv[k] = T(0);
    if (e <= rows3) {
      if (rloc) {
        rv[k] = rloc[off + e];
      } else {
        const int gg = e < rows3 ? (e / m) * nu + nodes[e % m] : 3 * nu + i;
        rv[k] = r[gg];
      }
    }
  }
  if (gflag) return;
#pragma unroll
  for (int k = 0; k < 2; ++k)
    if (t + k * NT <= rows3) rl[t + k * NT] = rv[k];
  __syncthreads();
  for (int a0 = 0; a0 < m; a0 += R) {
    const int a = a0 + lr;
    T s0 = T(0), s1 = T(0), s2 = T(0);
    for (int c0 = b0; c0 < b1; c0 += CH) {
      if (a0 > 0 || c0 > b0) {
#pragma unroll
        for (int u = 0; u < CH; ++u) av[u] = (a < m && c0 + u < b1) ? A[size_t(c0 + u) * m + a] : T(0);
      }
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        if (c0 + u < b1) {
          s0 += av[u] * rl[c0 + u];
          s1 += av[u] * rl[m + c0 + u];
          s2 += av[u] * rl[2 * m + c0 + u];
        }
      }
    }
    part[q][0][lr] = s0;
    part[q][1][lr] = s1;
    part[q][2][lr] = s2;
    __syncthreads();
    for (int e = t; e < 3 * R; e += NT) {
      const int k = e / R, rr = e % R, aa = a0 + rr;
      if (aa < m) w[k * m + aa] = ((part[0][k][rr] + part[1][k][rr]) + part[2][k][rr]) + part[3][k][rr];
    }
    __syncthreads();
  }
  T d = T(0);
#pragma unroll
  for (int k = 0; k < E; ++k)
    if (t + k * NT < rows3) d += bbv[k] * w[t + k * NT];
  for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
  if ((t & 31) == 0) red[t >> 5] = d;
  __syncthreads();
  T dsum = T(0);
#pragma unroll
  for (int k = 0; k < NT / 32; ++k) dsum += red[k];
  const T p = si * (rl[rows3] - dsum);
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int e = t + k * NT;
    if (e < rows3) {
      const T u = damp * (w[e] - ttv[k] * p);
      if (x) x[g[k]] = xv[k] + u;
      else out[off + e] = u;
    }
  }
  if (t == 0) {
    if (x) x[3 * nu + i] = xp + damp * p;
    else out[off + rows3] = damp * p;
  }
}

// local residuals b - V x of the patches of one colour: one block per patch,
// four lanes per row (128 rows at a time), eight loads in flight per lane, the
// four partial sums combined by two shuffle steps
template <class T>
__global__ void __launch_bounds__(512) k_nodal_rhs(const int* __restrict__ guard, int cnt, const int* __restrict__ patches, int nu,
                                                   const int* __restrict__ vptr, const int* __restrict__ vidx,
                                                   const int* __restrict__ rp, const int* __restrict__ ci,
                                                   const T* __restrict__ v, const T* __restrict__ b,
                                                   const T* __restrict__ x, T* __restrict__ rloc) {
  if (guarded(guard)) return;  // uniform for the whole grid
  constexpr int L = 4, U = 8;  // lanes per row, loads in flight per lane
  const int idx = blockIdx.x;
  if (idx >= cnt) return;
  const int i = patches[idx];
  const int m = vptr[i + 1] - vptr[i];
  const int* nodes = vidx + vptr[i];
  const size_t off = 3 * size_t(vptr[i]) + i;
  const int lane = threadIdx.x & (L - 1);
  const int rows = 3 * m + 1;
  // every thread of the block runs the same number of passes (the shuffles
  // need whole groups)
  for (int e0 = 0; e0 < rows; e0 += int(blockDim.x) / L) {
    const int e = e0 + int(threadIdx.x) / L;
    const bool valid = e < rows;
    int g = 0, beg = 0, end = 0;
    if (valid) {
      g = e < 3 * m ? (e / m) * nu + nodes[e % m] : 3 * nu + i;
      beg = rp[g];
      end = rp[g + 1];
    }
    T s = T(0);
    for (int base = beg; base < end; base += L * U) {
      T vv[U], xv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int k = base + u * L + lane;
        const bool in = k < end;
        vv[u] = in ? v[k] : T(0);
        xv[u] = in ? x[ci[k]] : T(0);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) s += vv[u] * xv[u];
    }
    s += __shfl_xor_sync(0xffffffffu, s, 1, L);
    s += __shfl_xor_sync(0xffffffffu, s, 2, L);
    if (valid && lane == 0) rloc[off + e] = b[g] - s;
  }
}

template <class T>
static void nodal_jacobi(pm_ctx* c, DevNodalVanka& nv, const DevCsr& V, const T* ainv, const T* tb, const T* sinv,
                         T* sol, const T* b, T* x, T* r, T damp) {
  if constexpr (sizeof(T) == 8) csr_apply(c, V, EPI_DEFECT, x, r, b, 1.0);
  else csr_apply32(c, V, EPI_DEFECT, x, r, b, 1.0f);
  k_nodal_local<T><<<nv.np, kLocalThreads, 0, c->stream>>>(c->guard, nv.np, nullptr, nv.nu, nv.vptr.p, nv.vidx.p, nv.aoff.p,
                                                          ainv, tb, sinv, r, nullptr, sol, nullptr, damp);
  const int g = std::max(1, std::min((nv.n + 255) / 256, c->num_sms * 16));
  k_vanka_average<T><<<g, 256, 0, c->stream>>>(c->guard, nv.n, nv.inc_ptr.p, nv.inc_idx.p, nv.count.p, sol, x);
  PM_CHECK_LAUNCH();
  c->kernel_launches += 2;
}

// bloc[slot] = b[global row of the slot]
template <class T>
__global__ void k_gather_slots(const int* __restrict__ guard, int n, const int* __restrict__ rows,
                               const T* __restrict__ b, T* __restrict__ out) {
  if (guarded(guard)) return;  // uniform for the whole grid
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = b[rows[i]];
}

template <class T>
static void nodal_colored(pm_ctx* c, DevNodalVanka& nv, const DevCsr& V, const T* vals, const T* ainv, const T* tb,
                          const T* sinv, T* rloc, const T* b, T* x, T damp) {
  const int ncol = int(nv.color_ptr.size()) - 1;
  const T* rsv = nullptr;
  T* bl = nullptr;
  if constexpr (sizeof(T) == 4) {
    rsv = nv.rs_vals32.p;
    bl = nv.bloc32.p;
  } else {
    rsv = nv.rs_vals.p;
    bl = nv.bloc.p;
  }
  const bool sliced = nv.rs_ok && rsv && bl && c->nodal_sliced != 0;
  BlockMask mg{};
  mg.guard = c->guard;
  if (sliced) {
    const int n = int(nv.bslot.n);
    const int g = std::max(1, std::min((n + 255) / 256, c->num_sms * 8));
    k_gather_slots<T><<<g, 256, 0, c->stream>>>(c->guard, n, nv.bslot.p, b, bl);
    PM_CHECK_LAUNCH();
    c->kernel_launches++;
  }
  for (int k = 0; k < ncol; ++k) {
    const int beg = nv.color_ptr[k], cnt = nv.color_ptr[k + 1] - beg;
    if (!cnt) continue;
    const int* pts = nv.color_patches.p + beg;
    if (c->probe_nodal) {
      cudaEvent_t e0 = probe_event(c);
      PM_CUDA(cudaEventRecord(e0, c->stream));
      c->probe_events.push_back(e0);
      // algorithmic bytes of the pair: the rows' values, column indices and
      // gathered x, b, the local residuals written and read back, the
      // inverses (m^2), t and b vectors (6 m), 1/S, and x read and written
      const double eb = double(sizeof(T));
      c->probe_bytes.push_back(double(nv.color_entries[k]) * (2 * eb + 4) + double(nv.color_rows[k]) * 5 * eb +
                               double(nv.color_msq[k]) * eb + double(nv.color_nodes[k]) * 6 * eb + double(cnt) * eb);
    }
    if (sliced) {
      // the colour's local residuals as one sliced SpMV: rloc[slot] = bloc[slot] - (V x)[row]
      const int s0 = nv.color_slice[k], ns = nv.color_slice[k + 1] - s0;
      if (nv.rs_lanes == 8)
        sell_kernel<T, 8, 8, true, EPI_DEFECT><<<(ns + 3) / 4, 128, 0, c->stream>>>(
            ns, nv.rs_perm.p + size_t(s0) * 4, nv.rs_off.p + s0, nv.rs_cols.p, rsv, x, rloc, bl, nullptr, T(0), mg);
      else
        sell_kernel<T, 4, 8, true, EPI_DEFECT><<<(ns + 3) / 4, 128, 0, c->stream>>>(
            ns, nv.rs_perm.p + size_t(s0) * 8, nv.rs_off.p + s0, nv.rs_cols.p, rsv, x, rloc, bl, nullptr, T(0), mg);
    } else {
      k_nodal_rhs<T><<<cnt, 512, 0, c->stream>>>(c->guard, cnt, pts, nv.nu, nv.vptr.p, nv.vidx.p, V.row_ptr.p,
                                                  V.cols.p, vals, b, x, rloc);
    }
    k_nodal_local<T><<<cnt, kLocalThreads, 0, c->stream>>>(c->guard, cnt, pts, nv.nu, nv.vptr.p, nv.vidx.p, nv.aoff.p, ainv,
                                                          tb, sinv, nullptr, rloc, nullptr, x, damp);
    c->kernel_launches += 2;
    if (c->probe_nodal) {
      cudaEvent_t e1 = probe_event(c);
      PM_CUDA(cudaEventRecord(e1, c->stream));
      c->probe_events.push_back(e1);
    }
  }
  PM_CHECK_LAUNCH();
}

void DevNodalVanka::sweep_jacobi(pm_ctx* c, const DevCsr& V, const double* b, double* x, double* r, double damp) {
  nodal_jacobi<double>(c, *this, V, ainv.p, tb.p, sinv.p, sol.p, b, x, r, damp);
}
void DevNodalVanka::sweep_jacobi32(pm_ctx* c, const DevCsr& V, const float* b, float* x, float* r, float damp) {
  nodal_jacobi<float>(c, *this, V, ainv32.p, tb32.p, sinv32.p, sol32.p, b, x, r, damp);
}
void DevNodalVanka::sweep_colored(pm_ctx* c, const DevCsr& V, const double* b, double* x, double damp) {
  nodal_colored<double>(c, *this, V, V.vals.p, ainv.p, tb.p, sinv.p, sol.p, b, x, damp);
}
void DevNodalVanka::sweep_colored32(pm_ctx* c, const DevCsr& V, const float* b, float* x, float damp) {
  nodal_colored<float>(c, *this, V, V.vals32.p, ainv32.p, tb32.p, sinv32.p, sol32.p, b, x, damp);
}

}  // namespace pm
