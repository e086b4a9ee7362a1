// Element assembly of convection-diffusion systems on the device.
//
// Restates the ParMooN element loop for the Galerkin convection-diffusion form:
//   Assemble3D (src/AssembleRoutines/Assemble3D.C:228-470) / Assemble2D
//   (src/AssembleRoutines/Assemble2D.C:6940-7889), LocalAssembling::GetLocalForms
//   (src/AssembleRoutines/LocalAssembling.C:669-765) and
//   BilinearAssembleGalerkin<2,3> (src/AssembleRoutines/ConvDiff.C:1794-1856):
//     K_ij += Mult_q [eps grad phi_i . grad phi_j + (b . grad phi_j) phi_i + c phi_j phi_i]
//     F_i  += Mult_q phi_i f,      Mult_q = w_q |det J|
// on affine quadrilaterals/hexahedra (QuadAffin / HexaAffin reference maps,
// src/FE/QuadAffin.C:614, src/FE/HexaAffin.C:858) with tensor Gauss rules
// (src/QuadFormulas/QuadFormulaHexa.C:41-120, QuadFormulaQuad.C:43).
//
// Stage 1 computes every element matrix into a scratch array, one group of
// threads per cell. Stage 2 gathers them into the CSR values: every entry sums
// its contributions in cell order - the order in which the reference's scatter
// adds them - so the result is deterministic and does not depend on atomics.
#include <cmath>
#include <vector>

#include "pm_assemble.h"
#include "pm_tetra.h"

namespace pm {

// 1D Gauss rules in the reference's point order
static void gauss1d(int n, std::vector<double>& x, std::vector<double>& w) {
  if (n == 2) {
    x = {-0.5773502691896257645091489, 0.5773502691896257645091489};
    w = {1.0, 1.0};
  } else if (n == 3) {
    x = {-0.7745966692414833770358530, 0.0, 0.7745966692414833770358530};
    w = {0.5555555555555555555555558, 0.8888888888888888888888888, 0.5555555555555555555555558};
  } else if (n == 4) {
    x = {0.33998104358485626480266576, 0.86113631159405257522394649,
         -0.86113631159405257522394649, -0.33998104358485626480266576};
    w = {0.652145154862546142626936051, 0.347854845137453857373063949,
         0.347854845137453857373063949, 0.652145154862546142626936051};
  } else {
    throw Error(PM_E_UNSUPPORTED, "tensor Gauss rules with 2, 3 or 4 points per direction");
  }
}

static void lag1d(int k, double x, double* l, double* dl) {
  if (k == 1) {
    l[0] = 0.5 * (1.0 - x);
    l[1] = 0.5 * (1.0 + x);
    dl[0] = -0.5;
    dl[1] = 0.5;
  } else {
    l[0] = 0.5 * x * (x - 1.0);
    l[1] = 1.0 - x * x;
    l[2] = 0.5 * x * (x + 1.0);
    dl[0] = x - 0.5;
    dl[1] = -2.0 * x;
    dl[2] = x + 0.5;
  }
}

void build_qk_tables(int dim, int k, int qn, RefTables& t) {
  std::vector<double> x1, w1;
  gauss1d(qn, x1, w1);
  const int nb1 = k + 1;
  t.dim = dim;
  t.nb = dim == 2 ? nb1 * nb1 : nb1 * nb1 * nb1;
  t.nq = dim == 2 ? qn * qn : qn * qn * qn;
  t.w.assign(t.nq, 0.0);
  t.xi.assign(size_t(t.nq) * 3, 0.0);
  t.phi.assign(size_t(t.nq) * t.nb, 0.0);
  t.dphi.assign(size_t(3) * t.nq * t.nb, 0.0);
  int q = 0;
  for (int i = 0; i < (dim == 3 ? qn : 1); ++i)
    for (int j = 0; j < qn; ++j)
      for (int kk = 0; kk < qn; ++kk, ++q) {
        const double xs = x1[kk], ys = x1[j], zs = dim == 3 ? x1[i] : 0.0;
        t.xi[q * 3 + 0] = xs;
        t.xi[q * 3 + 1] = ys;
        t.xi[q * 3 + 2] = zs;
        t.w[q] = dim == 3 ? w1[i] * w1[j] * w1[kk] : w1[j] * w1[kk];
        double lx[3], ly[3], lz[3] = {1, 1, 1}, dx[3], dy[3], dz[3] = {0, 0, 0};
        lag1d(k, xs, lx, dx);
        lag1d(k, ys, ly, dy);
        if (dim == 3) lag1d(k, zs, lz, dz);
        int m = 0;
        for (int c = 0; c < (dim == 3 ? nb1 : 1); ++c)
          for (int b = 0; b < nb1; ++b)
            for (int a = 0; a < nb1; ++a, ++m) {
              const double zc = dim == 3 ? lz[c] : 1.0;
              t.phi[size_t(q) * t.nb + m] = lx[a] * ly[b] * zc;
              t.dphi[(size_t(0) * t.nq + q) * t.nb + m] = dx[a] * ly[b] * zc;
              t.dphi[(size_t(1) * t.nq + q) * t.nb + m] = lx[a] * dy[b] * zc;
              if (dim == 3) t.dphi[(size_t(2) * t.nq + q) * t.nb + m] = lx[a] * ly[b] * dz[c];
            }
      }
}

// P1 / P2 tables on a tetrahedral rule: qn = 11 (P4Tetra) or 15 (P5Tetra)
// points; the same layout as build_qk_tables (dim 3)
void build_pk_tables(int elem, int qn, RefTables& t) {
  if (qn != kP4n && qn != kP5n) throw Error(PM_E_UNSUPPORTED, "tetrahedral rules with 11 or 15 points");
  const double* X = qn == kP4n ? kP4x : kP5x;
  const double* Y = qn == kP4n ? kP4y : kP5y;
  const double* Z = qn == kP4n ? kP4z : kP5z;
  const double* W = qn == kP4n ? kP4w : kP5w;
  t.dim = 3;
  t.nb = elem == 12 ? 10 : 4;
  t.nq = qn;
  t.w.assign(W, W + qn);
  t.xi.assign(size_t(qn) * 3, 0.0);
  t.phi.assign(size_t(qn) * t.nb, 0.0);
  t.dphi.assign(size_t(3) * qn * t.nb, 0.0);
  for (int q = 0; q < qn; ++q) {
    t.xi[q * 3 + 0] = X[q];
    t.xi[q * 3 + 1] = Y[q];
    t.xi[q * 3 + 2] = Z[q];
    double v[10], dx[10], dy[10], dz[10];
    if (elem == 12) p2_eval(X[q], Y[q], Z[q], v, dx, dy, dz);
    else p1_eval(X[q], Y[q], Z[q], v, dx, dy, dz);
    for (int i = 0; i < t.nb; ++i) {
      t.phi[size_t(q) * t.nb + i] = v[i];
      t.dphi[(size_t(0) * qn + q) * t.nb + i] = dx[i];
      t.dphi[(size_t(1) * qn + q) * t.nb + i] = dy[i];
      t.dphi[(size_t(2) * qn + q) * t.nb + i] = dz[i];
    }
  }
}

void build_element_tables(int dim, int elem, int qn, RefTables& t) {
  if (elem == 11 || elem == 12) build_pk_tables(elem, qn, t);
  else build_qk_tables(dim, elem, qn, t);
}

// -------------------------------------------------------------- kernels ----
struct CdCoef {
  double eps, b0, b1, b2, c, fconst;
  int manufactured;  // 0: f = fconst; 1: sine exact solution; 2: quadratic exact solution
  double poly[10];   // 1, x, y, z, x^2, y^2, z^2, xy, xz, yz
  double src[10];    // added to f (time derivative of the exact solution)
};

static CdCoef make_coef(const pm_cd_coeffs& cf) {
  CdCoef k{cf.eps, cf.b[0], cf.b[1], cf.b[2], cf.c, cf.f_const, cf.manufactured, {}, {}};
  if (cf.manufactured == 2)
    for (int i = 0; i < 10; ++i) {
      k.poly[i] = cf.poly[i];
      k.src[i] = cf.poly_src[i];
    }
  return k;
}

// value of the quadratic exact solution (x[2] = 0 in 2D)
__host__ __device__ __forceinline__ double poly_u(const double* p, const double* x) {
  double u = p[0];
  u += p[1] * x[0];
  u += p[2] * x[1];
  u += p[3] * x[2];
  u += p[4] * x[0] * x[0];
  u += p[5] * x[1] * x[1];
  u += p[6] * x[2] * x[2];
  u += p[7] * x[0] * x[1];
  u += p[8] * x[0] * x[2];
  u += p[9] * x[1] * x[2];
  return u;
}

// f = -eps Lap u + b.grad u + c u of the quadratic exact solution, in the
// order of the sine branch (the examples' BilinearCoeffs)
__device__ __forceinline__ double poly_rhs(const CdCoef& k, int dim, const double* xin) {
  const double x[3] = {xin[0], xin[1], dim == 3 ? xin[2] : 0.0};
  const double* p = k.poly;
  const double u = poly_u(p, x);
  const double ux = p[1] + 2 * p[4] * x[0] + p[7] * x[1] + p[8] * x[2];
  const double uy = p[2] + 2 * p[5] * x[1] + p[7] * x[0] + p[9] * x[2];
  const double uz = p[3] + 2 * p[6] * x[2] + p[8] * x[0] + p[9] * x[1];
  const double lap = dim == 3 ? 2 * (p[4] + p[5] + p[6]) : 2 * (p[4] + p[5]);
  double f = -k.eps * lap;
  f += k.b0 * ux + k.b1 * uy + (dim == 3 ? k.b2 * uz : 0.0);
  f += k.c * u;
  f += poly_u(k.src, x);
  return f;
}

// affine map of cell `cell`: origin and Jacobian columns (QuadAffin/HexaAffin;
// TetraAffin, src/FE/TetraAffin.C: x = v0 + [v1-v0, v2-v0, v3-v0] xi on the
// unit simplex, when NV = 4 in 3D)
template <int DIM, int NV = DIM == 2 ? 4 : 8>
__device__ __forceinline__ void affine_map(const double* __restrict__ v, double* x0, double J[3][3]) {
  if (DIM == 3 && NV == 4) {
    for (int d = 0; d < 3; ++d) {
      x0[d] = v[d];
      J[d][0] = v[3 + d] - v[d];
      J[d][1] = v[6 + d] - v[d];
      J[d][2] = v[9 + d] - v[d];
    }
  } else if (DIM == 2) {
    // vertices 0,1,3: xc0 = (x1+x3)/2, xc1 = (x1-x0)/2, xc2 = (x3-x0)/2
    for (int d = 0; d < 2; ++d) {
      x0[d] = (v[2 + d] + v[6 + d]) * 0.5;
      J[d][0] = (v[2 + d] - v[d]) * 0.5;
      J[d][1] = (v[6 + d] - v[d]) * 0.5;
    }
  } else {
    for (int d = 0; d < 3; ++d) {
      x0[d] = (v[3 + d] + v[9 + d] + v[12 + d] - v[d]) * 0.5;
      J[d][0] = (v[3 + d] - v[d]) * 0.5;
      J[d][1] = (v[9 + d] - v[d]) * 0.5;
      J[d][2] = (v[12 + d] - v[d]) * 0.5;
    }
  }
}

__device__ __forceinline__ double rhs_value(const CdCoef& k, int dim, const double* x) {
  if (!k.manufactured) return k.fconst;
  if (k.manufactured == 2) return poly_rhs(k, dim, x);
  const double p = 3.14159265358979323846;
  // exact solution u = prod sin(pi x_d): values, gradient, Laplacian
  double s[3], co[3];
  for (int d = 0; d < dim; ++d) {
    s[d] = sin(p * x[d]);
    co[d] = cos(p * x[d]);
  }
  double u, ux, uy, uz = 0.0, lap;
  if (dim == 2) {
    u = s[0] * s[1];
    ux = p * co[0] * s[1];
    uy = p * s[0] * co[1];
    lap = -2 * p * p * s[0] * s[1];
  } else {
    u = s[0] * s[1] * s[2];
    ux = p * co[0] * s[1] * s[2];
    uy = p * s[0] * co[1] * s[2];
    uz = p * s[0] * s[1] * co[2];
    lap = -3 * p * p * s[0] * s[1] * s[2];
  }
  double f = -k.eps * lap;
  f += k.b0 * ux + k.b1 * uy + (dim == 3 ? k.b2 * uz : 0.0);
  f += k.c * u;
  return f;
}

// the same right-hand side with sin(pi x) and cos(pi x) from one sincospi call
__device__ __forceinline__ double rhs_value_pi(const CdCoef& k, int dim, const double* x) {
  if (!k.manufactured) return k.fconst;
  if (k.manufactured == 2) return poly_rhs(k, dim, x);
  const double p = 3.14159265358979323846;
  double s[3], co[3];
  for (int d = 0; d < dim; ++d) sincospi(x[d], &s[d], &co[d]);
  double u, ux, uy, uz = 0.0, lap;
  if (dim == 2) {
    u = s[0] * s[1];
    ux = p * co[0] * s[1];
    uy = p * s[0] * co[1];
    lap = -2 * p * p * s[0] * s[1];
  } else {
    u = s[0] * s[1] * s[2];
    ux = p * co[0] * s[1] * s[2];
    uy = p * s[0] * co[1] * s[2];
    uz = p * s[0] * s[1] * co[2];
    lap = -3 * p * p * s[0] * s[1] * s[2];
  }
  double f = -k.eps * lap;
  f += k.b0 * ux + k.b1 * uy + (dim == 3 ? k.b2 * uz : 0.0);
  f += k.c * u;
  return f;
}

// One group of TPC threads per cell, CPB cells per block. Shared memory per
// cell: A[q][i][4] = Mult_q (eps dphi_i, phi_i), B[q][j][4] = (dphi_j, b.dphi_j + c phi_j);
// K_ij = sum_q sum_d A[q][i][d] B[q][j][d].
template <int DIM, int NB, int NQ, int CPB, int NV = DIM == 2 ? 4 : 8>
__global__ void __launch_bounds__(256) k_elem_cd(int n_cells, const double* __restrict__ verts,
                                                 const double* __restrict__ ref, CdCoef co,
                                                 double* __restrict__ K, double* __restrict__ F) {
  extern __shared__ double smem[];
  constexpr int TPC = 256 / CPB;
  const int slot = threadIdx.x / TPC;
  const int t = threadIdx.x % TPC;
  const int cell = blockIdx.x * CPB + slot;
  double* A = smem + size_t(slot) * (2 * NQ * NB * 4 + NQ);
  double* B = A + NQ * NB * 4;
  double* fq = B + NQ * NB * 4;  // Mult_q * f(x_q)
  const double* phi = ref;
  const double* dphi = ref + NQ * NB;
  const double* w = ref + 4 * NQ * NB;
  const double* xi = w + NQ;
  const bool valid = cell < n_cells;
  double x0[3] = {0, 0, 0}, J[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  if (valid) affine_map<DIM, NV>(verts + (size_t)cell * NV * DIM, x0, J);
  // inverse transpose and |det J|
  double G[3][3], det;
  if (DIM == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double r = 1.0 / det;
    // grad phi = J^{-T} grad_ref phi
    G[0][0] = J[1][1] * r;  G[0][1] = -J[1][0] * r;
    G[1][0] = -J[0][1] * r; G[1][1] = J[0][0] * r;
  } else {
    det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
          J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    const double r = 1.0 / det;
    // (J^{-1})^T = cofactor(J) / det
    G[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * r;
    G[0][1] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]) * r;
    G[0][2] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * r;
    G[1][0] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) * r;
    G[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
    G[1][2] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) * r;
    G[2][0] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
    G[2][1] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) * r;
    G[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
  }
  const double adet = fabs(det);
  // stage A: per (q, i) physical derivatives
  for (int e = t; e < NQ * NB; e += TPC) {
    const int q = e / NB, i = e % NB;
    double g[3] = {0, 0, 0};
    double dr[3];
    for (int a = 0; a < DIM; ++a) dr[a] = dphi[(a * NQ + q) * NB + i];
    for (int d = 0; d < DIM; ++d) {
      double s = 0.0;
      for (int a = 0; a < DIM; ++a) s += G[d][a] * dr[a];
      g[d] = s;
    }
    const double ph = phi[q * NB + i];
    const double mult = w[q] * adet;
    double* Ai = A + (q * NB + i) * 4;
    double* Bi = B + (q * NB + i) * 4;
    Ai[0] = mult * co.eps * g[0];
    Ai[1] = mult * co.eps * g[1];
    Ai[2] = DIM == 3 ? mult * co.eps * g[2] : 0.0;
    Ai[3] = mult * ph;
    Bi[0] = g[0];
    Bi[1] = g[1];
    Bi[2] = DIM == 3 ? g[2] : 0.0;
    Bi[3] = co.b0 * g[0] + co.b1 * g[1] + (DIM == 3 ? co.b2 * g[2] : 0.0) + co.c * ph;
  }
  for (int q = t; q < NQ; q += TPC) {
    double x[3];
    for (int d = 0; d < DIM; ++d) {
      double s = x0[d];
      for (int a = 0; a < DIM; ++a) s += J[d][a] * xi[q * 3 + a];
      x[d] = s;
    }
    fq[q] = w[q] * adet * rhs_value(co, DIM, x);
  }
  __syncthreads();
  if (!valid) return;
  double* Kc = K + (size_t)cell * NB * NB;
  for (int p = t; p < NB * NB; p += TPC) {
    const int i = p / NB, j = p % NB;
    double s = 0.0;
#pragma unroll 3
    for (int q = 0; q < NQ; ++q) {
      const double* Ai = A + (q * NB + i) * 4;
      const double* Bj = B + (q * NB + j) * 4;
      s += Ai[0] * Bj[0] + Ai[1] * Bj[1] + Ai[2] * Bj[2] + Ai[3] * Bj[3];
    }
    Kc[p] = s;
  }
  for (int i = t; i < NB; i += TPC) {
    double s = 0.0;
    for (int q = 0; q < NQ; ++q) s += fq[q] * phi[q * NB + i];
    F[(size_t)cell * NB + i] = s;
  }
}

// Reference-tensor element kernel. On an affine cell with cell-constant eps,
// b, c the quadrature sum of BilinearAssembleGalerkin factors into
//   K_e = |det J| ( sum_{a<=b} A_ab S_ab + sum_a beta_a C_a + c M ),
//   A_ab = eps sum_d G_da G_db,  beta_a = sum_d b_d G_da,  G = J^{-T},
// with the reference tensors S, C, M (sums over the same quadrature points,
// computed once per element type). This is the same quadrature applied in a
// different summation order: NT FMAs per entry instead of 4 per quadrature
// point. The right-hand side keeps the per-point loop (f varies in the cell).
template <int DIM, int NB, int NQ, int CHUNK, int NV = DIM == 2 ? 4 : 8>
__global__ void __launch_bounds__(256) k_elem_cd_tensor(int n_cells, const double* __restrict__ verts,
                                                        const double* __restrict__ ref,
                                                        const double* __restrict__ T, CdCoef co,
                                                        double* __restrict__ K, double* __restrict__ F) {
  constexpr int NT = DIM * (DIM + 1) / 2 + DIM + 1;
  __shared__ double coef[CHUNK][NT];
  __shared__ double fq[CHUNK][NQ];
  __shared__ double geo[CHUNK][13];  // x0, J (row-major), |det J|
  const double* phi = ref;
  const double* w = ref + 4 * NQ * NB;
  const double* xi = w + NQ;
  const int c0 = blockIdx.x * CHUNK;
  const int nc = min(CHUNK, n_cells - c0);
  const int t = threadIdx.x;
  double x0[3] = {0, 0, 0}, J[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  // per-cell coefficients (one thread per cell)
  if (t < nc) {
    affine_map<DIM, NV>(verts + (size_t)(c0 + t) * NV * DIM, x0, J);
    double G[3][3] = {{0}}, det;
    if (DIM == 2) {
      det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      const double r = 1.0 / det;
      G[0][0] = J[1][1] * r;  G[0][1] = -J[1][0] * r;
      G[1][0] = -J[0][1] * r; G[1][1] = J[0][0] * r;
    } else {
      det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
            J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
            J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      const double r = 1.0 / det;
      G[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * r;
      G[0][1] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]) * r;
      G[0][2] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * r;
      G[1][0] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) * r;
      G[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
      G[1][2] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) * r;
      G[2][0] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
      G[2][1] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) * r;
      G[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
    }
    const double adet = fabs(det);
    const double bv[3] = {co.b0, co.b1, co.b2};
    int k = 0;
    for (int a = 0; a < DIM; ++a)
      for (int b = a; b < DIM; ++b) {
        double s = 0.0;
        for (int d = 0; d < DIM; ++d) s += G[d][a] * G[d][b];
        coef[t][k++] = adet * co.eps * s;
      }
    for (int a = 0; a < DIM; ++a) {
      double s = 0.0;
      for (int d = 0; d < DIM; ++d) s += bv[d] * G[d][a];
      coef[t][k++] = adet * s;
    }
    coef[t][k] = adet * co.c;
    for (int d = 0; d < 3; ++d) {
      geo[t][d] = x0[d];
      for (int a = 0; a < 3; ++a) geo[t][3 + d * 3 + a] = J[d][a];
    }
    geo[t][12] = adet;
  }
  __syncthreads();
  // quadrature weights times |det J| times f at the mapped points, one
  // (cell, point) pair per thread
  for (int e = t; e < nc * NQ; e += blockDim.x) {
    const int cl = e / NQ, q = e % NQ;
    double x[3];
    for (int d = 0; d < DIM; ++d) {
      double s = geo[cl][d];
      for (int a = 0; a < DIM; ++a) s += geo[cl][3 + d * 3 + a] * xi[q * 3 + a];
      x[d] = s;
    }
    fq[cl][q] = w[q] * geo[cl][12] * rhs_value_pi(co, DIM, x);
  }
  __syncthreads();
  for (int e = t; e < nc * NB * NB; e += blockDim.x) {
    const int cl = e / (NB * NB), p = e % (NB * NB);
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < NT; ++k) s = fma(coef[cl][k], __ldg(T + k * NB * NB + p), s);
    K[(size_t)(c0 + cl) * NB * NB + p] = s;
  }
  for (int e = t; e < nc * NB; e += blockDim.x) {
    const int cl = e / NB, i = e % NB;
    double s = 0.0;
    for (int q = 0; q < NQ; ++q) s += fq[cl][q] * phi[q * NB + i];
    F[(size_t)(c0 + cl) * NB + i] = s;
  }
}

void build_ref_tensors(const RefTables& t, std::vector<double>& out) {
  const int D = t.dim, nb = t.nb, nq = t.nq;
  const int nt = n_ref_tensors(D);
  out.assign(size_t(nt) * nb * nb, 0.0);
  auto dphi = [&](int a, int q, int i) { return t.dphi[(size_t(a) * nq + q) * nb + i]; };
  int k = 0;
  for (int a = 0; a < D; ++a)
    for (int b = a; b < D; ++b, ++k)
      for (int i = 0; i < nb; ++i)
        for (int j = 0; j < nb; ++j) {
          double s = 0.0;
          for (int q = 0; q < nq; ++q) {
            s += t.w[q] * dphi(a, q, i) * dphi(b, q, j);
            if (a != b) s += t.w[q] * dphi(b, q, i) * dphi(a, q, j);
          }
          out[(size_t(k) * nb + i) * nb + j] = s;
        }
  for (int a = 0; a < D; ++a, ++k)
    for (int i = 0; i < nb; ++i)
      for (int j = 0; j < nb; ++j) {
        double s = 0.0;
        for (int q = 0; q < nq; ++q) s += t.w[q] * t.phi[size_t(q) * nb + i] * dphi(a, q, j);
        out[(size_t(k) * nb + i) * nb + j] = s;
      }
  for (int i = 0; i < nb; ++i)
    for (int j = 0; j < nb; ++j) {
      double s = 0.0;
      for (int q = 0; q < nq; ++q) s += t.w[q] * t.phi[size_t(q) * nb + i] * t.phi[size_t(q) * nb + j];
      out[(size_t(k) * nb + i) * nb + j] = s;
    }
}

template <int DIM, int NB, int NQ, int NV = DIM == 2 ? 4 : 8>
static void launch_elem_tensor(pm_ctx* c, int n_cells, const double* verts, const double* ref,
                               const double* T, const CdCoef& co, double* K, double* F) {
  constexpr int CHUNK = 64;
  const int grid = (n_cells + CHUNK - 1) / CHUNK;
  k_elem_cd_tensor<DIM, NB, NQ, CHUNK, NV><<<grid, 256, 0, c->stream>>>(n_cells, verts, ref, T, co, K, F);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

// stage 2: CSR values from the element matrices, in cell order
__global__ void k_gather(int nnz, const int* __restrict__ ptr, const int* __restrict__ idx,
                         const double* __restrict__ K, double* __restrict__ vals) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int t = ptr[e]; t < ptr[e + 1]; ++t) s += K[idx[t]];
    vals[e] = s;
  }
}

__global__ void k_set_unit(int n, const int* __restrict__ pos, double* __restrict__ vals) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) vals[pos[i]] = 1.0;
}

template <int DIM, int NB, int NQ, int CPB, int NV = DIM == 2 ? 4 : 8>
static void launch_elem(pm_ctx* c, int n_cells, const double* verts, const double* ref,
                        const CdCoef& co, double* K, double* F) {
  const size_t sm = size_t(CPB) * (2 * NQ * NB * 4 + NQ) * sizeof(double);
  auto kern = k_elem_cd<DIM, NB, NQ, CPB, NV>;
  if (sm > 48 * 1024) PM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm)));
  const int grid = (n_cells + CPB - 1) / CPB;
  kern<<<grid, 256, sm, c->stream>>>(n_cells, verts, ref, co, K, F);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

// Dirichlet values g = u(node) of the quadratic exact solution at the
// non-active DOFs (their rows are unit rows; the gather left their rhs 0)
__global__ void k_dirichlet_poly(int nb, int n_active, const double* __restrict__ xyz, CdCoef co,
                                 double* __restrict__ rhs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double x[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
  rhs[n_active + i] = poly_u(co.poly, x);
}

double poly_value_host(const double* p, const double* x) { return poly_u(p, x); }

// Exact solution of the coefficient kind and its gradient at x: the sine
// solution prod sin(pi x_d), the quadratic polynomial, or zero when the
// right-hand side is a constant (the examples without a known solution set
// their Exact to zero). out = (u, u_x, u_y, u_z).
__device__ __forceinline__ void exact_value(const CdCoef& k, int dim, const double* xin, double* out) {
  const double x[3] = {xin[0], xin[1], dim == 3 ? xin[2] : 0.0};
  out[0] = out[1] = out[2] = out[3] = 0.0;
  if (k.manufactured == 2) {
    const double* p = k.poly;
    out[0] = poly_u(p, x);
    out[1] = p[1] + 2 * p[4] * x[0] + p[7] * x[1] + p[8] * x[2];
    out[2] = p[2] + 2 * p[5] * x[1] + p[7] * x[0] + p[9] * x[2];
    out[3] = dim == 3 ? p[3] + 2 * p[6] * x[2] + p[8] * x[0] + p[9] * x[1] : 0.0;
  } else if (k.manufactured == 1) {
    const double pi = 3.14159265358979323846;
    double s[3], co[3];
    for (int d = 0; d < dim; ++d) {
      s[d] = sin(pi * x[d]);
      co[d] = cos(pi * x[d]);
    }
    if (dim == 2) {
      out[0] = s[0] * s[1];
      out[1] = pi * co[0] * s[1];
      out[2] = pi * s[0] * co[1];
    } else {
      out[0] = s[0] * s[1] * s[2];
      out[1] = pi * co[0] * s[1] * s[2];
      out[2] = pi * s[0] * co[1] * s[2];
      out[3] = pi * s[0] * s[1] * co[2];
    }
  }
}

// Neumann boundary integral (Assemble2D.C:716-757): for every edge on a
// Neumann side, rhs_i += sum_l g(x_l) hE w_l phi_i(xi_l) over the line Gauss
// rule of degree 2k (Gauss2 for Q1, Gauss3 for Q2), hE half the edge length,
// xi_l on edge m of [-1,1]^2 (vertex m to m+1, BaseFunct2D.C:87-118), only for
// active DOFs. g = eps grad u . n is the Neumann datum of the exact solution
// (SineLaplace's BoundValue on x = 1). One thread per DOF on a Neumann edge
// adds its edges in cell order, so the sum is deterministic.
struct LineRule {
  int n;
  double z[4], w[4];
};

template <int K>
__global__ void k_neumann_rhs(int nt, const int* __restrict__ dof, const int* __restrict__ ptr,
                              const int* __restrict__ cell, const int* __restrict__ code,
                              const double* __restrict__ verts, CdCoef co, LineRule lr,
                              double* __restrict__ rhs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const int g = dof[t];
  double acc = rhs[g];
  for (int e = ptr[t]; e < ptr[t + 1]; ++e) {
    const int c = cell[e], cd = code[e];
    const int m = cd & 3, side = (cd >> 2) & 3, loc = cd >> 4;
    const int m1 = (m + 1) & 3;
    const double* v = verts + size_t(c) * 8;
    const double ax = v[2 * m], ay = v[2 * m + 1], bx = v[2 * m1], by = v[2 * m1 + 1];
    const double hE = sqrt((bx - ax) * (bx - ax) + (by - ay) * (by - ay)) / 2;
    // reference vertices (-1,-1) (1,-1) (1,1) (-1,1)
    const double r0x = (m == 1 || m == 2) ? 1.0 : -1.0, r0y = m >= 2 ? 1.0 : -1.0;
    const double r1x = (m1 == 1 || m1 == 2) ? 1.0 : -1.0, r1y = m1 >= 2 ? 1.0 : -1.0;
    const int a = loc % (K + 1), b = loc / (K + 1);
    for (int l = 0; l < lr.n; ++l) {
      const double f = 0.5 * (lr.z[l] + 1.0);
      const double xi = r0x + f * (r1x - r0x), eta = r0y + f * (r1y - r0y);
      double lx[3], ly[3];
      if (K == 1) {
        lx[0] = 0.5 * (1.0 - xi); lx[1] = 0.5 * (1.0 + xi);
        ly[0] = 0.5 * (1.0 - eta); ly[1] = 0.5 * (1.0 + eta);
      } else {
        lx[0] = 0.5 * xi * (xi - 1.0); lx[1] = 1.0 - xi * xi; lx[2] = 0.5 * xi * (xi + 1.0);
        ly[0] = 0.5 * eta * (eta - 1.0); ly[1] = 1.0 - eta * eta; ly[2] = 0.5 * eta * (eta + 1.0);
      }
      const double x[3] = {ax + f * (bx - ax), ay + f * (by - ay), 0.0};
      double u[4];
      exact_value(co, 2, x, u);
      // outward normals of the sides y=0, x=1, y=1, x=0
      const double gn = side == 0 ? -u[2] : side == 1 ? u[1] : side == 2 ? u[2] : -u[1];
      double sv = co.eps * gn;
      sv *= hE * lr.w[l];
      acc += sv * (lx[a] * ly[b]);
    }
  }
  rhs[g] = acc;
}

void launch_neumann_values(pm_ctx* c, const DevAssemblyLevel& L, const pm_cd_coeffs& cf, double* rhs) {
  const int nt = int(L.nm_dof.n);
  // homogeneous Neumann data when the solution is not known (constant f)
  if (nt == 0 || cf.manufactured == 0) return;
  const int k = L.nloc == 9 ? 2 : 1;
  std::vector<double> z, w;
  gauss1d(k + 1, z, w);
  LineRule lr{};
  lr.n = k + 1;
  for (int l = 0; l < lr.n; ++l) {
    lr.z[l] = z[l];
    lr.w[l] = w[l];
  }
  const CdCoef co = make_coef(cf);
  const int grid = (nt + 127) / 128;
  if (k == 1)
    k_neumann_rhs<1><<<grid, 128, 0, c->stream>>>(nt, L.nm_dof.p, L.nm_ptr.p, L.nm_cell.p, L.nm_code.p,
                                                   L.verts.p, co, lr, rhs);
  else
    k_neumann_rhs<2><<<grid, 128, 0, c->stream>>>(nt, L.nm_dof.p, L.nm_ptr.p, L.nm_cell.p, L.nm_code.p,
                                                   L.verts.p, co, lr, rhs);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

// Error functional of ConvectionDiffusion<d>::output (ConvectionDiffusion.C:213-283):
// TFEFunction{2,3}D::GetErrors (FEFunction2D.C:318-575, FEFunction3D.C:80-245)
// with conv_diff_l2_h1_linf_error (ConvDiff.C:2134-2185). Per cell and
// quadrature point, e = u_h - u, w = weight |det J|:
//   L2^2 += w e^2,  H1^2 += w |grad e|^2,  L_inf = max |e|,
//   SD^2 += w (eps |grad e|^2 + c e^2 + delta (b . grad e)^2)
// with the SUPG parameter delta of Compute_SDFEM_delta (ConvDiff.C:273-360)
// at the reference's defaults (SDFEM_TYPE 2, DELTA0 1, polynomial degree 1,
// CELL_MEASURE 0: hK = cell diameter). One thread per cell; each block sums
// its cells by a fixed tree into one partial, a second kernel sums the
// partials in a fixed order: the result does not depend on scheduling.
template <int DIM, int NB, int NQ, int NV = DIM == 2 ? 4 : 8>
__global__ void __launch_bounds__(128) k_cd_errors(int n_cells, const double* __restrict__ verts,
                                                   const int* __restrict__ dofmap, const double* __restrict__ u,
                                                   const double* __restrict__ ref, CdCoef co,
                                                   double* __restrict__ partial) {
  __shared__ double red[4][128];
  const int cell = blockIdx.x * 128 + threadIdx.x;
  double loc[4] = {0.0, 0.0, 0.0, 0.0};
  if (cell < n_cells) {
    const double* v = verts + size_t(cell) * NV * DIM;
    double x0[3] = {0, 0, 0}, J[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    affine_map<DIM, NV>(v, x0, J);
    double G[3][3] = {{0}}, det;
    if (DIM == 2) {
      det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      const double r = 1.0 / det;
      G[0][0] = J[1][1] * r;  G[0][1] = -J[1][0] * r;
      G[1][0] = -J[0][1] * r; G[1][1] = J[0][0] * r;
    } else {
      det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
            J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
            J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      const double r = 1.0 / det;
      G[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * r;
      G[0][1] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]) * r;
      G[0][2] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * r;
      G[1][0] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) * r;
      G[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
      G[1][2] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) * r;
      G[2][0] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
      G[2][1] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) * r;
      G[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
    }
    const double adet = fabs(det);
    // cell diameter: the largest distance between two vertices
    double hk2 = 0.0;
    for (int i = 0; i < NV; ++i)
      for (int j = i + 1; j < NV; ++j) {
        double s = 0.0;
        for (int d = 0; d < DIM; ++d) s += (v[i * DIM + d] - v[j * DIM + d]) * (v[i * DIM + d] - v[j * DIM + d]);
        hk2 = fmax(hk2, s);
      }
    const double hK = sqrt(hk2);
    const double bv[3] = {co.b0, co.b1, DIM == 3 ? co.b2 : 0.0};
    const double eps = fabs(co.eps) < 1e-20 ? 1e-20 : co.eps;
    const double norm_b = sqrt(bv[0] * bv[0] + bv[1] * bv[1] + bv[2] * bv[2]);
    double delta = 0.0;
    if (norm_b > 0) {
      const double alpha = norm_b * hK / (2 * eps);
      delta = hK * (1 / tanh(alpha) - 1 / alpha) / (2 * norm_b);
    }
    double uc[NB];
    for (int i = 0; i < NB; ++i) uc[i] = u[dofmap[size_t(cell) * NB + i]];
    const double* phi = ref;
    const double* dphi = ref + NQ * NB;
    const double* w = ref + 4 * NQ * NB;
    const double* xi = w + NQ;
    for (int q = 0; q < NQ; ++q) {
      double val = 0.0, dr[3] = {0.0, 0.0, 0.0};
      for (int i = 0; i < NB; ++i) {
        val += uc[i] * phi[q * NB + i];
        for (int a = 0; a < DIM; ++a) dr[a] += uc[i] * dphi[(a * NQ + q) * NB + i];
      }
      double grad[3] = {0.0, 0.0, 0.0};
      for (int d = 0; d < DIM; ++d)
        for (int a = 0; a < DIM; ++a) grad[d] += G[d][a] * dr[a];
      double x[3];
      for (int d = 0; d < DIM; ++d) {
        double s = x0[d];
        for (int a = 0; a < DIM; ++a) s += J[d][a] * xi[q * 3 + a];
        x[d] = s;
      }
      double ex[4];
      exact_value(co, DIM, x, ex);
      const double wq = w[q] * adet;
      const double e0 = val - ex[0];
      const double e1 = grad[0] - ex[1], e2 = grad[1] - ex[2], e3 = DIM == 3 ? grad[2] - ex[3] : 0.0;
      loc[0] += wq * e0 * e0;
      loc[1] += wq * (e1 * e1 + e2 * e2 + e3 * e3);
      const double e4 = bv[0] * e1 + bv[1] * e2 + bv[2] * e3;
      loc[2] += wq * (co.eps * (e1 * e1 + e2 * e2 + e3 * e3) + co.c * e0 * e0 + delta * e4 * e4);
      loc[3] = fmax(loc[3], fabs(e0));
    }
  }
  for (int k = 0; k < 4; ++k) red[k][threadIdx.x] = loc[k];
  __syncthreads();
  for (int s = 64; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      for (int k = 0; k < 3; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + s];
      red[3][threadIdx.x] = fmax(red[3][threadIdx.x], red[3][threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) partial[size_t(blockIdx.x) * 4 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void __launch_bounds__(256) k_cd_errors_finish(int nparts, const double* __restrict__ partial,
                                                          double* __restrict__ out) {
  __shared__ double red[4][256];
  double loc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < nparts; i += 256) {
    for (int k = 0; k < 3; ++k) loc[k] += partial[size_t(i) * 4 + k];
    loc[3] = fmax(loc[3], partial[size_t(i) * 4 + 3]);
  }
  for (int k = 0; k < 4; ++k) red[k][threadIdx.x] = loc[k];
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      for (int k = 0; k < 3; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + s];
      red[3][threadIdx.x] = fmax(red[3][threadIdx.x], red[3][threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 3) out[threadIdx.x] = sqrt(red[threadIdx.x][0]);
  if (threadIdx.x == 3) out[3] = red[3][0];
}

int error_blocks(int n_cells) { return (n_cells + 127) / 128; }

void launch_cd_errors(pm_ctx* c, int dim, int k, int qn, int n_cells, const double* verts, const int* dofmap,
                      const double* u, const DevRefTables& rt, const pm_cd_coeffs& cf, double* partial,
                      double* out) {
  const CdCoef co = make_coef(cf);
  const int grid = error_blocks(n_cells);
  if (dim == 2 && k == 1 && qn == 2) k_cd_errors<2, 4, 4><<<grid, 128, 0, c->stream>>>(n_cells, verts, dofmap, u, rt.data.p, co, partial);
  else if (dim == 2 && k == 1 && qn == 3) k_cd_errors<2, 4, 9><<<grid, 128, 0, c->stream>>>(n_cells, verts, dofmap, u, rt.data.p, co, partial);
  else if (dim == 2 && k == 2 && qn == 3) k_cd_errors<2, 9, 9><<<grid, 128, 0, c->stream>>>(n_cells, verts, dofmap, u, rt.data.p, co, partial);
  else if (dim == 2 && k == 2 && qn == 4) k_cd_errors<2, 9, 16><<<grid, 128, 0, c->stream>>>(n_cells, verts, dofmap, u, rt.data.p, co, partial);
  else if (dim == 3 && k == 1 && qn == 3) k_cd_errors<3, 8, 27><<<grid, 128, 0, c->stream>>>(n_cells, verts, dofmap, u, rt.data.p, co, partial);
  else if (dim == 3 && k == 1 && qn == 2) k_cd_errors<3, 8, 8><<<grid, 128, 0, c->stream>>>(n_cells, verts, dofmap, u, rt.data.p, co, partial);
  else if (dim == 3 && k == 2 && qn == 4) k_cd_errors<3, 27, 64><<<grid, 128, 0, c->stream>>>(n_cells, verts, dofmap, u, rt.data.p, co, partial);
  else if (dim == 3 && k == 2 && qn == 3) k_cd_errors<3, 27, 27><<<grid, 128, 0, c->stream>>>(n_cells, verts, dofmap, u, rt.data.p, co, partial);
  else if (k == 11 && qn == 11) k_cd_errors<3, 4, 11, 4><<<grid, 128, 0, c->stream>>>(n_cells, verts, dofmap, u, rt.data.p, co, partial);
  else if (k == 11 && qn == 15) k_cd_errors<3, 4, 15, 4><<<grid, 128, 0, c->stream>>>(n_cells, verts, dofmap, u, rt.data.p, co, partial);
  else if (k == 12 && qn == 11) k_cd_errors<3, 10, 11, 4><<<grid, 128, 0, c->stream>>>(n_cells, verts, dofmap, u, rt.data.p, co, partial);
  else if (k == 12 && qn == 15) k_cd_errors<3, 10, 15, 4><<<grid, 128, 0, c->stream>>>(n_cells, verts, dofmap, u, rt.data.p, co, partial);
  else throw Error(PM_E_UNSUPPORTED, "error functional: element / quadrature combination not compiled");
  PM_CHECK_LAUNCH();
  k_cd_errors_finish<<<1, 256, 0, c->stream>>>(grid, partial, out);
  PM_CHECK_LAUNCH();
  c->kernel_launches += 2;
}

void launch_dirichlet_values(pm_ctx* c, const DevAssemblyLevel& L, const pm_cd_coeffs& cf, double* rhs) {
  const int nb = int(L.bnd_xyz.n / 3);
  if (cf.manufactured != 2 || nb == 0) return;
  k_dirichlet_poly<<<(nb + 255) / 256, 256, 0, c->stream>>>(nb, L.n_active, L.bnd_xyz.p, make_coef(cf), rhs);
  PM_CHECK_LAUNCH();
  c->kernel_launches++;
}

void DevAssemblyLevel::upload(pm_ctx* c, const DiscLevel& L, int dim, int nvc) {
  n_cells = L.n_cells;
  nloc = L.space.nloc;
  n_dofs = L.sys.n_rows;
  n_active = L.sys.n_active;
  bnd_xyz.upload(L.bnd_xyz, c->stream);
  verts.upload(L.verts, c->stream);
  gat_ptr.upload(L.gat_ptr, c->stream);
  gat_idx.upload(L.gat_idx, c->stream);
  rgat_ptr.upload(L.rgat_ptr, c->stream);
  rgat_idx.upload(L.rgat_idx, c->stream);
  diag_pos.upload(L.diag_pos, c->stream);
  nm_dof.upload(L.nm_dof, c->stream);
  nm_ptr.upload(L.nm_ptr, c->stream);
  nm_cell.upload(L.nm_cell, c->stream);
  nm_code.upload(L.nm_code, c->stream);
  (void)dim;
  (void)nvc;
}

void DevAssemblyLevel::scratch_sizes(size_t& k_elems, size_t& f_elems) const {
  k_elems = size_t(n_cells) * nloc * nloc;
  f_elems = size_t(n_cells) * nloc;
}

// Element matrices and element right-hand sides of one level into K and F: by
// the reference-tensor contraction (default) or, with the context option
// assembly_quadrature_loop, by the per-quadrature-point loop. Shared by
// pm_assemble_cd / pm_problem_assemble and the allocation-free entry point,
// so both give the same bits.
void launch_cd_elements(pm_ctx* c, const DevAssemblyLevel& L, int dim, int k, int qn,
                        const pm_cd_coeffs& cf, const DevRefTables& rt, double* K, double* F) {
  const CdCoef co = make_coef(cf);
  const double* T = rt.tensors.p;
  if (!c->assembly_quadrature_loop && T) {
    if (dim == 2 && k == 1 && qn == 3) launch_elem_tensor<2, 4, 9>(c, L.n_cells, L.verts.p, rt.data.p, T, co, K, F);
    else if (dim == 2 && k == 1 && qn == 2) launch_elem_tensor<2, 4, 4>(c, L.n_cells, L.verts.p, rt.data.p, T, co, K, F);
    else if (dim == 2 && k == 2 && qn == 3) launch_elem_tensor<2, 9, 9>(c, L.n_cells, L.verts.p, rt.data.p, T, co, K, F);
    else if (dim == 2 && k == 2 && qn == 4) launch_elem_tensor<2, 9, 16>(c, L.n_cells, L.verts.p, rt.data.p, T, co, K, F);
    else if (dim == 3 && k == 1 && qn == 2) launch_elem_tensor<3, 8, 8>(c, L.n_cells, L.verts.p, rt.data.p, T, co, K, F);
    else if (dim == 3 && k == 1 && qn == 3) launch_elem_tensor<3, 8, 27>(c, L.n_cells, L.verts.p, rt.data.p, T, co, K, F);
    else if (dim == 3 && k == 2 && qn == 3) launch_elem_tensor<3, 27, 27>(c, L.n_cells, L.verts.p, rt.data.p, T, co, K, F);
    else if (dim == 3 && k == 2 && qn == 4) launch_elem_tensor<3, 27, 64>(c, L.n_cells, L.verts.p, rt.data.p, T, co, K, F);
    else if (k == 11 && qn == 11) launch_elem_tensor<3, 4, 11, 4>(c, L.n_cells, L.verts.p, rt.data.p, T, co, K, F);
    else if (k == 11 && qn == 15) launch_elem_tensor<3, 4, 15, 4>(c, L.n_cells, L.verts.p, rt.data.p, T, co, K, F);
    else if (k == 12 && qn == 11) launch_elem_tensor<3, 10, 11, 4>(c, L.n_cells, L.verts.p, rt.data.p, T, co, K, F);
    else if (k == 12 && qn == 15) launch_elem_tensor<3, 10, 15, 4>(c, L.n_cells, L.verts.p, rt.data.p, T, co, K, F);
    else throw Error(PM_E_UNSUPPORTED, "element / quadrature combination not compiled");
  } else if (dim == 2 && k == 1 && qn == 3) launch_elem<2, 4, 9, 16>(c, L.n_cells, L.verts.p, rt.data.p, co, K, F);
  else if (dim == 2 && k == 1 && qn == 2) launch_elem<2, 4, 4, 16>(c, L.n_cells, L.verts.p, rt.data.p, co, K, F);
  else if (dim == 2 && k == 2 && qn == 3) launch_elem<2, 9, 9, 4>(c, L.n_cells, L.verts.p, rt.data.p, co, K, F);
  else if (dim == 2 && k == 2 && qn == 4) launch_elem<2, 9, 16, 4>(c, L.n_cells, L.verts.p, rt.data.p, co, K, F);
  else if (dim == 3 && k == 1 && qn == 2) launch_elem<3, 8, 8, 4>(c, L.n_cells, L.verts.p, rt.data.p, co, K, F);
  else if (dim == 3 && k == 1 && qn == 3) launch_elem<3, 8, 27, 2>(c, L.n_cells, L.verts.p, rt.data.p, co, K, F);
  else if (dim == 3 && k == 2 && qn == 3) launch_elem<3, 27, 27, 1>(c, L.n_cells, L.verts.p, rt.data.p, co, K, F);
  else if (dim == 3 && k == 2 && qn == 4) launch_elem<3, 27, 64, 1>(c, L.n_cells, L.verts.p, rt.data.p, co, K, F);
  else if (k == 11 && qn == 11) launch_elem<3, 4, 11, 16, 4>(c, L.n_cells, L.verts.p, rt.data.p, co, K, F);
  else if (k == 11 && qn == 15) launch_elem<3, 4, 15, 16, 4>(c, L.n_cells, L.verts.p, rt.data.p, co, K, F);
  else if (k == 12 && qn == 11) launch_elem<3, 10, 11, 4, 4>(c, L.n_cells, L.verts.p, rt.data.p, co, K, F);
  else if (k == 12 && qn == 15) launch_elem<3, 10, 15, 4, 4>(c, L.n_cells, L.verts.p, rt.data.p, co, K, F);
  else throw Error(PM_E_UNSUPPORTED, "element / quadrature combination not compiled");
}

void assemble_cd_level(pm_ctx* c, const DevAssemblyLevel& L, int dim, int elem, int qn,
                       const pm_cd_coeffs& cf, const DevRefTables& rt, DevCsr& A, double* rhs,
                       double* K, double* F) {
  launch_cd_elements(c, L, dim, elem, qn, cf, rt, K, F);
  const int nnz = int(A.nnz);
  k_gather<<<std::max(1, std::min((nnz + 255) / 256, c->num_sms * 16)), 256, 0, c->stream>>>(
      nnz, L.gat_ptr.p, L.gat_idx.p, K, A.vals.p);
  PM_CHECK_LAUNCH();
  const int nd = int(L.diag_pos.n);
  if (nd) {
    k_set_unit<<<(nd + 255) / 256, 256, 0, c->stream>>>(nd, L.diag_pos.p, A.vals.p);
    PM_CHECK_LAUNCH();
  }
  const int n = L.n_dofs;
  k_gather<<<std::max(1, std::min((n + 255) / 256, c->num_sms * 16)), 256, 0, c->stream>>>(
      n, L.rgat_ptr.p, L.rgat_idx.p, F, rhs);
  PM_CHECK_LAUNCH();
  c->kernel_launches += nd ? 3 : 2;
  launch_dirichlet_values(c, L, cf, rhs);
  launch_neumann_values(c, L, cf, rhs);
  A.values_changed(c);
}

void DevRefTables::upload(pm_ctx* c, const RefTables& t) {
  // layout: phi[nq][nb], dphi[3][nq][nb], w[nq], xi[nq][3]
  std::vector<double> h;
  h.insert(h.end(), t.phi.begin(), t.phi.end());
  h.insert(h.end(), t.dphi.begin(), t.dphi.end());
  h.insert(h.end(), t.w.begin(), t.w.end());
  h.insert(h.end(), t.xi.begin(), t.xi.end());
  data.upload(h, c->stream);
  nb = t.nb;
  nq = t.nq;
  std::vector<double> tens;
  build_ref_tensors(t, tens);
  tensors.upload(tens, c->stream);
  nt = n_ref_tensors(t.dim);
}

}  // namespace pm

// ---------------------------------------------------------------------------
// Assembly without device allocation.
//
// pm_assemble_cd allocates its scratch (the element matrices and element
// right-hand sides of a level) with cudaMalloc on every call. Some callers
// cannot do that: a serving worker that must not stall other requests (a
// cudaMalloc may synchronise the device), code running under a fixed memory
// budget that was reserved up front, or a host that allocates all device
// memory itself. pm_assemble_cd_noalloc runs the same element and gather
// kernels with the scratch placed in the file-scope array below instead.
//
// The array holds kNoAllocScratchDoubles doubles (4 Mi doubles = 32 MiB). Every
// GPU that loads this library holds it until the process exits. A level needs
// n_cells*nloc*nloc + n_cells*nloc doubles, e.g. 3.1 Mi for 16^3 Q2 hexahedra;
// larger levels are rejected with PM_E_INVALID.
#include <mutex>

#include "pm_problem.h"

namespace {
constexpr size_t kNoAllocScratchDoubles = size_t(4) << 20;
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
double* g_noalloc_scratch_addr[kMaxDevices] = {nullptr};
}  // namespace

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

// Device address of the scratch array on `device`. In host code the name
// g_noalloc_scratch is only a host-side stand-in, not a device address, so
// the address is looked up once per device with that device current.
static int noalloc_scratch(int device, double** out, std::string& err) {
  if (device < 0 || device >= kMaxDevices) {
    err = "device index out of range";
    return PM_E_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_scratch_addr[device]) {
    int prev = -1;
    cudaError_t e = cudaGetDevice(&prev);
    if (e == cudaSuccess && prev != device) e = cudaSetDevice(device);
    void* ptr = nullptr;
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    if (e != cudaSuccess || !ptr) {
      err = std::string("cudaGetSymbolAddress of the assembly scratch failed: ") + cudaGetErrorString(e);
      cudaGetLastError();
      return PM_E_CUDA;
    }
    g_noalloc_scratch_addr[device] = static_cast<double*>(ptr);
  }
  *out = g_noalloc_scratch_addr[device];
  return PM_OK;
}


/* Assembly of one level of a convection-diffusion problem into caller-owned
 * device arrays, with no device allocation (see the comment block above).
 * vals_dev receives the level matrix values in the level's CSR order (nnz
 * doubles), rhs_dev the right-hand side (n_dofs doubles). coeffs == NULL uses
 * the problem's coefficients. Runs on the problem's context stream.
 *
 * The first call on a device looks up the scratch address (cudaGetSymbolAddress);
 * make that first call before any stream capture. All calls share the one
 * scratch array, which keeps the last call's contents: the element kernels
 * overwrite every scratch entry a call reads, so nothing needs clearing, but
 * calls whose work overlaps on the GPU (other streams or host threads) race
 * on the array and must be serialised by the caller. */
extern "C" int pm_assemble_cd_noalloc(pm_problem* p, int level, const pm_cd_coeffs* coeffs,
                                      double* vals_dev, double* rhs_dev) {
  if (!p || !vals_dev || !rhs_dev) return PM_E_INVALID;
  pm_ctx* c = p->ctx;
  try {
    if (p->kind != 0) {
      c->last_error = "pm_assemble_cd_noalloc: convection-diffusion problems only";
      return PM_E_UNSUPPORTED;
    }
    if (level < 0 || level >= int(p->alev.size())) {
      c->last_error = "level out of range";
      return PM_E_INVALID;
    }
    const pm::DevAssemblyLevel& L = p->alev[level];
    const size_t kn = size_t(L.n_cells) * L.nloc * L.nloc, fn = size_t(L.n_cells) * L.nloc;
    if (kn + fn > kNoAllocScratchDoubles) {
      c->last_error = "level needs " + std::to_string(kn + fn) +
                      " doubles of assembly scratch; the allocation-free assembly holds at most " +
                      std::to_string(kNoAllocScratchDoubles) + " (32 MiB)";
      return PM_E_INVALID;
    }
    double* scratch = nullptr;
    int rc = noalloc_scratch(c->device, &scratch, c->last_error);
    if (rc != PM_OK) return rc;
    double* K = scratch;
    double* F = scratch + kn;
    const pm::Disc& D = *p->disc->d;
    pm::launch_cd_elements(c, L, D.dim(), D.elem, p->qn, coeffs ? *coeffs : p->coeffs, p->ref, K, F);
    const int nnz = int(p->mats[level]->csr.nnz);
    pm::k_gather<<<std::max(1, std::min((nnz + 255) / 256, c->num_sms * 16)), 256, 0, c->stream>>>(
        nnz, L.gat_ptr.p, L.gat_idx.p, K, vals_dev);
    const int nd = int(L.diag_pos.n);
    if (nd) pm::k_set_unit<<<(nd + 255) / 256, 256, 0, c->stream>>>(nd, L.diag_pos.p, vals_dev);
    const int n = L.n_dofs;
    pm::k_gather<<<std::max(1, std::min((n + 255) / 256, c->num_sms * 16)), 256, 0, c->stream>>>(
        n, L.rgat_ptr.p, L.rgat_idx.p, F, rhs_dev);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      c->last_error = std::string("kernel launch failed: ") + cudaGetErrorString(e);
      return PM_E_CUDA;
    }
    c->kernel_launches += nd ? 3 : 2;
    pm::launch_dirichlet_values(c, L, coeffs ? *coeffs : p->coeffs, rhs_dev);
    pm::launch_neumann_values(c, L, coeffs ? *coeffs : p->coeffs, rhs_dev);
    return PM_OK;
  } catch (const pm::Error& e) {
    c->last_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    c->last_error = e.what();
    return PM_E_INVALID;
  }
}
