/*
 * oracle.c - CPU restatement of ParMooN's solve path, used ONLY as the checker
 * of the GPU library (tests, __graft_entry__.smoke, and bench.py's CPU
 * baseline). It is test infrastructure, never part of the product path.
 *
 * Each function follows the reference routine named in its comment, in the
 * same loop and operation order (sequential sums, cell-wise scatter with a
 * linear search of the CSR row, cell-wise grid transfer with multiplicity
 * averaging, literal multigrid cycle control, literal flexible GMRES).
 * Reference paths are relative to the ParMooN source tree.
 *
 * Third-party arithmetic the reference delegates: the coarse direct solve
 * (UMFPACK, src/Solver/DirectSolver.C:325-433) and Vanka's local LU (LAPACK
 * dgetrf/dgetrs, src/Matrix/DenseMatrix.C:136-177) are restated here as a dense
 * LU with partial pivoting; their internals are not pinned to those libraries.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define MAXNB 64
#define MAXQ 64

/* ------------------------------------------------------------ BLAS-1 ------
 * Ddot / Dnorm / Daxpy (src/FE/Blas1.C:14-115): sequential left-to-right. */
double orc_dot(int n, const double* x, const double* y) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += x[i] * y[i];
  return s;
}
double orc_norm(int n, const double* x) { return sqrt(orc_dot(n, x, x)); }
static void axpy(int n, double a, const double* x, double* y) {
  for (int i = 0; i < n; ++i) y[i] += a * x[i];
}

/* ------------------------------------------------------------ SpMV --------
 * FEMatrix::multiplyActive (src/Matrix/FEMatrix.C:186-198) on rows < n_active,
 * then BlockVector::addScaledNonActive (src/Matrix/BlockVector.C:212) on the
 * remaining rows: BlockFEMatrix::apply_scaled_add (BlockFEMatrix.C:863). The
 * active flags allow block vectors with several non-active tails. */
void orc_apply_scaled_add(int n_rows, const unsigned char* active, const int* rp, const int* ci,
                          const double* v, const double* x, double* y, double a) {
  for (int i = 0; i < n_rows; ++i) {
    if (!active[i]) continue;
    double val = 0.0;
    for (int j = rp[i]; j < rp[i + 1]; ++j) val += v[j] * x[ci[j]];
    y[i] += a * val;
  }
  for (int i = 0; i < n_rows; ++i)
    if (!active[i]) y[i] += a * x[i];
}

/* TMatrix::multiply (src/Matrix/Matrix.C:430-451): every row */
void orc_multiply(int n_rows, const int* rp, const int* ci, const double* v, const double* x,
                  double* y, double a) {
  if (a == 0.0) return;
  for (int i = 0; i < n_rows; ++i) {
    double val = 0.0;
    for (int j = rp[i]; j < rp[i + 1]; ++j) val += v[j] * x[ci[j]];
    y[i] += a * val;
  }
}

/* ------------------------------------------------------- quadrature -------
 * QuadFormulaQuad::Gauss3 (src/QuadFormulas/QuadFormulaQuad.C:43),
 * QuadFormulaHexa::Gauss2/3/4 (src/QuadFormulas/QuadFormulaHexa.C:41-120):
 * point l = i*n*n + j*n + k has x = onexi[k], y = onexi[j], z = onexi[i]. */
static int gauss_rule(int dim, int n, double* xq, double* wq) {
  double ox[4], ow[4];
  if (n == 2) {
    ox[0] = -0.5773502691896257645091489; ox[1] = 0.5773502691896257645091489;
    ow[0] = 1.0; ow[1] = 1.0;
  } else if (n == 3) {
    ox[0] = -0.7745966692414833770358530; ox[1] = 0.0; ox[2] = 0.7745966692414833770358530;
    ow[0] = 0.5555555555555555555555558; ow[1] = 0.8888888888888888888888888;
    ow[2] = 0.5555555555555555555555558;
  } else if (n == 4) {
    ox[0] = 0.33998104358485626480266576; ox[1] = 0.86113631159405257522394649;
    ox[2] = -0.86113631159405257522394649; ox[3] = -0.33998104358485626480266576;
    ow[0] = 0.652145154862546142626936051; ow[1] = 0.347854845137453857373063949;
    ow[2] = 0.347854845137453857373063949; ow[3] = 0.652145154862546142626936051;
  } else {
    return -1;
  }
  int l = 0;
  if (dim == 2) {
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < n; ++k, ++l) {
        xq[3 * l] = ox[k]; xq[3 * l + 1] = ox[j]; xq[3 * l + 2] = 0.0;
        wq[l] = ow[j] * ow[k];
      }
  } else {
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k, ++l) {
          xq[3 * l] = ox[k]; xq[3 * l + 1] = ox[j]; xq[3 * l + 2] = ox[i];
          wq[l] = ow[i] * ow[j] * ow[k];
        }
  }
  return l;
}

/* Qk basis (tensor Lagrange, local DOFs lexicographic with xi fastest as in
 * include/FE2D/BF_C_Q_Q1_2D.h, BF_C_Q_Q2_2D.h, include/FE3D/BF_C_H_Q1_3D.h,
 * BF_C_H_Q2_3D.h): values and reference derivatives */
static void q1d(int k, double x, double* l, double* d) {
  if (k == 1) {
    l[0] = 0.5 * (1 - x); l[1] = 0.5 * (1 + x);
    d[0] = -0.5; d[1] = 0.5;
  } else {
    l[0] = 0.5 * x * (x - 1); l[1] = 1 - x * x; l[2] = 0.5 * x * (x + 1);
    d[0] = x - 0.5; d[1] = -2 * x; d[2] = x + 0.5;
  }
}
static int qk_eval(int dim, int k, const double* xi, double* phi, double* dx, double* dy, double* dz) {
  double lx[3], ly[3], lz[3], ddx[3], ddy[3], ddz[3];
  q1d(k, xi[0], lx, ddx);
  q1d(k, xi[1], ly, ddy);
  if (dim == 3) q1d(k, xi[2], lz, ddz);
  int m = 0;
  for (int c = 0; c < (dim == 3 ? k + 1 : 1); ++c)
    for (int b = 0; b <= k; ++b)
      for (int a = 0; a <= k; ++a, ++m) {
        double zc = dim == 3 ? lz[c] : 1.0;
        phi[m] = lx[a] * ly[b] * zc;
        if (dx) {
          dx[m] = ddx[a] * ly[b] * zc;
          dy[m] = lx[a] * ddy[b] * zc;
          if (dim == 3) dz[m] = lx[a] * ly[b] * ddz[c];
        }
      }
  return m;
}

/* exact solution u = prod sin(pi x_d) and f = -eps*Lap u + b.grad u + c u in
 * the order of the example callbacks (include/Examples/CD_2D/SineLaplace.h) */
/* quadratic exact solution u = p0 + p1 x + p2 y + p3 z + p4 x^2 + p5 y^2 +
 * p6 z^2 + p7 xy + p8 xz + p9 yz (the test_p0 / test_p1 / test_p2 examples of
 * src/Examples/Example_CD3D.C:164-193 are of this form) */
double orc_poly_u(const double* p, const double* x) {
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

double orc_poly_rhs(int dim, const double* xin, double eps, const double* b, double c, const double* p,
                    const double* src) {
  const double x[3] = {xin[0], xin[1], dim == 3 ? xin[2] : 0.0};
  const double u = orc_poly_u(p, x);
  const double ux = p[1] + 2 * p[4] * x[0] + p[7] * x[1] + p[8] * x[2];
  const double uy = p[2] + 2 * p[5] * x[1] + p[7] * x[0] + p[9] * x[2];
  const double uz = p[3] + 2 * p[6] * x[2] + p[8] * x[0] + p[9] * x[1];
  const double lap = dim == 3 ? 2 * (p[4] + p[5] + p[6]) : 2 * (p[4] + p[5]);
  double f = -eps * lap;
  f += b[0] * ux + b[1] * uy + (dim == 3 ? b[2] * uz : 0.0);
  f += c * u;
  if (src) f += orc_poly_u(src, x);
  return f;
}

static double rhs_f(int dim, const double* x, double eps, const double* b, double c, int manuf,
                    double fconst, const double* poly) {
  if (!manuf) return fconst;
  if (manuf == 2) return orc_poly_rhs(dim, x, eps, b, c, poly, poly ? poly + 10 : NULL);
  const double p = 3.14159265358979323846;
  double u, ux, uy, uz = 0, lap;
  if (dim == 2) {
    u = sin(p * x[0]) * sin(p * x[1]);
    ux = p * cos(p * x[0]) * sin(p * x[1]);
    uy = p * sin(p * x[0]) * cos(p * x[1]);
    lap = -2 * p * p * sin(p * x[0]) * sin(p * x[1]);
  } else {
    u = sin(p * x[0]) * sin(p * x[1]) * sin(p * x[2]);
    ux = p * cos(p * x[0]) * sin(p * x[1]) * sin(p * x[2]);
    uy = p * sin(p * x[0]) * cos(p * x[1]) * sin(p * x[2]);
    uz = p * sin(p * x[0]) * sin(p * x[1]) * cos(p * x[2]);
    lap = -3 * p * p * sin(p * x[0]) * sin(p * x[1]) * sin(p * x[2]);
  }
  double f = -eps * lap;
  f += b[0] * ux + b[1] * uy + (dim == 3 ? b[2] * uz : 0.0);
  f += c * u;
  return f;
}

/* ------------------------------------------------------- assembly ---------
 * Assemble2D/Assemble3D (src/AssembleRoutines/Assemble3D.C:228-470) with
 * LocalAssembling::GetLocalForms (LocalAssembling.C:669-765) and
 * BilinearAssembleGalerkin<d> (ConvDiff.C:1794-1856). Affine cells: QuadAffin
 * (src/FE/QuadAffin.C:614) / HexaAffin (src/FE/HexaAffin.C:858).
 * verts: n_cells * nv * dim; dofmap: n_cells * nloc. vals / rhs are reset. */
int orc_assemble_cd_poly(int dim, int k, int qn, int n_cells, const double* verts, int nloc,
                         const int* dofmap, int n_rows, int n_active, const int* rp, const int* ci,
                         double eps, const double* b, double c, int manuf, double fconst, const double* poly,
                         double* vals, double* rhs);

int orc_assemble_cd(int dim, int k, int qn, int n_cells, const double* verts, int nloc,
                    const int* dofmap, int n_rows, int n_active, const int* rp, const int* ci,
                    double eps, const double* b, double c, int manuf, double fconst, double* vals,
                    double* rhs) {
  if (manuf == 2) return -2; /* the polynomial needs orc_assemble_cd_poly */
  return orc_assemble_cd_poly(dim, k, qn, n_cells, verts, nloc, dofmap, n_rows, n_active, rp, ci, eps, b, c,
                              manuf, fconst, NULL, vals, rhs);
}

/* the same; manuf = 2 takes f from the quadratic exact solution poly[0..9]
 * plus the source polynomial poly[10..19] (the time derivative of a
 * time-dependent exact solution); the Dirichlet values are set by the
 * caller: the non-active rhs entries stay 0 */
int orc_assemble_cd_poly(int dim, int k, int qn, int n_cells, const double* verts, int nloc,
                         const int* dofmap, int n_rows, int n_active, const int* rp, const int* ci,
                         double eps, const double* b, double c, int manuf, double fconst, const double* poly,
                         double* vals, double* rhs) {
  if (manuf == 2 && !poly) return -2;
  double xq[3 * MAXQ], wq[MAXQ];
  const int nq = gauss_rule(dim, qn, xq, wq);
  if (nq < 0) return -1;
  const int nv = dim == 2 ? 4 : 8;
  static double phi[MAXQ][MAXNB], dxr[MAXQ][MAXNB], dyr[MAXQ][MAXNB], dzr[MAXQ][MAXNB];
  for (int q = 0; q < nq; ++q) {
    int m = qk_eval(dim, k, xq + 3 * q, phi[q], dxr[q], dyr[q], dzr[q]);
    if (m != nloc) return -2;
  }
  memset(vals, 0, sizeof(double) * (size_t)rp[n_rows]);
  memset(rhs, 0, sizeof(double) * (size_t)n_rows);
  double Kloc[MAXNB][MAXNB], Floc[MAXNB];
  for (int cell = 0; cell < n_cells; ++cell) {
    const double* v = verts + (size_t)cell * nv * dim;
    double x0[3], J[3][3] = {{0}};
    if (dim == 2) {
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
    double det, G[3][3];
    if (dim == 2) {
      det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      G[0][0] = J[1][1] / det; G[0][1] = -J[1][0] / det;
      G[1][0] = -J[0][1] / det; G[1][1] = J[0][0] / det;
    } else {
      det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
            J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
            J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      G[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
      G[0][1] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]) / det;
      G[0][2] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
      G[1][0] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) / det;
      G[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
      G[1][2] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) / det;
      G[2][0] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
      G[2][1] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) / det;
      G[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    }
    const double adet = fabs(det);
    for (int i = 0; i < nloc; ++i) {
      Floc[i] = 0.0;
      for (int j = 0; j < nloc; ++j) Kloc[i][j] = 0.0;
    }
    for (int q = 0; q < nq; ++q) {
      double X[3] = {x0[0], x0[1], dim == 3 ? x0[2] : 0.0};
      for (int d = 0; d < dim; ++d)
        for (int a = 0; a < dim; ++a) X[d] += J[d][a] * xq[3 * q + a];
      const double f = rhs_f(dim, X, eps, b, c, manuf, fconst, poly);
      const double Mult = wq[q] * adet;
      double ux[MAXNB], uy[MAXNB], uz[MAXNB];
      for (int i = 0; i < nloc; ++i) {
        const double r[3] = {dxr[q][i], dyr[q][i], dim == 3 ? dzr[q][i] : 0.0};
        ux[i] = G[0][0] * r[0] + G[0][1] * r[1] + (dim == 3 ? G[0][2] * r[2] : 0.0);
        uy[i] = G[1][0] * r[0] + G[1][1] * r[1] + (dim == 3 ? G[1][2] * r[2] : 0.0);
        uz[i] = dim == 3 ? G[2][0] * r[0] + G[2][1] * r[1] + G[2][2] * r[2] : 0.0;
      }
      const double* u = phi[q];
      for (int i = 0; i < nloc; ++i) {
        Floc[i] += Mult * u[i] * f;
        for (int j = 0; j < nloc; ++j) {
          double val;
          if (dim == 2) {
            val = eps * (ux[i] * ux[j] + uy[i] * uy[j]);
            val += (b[0] * ux[j] + b[1] * uy[j]) * u[i];
            val += c * u[j] * u[i];
            val *= Mult;
            Kloc[i][j] += val;
          } else {
            val = eps * (ux[i] * ux[j] + uy[i] * uy[j] + uz[i] * uz[j]);
            val += (b[0] * ux[j] + b[1] * uy[j] + b[2] * uz[j]) * u[i];
            val += c * u[j] * u[i];
            Kloc[i][j] += val * Mult;
          }
        }
      }
    }
    /* scatter (Assemble3D.C:346-404) */
    const int* DOF = dofmap + (size_t)cell * nloc;
    for (int m = 0; m < nloc; ++m) {
      int l = DOF[m];
      if (l < n_active) {
        for (int kk = 0; kk < nloc; ++kk) {
          int found = 0;
          for (int n = rp[l]; n < rp[l + 1]; ++n)
            if (DOF[kk] == ci[n]) {
              vals[n] += Kloc[m][kk];
              found = 1;
              break;
            }
          if (!found) return -3;
        }
        rhs[l] += Floc[m];
      } else {
        for (int n = rp[l]; n < rp[l + 1]; ++n)
          if (ci[n] == l) {
            vals[n] = 1.0;
            break;
          }
      }
    }
  }
  return 0;
}

/* ---------------------------------------------------- grid transfer -------
 * GridTransfer::Prolongate / DefectRestriction for nested uniform meshes
 * (src/Multigrid/GridTransfer.C:665-941 and 943-1216): per fine cell, the
 * local prolongation matrix QQ (fine nodal functionals applied to the
 * parent's basis, FEDatabase3D.C:1606) maps the parent's coarse values; fine
 * values are averaged over the cells sharing them. Restriction divides the
 * fine defect by that multiplicity and applies QQ^T. */
typedef struct {
  int dim, k;  /* k: Qk degree; for tetrahedra k = 11 (P1) or 12 (P2) */
  int n_fine_cells, nloc;
  const int* fine_dofmap;
  const int* coarse_dofmap;
  const int* parent;
  const double* fine_verts;
  const double* coarse_verts;
  int n_fine, n_coarse;
} orc_transfer;

/* P1 / P2 on the reference tetrahedron (include/FE3D/BF_C_T_P1_3D.h,
 * BF_C_T_P2_3D.h): values at (x, y, z) in local DOF order */
static void tet_eval(int elem, double x, double y, double z, double* v) {
  if (elem == 11) {
    v[0] = 1 - x - y - z; v[1] = x; v[2] = y; v[3] = z;
    return;
  }
  v[0] = 1 - 3 * x - 3 * y - 3 * z + 2 * x * x + 4 * x * y + 4 * x * z + 2 * y * y + 4 * y * z + 2 * z * z;
  v[1] = 4 * x - 4 * x * x - 4 * x * y - 4 * x * z;
  v[2] = -x + 2 * x * x;
  v[3] = 4 * y - 4 * x * y - 4 * y * y - 4 * y * z;
  v[4] = 4 * x * y;
  v[5] = -y + 2 * y * y;
  v[6] = 4 * z - 4 * x * z - 4 * y * z - 4 * z * z;
  v[7] = 4 * x * z;
  v[8] = 4 * y * z;
  v[9] = -z + 2 * z * z;
}

/* nodes of a tetrahedral cell in local DOF order: P1 vertices; P2 v0, m01,
 * v1, m02, m12, v2, m03, m13, m23, v3 */
static void tet_nodes(int elem, const double* v, double X[][3]) {
  static const int pr[10][2] = {{0, 0}, {0, 1}, {1, 1}, {0, 2}, {1, 2}, {2, 2}, {0, 3}, {1, 3}, {2, 3}, {3, 3}};
  if (elem == 11) {
    for (int m = 0; m < 4; ++m)
      for (int d = 0; d < 3; ++d) X[m][d] = v[m * 3 + d];
    return;
  }
  for (int m = 0; m < 10; ++m)
    for (int d = 0; d < 3; ++d) X[m][d] = 0.5 * (v[pr[m][0] * 3 + d] + v[pr[m][1] * 3 + d]);
}

/* barycentric-type reference coordinates of x in the tetrahedron v */
static void tet_ref(const double* v, const double* x, double* xi) {
  double A[3][3], r[3];
  for (int d = 0; d < 3; ++d) {
    A[d][0] = v[3 + d] - v[d];
    A[d][1] = v[6 + d] - v[d];
    A[d][2] = v[9 + d] - v[d];
    r[d] = x[d] - v[d];
  }
  double det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
               A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
  for (int kk = 0; kk < 3; ++kk) {
    double B[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) B[i][j] = (j == kk) ? r[i] : A[i][j];
    xi[kk] = (B[0][0] * (B[1][1] * B[2][2] - B[1][2] * B[2][1]) - B[0][1] * (B[1][0] * B[2][2] - B[1][2] * B[2][0]) +
              B[0][2] * (B[1][0] * B[2][1] - B[1][1] * B[2][0])) / det;
  }
}

static void ref_coords(int dim, const double* v, const double* x, double* xi) {
  /* solve x = v0 + A t, A = [v1-v0, v3-v0(, v4-v0)], xi = 2t - 1 */
  if (dim == 2) {
    double a00 = v[2] - v[0], a10 = v[3] - v[1], a01 = v[6] - v[0], a11 = v[7] - v[1];
    double r0 = x[0] - v[0], r1 = x[1] - v[1];
    double det = a00 * a11 - a01 * a10;
    xi[0] = 2.0 * ((r0 * a11 - a01 * r1) / det) - 1.0;
    xi[1] = 2.0 * ((a00 * r1 - r0 * a10) / det) - 1.0;
  } else {
    double A[3][3], r[3];
    for (int d = 0; d < 3; ++d) {
      A[d][0] = v[3 + d] - v[d];
      A[d][1] = v[9 + d] - v[d];
      A[d][2] = v[12 + d] - v[d];
      r[d] = x[d] - v[d];
    }
    double det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
                 A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                 A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
    for (int kk = 0; kk < 3; ++kk) {
      double B[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) B[i][j] = (j == kk) ? r[i] : A[i][j];
      double dk = B[0][0] * (B[1][1] * B[2][2] - B[1][2] * B[2][1]) -
                  B[0][1] * (B[1][0] * B[2][2] - B[1][2] * B[2][0]) +
                  B[0][2] * (B[1][0] * B[2][1] - B[1][1] * B[2][0]);
      xi[kk] = 2.0 * (dk / det) - 1.0;
    }
  }
}

/* QQ[j][kk] of fine cell `cell`: coarse basis kk at fine node j */
static void local_qq(const orc_transfer* t, int cell, double QQ[MAXNB][MAXNB]) {
  if (t->k >= 11) {
    /* tetrahedra: fine nodes in the parent's reference coordinates */
    const double* fv = t->fine_verts + (size_t)cell * 12;
    const double* cv = t->coarse_verts + (size_t)t->parent[cell] * 12;
    double X[10][3];
    tet_nodes(t->k, fv, X);
    for (int m = 0; m < t->nloc; ++m) {
      double xi[3];
      tet_ref(cv, X[m], xi);
      tet_eval(t->k, xi[0], xi[1], xi[2], QQ[m]);
    }
    return;
  }
  const int nv = t->dim == 2 ? 4 : 8;
  const double* fv = t->fine_verts + (size_t)cell * nv * t->dim;
  const double* cv = t->coarse_verts + (size_t)t->parent[cell] * nv * t->dim;
  int m = 0;
  const int kk = t->k;
  for (int c = 0; c < (t->dim == 3 ? kk + 1 : 1); ++c)
    for (int b = 0; b <= kk; ++b)
      for (int a = 0; a <= kk; ++a, ++m) {
        /* fine node m in physical coordinates: x0 + (x1-x0) a/k + ... */
        double X[3];
        for (int d = 0; d < t->dim; ++d) {
          X[d] = fv[d] + (fv[t->dim + d] - fv[d]) * a / kk + (fv[3 * t->dim + d] - fv[d]) * b / kk;
          if (t->dim == 3) X[d] += (fv[12 + d] - fv[d]) * c / kk;
        }
        double xi[3];
        ref_coords(t->dim, cv, X, xi);
        qk_eval(t->dim, kk, xi, QQ[m], NULL, NULL, NULL);
      }
}

void orc_prolongate(const orc_transfer* t, const double* coarse, double* fine) {
  double* aux = (double*)calloc((size_t)t->n_fine, sizeof(double));
  memset(fine, 0, sizeof(double) * (size_t)t->n_fine);
  for (int i = 0; i < t->n_fine_cells; ++i)
    for (int j = 0; j < t->nloc; ++j) aux[t->fine_dofmap[(size_t)i * t->nloc + j]] += 1;
  double QQ[MAXNB][MAXNB];
  for (int i = 0; i < t->n_fine_cells; ++i) {
    local_qq(t, i, QQ);
    const int* cd = t->coarse_dofmap + (size_t)t->parent[i] * t->nloc;
    const int* fd = t->fine_dofmap + (size_t)i * t->nloc;
    for (int j = 0; j < t->nloc; ++j) {
      double s = 0.0;
      for (int kk = 0; kk < t->nloc; ++kk) s += QQ[j][kk] * coarse[cd[kk]];
      fine[fd[j]] += s;
    }
  }
  for (int i = 0; i < t->n_fine; ++i) fine[i] /= aux[i];
  free(aux);
}

void orc_restrict(const orc_transfer* t, double* coarse, const double* fine) {
  double* aux = (double*)calloc((size_t)t->n_fine, sizeof(double));
  double* fc = (double*)malloc(sizeof(double) * (size_t)t->n_fine);
  memcpy(fc, fine, sizeof(double) * (size_t)t->n_fine);
  memset(coarse, 0, sizeof(double) * (size_t)t->n_coarse);
  for (int i = 0; i < t->n_fine_cells; ++i)
    for (int j = 0; j < t->nloc; ++j) aux[t->fine_dofmap[(size_t)i * t->nloc + j]] += 1;
  for (int i = 0; i < t->n_fine; ++i) fc[i] /= aux[i];
  double QQ[MAXNB][MAXNB];
  for (int i = 0; i < t->n_fine_cells; ++i) {
    local_qq(t, i, QQ);
    const int* cd = t->coarse_dofmap + (size_t)t->parent[i] * t->nloc;
    const int* fd = t->fine_dofmap + (size_t)i * t->nloc;
    for (int kk = 0; kk < t->nloc; ++kk) {
      double s = 0.0;
      for (int j = 0; j < t->nloc; ++j) s += QQ[j][kk] * fc[fd[j]];
      coarse[cd[kk]] += s;
    }
  }
  free(aux);
  free(fc);
}

/* ---------------------------------------------------- dense LU ------------
 * stand-in for UMFPACK (DirectSolver) and LAPACK dgetrf/dgetrs: row-major LU
 * with partial pivoting */
int orc_lu_factor(int n, double* a, int* piv) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = fabs(a[(size_t)k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (fabs(a[(size_t)i * n + k]) > best) { best = fabs(a[(size_t)i * n + k]); p = i; }
    piv[k] = p;
    if (best == 0.0) return k + 1;
    if (p != k)
      for (int j = 0; j < n; ++j) {
        double t = a[(size_t)k * n + j];
        a[(size_t)k * n + j] = a[(size_t)p * n + j];
        a[(size_t)p * n + j] = t;
      }
    const double d = a[(size_t)k * n + k];
    for (int i = k + 1; i < n; ++i) {
      const double l = a[(size_t)i * n + k] / d;
      a[(size_t)i * n + k] = l;
      if (l != 0.0)
        for (int j = k + 1; j < n; ++j) a[(size_t)i * n + j] -= l * a[(size_t)k * n + j];
    }
  }
  return 0;
}

void orc_lu_solve(int n, const double* a, const int* piv, double* b) {
  for (int k = 0; k < n; ++k)
    if (piv[k] != k) { double t = b[k]; b[k] = b[piv[k]]; b[piv[k]] = t; }
  for (int i = 0; i < n; ++i) {
    double s = b[i];
    for (int j = 0; j < i; ++j) s -= a[(size_t)i * n + j] * b[j];
    b[i] = s;
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < n; ++j) s -= a[(size_t)i * n + j] * b[j];
    b[i] = s / a[(size_t)i * n + i];
  }
}

/* ------------------------------------------------------- multigrid --------
 * Multigrid (src/Multigrid/Multigrid.C:68-420), CycleControl
 * (src/Multigrid/CycleControl.C:17-110), MultigridLevel::calculate_defect
 * (MultigridLevel.C:131), JacobiSmoother::smooth (JacobiSmoother.C:22),
 * DirectSmoother (DirectSmoother.C:25). Level 0 is the coarsest. */
typedef struct {
  int n, n_active;
  const int *rp, *ci;
  const double* v;
  unsigned char* active;
  double *rhs, *sol, *defect, *diag;
  double* lu;
  int* piv;
  /* transfer to the next finer level, one per block of the block vector */
  orc_transfer up[4];
  int n_up, foff[4], coff[4];
  /* saddle point levels: projected combined matrix and cell-Vanka patches */
  const int *vrp, *vci;
  const double* vv;
  const int* patch;
  const int* patch_ptr; /* NULL: 34 DOFs per patch */
  int n_patches;
  const int *color_ptr, *color_cells;
  int n_colors;
  const int* n_freeze;
  void* store; /* stored local factorisations */
  const int* sor_order; /* rows in the order of the SOR sweep (NULL: 0..n-1) */
} orc_level;

enum { SM_JAC = 0, SM_DIR = 1, SM_VANKA = 2, SM_VANKA_JAC = 3, SM_VANKA_COLOR = 4, SM_SOR = 5, SM_SSOR = 6 };

/* TMatrix::sor_sweep (src/Matrix/Matrix.C:943-1031): for every row in turn,
 * s = b_row - sum_k a_row,k x_k (left to right), x_row += omega s / a_row,row;
 * flag 0 forward, 1 backward, 2 forward then backward (SSOR). The rows are
 * visited in `order` (NULL: the natural order, the reference's); the GPU's
 * multicolour sweep is this sweep in colour order. Returns -1 on a zero
 * diagonal entry (the reference throws). */
int orc_sor_sweep(int n, const int* rp, const int* ci, const double* v, const double* b, double* x, double omega,
                  const int* order, int flag) {
  double* diag = (double*)calloc((size_t)n, sizeof(double));
  for (int i = 0; i < n; ++i)
    for (int k = rp[i]; k < rp[i + 1]; ++k)
      if (ci[k] == i) diag[i] = v[k];
  for (int i = 0; i < n; ++i)
    if (diag[i] == 0.0) { free(diag); return -1; }
  for (int sweep = 0; sweep < (flag == 2 ? 2 : 1); ++sweep) {
    const int backward = flag == 1 || (flag == 2 && sweep == 1);
    for (int r = 0; r < n; ++r) {
      const int q = backward ? n - 1 - r : r;
      const int row = order ? order[q] : q;
      double s = b[row];
      for (int k = rp[row]; k < rp[row + 1]; ++k) s -= v[k] * x[ci[k]];
      x[row] = x[row] + omega * s / diag[row];
    }
  }
  free(diag);
  return 0;
}

void* orc_vanka_store_create(int n_patches);
void orc_vanka_store_destroy(void* st);

typedef struct {
  int n_levels;
  orc_level* lv;
  int n_pre, n_post, coarse_max_it, cycle; /* cycle: 0 V, 1 W, 2 F */
  double jacobi_damp, correction_damp, coarse_residual, vanka_damp, sor_omega;
  int coarse_direct;
  int smoother, smoother_coarse;
  int* control;
  int n_control;
} orc_mg;

enum { D_DUMMY = 0, D_DOWN = 1, D_UP = 2, D_END = 3 };

static void fill_rec(orc_mg* m, int* rec, int level) {
  if (level == 0) { m->control[m->n_control++] = D_UP; return; }
  for (int j = 0; j < rec[level]; ++j) {
    m->control[m->n_control++] = D_DOWN;
    fill_rec(m, rec, level - 1);
  }
  if (m->cycle == 2) rec[level] = 1;
  m->control[m->n_control++] = (level == m->n_levels - 1) ? D_END : D_UP;
}

orc_mg* orc_mg_create(int n_levels, int n_pre, int n_post, double jacobi_damp, double correction_damp,
                      int cycle, int coarse_direct, int coarse_max_it, double coarse_residual) {
  orc_mg* m = (orc_mg*)calloc(1, sizeof(orc_mg));
  m->n_levels = n_levels;
  m->lv = (orc_level*)calloc((size_t)n_levels, sizeof(orc_level));
  m->n_pre = n_pre;
  m->n_post = n_post;
  m->jacobi_damp = jacobi_damp;
  m->correction_damp = correction_damp;
  m->cycle = cycle;
  m->coarse_direct = coarse_direct;
  m->coarse_max_it = coarse_max_it;
  m->coarse_residual = coarse_residual;
  m->smoother = SM_JAC;
  m->smoother_coarse = coarse_direct ? SM_DIR : SM_JAC;
  m->vanka_damp = 1.0;
  m->sor_omega = 1.5;
  int* rec = (int*)malloc(sizeof(int) * (size_t)n_levels);
  for (int i = 0; i < n_levels; ++i) rec[i] = cycle == 0 ? 1 : 2;
  rec[n_levels - 1] = 1;
  m->control = (int*)malloc(sizeof(int) * 100000);
  m->control[m->n_control++] = D_DUMMY;
  fill_rec(m, rec, n_levels - 1);
  free(rec);
  return m;
}

/* level matrix (active flags per row), plus the transfer to the finer level */
int orc_mg_set_level(orc_mg* m, int l, int n, const unsigned char* active, const int* rp, const int* ci,
                     const double* v) {
  orc_level* L = &m->lv[l];
  L->n = n;
  L->rp = rp;
  L->ci = ci;
  L->v = v;
  L->active = (unsigned char*)malloc((size_t)n);
  memcpy(L->active, active, (size_t)n);
  L->n_active = 0;
  for (int i = 0; i < n; ++i) L->n_active += active[i];
  L->rhs = (double*)calloc((size_t)n, sizeof(double));
  L->sol = (double*)calloc((size_t)n, sizeof(double));
  L->defect = (double*)calloc((size_t)n, sizeof(double));
  L->diag = (double*)calloc((size_t)n, sizeof(double));
  for (int i = 0; i < n; ++i)
    for (int k = rp[i]; k < rp[i + 1]; ++k)
      if (ci[k] == i) L->diag[i] = v[k];
  return 0;
}

/* smoothers: 0 Jacobi, 1 direct, 2 cell Vanka (cell order), 3 cell Vanka
 * Jacobi, 4 cell Vanka in colour order */
void orc_mg_set_smoothers(orc_mg* m, int fine, int coarse, double vanka_damp) {
  m->smoother = fine;
  m->smoother_coarse = coarse;
  m->coarse_direct = coarse == SM_DIR;
  m->vanka_damp = vanka_damp;
}

/* SOR / SSOR smoother: the row order of level l's sweeps and the
 * overrelaxation parameter (sor_omega) */
void orc_mg_set_sor(orc_mg* m, int l, const int* order, double omega) {
  m->lv[l].sor_order = order;
  m->sor_omega = omega;
}

/* saddle point level: projected combined matrix (get_combined_matrix) and the
 * Vanka patches (sorted combined DOFs; patch_ptr NULL: 34 per cell) with their
 * colouring */
void orc_mg_set_vanka(orc_mg* m, int l, const int* vrp, const int* vci, const double* vv, const int* patch,
                      int n_patches, const int* color_ptr, const int* color_cells, int n_colors,
                      const int* n_freeze, const int* patch_ptr) {
  orc_level* L = &m->lv[l];
  L->vrp = vrp; L->vci = vci; L->vv = vv;
  L->patch = patch; L->n_patches = n_patches; L->patch_ptr = patch_ptr;
  L->color_ptr = color_ptr; L->color_cells = color_cells; L->n_colors = n_colors;
  L->n_freeze = n_freeze;
  orc_vanka_store_destroy(L->store);
  L->store = orc_vanka_store_create(n_patches);
}

/* DirectSolver on get_combined_matrix of the coarsest level: the projected
 * matrix when given, else the system with unit rows for non-actives */
int orc_mg_finalize(orc_mg* m) {
  orc_level* L = &m->lv[0];
  if (!m->coarse_direct) return 0;
  const int n = L->n;
  free(L->lu);
  free(L->piv);
  L->lu = (double*)calloc((size_t)n * n, sizeof(double));
  L->piv = (int*)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; ++i) {
    if (L->vrp) {
      for (int k = L->vrp[i]; k < L->vrp[i + 1]; ++k) L->lu[(size_t)i * n + L->vci[k]] = L->vv[k];
    } else {
      if (!L->active[i]) { L->lu[(size_t)i * n + i] = 1.0; continue; }
      for (int k = L->rp[i]; k < L->rp[i + 1]; ++k) L->lu[(size_t)i * n + L->ci[k]] = L->v[k];
    }
  }
  return orc_lu_factor(n, L->lu, L->piv) ? -1 : 0;
}

void orc_mg_set_transfer_block(orc_mg* m, int l, int block, int fine_off, int coarse_off, int dim, int k,
                               int n_fine_cells, int nloc, const int* fine_dofmap, const int* coarse_dofmap,
                               const int* parent, const double* fine_verts, const double* coarse_verts,
                               int n_fine, int n_coarse) {
  orc_level* L = &m->lv[l];
  orc_transfer* t = &L->up[block];
  t->dim = dim; t->k = k; t->n_fine_cells = n_fine_cells; t->nloc = nloc;
  t->fine_dofmap = fine_dofmap; t->coarse_dofmap = coarse_dofmap; t->parent = parent;
  t->fine_verts = fine_verts; t->coarse_verts = coarse_verts;
  t->n_fine = n_fine; t->n_coarse = n_coarse;
  L->foff[block] = fine_off;
  L->coff[block] = coarse_off;
  if (block + 1 > L->n_up) L->n_up = block + 1;
}

void orc_mg_set_transfer(orc_mg* m, int l, int dim, int k, int n_fine_cells, int nloc, const int* fine_dofmap,
                         const int* coarse_dofmap, const int* parent, const double* fine_verts,
                         const double* coarse_verts, int n_fine, int n_coarse) {
  orc_mg_set_transfer_block(m, l, 0, 0, 0, dim, k, n_fine_cells, nloc, fine_dofmap, coarse_dofmap, parent,
                            fine_verts, coarse_verts, n_fine, n_coarse);
}

void orc_mg_destroy(orc_mg* m) {
  for (int l = 0; l < m->n_levels; ++l) {
    orc_level* L = &m->lv[l];
    free(L->active); free(L->rhs); free(L->sol); free(L->defect); free(L->diag);
    free(L->lu); free(L->piv);
    orc_vanka_store_destroy(L->store);
  }
  free(m->lv);
  free(m->control);
  free(m);
}

static double calc_defect(orc_level* L) {
  memcpy(L->defect, L->rhs, sizeof(double) * (size_t)L->n);
  orc_apply_scaled_add(L->n, L->active, L->rp, L->ci, L->v, L->sol, L->defect, -1.0);
  return sqrt(orc_dot(L->n, L->defect, L->defect));
}

void orc_vanka_sweep_var(int type, int n_patches, const int* ptr, const int* patch, int n, const int* rp,
                         const int* ci, const double* v, const double* b, double* x, double damp,
                         const int* color_ptr, const int* color_cells, int n_colors, const int* n_freeze,
                         void* store);


static void smooth(orc_mg* m, int l) {
  orc_level* L = &m->lv[l];
  const int code = l == 0 ? m->smoother_coarse : m->smoother;
  if (code == SM_DIR) {
    memcpy(L->sol, L->rhs, sizeof(double) * (size_t)L->n);
    orc_lu_solve(L->n, L->lu, L->piv, L->sol);
    return;
  }
  if (code == SM_VANKA || code == SM_VANKA_JAC || code == SM_VANKA_COLOR) {
    orc_vanka_sweep_var(code == SM_VANKA ? 0 : code == SM_VANKA_JAC ? 1 : 2, L->n_patches, L->patch_ptr, L->patch, L->n, L->vrp,
                    L->vci, L->vv, L->rhs, L->sol, m->vanka_damp, L->color_ptr, L->color_cells, L->n_colors,
                    L->n_freeze, L->store);
    return;
  }
  if (code == SM_SOR || code == SM_SSOR) {
    /* SORSmoother::smooth (src/Multigrid/SORSmoother.C:29): one sweep of
     * Iteration_sor::apply_smoother, SOR forward (0) or SSOR (2) */
    orc_sor_sweep(L->n, L->rp, L->ci, L->v, L->rhs, L->sol, m->sor_omega, L->sor_order, code == SM_SOR ? 0 : 2);
    return;
  }
  /* JacobiSmoother::smooth */
  double* d = (double*)malloc(sizeof(double) * (size_t)L->n);
  memcpy(d, L->rhs, sizeof(double) * (size_t)L->n);
  orc_apply_scaled_add(L->n, L->active, L->rp, L->ci, L->v, L->sol, d, -1.0);
  for (int j = 0; j < L->n; ++j) d[j] /= L->diag[j];
  axpy(L->n, m->jacobi_damp, d, L->sol);
  free(d);
}

static void prolong_add(orc_mg* m, int l) {
  orc_level* C = &m->lv[l];
  orc_level* F = &m->lv[l + 1];
  double* tmp = (double*)malloc(sizeof(double) * (size_t)F->n);
  for (int b = 0; b < C->n_up; ++b)
    orc_prolongate(&C->up[b], C->sol + C->coff[b], tmp + C->foff[b]);
  /* damped addition on the actives (Multigrid.C:357-418) */
  for (int j = 0; j < F->n; ++j)
    if (F->active[j]) F->sol[j] += m->correction_damp * tmp[j];
  free(tmp);
}

static int cycle_step(orc_mg* m, int step, int level) {
  if (level == 0) {
    double res = 1e10;
    calc_defect(&m->lv[0]);
    for (int i = 0; i < m->coarse_max_it && res > m->coarse_residual; ++i) {
      smooth(m, 0);
      res = calc_defect(&m->lv[0]);
    }
    prolong_add(m, 0);
    return 1;
  }
  int from_below = m->control[step - 1] == D_UP;
  int up = m->control[step] == D_UP;
  int down = m->control[step] == D_DOWN;
  if (from_below)
    for (int i = 0; i < m->n_post; ++i) smooth(m, level);
  if (down) {
    for (int i = 0; i < m->n_pre; ++i) smooth(m, level);
    calc_defect(&m->lv[level]);
    orc_level* C = &m->lv[level - 1];
    memset(C->sol, 0, sizeof(double) * (size_t)C->n);
    for (int b = 0; b < C->n_up; ++b)
      orc_restrict(&C->up[b], C->rhs + C->coff[b], m->lv[level].defect + C->foff[b]);
    for (int j = 0; j < C->n; ++j)
      if (!C->active[j]) C->rhs[j] = 0.0; /* ResetNonActive */
    return level - 1;
  }
  if (up) {
    prolong_add(m, level);
    return level + 1;
  }
  return -1;
}

/* Iteration_multigrid::apply (src/Solver/Iteration_multigrid.C:22-32) */
void orc_mg_apply(orc_mg* m, const double* z, double* r) {
  orc_level* T = &m->lv[m->n_levels - 1];
  memcpy(T->rhs, z, sizeof(double) * (size_t)T->n);
  for (int j = 0; j < T->n; ++j) T->sol[j] = T->active[j] ? 0.0 : T->rhs[j];
  int level = m->n_levels - 1;
  for (int step = 1; step < m->n_control && level >= 0; ++step) level = cycle_step(m, step, level);
  memcpy(r, T->sol, sizeof(double) * (size_t)T->n);
}

/* ---------------------------------------------------- Krylov ---------------
 * IterativeMethod::converged (include/Solver/IterativeMethod.h:81-140) */
typedef struct {
  double tol, reduction, divergence, stagnation;
  int max_it, min_it, restart;
  double initial, previous;
  int last_it;
  double last_res;
  double* history;
  int n_history, cap_history;
  int status; /* 0 ok, 3 diverged, 4 breakdown */
} orc_krylov;

static int converged(orc_krylov* k, double r, int it) {
  if (it == 0) { k->initial = r; k->previous = r; k->n_history = 0; }
  if (k->history && k->n_history < k->cap_history) k->history[k->n_history++] = r;
  int small = r < k->tol;
  int red = r < k->reduction * k->initial;
  int enough = it > k->min_it || k->min_it == 0;
  int stag = r > k->stagnation * k->previous;
  int div = r > k->divergence * k->initial;
  int conv = (small || red || stag || div) && enough;
  if (it == k->max_it) conv = 1;
  k->previous = r;
  k->last_it = it;
  k->last_res = r;
  if (div) { k->status = 3; return 1; }
  return conv;
}

typedef struct {
  int n;
  const unsigned char* active;
  const int *rp, *ci;
  const double* v;
  orc_mg* mg; /* NULL: no preconditioner */
  /* SOR / SSOR preconditioner (Iteration_sor::apply): sor_flag 0 or 2, -1 none */
  int sor_flag;
  const int* sor_order;
  double sor_omega;
} orc_system;

static void sys_apply_scaled_add(const orc_system* s, const double* x, double* y, double a) {
  orc_apply_scaled_add(s->n, s->active, s->rp, s->ci, s->v, x, y, a);
}
static void prec_apply(const orc_system* s, const double* z, double* r) {
  if (s->mg) orc_mg_apply(s->mg, z, r);
  else if (s->sor_flag >= 0) {
    /* Iteration_sor::apply (src/Solver/Iteration_sor.C:75): r = 0, one sweep */
    memset(r, 0, sizeof(double) * (size_t)s->n);
    orc_sor_sweep(s->n, s->rp, s->ci, s->v, z, r, s->sor_omega, s->sor_order, s->sor_flag);
  } else memcpy(r, z, sizeof(double) * (size_t)s->n);
}

static void gen_rot(double dx, double dy, double* cs, double* sn) {
  if (dy == 0.0) { *cs = 1.0; *sn = 0.0; }
  else if (fabs(dy) > fabs(dx)) { double t = dx / dy; *sn = 1.0 / sqrt(1.0 + t * t); *cs = t * *sn; }
  else { double t = dy / dx; *cs = 1.0 / sqrt(1.0 + t * t); *sn = t * *cs; }
}
static void app_rot(double* dx, double* dy, double cs, double sn) {
  double t = cs * *dx + sn * *dy;
  *dy = -sn * *dx + cs * *dy;
  *dx = t;
}

/* Iteration_gmres::flexible_gmres (src/Solver/Iteration_gmres.C:376-532) */
int orc_fgmres(const orc_system* s, orc_krylov* k, const double* rhs, double* sol) {
  const int n = s->n, m = k->restart;
  double* r = (double*)malloc(sizeof(double) * (size_t)n);
  double* V = (double*)malloc(sizeof(double) * (size_t)n * (m + 1));
  double* Z = (double*)malloc(sizeof(double) * (size_t)n * (m + 1));
  double* H = (double*)calloc((size_t)(m + 1) * (m + 1), sizeof(double)); /* H[row*(m+1)+col] */
  double* sv = (double*)calloc((size_t)m + 1, sizeof(double));
  double* cs = (double*)calloc((size_t)m + 1, sizeof(double));
  double* sn = (double*)calloc((size_t)m + 1, sizeof(double));
  double* y = (double*)calloc((size_t)m + 1, sizeof(double));
  k->status = 0;
  memcpy(r, rhs, sizeof(double) * (size_t)n);
  sys_apply_scaled_add(s, sol, r, -1.0);
  double resid = orc_norm(n, r), beta = resid;
  int ret = 0;
  if (converged(k, resid, 0)) goto done;
  int j = 1;
  while (j <= k->max_it) {
    for (int t = 0; t < n; ++t) V[t] = r[t];
    { const double sc = 1.0 / beta; for (int t = 0; t < n; ++t) V[t] *= sc; }
    for (int t = 0; t <= m; ++t) sv[t] = 0.0;
    sv[0] = beta;
    int i;
    for (i = 0; i < m && j <= k->max_it; ++i, ++j) {
      double* zi = Z + (size_t)i * n;
      for (int t = 0; t < n; ++t) zi[t] = 0.0;
      prec_apply(s, V + (size_t)i * n, zi);
      for (int t = 0; t < n; ++t) r[t] = 0.0;
      sys_apply_scaled_add(s, zi, r, 1.0); /* apply: reset + apply_scaled_add(.,1) */
      for (int kk = 0; kk <= i; ++kk) {
        double h = orc_dot(n, r, V + (size_t)kk * n);
        H[kk * (m + 1) + i] = h;
        axpy(n, -h, V + (size_t)kk * n, r);
      }
      double hn = orc_norm(n, r);
      H[(i + 1) * (m + 1) + i] = hn;
      if (hn == 0.0) { k->status = 4; ret = 4; goto done; }
      { double* vn = V + (size_t)(i + 1) * n; const double sc = 1.0 / hn;
        for (int t = 0; t < n; ++t) vn[t] = r[t] * sc; }
      for (int kk = 0; kk < i; ++kk) app_rot(&H[kk * (m + 1) + i], &H[(kk + 1) * (m + 1) + i], cs[kk], sn[kk]);
      gen_rot(H[i * (m + 1) + i], H[(i + 1) * (m + 1) + i], &cs[i], &sn[i]);
      app_rot(&H[i * (m + 1) + i], &H[(i + 1) * (m + 1) + i], cs[i], sn[i]);
      app_rot(&sv[i], &sv[i + 1], cs[i], sn[i]);
      resid = fabs(sv[i + 1]);
      if (converged(k, resid, j)) {
        for (int t = 0; t <= i; ++t) y[t] = sv[t];
        for (int a = i; a >= 0; --a) {
          y[a] /= H[a * (m + 1) + a];
          for (int b = a - 1; b >= 0; --b) y[b] -= H[b * (m + 1) + a] * y[a];
        }
        for (int t = 0; t < n; ++t) r[t] = 0.0;
        for (int a = 0; a <= i; ++a) axpy(n, y[a], Z + (size_t)a * n, r);
        for (int t = 0; t < n; ++t) sol[t] += r[t];
        goto done;
      }
    }
    for (int t = 0; t < m; ++t) y[t] = sv[t];
    for (int a = m - 1; a >= 0; --a) {
      y[a] /= H[a * (m + 1) + a];
      for (int b = a - 1; b >= 0; --b) y[b] -= H[b * (m + 1) + a] * y[a];
    }
    for (int t = 0; t < n; ++t) r[t] = 0.0;
    for (int a = 0; a < m; ++a) axpy(n, y[a], Z + (size_t)a * n, r);
    for (int t = 0; t < n; ++t) sol[t] += r[t];
    memcpy(r, rhs, sizeof(double) * (size_t)n);
    sys_apply_scaled_add(s, sol, r, -1.0);
    beta = orc_norm(n, r);
    if (converged(k, resid, j)) goto done;
  }
done:
  if (k->status) ret = k->status;
  free(r); free(V); free(Z); free(H); free(sv); free(cs); free(sn); free(y);
  return ret;
}

/* Iteration_cg::iterate (src/Solver/Iteration_cg.C:22-79) */
int orc_cg(const orc_system* s, orc_krylov* k, const double* rhs, double* sol) {
  const int n = s->n;
  double* r = (double*)malloc(sizeof(double) * (size_t)n);
  double* z = (double*)malloc(sizeof(double) * (size_t)n);
  double* p = (double*)malloc(sizeof(double) * (size_t)n);
  double* q = (double*)malloc(sizeof(double) * (size_t)n);
  k->status = 0;
  memcpy(r, rhs, sizeof(double) * (size_t)n);
  sys_apply_scaled_add(s, sol, r, -1.0);
  double normb = orc_norm(n, rhs);
  if (normb == 0.0) normb = 1.0;
  double resid = orc_norm(n, r) / normb, rho_1 = 0.0;
  if (!converged(k, resid, 0)) {
    for (int i = 1; i <= k->max_it; ++i) {
      prec_apply(s, r, z);
      double rho = orc_dot(n, r, z);
      if (i == 1) memcpy(p, z, sizeof(double) * (size_t)n);
      else { double beta = rho / rho_1; for (int t = 0; t < n; ++t) { p[t] *= beta; p[t] += z[t]; } }
      for (int t = 0; t < n; ++t) q[t] = 0.0;
      sys_apply_scaled_add(s, p, q, 1.0);
      double alpha = rho / orc_dot(n, p, q);
      axpy(n, alpha, p, sol);
      axpy(n, -alpha, q, r);
      resid = orc_norm(n, r) / normb;
      if (converged(k, resid, i)) break;
      rho_1 = rho;
    }
  }
  free(r); free(z); free(p); free(q);
  return k->status;
}

/* Iteration_bicgstab::iterate (src/Solver/Iteration_bicgstab.C:28-206) */
int orc_bicgstab(const orc_system* s, orc_krylov* k, const double* rhs, double* sol) {
  const int n = s->n;
  double* buf = (double*)malloc(sizeof(double) * (size_t)n * 8);
  double *r = buf, *rt = buf + n, *p = buf + 2 * (size_t)n, *ph = buf + 3 * (size_t)n, *sv = buf + 4 * (size_t)n,
         *sh = buf + 5 * (size_t)n, *t = buf + 6 * (size_t)n, *v = buf + 7 * (size_t)n;
  double rho_2 = 1.0, alpha = 1.0, omega = 1.0;
  k->status = 0;
  memcpy(r, rhs, sizeof(double) * (size_t)n);
  sys_apply_scaled_add(s, sol, r, -1.0);
  memcpy(rt, r, sizeof(double) * (size_t)n);
  double normb = orc_norm(n, rhs);
  if (normb == 0.0) normb = 1.0;
  double resid = orc_norm(n, r) / normb;
  if (!converged(k, resid, 0)) {
    for (int i = 1; i <= k->max_it; ++i) {
      double rho_1 = orc_dot(n, rt, r);
      if (rho_1 == 0.0) { k->last_it = i; k->last_res = orc_norm(n, r) / normb; break; }
      if (i == 1) memcpy(p, r, sizeof(double) * (size_t)n);
      else {
        double beta = (rho_1 / rho_2) * (alpha / omega);
        axpy(n, -omega, v, p);
        for (int q = 0; q < n; ++q) { p[q] *= beta; p[q] += r[q]; }
      }
      prec_apply(s, p, ph);
      for (int q = 0; q < n; ++q) v[q] = 0.0;
      sys_apply_scaled_add(s, ph, v, 1.0);
      alpha = rho_1 / orc_dot(n, rt, v);
      memcpy(sv, r, sizeof(double) * (size_t)n);
      axpy(n, -alpha, v, sv);
      resid = orc_norm(n, sv) / normb;
      if (converged(k, resid, i)) { axpy(n, alpha, ph, sol); break; }
      prec_apply(s, sv, sh);
      for (int q = 0; q < n; ++q) t[q] = 0.0;
      sys_apply_scaled_add(s, sh, t, 1.0);
      omega = orc_dot(n, t, sv) / orc_dot(n, t, t);
      axpy(n, alpha, ph, sol);
      axpy(n, omega, sh, sol);
      memcpy(r, sv, sizeof(double) * (size_t)n);
      axpy(n, -omega, t, r);
      rho_2 = rho_1;
      resid = orc_norm(n, r) / normb;
      if (converged(k, resid, i)) break;
      if (omega == 0.0) { k->status = 4; break; }
    }
  }
  free(buf);
  return k->status;
}

/* flat entry point for ctypes: solver 0 fgmres, 1 cg, 2 bicgstab */
int orc_krylov_solve_sor(int method, int n, const unsigned char* active, const int* rp, const int* ci,
                         const double* v, orc_mg* mg, int sor_flag, const int* sor_order, double sor_omega,
                         double tol, double reduction, int max_it, int min_it, int restart, const double* rhs,
                         double* sol, int* iterations, double* residual, double* history, int cap_history,
                         int* n_history);

int orc_krylov_solve(int method, int n, const unsigned char* active, const int* rp, const int* ci,
                     const double* v, orc_mg* mg, double tol, double reduction, int max_it, int min_it,
                     int restart, const double* rhs, double* sol, int* iterations, double* residual,
                     double* history, int cap_history, int* n_history) {
  return orc_krylov_solve_sor(method, n, active, rp, ci, v, mg, -1, NULL, 0.0, tol, reduction, max_it, min_it,
                              restart, rhs, sol, iterations, residual, history, cap_history, n_history);
}

/* the same with the SOR (sor_flag 0) or SSOR (2) preconditioner when mg is
 * NULL; the sweeps visit the rows in sor_order */
int orc_krylov_solve_sor(int method, int n, const unsigned char* active, const int* rp, const int* ci,
                         const double* v, orc_mg* mg, int sor_flag, const int* sor_order, double sor_omega,
                         double tol, double reduction, int max_it, int min_it, int restart, const double* rhs,
                         double* sol, int* iterations, double* residual, double* history, int cap_history,
                         int* n_history) {
  orc_system s = {n, active, rp, ci, v, mg, sor_flag, sor_order, sor_omega};
  orc_krylov k;
  memset(&k, 0, sizeof(k));
  k.tol = tol; k.reduction = reduction; k.divergence = 1e10; k.stagnation = 1e10;
  k.max_it = max_it; k.min_it = min_it; k.restart = restart;
  k.history = history; k.cap_history = cap_history;
  int st = method == 0 ? orc_fgmres(&s, &k, rhs, sol) : method == 1 ? orc_cg(&s, &k, rhs, sol)
                                                                      : orc_bicgstab(&s, &k, rhs, sol);
  if (iterations) *iterations = k.last_it;
  if (residual) *residual = k.last_res;
  if (n_history) *n_history = k.n_history;
  return st;
}

/* flat wrappers of the grid transfer for ctypes */
void orc_prolongate_flat(int dim, int k, int n_fine_cells, int nloc, const int* fine_dofmap,
                         const int* coarse_dofmap, const int* parent, const double* fine_verts,
                         const double* coarse_verts, int n_fine, int n_coarse, const double* coarse,
                         double* fine) {
  orc_transfer t = {dim, k, n_fine_cells, nloc, fine_dofmap, coarse_dofmap, parent,
                    fine_verts, coarse_verts, n_fine, n_coarse};
  orc_prolongate(&t, coarse, fine);
}

void orc_restrict_flat(int dim, int k, int n_fine_cells, int nloc, const int* fine_dofmap,
                       const int* coarse_dofmap, const int* parent, const double* fine_verts,
                       const double* coarse_verts, int n_fine, int n_coarse, double* coarse,
                       const double* fine) {
  orc_transfer t = {dim, k, n_fine_cells, nloc, fine_dofmap, coarse_dofmap, parent,
                    fine_verts, coarse_verts, n_fine, n_coarse};
  orc_restrict(&t, coarse, fine);
}

/* ------------------------------------------------------ cell Vanka ---------
 * VankaSmoother::smooth (src/Multigrid/VankaSmoother.C:110-292) on the
 * projected combined matrix. type 0: CELL (multiplicative, cells in order),
 * type 1: CELL_JACOBI (global residual once, corrections averaged over the
 * patches sharing a DOF), type 2: CELL in colour order (all local right-hand
 * sides of a colour from the same iterate, then the colour's updates).
 *
 * Frozen pressure DOFs: a cell with a single active velocity node (3 active
 * velocity rows against 4 pressure columns) has an exactly singular local
 * matrix, on which the reference's LAPACK LU throws or returns a blown-up
 * correction. n_freeze[cell] (4 - 3 x active velocity nodes, clamped to
 * 0..4) trailing pressure entries of the sorted patch are decoupled (unit
 * row and column) and receive no update. n_freeze == NULL keeps every
 * local matrix as the reference builds it. */
/* patch p: dofs[ptr[p] .. ptr[p+1]), sorted combined DOFs */
static void vanka_local_matrix(const int* dof, int sz, const int* rp, const int* ci, const double* v, int nf,
                               double* M) {
  for (size_t e = 0; e < (size_t)sz * sz; ++e) M[e] = 0.0;
  for (int r = 0; r < sz; ++r) {
    const int rg = dof[r];
    int c = 0;
    for (int j = rp[rg]; j < rp[rg + 1]; ++j) {
      const double entry = v[j];
      if (entry == 0) continue; /* don't copy zeroes */
      const int cg = ci[j];
      while (dof[c] < cg) {
        ++c;
        if (c == sz) break;
      }
      if (c == sz) break;
      if (dof[c] == cg) M[(size_t)r * sz + c] = entry;
    }
  }
  for (int f = sz - nf; f < sz; ++f) {
    for (int k = 0; k < sz; ++k) M[(size_t)f * sz + k] = M[(size_t)k * sz + f] = 0.0;
    M[(size_t)f * sz + f] = 1.0;
  }
}

/* stored local factorisations (the reference's *_store Vanka variants; the
 * factors do not change while the matrix is the same, so results agree with
 * refactorising every sweep) */
typedef struct {
  int n_patches;
  double** lu;
  int** piv;
} orc_vanka_store;

static orc_vanka_store* vanka_store_new(int n_patches) {
  orc_vanka_store* st = (orc_vanka_store*)calloc(1, sizeof(orc_vanka_store));
  st->n_patches = n_patches;
  st->lu = (double**)calloc((size_t)n_patches, sizeof(double*));
  st->piv = (int**)calloc((size_t)n_patches, sizeof(int*));
  return st;
}

static void vanka_store_free(orc_vanka_store* st) {
  if (!st) return;
  for (int p = 0; p < st->n_patches; ++p) {
    free(st->lu[p]);
    free(st->piv[p]);
  }
  free(st->lu);
  free(st->piv);
  free(st);
}

static void vanka_local_solve(orc_vanka_store* st, int p, const int* dof, int sz, const int* rp, const int* ci,
                              const double* v, int nf, double* loc) {
  double* M;
  int* piv;
  if (st && st->lu[p]) {
    M = st->lu[p];
    piv = st->piv[p];
  } else {
    M = (double*)malloc(sizeof(double) * (size_t)sz * sz);
    piv = (int*)malloc(sizeof(int) * (size_t)sz);
    vanka_local_matrix(dof, sz, rp, ci, v, nf, M);
    orc_lu_factor(sz, M, piv);
  }
  orc_lu_solve(sz, M, piv, loc);
  for (int f = sz - nf; f < sz; ++f) loc[f] = 0.0;
  if (st) {
    st->lu[p] = M;
    st->piv[p] = piv;
  } else {
    free(M);
    free(piv);
  }
}

static void vanka_local_rhs(const int* dof, int sz, const int* rp, const int* ci, const double* v, const double* b,
                            const double* x, double* loc) {
  for (int r = 0; r < sz; ++r) {
    const int rg = dof[r];
    double t = b[rg];
    for (int j = rp[rg]; j < rp[rg + 1]; ++j) t -= v[j] * x[ci[j]];
    loc[r] = t;
  }
}

/* patches of any size: ptr == NULL means 34 DOFs per patch (cell patches of
 * P2/P1 tetrahedra) */
void orc_vanka_sweep_var(int type, int n_patches, const int* ptr, const int* patch, int n, const int* rp,
                         const int* ci, const double* v, const double* b, double* x, double damp,
                         const int* color_ptr, const int* color_cells, int n_colors, const int* n_freeze,
                         void* store) {
  orc_vanka_store* st = (orc_vanka_store*)store;
#define PB(p) (ptr ? ptr[p] : 34 * (p))
#define PS(p) (ptr ? ptr[(p) + 1] - ptr[p] : 34)
  int maxsz = 0;
  for (int p = 0; p < n_patches; ++p)
    if (PS(p) > maxsz) maxsz = PS(p);
  double* loc = (double*)malloc(sizeof(double) * (size_t)(maxsz > 0 ? maxsz : 1));
  if (type == 1) {
    double* res = (double*)malloc(sizeof(double) * (size_t)n);
    double* upd = (double*)calloc((size_t)n, sizeof(double));
    double* cnt = (double*)calloc((size_t)n, sizeof(double));
    memcpy(res, b, sizeof(double) * (size_t)n);
    orc_multiply(n, rp, ci, v, x, res, -1.0);
    for (int p = 0; p < n_patches; ++p) {
      const int* dof = patch + PB(p);
      const int sz = PS(p);
      for (int r = 0; r < sz; ++r) loc[r] = res[dof[r]];
      vanka_local_solve(st, p, dof, sz, rp, ci, v, n_freeze ? n_freeze[p] : 0, loc);
      for (int r = 0; r < sz; ++r) {
        upd[dof[r]] += damp * loc[r];
        cnt[dof[r]] += 1;
      }
    }
    for (int i = 0; i < n; ++i)
      if (cnt[i] != 0) x[i] += upd[i] / cnt[i];
    free(res); free(upd); free(cnt); free(loc);
    return;
  }
  if (type == 0) {
    for (int p = 0; p < n_patches; ++p) {
      const int* dof = patch + PB(p);
      const int sz = PS(p);
      vanka_local_rhs(dof, sz, rp, ci, v, b, x, loc);
      vanka_local_solve(st, p, dof, sz, rp, ci, v, n_freeze ? n_freeze[p] : 0, loc);
      for (int r = 0; r < sz; ++r) x[dof[r]] += damp * loc[r];
    }
    free(loc);
    return;
  }
  /* colour order */
  for (int k = 0; k < n_colors; ++k) {
    const int beg = color_ptr[k], end = color_ptr[k + 1];
    size_t tot = 0;
    for (int q = beg; q < end; ++q) tot += (size_t)PS(color_cells[q]);
    double* rl = (double*)malloc(sizeof(double) * (tot > 0 ? tot : 1));
    size_t off = 0;
    for (int q = beg; q < end; ++q) {
      const int p = color_cells[q];
      vanka_local_rhs(patch + PB(p), PS(p), rp, ci, v, b, x, rl + off);
      off += (size_t)PS(p);
    }
    off = 0;
    for (int q = beg; q < end; ++q) {
      const int p = color_cells[q];
      const int* dof = patch + PB(p);
      const int sz = PS(p);
      double* l = rl + off;
      vanka_local_solve(st, p, dof, sz, rp, ci, v, n_freeze ? n_freeze[p] : 0, l);
      for (int r = 0; r < sz; ++r) x[dof[r]] += damp * l[r];
      off += (size_t)sz;
    }
    free(rl);
  }
  free(loc);
#undef PB
#undef PS
}

void* orc_vanka_store_create(int n_patches) { return vanka_store_new(n_patches); }
void orc_vanka_store_destroy(void* st) { vanka_store_free((orc_vanka_store*)st); }

void orc_vanka_sweep(int type, int n_patches, const int* patch, int n, const int* rp, const int* ci,
                     const double* v, const double* b, double* x, double damp, const int* color_ptr,
                     const int* color_cells, int n_colors, const int* n_freeze) {
  orc_vanka_sweep_var(type, n_patches, NULL, patch, n, rp, ci, v, b, x, damp, color_ptr, color_cells, n_colors,
                      n_freeze, NULL);
}

/* ---------------------------------------------------- Stokes assembly ------
 * Assemble3D with the NSE Galerkin local forms for Stokes, Laplace form
 * (NSLaplaceGradGrad, NSDivergenceBlocks with sign 1, NSGradientBlocks,
 * NSRightHandSide: src/AssembleRoutinesSaddle/NSE_local_assembling_routines.C
 * :82-254), P2/P1 on affine tetrahedra with the P4Tetra rule
 * (src/QuadFormulas/QuadFormulaTetra.C:73). cdof: 34 combined DOFs per cell
 * ([u1 | u2 | u3 | p] numbering). Right-hand side of the manufactured
 * solution u = curl(psi (1,1,1)), psi = (sin pi x sin pi y sin pi z)^2,
 * p = x + y + z - 3/2. */
static void stokes_f(double nu, const double* x, double* f, int example) {
  if (example == -3) {
    /* include/Examples/NSE_3D/test_u_2_p_1.h: u = (y^2, xz, -y^2),
     * p = x + y + z - 3/2: f = -nu Lap u + grad p */
    f[0] = -nu * 2.0 + 1.0;
    f[1] = -nu * 0.0 + 1.0;
    f[2] = -nu * -2.0 + 1.0;
    return;
  }
  const double p = 3.14159265358979323846;
  double S[3], S1[3], S2[3], S3[3];
  for (int d = 0; d < 3; ++d) {
    const double s = sin(p * x[d]);
    S[d] = s * s;
    S1[d] = p * sin(2 * p * x[d]);
    S2[d] = 2 * p * p * cos(2 * p * x[d]);
    S3[d] = -4 * p * p * p * sin(2 * p * x[d]);
  }
  const double lx = S3[0] * S[1] * S[2] + S1[0] * S2[1] * S[2] + S1[0] * S[1] * S2[2];
  const double ly = S2[0] * S1[1] * S[2] + S[0] * S3[1] * S[2] + S[0] * S1[1] * S2[2];
  const double lz = S2[0] * S[1] * S1[2] + S[0] * S2[1] * S1[2] + S[0] * S[1] * S3[2];
  f[0] = -nu * (ly - lz) + 1.0;
  f[1] = -nu * (lz - lx) + 1.0;
  f[2] = -nu * (lx - ly) + 1.0;
}

static const double P4W[11] = {-.0131555555555555555555555555556, .00762222222222222222222222222222,
  .00762222222222222222222222222222, .00762222222222222222222222222222, .00762222222222222222222222222222,
  .0248888888888888888888888888889, .0248888888888888888888888888889, .0248888888888888888888888888889,
  .0248888888888888888888888888889, .0248888888888888888888888888889, .0248888888888888888888888888889};
static const double P4X[11] = {.25, .0714285714285714285714285714286, .785714285714285714285714285714,
  .0714285714285714285714285714286, .0714285714285714285714285714286, .399403576166799204996102147462,
  .399403576166799204996102147462, .100596423833200795003897852538, .100596423833200795003897852538,
  .100596423833200795003897852538, .399403576166799204996102147462};
static const double P4Y[11] = {.25, .0714285714285714285714285714286, .0714285714285714285714285714286,
  .785714285714285714285714285714, .0714285714285714285714285714286, .399403576166799204996102147462,
  .100596423833200795003897852538, .399403576166799204996102147462, .100596423833200795003897852538,
  .399403576166799204996102147462, .100596423833200795003897852538};
static const double P4Z[11] = {.25, .0714285714285714285714285714286, .0714285714285714285714285714286,
  .0714285714285714285714285714286, .785714285714285714285714285714, .100596423833200795003897852538,
  .399403576166799204996102147462, .399403576166799204996102147462, .399403576166799204996102147462,
  .100596423833200795003897852538, .100596423833200795003897852538};

static void p2_grad(double x, double y, double z, double* dx, double* dy, double* dz) {
  const double g0 = -3 + 4 * x + 4 * y + 4 * z;
  const double a[10] = {g0, 4 - 8 * x - 4 * y - 4 * z, -1 + 4 * x, -4 * y, 4 * y, 0, -4 * z, 4 * z, 0, 0};
  const double b[10] = {g0, -4 * x, 0, 4 - 4 * x - 8 * y - 4 * z, 4 * x, -1 + 4 * y, -4 * z, 0, 4 * z, 0};
  const double c[10] = {g0, -4 * x, 0, -4 * y, 0, 0, 4 - 4 * x - 4 * y - 8 * z, 4 * x, 4 * y, -1 + 4 * z};
  for (int i = 0; i < 10; ++i) { dx[i] = a[i]; dy[i] = b[i]; dz[i] = c[i]; }
}

static int add_entry(const int* rp, const int* ci, double* vals, int row, int col, double val) {
  for (int n = rp[row]; n < rp[row + 1]; ++n)
    if (ci[n] == col) { vals[n] += val; return 0; }
  return -1;
}

int orc_assemble_stokes_ex(int n_cells, const double* verts, double nu, const int* cdof, int n_rows,
                           const unsigned char* active, const int* rp, const int* ci, double* vals, double* rhs,
                           int example);
int orc_assemble_stokes(int n_cells, const double* verts, double nu, const int* cdof, int n_rows,
                        const unsigned char* active, const int* rp, const int* ci, double* vals, double* rhs) {
  return orc_assemble_stokes_ex(n_cells, verts, nu, cdof, n_rows, active, rp, ci, vals, rhs, 0);
}

/* the same for example 0 (manufactured) or -3 (polynomial; the Dirichlet
 * values are set by the caller) */
int orc_assemble_stokes_ex(int n_cells, const double* verts, double nu, const int* cdof, int n_rows,
                           const unsigned char* active, const int* rp, const int* ci, double* vals, double* rhs,
                           int example) {
  memset(vals, 0, sizeof(double) * (size_t)rp[n_rows]);
  memset(rhs, 0, sizeof(double) * (size_t)n_rows);
  for (int cell = 0; cell < n_cells; ++cell) {
    const double* v = verts + (size_t)cell * 12;
    double J[3][3];
    for (int d = 0; d < 3; ++d) {
      J[d][0] = v[3 + d] - v[d]; J[d][1] = v[6 + d] - v[d]; J[d][2] = v[9 + d] - v[d];
    }
    const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                       J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    double G[3][3];
    G[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
    G[0][1] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]) / det;
    G[0][2] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
    G[1][0] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) / det;
    G[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    G[1][2] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) / det;
    G[2][0] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    G[2][1] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) / det;
    G[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    const double adet = fabs(det);
    double A[10][10] = {{0}}, B[3][4][10] = {{{0}}}, BT[3][10][4] = {{{0}}}, F[3][10] = {{0}};
    for (int q = 0; q < 11; ++q) {
      const double xi = P4X[q], et = P4Y[q], ze = P4Z[q];
      double rx[10], ry[10], rz[10], ux[10], uy[10], uz[10], u[10], ps[4];
      tet_eval(12, xi, et, ze, u);
      tet_eval(11, xi, et, ze, ps);
      p2_grad(xi, et, ze, rx, ry, rz);
      for (int i = 0; i < 10; ++i) {
        ux[i] = G[0][0] * rx[i] + G[0][1] * ry[i] + G[0][2] * rz[i];
        uy[i] = G[1][0] * rx[i] + G[1][1] * ry[i] + G[1][2] * rz[i];
        uz[i] = G[2][0] * rx[i] + G[2][1] * ry[i] + G[2][2] * rz[i];
      }
      double X[3];
      for (int d = 0; d < 3; ++d) X[d] = v[d] + J[d][0] * xi + J[d][1] * et + J[d][2] * ze;
      double f[3];
      stokes_f(nu, X, f, example);
      const double Mult = P4W[q] * adet;
      for (int i = 0; i < 10; ++i)
        for (int j = 0; j < 10; ++j) A[i][j] += Mult * nu * (ux[i] * ux[j] + uy[i] * uy[j] + uz[i] * uz[j]);
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 10; ++j) {
          B[0][i][j] -= 1 * Mult * ps[i] * ux[j];
          B[1][i][j] -= 1 * Mult * ps[i] * uy[j];
          B[2][i][j] -= Mult * 1 * ps[i] * uz[j];
        }
      for (int i = 0; i < 10; ++i)
        for (int j = 0; j < 4; ++j) {
          BT[0][i][j] -= Mult * ps[j] * ux[i];
          BT[1][i][j] -= Mult * ps[j] * uy[i];
          BT[2][i][j] -= Mult * ps[j] * uz[i];
        }
      for (int i = 0; i < 10; ++i)
        for (int d = 0; d < 3; ++d) F[d][i] += Mult * u[i] * f[d];
    }
    const int* D = cdof + (size_t)cell * 34;
    for (int m = 0; m < 34; ++m) {
      const int r = D[m];
      if (!active[r]) {
        for (int n = rp[r]; n < rp[r + 1]; ++n)
          if (ci[n] == r) vals[n] = 1.0;
        continue;
      }
      for (int k = 0; k < 34; ++k) {
        const int bm = m < 30 ? m / 10 : 3, bk = k < 30 ? k / 10 : 3;
        double val;
        if (bm < 3 && bk < 3) {
          if (bm != bk) continue;
          val = A[m % 10][k % 10];
        } else if (bm < 3) {
          val = BT[bm][m % 10][k - 30];
        } else if (bk < 3) {
          val = B[bk][m - 30][k % 10];
        } else {
          continue;
        }
        if (add_entry(rp, ci, vals, r, D[k], val)) return -3;
      }
      if (m < 30) rhs[r] += F[m / 10][m % 10];
    }
  }
  return 0;
}
