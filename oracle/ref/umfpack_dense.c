/*
 * umfpack_dense.c - dense-LU stand-in behind umfpack.h (test infrastructure:
 * the oracle's build of the reference only).
 *
 * The matrix arrives in UMFPACK's compressed-column form (Ap column pointers,
 * Ai row indices). ParMooN hands its CSR arrays over unchanged and solves
 * with UMFPACK_At (src/Solver/DirectSolver.C:433), i.e. it solves its own CSR
 * system. The numeric phase scatters the matrix into a dense row-major array
 * and factorises it by Gaussian elimination with partial pivoting (largest
 * magnitude in the column, first row on ties); the solve phase runs the
 * triangular solves for A or A^T.
 */
#include "umfpack.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  long n;
} symbolic_t;

typedef struct {
  long n;
  double* lu;   /* n x n row-major, L unit lower (below the diagonal), U upper */
  long* perm;   /* row i of PA is row perm[i] of A */
  int singular;
} numeric_t;

static void defaults(double* c)
{
  if (c) for (int i = 0; i < UMFPACK_CONTROL; ++i) c[i] = 0.0;
}

static int symbolic(long n_row, long n_col, void** Symbolic, double* info)
{
  if (!Symbolic) return UMFPACK_ERROR_argument_missing;
  if (n_row <= 0 || n_col <= 0) return UMFPACK_ERROR_n_nonpositive;
  if (n_row != n_col) return UMFPACK_ERROR_invalid_matrix;
  symbolic_t* s = (symbolic_t*)malloc(sizeof(symbolic_t));
  if (!s) return UMFPACK_ERROR_out_of_memory;
  s->n = n_row;
  *Symbolic = s;
  if (info) memset(info, 0, sizeof(double) * UMFPACK_INFO);
  return UMFPACK_OK;
}

#define NUMERIC_BODY(IDX)                                                              \
  if (!Symbolic) return UMFPACK_ERROR_invalid_Symbolic_object;                         \
  if (!Numeric || !Ap || !Ai || !Ax) return UMFPACK_ERROR_argument_missing;            \
  long n = ((symbolic_t*)Symbolic)->n;                                                  \
  numeric_t* f = (numeric_t*)malloc(sizeof(numeric_t));                                \
  if (!f) return UMFPACK_ERROR_out_of_memory;                                          \
  f->n = n;                                                                            \
  f->lu = (double*)calloc((size_t)(n * n), sizeof(double));                            \
  f->perm = (long*)malloc(sizeof(long) * (size_t)n);                                   \
  f->singular = 0;                                                                     \
  if (!f->lu || !f->perm) return UMFPACK_ERROR_out_of_memory;                          \
  for (long j = 0; j < n; ++j)                                                         \
    for (IDX k = Ap[j]; k < Ap[j + 1]; ++k) f->lu[(long)Ai[k] * n + j] += Ax[k];       \
  factor(f);                                                                           \
  *Numeric = f;                                                                        \
  if (Info) {                                                                          \
    memset(Info, 0, sizeof(double) * UMFPACK_INFO);                                    \
    Info[UMFPACK_PEAK_MEMORY] = (double)(n * n) * 8.0;                                 \
    Info[UMFPACK_RCOND] = f->singular ? 0.0 : 1.0;                                     \
  }                                                                                    \
  return f->singular ? UMFPACK_WARNING_singular_matrix : UMFPACK_OK;

static void factor(numeric_t* f)
{
  long n = f->n;
  double* a = f->lu;
  for (long i = 0; i < n; ++i) f->perm[i] = i;
  for (long k = 0; k < n; ++k) {
    long p = k;
    double best = fabs(a[k * n + k]);
    for (long i = k + 1; i < n; ++i)
      if (fabs(a[i * n + k]) > best) { best = fabs(a[i * n + k]); p = i; }
    if (best == 0.0) { f->singular = 1; continue; }
    if (p != k) {
      for (long j = 0; j < n; ++j) {
        double t = a[k * n + j]; a[k * n + j] = a[p * n + j]; a[p * n + j] = t;
      }
      long t = f->perm[k]; f->perm[k] = f->perm[p]; f->perm[p] = t;
    }
    double piv = a[k * n + k];
    for (long i = k + 1; i < n; ++i) {
      double l = a[i * n + k] / piv;
      a[i * n + k] = l;
      if (l != 0.0)
        for (long j = k + 1; j < n; ++j) a[i * n + j] -= l * a[k * n + j];
    }
  }
}

/* PA = LU. sys A: x = U^-1 L^-1 P b. sys At: A^T = U^T L^T P, x = P^T L^-T U^-T b */
static int solve(int sys, numeric_t* f, double* x, const double* b)
{
  long n = f->n;
  const double* a = f->lu;
  double* w = (double*)malloc(sizeof(double) * (size_t)n);
  if (!w) return UMFPACK_ERROR_out_of_memory;
  if (sys == UMFPACK_A) {
    for (long i = 0; i < n; ++i) w[i] = b[f->perm[i]];
    for (long i = 0; i < n; ++i)
      for (long j = 0; j < i; ++j) w[i] -= a[i * n + j] * w[j];
    for (long i = n - 1; i >= 0; --i) {
      for (long j = i + 1; j < n; ++j) w[i] -= a[i * n + j] * w[j];
      w[i] /= a[i * n + i];
    }
    memcpy(x, w, sizeof(double) * (size_t)n);
  } else if (sys == UMFPACK_At) {
    for (long i = 0; i < n; ++i) w[i] = b[i];
    for (long i = 0; i < n; ++i) {          /* U^T w = b (lower triangular) */
      for (long j = 0; j < i; ++j) w[i] -= a[j * n + i] * w[j];
      w[i] /= a[i * n + i];
    }
    for (long i = n - 1; i >= 0; --i)       /* L^T v = w (unit upper) */
      for (long j = i + 1; j < n; ++j) w[i] -= a[j * n + i] * w[j];
    for (long i = 0; i < n; ++i) x[f->perm[i]] = w[i];
  } else {
    free(w);
    return UMFPACK_ERROR_invalid_system;
  }
  free(w);
  return f->singular ? UMFPACK_WARNING_singular_matrix : UMFPACK_OK;
}

static void free_numeric(void** Numeric)
{
  if (!Numeric || !*Numeric) return;
  numeric_t* f = (numeric_t*)*Numeric;
  free(f->lu);
  free(f->perm);
  free(f);
  *Numeric = 0;
}

static void free_symbolic(void** Symbolic)
{
  if (!Symbolic || !*Symbolic) return;
  free(*Symbolic);
  *Symbolic = 0;
}

void umfpack_di_defaults(double Control[UMFPACK_CONTROL]) { defaults(Control); }
void umfpack_dl_defaults(double Control[UMFPACK_CONTROL]) { defaults(Control); }

int umfpack_di_symbolic(int n_row, int n_col, const int Ap[], const int Ai[], const double Ax[],
                        void** Symbolic, const double Control[UMFPACK_CONTROL],
                        double Info[UMFPACK_INFO])
{
  (void)Ap; (void)Ai; (void)Ax; (void)Control;
  return symbolic(n_row, n_col, Symbolic, Info);
}

int umfpack_dl_symbolic(long n_row, long n_col, const long Ap[], const long Ai[],
                        const double Ax[], void** Symbolic, const double Control[UMFPACK_CONTROL],
                        double Info[UMFPACK_INFO])
{
  (void)Ap; (void)Ai; (void)Ax; (void)Control;
  return symbolic(n_row, n_col, Symbolic, Info);
}

int umfpack_di_numeric(const int Ap[], const int Ai[], const double Ax[], void* Symbolic,
                       void** Numeric, const double Control[UMFPACK_CONTROL],
                       double Info[UMFPACK_INFO])
{
  (void)Control;
  NUMERIC_BODY(int)
}

int umfpack_dl_numeric(const long Ap[], const long Ai[], const double Ax[], void* Symbolic,
                       void** Numeric, const double Control[UMFPACK_CONTROL],
                       double Info[UMFPACK_INFO])
{
  (void)Control;
  NUMERIC_BODY(long)
}

int umfpack_di_solve(int sys, const int Ap[], const int Ai[], const double Ax[], double X[],
                     const double B[], void* Numeric, const double Control[UMFPACK_CONTROL],
                     double Info[UMFPACK_INFO])
{
  (void)Ap; (void)Ai; (void)Ax; (void)Control; (void)Info;
  if (!Numeric) return UMFPACK_ERROR_invalid_Numeric_object;
  return solve(sys, (numeric_t*)Numeric, X, B);
}

int umfpack_dl_solve(int sys, const long Ap[], const long Ai[], const double Ax[], double X[],
                     const double B[], void* Numeric, const double Control[UMFPACK_CONTROL],
                     double Info[UMFPACK_INFO])
{
  (void)Ap; (void)Ai; (void)Ax; (void)Control; (void)Info;
  if (!Numeric) return UMFPACK_ERROR_invalid_Numeric_object;
  return solve(sys, (numeric_t*)Numeric, X, B);
}

void umfpack_di_free_symbolic(void** Symbolic) { free_symbolic(Symbolic); }
void umfpack_dl_free_symbolic(void** Symbolic) { free_symbolic(Symbolic); }
void umfpack_di_free_numeric(void** Numeric) { free_numeric(Numeric); }
void umfpack_dl_free_numeric(void** Numeric) { free_numeric(Numeric); }
