/*
 * lapack_shim.c - LAPACK entry points of the oracle's build of the reference
 * (test infrastructure only). The reference calls Fortran LAPACK (dgetrf_,
 * dgetrs_: src/Matrix/DenseMatrix.C:156-178, src/FE/LinAlg.C:98-286). No
 * system LAPACK is installed here; scipy's bundled OpenBLAS exports the same
 * Fortran-ABI routines with a "scipy_" prefix, and these wrappers forward to
 * them.
 */
extern void scipy_dgetrf_(int* m, int* n, double* a, int* lda, int* ipiv, int* info);
extern void scipy_dgetrs_(char* trans, int* n, int* nrhs, double* a, int* lda, int* ipiv,
                          double* b, int* ldb, int* info, long trans_len);
extern void scipy_dsyev_(char* jobz, char* uplo, int* n, double* a, int* lda, double* w,
                         double* work, int* lwork, int* info, long jobz_len, long uplo_len);
extern void scipy_dgemm_(char* ta, char* tb, int* m, int* n, int* k, double* alpha, double* a,
                         int* lda, double* b, int* ldb, double* beta, double* c, int* ldc,
                         long ta_len, long tb_len);

void dgetrf_(int* m, int* n, double* a, int* lda, int* ipiv, int* info)
{
  scipy_dgetrf_(m, n, a, lda, ipiv, info);
}

void dgetrs_(char* trans, int* n, int* nrhs, double* a, int* lda, int* ipiv, double* b, int* ldb,
             int* info)
{
  scipy_dgetrs_(trans, n, nrhs, a, lda, ipiv, b, ldb, info, 1);
}

void dsyev_(char* jobz, char* uplo, int* n, double* a, int* lda, double* w, double* work,
            int* lwork, int* info)
{
  scipy_dsyev_(jobz, uplo, n, a, lda, w, work, lwork, info, 1, 1);
}

void dgemm_(char* ta, char* tb, int* m, int* n, int* k, double* alpha, double* a, int* lda,
            double* b, int* ldb, double* beta, double* c, int* ldc)
{
  scipy_dgemm_(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, 1, 1);
}

/* Eigenvalue routines referenced by FindEigenValues (src/FE/LinAlg.C), which
 * is not on the solve path: present for the link, abort if ever called. */
#include <stdio.h>
#include <stdlib.h>
static void not_on_the_path(const char* name)
{
  fprintf(stderr, "oracle build of the reference: LAPACK %s is not provided\n", name);
  abort();
}
void dsptrd_(void) { not_on_the_path("dsptrd"); }
void dopgtr_(void) { not_on_the_path("dopgtr"); }
void dsteqr_(void) { not_on_the_path("dsteqr"); }
