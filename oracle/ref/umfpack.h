/*
 * umfpack.h - stand-in for the part of SuiteSparse UMFPACK's C interface that
 * ParMooN's DirectSolver calls (src/Solver/DirectSolver.C:277-441 of the
 * reference): umfpack_{di,dl}_{defaults,symbolic,numeric,solve,free_*}.
 *
 * Test infrastructure only (the oracle's build of the reference). UMFPACK is
 * not vendored by the reference and not installed here; its published
 * interface is restated, and the factorisation is a dense LU with partial
 * pivoting (umfpack_dense.c), so the coarse solves agree with UMFPACK's up to
 * rounding, not bit for bit.
 */
#ifndef ORACLE_UMFPACK_STANDIN_H
#define ORACLE_UMFPACK_STANDIN_H

#ifdef __cplusplus
extern "C" {
#endif

#define UMFPACK_CONTROL 20
#define UMFPACK_INFO 90

/* status codes of the published interface */
#define UMFPACK_OK (0)
#define UMFPACK_WARNING_singular_matrix (1)
#define UMFPACK_WARNING_determinant_underflow (2)
#define UMFPACK_WARNING_determinant_overflow (3)
#define UMFPACK_ERROR_out_of_memory (-1)
#define UMFPACK_ERROR_invalid_Numeric_object (-3)
#define UMFPACK_ERROR_invalid_Symbolic_object (-4)
#define UMFPACK_ERROR_argument_missing (-5)
#define UMFPACK_ERROR_n_nonpositive (-6)
#define UMFPACK_ERROR_invalid_matrix (-8)
#define UMFPACK_ERROR_different_pattern (-11)
#define UMFPACK_ERROR_invalid_system (-13)
#define UMFPACK_ERROR_invalid_permutation (-15)
#define UMFPACK_ERROR_file_IO (-17)
#define UMFPACK_ERROR_internal_error (-911)

/* systems: A x = b and A^T x = b for the compressed-column matrix A */
#define UMFPACK_A (0)
#define UMFPACK_At (1)

/* Info entries read by the caller */
#define UMFPACK_PEAK_MEMORY 41
#define UMFPACK_RCOND 67

void umfpack_di_defaults(double Control[UMFPACK_CONTROL]);
int umfpack_di_symbolic(int n_row, int n_col, const int Ap[], const int Ai[], const double Ax[],
                        void** Symbolic, const double Control[UMFPACK_CONTROL],
                        double Info[UMFPACK_INFO]);
int umfpack_di_numeric(const int Ap[], const int Ai[], const double Ax[], void* Symbolic,
                       void** Numeric, const double Control[UMFPACK_CONTROL],
                       double Info[UMFPACK_INFO]);
int umfpack_di_solve(int sys, const int Ap[], const int Ai[], const double Ax[], double X[],
                     const double B[], void* Numeric, const double Control[UMFPACK_CONTROL],
                     double Info[UMFPACK_INFO]);
void umfpack_di_free_symbolic(void** Symbolic);
void umfpack_di_free_numeric(void** Numeric);

void umfpack_dl_defaults(double Control[UMFPACK_CONTROL]);
int umfpack_dl_symbolic(long n_row, long n_col, const long Ap[], const long Ai[],
                        const double Ax[], void** Symbolic, const double Control[UMFPACK_CONTROL],
                        double Info[UMFPACK_INFO]);
int umfpack_dl_numeric(const long Ap[], const long Ai[], const double Ax[], void* Symbolic,
                       void** Numeric, const double Control[UMFPACK_CONTROL],
                       double Info[UMFPACK_INFO]);
int umfpack_dl_solve(int sys, const long Ap[], const long Ai[], const double Ax[], double X[],
                     const double B[], void* Numeric, const double Control[UMFPACK_CONTROL],
                     double Info[UMFPACK_INFO]);
void umfpack_dl_free_symbolic(void** Symbolic);
void umfpack_dl_free_numeric(void** Numeric);

#ifdef __cplusplus
}
#endif
#endif
