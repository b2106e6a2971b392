/* Test infrastructure only: the four LAPACKE routines of the reference's kjg_gsl.c, taken from
 * the OpenBLAS that scipy bundles (exported with a scipy_ prefix, 32-bit integers). */
#ifndef GSL_SHIM_LAPACKE_H
#define GSL_SHIM_LAPACKE_H
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
typedef int lapack_int;
lapack_int scipy_LAPACKE_dgesvd(int matrix_layout, char jobu, char jobvt, lapack_int m,
                                lapack_int n, double *a, lapack_int lda, double *s, double *u,
                                lapack_int ldu, double *vt, lapack_int ldvt, double *superb);
double scipy_LAPACKE_dlange(int matrix_layout, char norm, lapack_int m, lapack_int n,
                            const double *a, lapack_int lda);
lapack_int scipy_LAPACKE_dgeqrf(int matrix_layout, lapack_int m, lapack_int n, double *a,
                                lapack_int lda, double *tau);
lapack_int scipy_LAPACKE_dorgqr(int matrix_layout, lapack_int m, lapack_int n, lapack_int k,
                                double *a, lapack_int lda, const double *tau);
#define LAPACKE_dgesvd scipy_LAPACKE_dgesvd
#define LAPACKE_dlange scipy_LAPACKE_dlange
#define LAPACKE_dgeqrf scipy_LAPACKE_dgeqrf
#define LAPACKE_dorgqr scipy_LAPACKE_dorgqr
#endif
