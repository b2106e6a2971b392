/* Test infrastructure only: gsl_blas_dgemm (GSL's documented BLAS interface) with the CBLAS
 * transpose codes, backed by the CBLAS dgemm of the OpenBLAS that scipy bundles. */
#ifndef GSL_SHIM_BLAS_H
#define GSL_SHIM_BLAS_H
#include <gsl/gsl_matrix.h>
#include <gsl/gsl_vector.h>

enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
typedef enum CBLAS_TRANSPOSE CBLAS_TRANSPOSE_t;

int gsl_blas_dgemm(CBLAS_TRANSPOSE_t TransA, CBLAS_TRANSPOSE_t TransB, double alpha,
                   const gsl_matrix *A, const gsl_matrix *B, double beta, gsl_matrix *C);
#endif
