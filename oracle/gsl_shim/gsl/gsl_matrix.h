/* Test infrastructure only: the part of GSL's public matrix API (gsl_matrix_double.h) that the
 * reference's fastmode (src/ksrc/kjg_fpca.c, kjg_gsl.c) uses, declared from GSL's documented
 * interface so that the reference builds without GSL (oracle/build_ref.sh).  Row-major
 * matrices with a row stride `tda`, as in GSL. */
#ifndef GSL_SHIM_MATRIX_H
#define GSL_SHIM_MATRIX_H
#include <stddef.h>

typedef struct {
  size_t size1, size2, tda;
  double *data;
  void *block;
  int owner;
} gsl_matrix;

typedef struct {
  gsl_matrix matrix;
} gsl_matrix_view;

typedef struct {
  gsl_matrix matrix;
} gsl_matrix_const_view;

gsl_matrix *gsl_matrix_alloc(size_t n1, size_t n2);
void gsl_matrix_free(gsl_matrix *m);
gsl_matrix_view gsl_matrix_submatrix(gsl_matrix *m, size_t k1, size_t k2, size_t n1, size_t n2);
gsl_matrix_const_view gsl_matrix_const_submatrix(const gsl_matrix *m, size_t k1, size_t k2,
                                                 size_t n1, size_t n2);
gsl_matrix_view gsl_matrix_view_array(double *base, size_t n1, size_t n2);
int gsl_matrix_scale(gsl_matrix *a, const double x);
int gsl_matrix_memcpy(gsl_matrix *dest, const gsl_matrix *src);
void gsl_matrix_set_zero(gsl_matrix *m);
double *gsl_matrix_ptr(gsl_matrix *m, const size_t i, const size_t j);
double gsl_matrix_get(const gsl_matrix *m, const size_t i, const size_t j);
void gsl_matrix_set(gsl_matrix *m, const size_t i, const size_t j, const double x);
#endif
