/* Test infrastructure only: the part of GSL's public vector API (gsl_vector_double.h) that
 * the reference's fastmode uses, declared from GSL's documented interface. */
#ifndef GSL_SHIM_VECTOR_H
#define GSL_SHIM_VECTOR_H
#include <stddef.h>

typedef struct {
  size_t size, stride;
  double *data;
  void *block;
  int owner;
} gsl_vector;

typedef struct {
  gsl_vector vector;
} gsl_vector_view;

gsl_vector *gsl_vector_alloc(const size_t n);
void gsl_vector_free(gsl_vector *v);
gsl_vector_view gsl_vector_subvector(gsl_vector *v, size_t i, size_t n);
gsl_vector_view gsl_vector_view_array(double *base, size_t n);
int gsl_vector_mul(gsl_vector *a, const gsl_vector *b);
int gsl_vector_scale(gsl_vector *a, const double x);
int gsl_vector_memcpy(gsl_vector *dest, const gsl_vector *src);
double gsl_vector_get(const gsl_vector *v, const size_t i);
void gsl_vector_set(gsl_vector *v, const size_t i, double x);
#endif
