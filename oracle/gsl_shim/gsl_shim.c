/* Test infrastructure only (oracle/_ref build): implementations of the GSL API subset declared
 * in oracle/gsl_shim/gsl/ -- matrix and vector views, gsl_blas_dgemm over CBLAS, and GSL's
 * default generator mt19937 -- so that the reference's fastmode (src/ksrc/kjg_fpca.c,
 * kjg_gsl.c) links without GSL.
 *
 * mt19937: the Matsumoto-Nishimura generator (ACM TOMACS 8(1), 1998) with its 2002
 * initialisation, which is how GSL documents gsl_rng_mt19937 ("the seeding procedure ... of
 * the 2002 version"); GSL maps the seed 0 to its default 4357.  gsl_rng_uniform returns the
 * 32-bit output divided by 2^32 and gsl_rng_uniform_pos repeats it until the value is not 0. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <gsl/gsl_blas.h>
#include <gsl/gsl_matrix.h>
#include <gsl/gsl_rng.h>
#include <gsl/gsl_vector.h>

/* ---- matrices ------------------------------------------------------------------------ */
gsl_matrix *gsl_matrix_alloc(size_t n1, size_t n2)
{
  gsl_matrix *m = (gsl_matrix *)calloc(1, sizeof(gsl_matrix));
  m->data = (double *)calloc(n1 * n2 ? n1 * n2 : 1, sizeof(double));
  m->size1 = n1;
  m->size2 = n2;
  m->tda = n2;
  m->owner = 1;
  return m;
}

void gsl_matrix_free(gsl_matrix *m)
{
  if (!m) return;
  if (m->owner) free(m->data);
  free(m);
}

gsl_matrix_view gsl_matrix_submatrix(gsl_matrix *m, size_t k1, size_t k2, size_t n1, size_t n2)
{
  gsl_matrix_view v;
  memset(&v, 0, sizeof v);
  v.matrix.data = m->data + k1 * m->tda + k2;
  v.matrix.size1 = n1;
  v.matrix.size2 = n2;
  v.matrix.tda = m->tda;
  return v;
}

gsl_matrix_const_view gsl_matrix_const_submatrix(const gsl_matrix *m, size_t k1, size_t k2,
                                                 size_t n1, size_t n2)
{
  gsl_matrix_const_view v;
  memset(&v, 0, sizeof v);
  v.matrix.data = m->data + k1 * m->tda + k2;
  v.matrix.size1 = n1;
  v.matrix.size2 = n2;
  v.matrix.tda = m->tda;
  return v;
}

gsl_matrix_view gsl_matrix_view_array(double *base, size_t n1, size_t n2)
{
  gsl_matrix_view v;
  memset(&v, 0, sizeof v);
  v.matrix.data = base;
  v.matrix.size1 = n1;
  v.matrix.size2 = n2;
  v.matrix.tda = n2;
  return v;
}

int gsl_matrix_scale(gsl_matrix *a, const double x)
{
  for (size_t i = 0; i < a->size1; ++i)
    for (size_t j = 0; j < a->size2; ++j) a->data[i * a->tda + j] *= x;
  return 0;
}

int gsl_matrix_memcpy(gsl_matrix *dest, const gsl_matrix *src)
{
  if (dest->size1 != src->size1 || dest->size2 != src->size2) return 19; /* GSL_EBADLEN */
  for (size_t i = 0; i < src->size1; ++i)
    memcpy(dest->data + i * dest->tda, src->data + i * src->tda, src->size2 * sizeof(double));
  return 0;
}

void gsl_matrix_set_zero(gsl_matrix *m)
{
  for (size_t i = 0; i < m->size1; ++i) memset(m->data + i * m->tda, 0, m->size2 * sizeof(double));
}

double *gsl_matrix_ptr(gsl_matrix *m, const size_t i, const size_t j)
{
  return m->data + i * m->tda + j;
}

double gsl_matrix_get(const gsl_matrix *m, const size_t i, const size_t j)
{
  return m->data[i * m->tda + j];
}

void gsl_matrix_set(gsl_matrix *m, const size_t i, const size_t j, const double x)
{
  m->data[i * m->tda + j] = x;
}

/* ---- vectors ------------------------------------------------------------------------- */
gsl_vector *gsl_vector_alloc(const size_t n)
{
  gsl_vector *v = (gsl_vector *)calloc(1, sizeof(gsl_vector));
  v->data = (double *)calloc(n ? n : 1, sizeof(double));
  v->size = n;
  v->stride = 1;
  v->owner = 1;
  return v;
}

void gsl_vector_free(gsl_vector *v)
{
  if (!v) return;
  if (v->owner) free(v->data);
  free(v);
}

gsl_vector_view gsl_vector_subvector(gsl_vector *v, size_t i, size_t n)
{
  gsl_vector_view w;
  memset(&w, 0, sizeof w);
  w.vector.data = v->data + i * v->stride;
  w.vector.size = n;
  w.vector.stride = v->stride;
  return w;
}

gsl_vector_view gsl_vector_view_array(double *base, size_t n)
{
  gsl_vector_view w;
  memset(&w, 0, sizeof w);
  w.vector.data = base;
  w.vector.size = n;
  w.vector.stride = 1;
  return w;
}

int gsl_vector_mul(gsl_vector *a, const gsl_vector *b)
{
  for (size_t i = 0; i < a->size; ++i) a->data[i * a->stride] *= b->data[i * b->stride];
  return 0;
}

int gsl_vector_scale(gsl_vector *a, const double x)
{
  for (size_t i = 0; i < a->size; ++i) a->data[i * a->stride] *= x;
  return 0;
}

int gsl_vector_memcpy(gsl_vector *dest, const gsl_vector *src)
{
  if (dest->size != src->size) return 19;
  for (size_t i = 0; i < src->size; ++i) dest->data[i * dest->stride] = src->data[i * src->stride];
  return 0;
}

double gsl_vector_get(const gsl_vector *v, const size_t i) { return v->data[i * v->stride]; }

void gsl_vector_set(gsl_vector *v, const size_t i, double x) { v->data[i * v->stride] = x; }

/* ---- BLAS ---------------------------------------------------------------------------- */
void scipy_cblas_dgemm(int order, int transa, int transb, int m, int n, int k, double alpha,
                       const double *a, int lda, const double *b, int ldb, double beta, double *c,
                       int ldc);

int gsl_blas_dgemm(CBLAS_TRANSPOSE_t TransA, CBLAS_TRANSPOSE_t TransB, double alpha,
                   const gsl_matrix *A, const gsl_matrix *B, double beta, gsl_matrix *C)
{
  const size_t M = C->size1, N = C->size2;
  const size_t K = TransA == CblasNoTrans ? A->size2 : A->size1;
  const size_t KB = TransB == CblasNoTrans ? B->size1 : B->size2;
  const size_t MA = TransA == CblasNoTrans ? A->size1 : A->size2;
  const size_t NB = TransB == CblasNoTrans ? B->size2 : B->size1;
  if (K != KB || M != MA || N != NB) {
    fprintf(stderr, "gsl_blas_dgemm: invalid length\n");
    abort();
  }
  if (M == 0 || N == 0) return 0;
  scipy_cblas_dgemm(101 /* CblasRowMajor */, (int)TransA, (int)TransB, (int)M, (int)N, (int)K,
                    alpha, A->data, (int)A->tda, B->data, (int)B->tda, beta, C->data,
                    (int)C->tda);
  return 0;
}

/* ---- mt19937 ------------------------------------------------------------------------- */
#define MT_N 624
#define MT_M 397

typedef struct {
  unsigned long mt[MT_N];
  int mti;
} mt_state_t;

static void mt_set(void *vs, unsigned long s)
{
  mt_state_t *st = (mt_state_t *)vs;
  if (s == 0) s = 4357;
  st->mt[0] = s & 0xffffffffUL;
  int i;
  for (i = 1; i < MT_N; ++i)
    st->mt[i] = (1812433253UL * (st->mt[i - 1] ^ (st->mt[i - 1] >> 30)) + (unsigned long)i) &
                0xffffffffUL;
  st->mti = i;
}

static unsigned long mt_get(void *vs)
{
  mt_state_t *st = (mt_state_t *)vs;
  const unsigned long upper = 0x80000000UL, lower = 0x7fffffffUL, a = 0x9908b0dfUL;
  if (st->mti >= MT_N) {
    int kk;
    unsigned long y;
    for (kk = 0; kk < MT_N - MT_M; ++kk) {
      y = (st->mt[kk] & upper) | (st->mt[kk + 1] & lower);
      st->mt[kk] = st->mt[kk + MT_M] ^ (y >> 1) ^ ((y & 1UL) ? a : 0UL);
    }
    for (; kk < MT_N - 1; ++kk) {
      y = (st->mt[kk] & upper) | (st->mt[kk + 1] & lower);
      st->mt[kk] = st->mt[kk + (MT_M - MT_N)] ^ (y >> 1) ^ ((y & 1UL) ? a : 0UL);
    }
    y = (st->mt[MT_N - 1] & upper) | (st->mt[0] & lower);
    st->mt[MT_N - 1] = st->mt[MT_M - 1] ^ (y >> 1) ^ ((y & 1UL) ? a : 0UL);
    st->mti = 0;
  }
  unsigned long k = st->mt[st->mti++];
  k ^= (k >> 11);
  k ^= (k << 7) & 0x9d2c5680UL;
  k ^= (k << 15) & 0xefc60000UL;
  k ^= (k >> 18);
  return k & 0xffffffffUL;
}

static double mt_get_double(void *vs) { return (double)mt_get(vs) / 4294967296.0; }

static const gsl_rng_type mt_type = {"mt19937", 0xffffffffUL, 0, sizeof(mt_state_t),
                                     mt_set, mt_get, mt_get_double};

const gsl_rng_type *gsl_rng_mt19937 = &mt_type;
const gsl_rng_type *gsl_rng_default = &mt_type;
unsigned long gsl_rng_default_seed = 0;

const gsl_rng_type *gsl_rng_env_setup(void)
{
  const char *t = getenv("GSL_RNG_TYPE");
  if (t && strcmp(t, "mt19937") != 0) {
    fprintf(stderr, "GSL_RNG_TYPE=%s: only mt19937 is available here\n", t);
    abort();
  }
  const char *s = getenv("GSL_RNG_SEED");
  if (s) gsl_rng_default_seed = strtoul(s, NULL, 0);
  return gsl_rng_default;
}

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T)
{
  gsl_rng *r = (gsl_rng *)calloc(1, sizeof(gsl_rng));
  r->type = T;
  r->state = calloc(1, T->size);
  gsl_rng_set(r, gsl_rng_default_seed);
  return r;
}

void gsl_rng_free(gsl_rng *r)
{
  if (!r) return;
  free(r->state);
  free(r);
}

void gsl_rng_set(const gsl_rng *r, unsigned long seed) { r->type->set(r->state, seed); }

unsigned long gsl_rng_get(const gsl_rng *r) { return r->type->get(r->state); }

double gsl_rng_uniform(const gsl_rng *r) { return r->type->get_double(r->state); }

double gsl_rng_uniform_pos(const gsl_rng *r)
{
  double x;
  do {
    x = r->type->get_double(r->state);
  } while (x == 0);
  return x;
}

const char *gsl_rng_name(const gsl_rng *r) { return r->type->name; }
