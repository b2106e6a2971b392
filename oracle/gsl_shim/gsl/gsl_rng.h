/* Test infrastructure only: GSL's random number generator interface (gsl_rng.h) as documented,
 * with the one generator the reference's fastmode uses, GSL's default mt19937. */
#ifndef GSL_SHIM_RNG_H
#define GSL_SHIM_RNG_H
#include <stddef.h>

typedef struct {
  const char *name;
  unsigned long max, min;
  size_t size;
  void (*set)(void *state, unsigned long seed);
  unsigned long (*get)(void *state);
  double (*get_double)(void *state);
} gsl_rng_type;

typedef struct {
  const gsl_rng_type *type;
  void *state;
} gsl_rng;

extern const gsl_rng_type *gsl_rng_mt19937;
extern const gsl_rng_type *gsl_rng_default;
extern unsigned long gsl_rng_default_seed;

const gsl_rng_type *gsl_rng_env_setup(void);
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_free(gsl_rng *r);
void gsl_rng_set(const gsl_rng *r, unsigned long seed);
unsigned long gsl_rng_get(const gsl_rng *r);
double gsl_rng_uniform(const gsl_rng *r);
double gsl_rng_uniform_pos(const gsl_rng *r);
const char *gsl_rng_name(const gsl_rng *r);
#endif
