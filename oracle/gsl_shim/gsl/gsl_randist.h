/* Test infrastructure only: included by the reference's kjg_gsl.c; it uses none of GSL's
 * distributions (its Gaussian pairs are its own). */
#ifndef GSL_SHIM_RANDIST_H
#define GSL_SHIM_RANDIST_H
#include <gsl/gsl_rng.h>
#endif
