/* Test-infrastructure shim (point sources are not on the tested path). */
#ifndef SHIM_GSL_RANDIST_H
#define SHIM_GSL_RANDIST_H
#include "gsl_rng.h"
unsigned int gsl_ran_poisson(const gsl_rng *r, double mu);
#endif
