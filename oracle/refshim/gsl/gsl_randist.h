/* Empty stand-in: Tint.c and Integrand.c include it but call nothing from it. */
#ifndef WLREF_GSL_RANDIST_H
#define WLREF_GSL_RANDIST_H
#include "gsl_rng.h"
#endif
