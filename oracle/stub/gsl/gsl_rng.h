/* Opaque stand-in for the GSL RNG type: the reference likelihood core only
 * passes gsl_rng pointers through prototypes, never dereferences them. */
#ifndef ORACLE_STUB_GSL_RNG_H
#define ORACLE_STUB_GSL_RNG_H
typedef struct gsl_rng_s gsl_rng;
#endif
