/* Opaque stand-in for the GSL RNG type: the reference likelihood core only
 * passes gsl_rng pointers through prototypes, never dereferences them.  The
 * simulation (Pf/p4_treeSim.c) calls gsl_rng_uniform, which the oracle's
 * driver (ref_driver.c) defines over a counter-based stream. */
#ifndef ORACLE_STUB_GSL_RNG_H
#define ORACLE_STUB_GSL_RNG_H
typedef struct gsl_rng_s gsl_rng;
double gsl_rng_uniform(const gsl_rng *r);
#endif
