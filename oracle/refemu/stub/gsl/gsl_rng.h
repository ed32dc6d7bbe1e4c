/* Stand-in for GSL's gsl_rng.h, for compiling the reference driver's host
 * code (oracle/refemu/refhost_driver.c) where GSL is not installed.  The
 * generator behind it is refhost's own (not ranlxs2): the pins that use the
 * driver do not depend on its draws.  Oracle test infrastructure only. */
#ifndef PF_REFHOST_GSL_RNG_H
#define PF_REFHOST_GSL_RNG_H
typedef struct gsl_rng_type { int id; } gsl_rng_type;
typedef struct gsl_rng { unsigned long long s; } gsl_rng;
extern const gsl_rng_type *gsl_rng_ranlxs2;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(gsl_rng *r, unsigned long int seed);
double gsl_rng_uniform(gsl_rng *r);
void gsl_rng_free(gsl_rng *r);
#endif
