/* Stand-in for the nlopt header: the reference's BOBYQA paths
 * (Pf/p4_treeOpt.c: p4_allBOBYQAOptimize, p4_newtAndBOBYQAOpt) are compiled
 * but never called by the oracle, which runs p4_newtAndBrentPowellOpt (praxis
 * from Pf/brent.c).  nlopt is absent on this machine; the driver
 * (ref_driver.c) defines these entry points to fail. */
#ifndef ORACLE_STUB_NLOPT_H
#define ORACLE_STUB_NLOPT_H
typedef struct nlopt_opt_s *nlopt_opt;
typedef enum { NLOPT_FAILURE = -1, NLOPT_ROUNDOFF_LIMITED = -4, NLOPT_SUCCESS = 1 } nlopt_result;
typedef enum { NLOPT_LN_BOBYQA = 0 } nlopt_algorithm;
typedef double (*nlopt_func)(unsigned n, const double *x, double *gradient, void *func_data);
nlopt_opt nlopt_create(nlopt_algorithm algorithm, unsigned n);
void nlopt_destroy(nlopt_opt opt);
nlopt_result nlopt_set_lower_bounds(nlopt_opt opt, const double *lb);
nlopt_result nlopt_set_upper_bounds(nlopt_opt opt, const double *ub);
nlopt_result nlopt_set_max_objective(nlopt_opt opt, nlopt_func f, void *f_data);
nlopt_result nlopt_set_ftol_abs(nlopt_opt opt, double tol);
nlopt_result nlopt_optimize(nlopt_opt opt, double *x, double *opt_f);
#endif
