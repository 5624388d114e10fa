/* nlte_oracle.h -- CPU ORACLE interface for the NLTE path (test
 * infrastructure only). */
#ifndef PYRH_NLTE_ORACLE_H
#define PYRH_NLTE_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define NLTE_MAX_ACTIVE 16

/* line record (double[NL_NREC]) */
enum { NL_I = 0, NL_J, NL_LAMBDA0, NL_AJI, NL_BJI, NL_BIJ, NL_ISOFRAC, NL_NBLUE,
       NL_NLAMBDA, NL_SYMMETRIC, NL_NCOMP, NL_CSHIFT, NL_CFRAC, NL_VOIGT, NL_PRD,
       NL_POLARIZED, NL_NREC = 16 };
/* continuum record (double[NC_NREC]) */
enum { NC_I = 0, NC_J, NC_NBLUE, NC_NLAMBDA, NC_LAMBDA0, NC_HYDRO, NC_AOFF, NC_NREC = 8 };

typedef struct {
  int ndep, nspect, nrays, nlevel, nline, ncont, moving;
  const double *lambda;                 /* [nspect] nm */
  const double *muz, *wmu;              /* [nrays] */
  const double *height, *T, *vel, *vbroad;   /* [ndep] SI */
  const double *chi_c, *eta_c, *sca_c;  /* [nspect][ndep] */
  const int *bgline;                    /* [nspect] backgrflags: bit 0 hasline,
                                           bit 1 ispolarized */
  const double *nstar, *ntotal, *C;     /* [nlevel][ndep], [ndep], [nlevel^2][ndep] */
  const double *lines, *adamp;          /* [nline][NL_NREC], [nline][ndep] */
  const double *cont, *alpha;           /* [ncont][NC_NREC], concatenated */
  int ng_delay, ng_order, ng_period, isum, nmax_iter;
  double iter_limit;
} NlteProblem;

double oracle_voigt_armstrong(double a, double v);
void oracle_nlte_profiles(const NlteProblem *P, int nrays, const double *muz,
                          const double *wmu, double **phi, double *wphi);
void oracle_nlte_spectrum(const NlteProblem *P, const double *n, const double *Jold,
                          double *J_new, double *Gamma, double **phi, const double *wphi);
int oracle_stat_equil(const NlteProblem *P, const double *Gamma, double *n);
int oracle_nlte_iterate(const NlteProblem *P, double *n, double *J, double *dpops,
                        int *accelerated);
/* the same with the radiative rates (addtoRates, fillgamma.c:375-461) of
   the pass, [nline][2][ndep] followed by [ncont][2][ndep] */
void oracle_nlte_spectrum_rates(const NlteProblem *P, const double *n, const double *Jold,
                                double *J_new, double *Gamma, double **phi,
                                const double *wphi, double *rates);
int oracle_nlte_iterate_rates(const NlteProblem *P, double *n, double *J, double *dpops,
                              int *accelerated, double *rates);
void oracle_nlte_emergent(const NlteProblem *P, double mu_out, const double *n,
                          const double *J, double *Iout);

#ifdef __cplusplus
}
#endif
#endif
