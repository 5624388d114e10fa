/* rt_oracle.h -- CPU ORACLE interface (test infrastructure only).
 *
 * Line-constant record: double[RLK_NCONST] per Kurucz line, with the fields
 * of the reference's RLK_Line (rh/atom.h:156-167) after readKuruczLines()
 * (rh/kurucz.c:121-430) has derived them.
 */
#ifndef PYRH_RT_ORACLE_H
#define PYRH_RT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  RLK_LAMBDA0 = 0, RLK_PT_INDEX = 1, RLK_STAGE = 2, RLK_GI = 3, RLK_GJ = 4,
  RLK_EI = 5, RLK_EJ = 6, RLK_AJI = 7, RLK_BJI = 8, RLK_BIJ = 9,
  RLK_GRAD = 10, RLK_GSTARK = 11, RLK_GVDWAALS = 12, RLK_VDWAALS = 13,
  RLK_CROSS = 14, RLK_ALPHA = 15, RLK_ISOFRAC = 16, RLK_HFSFRAC = 17,
  RLK_POLARIZABLE = 18, RLK_WEIGHT = 19, RLK_CONTRIBUTES = 20,
  RLK_GL_I = 21, RLK_GL_J = 22, RLK_HAS_MODEL = 23, RLK_NCONST = 24
};

/* enum vdWaals of the reference (rh/atom.h:31) */
enum { RLK_VDW_UNSOLD = 0, RLK_VDW_RIDDER = 1, RLK_VDW_BARKLEM = 2, RLK_VDW_KURUCZ = 3 };

typedef struct {
  double T, ne, nHtot, np, vturb, vel, B, cos_gamma, cos_2chi, sin_2chi;
} OracleDepth;

/* One atmosphere in SI units (m, K, m^-3, m/s, T, rad), as the reference
   holds it after the unit conversion of pyrh_compute1dray.c:263-270. */
typedef struct {
  int ndep;
  double muz;
  const double *height, *T, *ne, *nHtot, *np, *vturb, *vel, *B, *gamma_B, *chi_B;
  const double *line_pops;     /* [nline][2][ndep]: n[stage][k], ln U(T[k]) */
} OracleAtmos;

typedef struct {
  int nline, maxcomp, magneto_optical, moving;
  int no_stokes;               /* STOKES_MODE = NO_STOKES: scalar solver */
  double vmicro_char;          /* [m/s] */
  const double *c;             /* [nline][RLK_NCONST] */
  const double *zeeman;        /* [nline][3][maxcomp]: q, shift, strength */
  const int *ncomp;            /* [nline] */
} OracleLines;

void oracle_humlicek(double a, double v, double *H, double *F);
double oracle_planck(double T, double lambda);
int oracle_lte_opacity(const OracleAtmos *A, const OracleLines *LN, int k,
                       double lambda, double *chi4, double *eta4, double *chip3);
double oracle_scalar_bezier3(int nd, const double *z, double imu,
                             const double *chi, const double *S,
                             double Bbot0, double Bbot1, int to_obs,
                             double *Iout, double *Psi);
double oracle_feautrier(int nd, const double *z, double muz, const double *chi,
                        const double *S, double Bbot0, double Bbot1,
                        double *P, double *Psi);
int oracle_lte_synth(const OracleAtmos *A, const OracleLines *LN, int nlam,
                     const double *lam, const double *chi_c, const double *eta_c,
                     int md_float, double *out);
int oracle_lte_synth_batch(int natm, int nthreads, const OracleAtmos *atms,
                           const OracleLines *LN, int nlam, const double *lam,
                           const double *chi_c, const double *eta_c,
                           int md_float, double *out);

#ifdef __cplusplus
}
#endif
#endif
