/* nlte_oracle.c -- CPU ORACLE for the NLTE MALI path (test infrastructure,
 * never shipped or measured as the product).  FP64 restatement of the
 * reference's lambda iteration for one active atom in a 1-D atmosphere,
 * starting from the state the reference's set-up leaves (populations,
 * collision matrix, background, line damping, continuum cross-sections).
 *
 * Parity pinned against the compiled reference (tests/golden/nlte_*.npz,
 * produced by tests/golden/make_golden.py).
 *
 * Restated (reference file:line):
 *   voigt_armstrong  rh/voigt.c:126-243 (Armstrong 1967, JQSRT 7, 61: K1 with
 *                    the odd Chebyshev expansion of Dawson's integral on
 *                    [0,5] and its asymptotic series above, K2/K3 with
 *                    20-point Gauss-Hermite quadrature)
 *   profiles         rh/profile.c:67-371 (field-free, moving atmosphere:
 *                    phi per (lambda, mu, direction, depth), wphi)
 *   opacity          rh/opacity.c:64-300 (active lines and continua)
 *   coupling         rh/fillgamma.c:251-332 (addtoCoupling)
 *   gamma            rh/fillgamma.c:82-246 (addtoGamma)
 *   formal           rh/rhf1d/formal.c:44-346 (Bezier branch with Psi for
 *                    both directions, Feautrier branch where no line is
 *                    active), rh/rhf1d/bezier_1D.c:306-541,
 *                    rh/rhf1d/feautrier.c:56-202
 *   stat_equil       rh/statequil.c:40-102, rh/ludcmp.c:36-177
 *   ng               rh/accelerate.c:34-146, rh/maxchange.c:32-50
 *   iterate          rh/iterate.c:48-143
 *   emergent         rh/rhf1d/pyrh_solveray.c:75-150 (one ray, fixed J)
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "nlte_oracle.h"
#include "rt_oracle.h"

#define CLIGHT      2.99792458E+08
#define HPLANCK     6.6260755E-34
#define KBOLTZMANN  1.380658E-23
#define NM_TO_M     1.0E-09
#define PI          3.14159265358979
#define SQRTPI      1.77245385090551

/* ------------------------------------------------------ Armstrong Voigt -- */

/* Chebyshev coefficients of Dawson(5x) in odd T_{2n+1}(x), x in [0,1]
   (computed from the definition of Dawson's integral). */
static const double DAWSON_CHEB[34] = {
  0.1999999999972224, -0.18400000000299979,
  0.15583999999650247, -0.12166400000439881,
  0.087708159994039123, -0.058514124808690643,
  0.036215730162391359, -0.020849765439803627,
  0.011196011634627011, -0.0056231896167108913,
  0.0026487634172264554, -0.0011732670757704463,
  0.00048995199780883401, -0.00019336308015277829,
  7.2287744678832942e-05, -2.565551249788587e-05,
  8.6620736840759859e-06, -2.7876379719252641e-06,
  8.5668736268524721e-07, -2.5184337837693224e-07,
  7.0936022149218665e-08, -1.917322572749502e-08,
  4.9801256466357896e-09, -1.2447733996061773e-09,
  2.9977766411656295e-10, -6.9644956269250685e-11,
  1.5626242538020159e-11, -3.3896879080452118e-12,
  7.1161574262122503e-13, -1.4472012169242576e-13,
  2.8536768232975401e-14, -5.4606927155058021e-15,
  1.0148769468261627e-15, -1.8333259200975614e-16};
/* positive nodes and weights of the 20-point Gauss-Hermite rule */
static const double GH_T[10] = {
  0.24534070830090124, 0.73747372854539439, 1.2340762153953231, 1.7385377121165861,
  2.2549740020892757, 2.7888060584281305, 3.3478545673832163, 3.9447640401156252,
  4.6036824495507442, 5.3874808900112328};
static const double GH_W[10] = {
  0.46224366960061009, 0.28667550536283415, 0.10901720602002329, 0.024810520887463643,
  0.0032437733422378567, 0.00022833863601635365, 7.8025564785320599e-06,
  1.0860693707692782e-07, 4.3993409922731747e-10, 2.2293936455341447e-13};

#define ARM_TINY 1.0E-08
#define TWOSQRTPI 1.12837917

static double voigt_k1(double a, double v)
{
  double a2 = a * a, v2 = v * v, u1, dn01, dn02;
  u1 = ((v2 - a2) > 70.0) ? 0.0 : exp(a2 - v2) * cos(2.0 * v * a);
  if (v > 5.0) {
    double r = 1.0 / v2;
    dn01 = -r * (0.5 + r * (0.75 + r * (1.875 + r * (6.5625 + r * (29.53125 +
           r * (1162.4218 + r * 1055.7421))))));
    dn02 = (1.0 - dn01) / (2.0 * v);
  } else {
    double b1 = 0.0, b2 = 0.0, b = 0.0, x = v / 5.0, coef = 4.0 * x * x - 2.0;
    for (int n = 33; n >= 0; n--) {
      b = coef * b1 - b2 + DAWSON_CHEB[n];
      b2 = b1;
      b1 = b;
    }
    dn02 = x * (b - b2);
    dn01 = 1.0 - 2.0 * v * dn02;
  }
  double funct = a * dn01;
  if (a > ARM_TINY) {
    double q = 1.0, an = a;
    for (int n = 2; n <= 50; n++) {
      double dn = (v * dn01 + dn02) * (-2.0 / n);
      dn02 = dn01;
      dn01 = dn;
      if (n % 2) {
        q = -q;
        an *= a2;
        double g = dn * an;
        funct += q * g;
        if (fabs(g / funct) <= ARM_TINY) return u1 - TWOSQRTPI * funct;
      }
    }
  }
  return u1 - TWOSQRTPI * funct;
}

static double voigt_k2(double a, double v)
{
  double g = 0.0, a2 = a * a;
  for (int n = 0; n < 10; n++) {
    double r = GH_T[n] - v, s = GH_T[n] + v;
    g += (4.0 * GH_T[n] * GH_T[n] - 2.0) *
         (r * atan(r / a) + s * atan(s / a) - 0.5 * a * (log(a2 + r * r) + log(a2 + s * s))) *
         GH_W[n];
  }
  return g / PI;
}

static double voigt_k3(double a, double v)
{
  double g = 0.0, a2 = a * a;
  for (int n = 0; n < 10; n++)
    g += (1.0 / ((v - GH_T[n]) * (v - GH_T[n]) + a2) +
          1.0 / ((v + GH_T[n]) * (v + GH_T[n]) + a2)) * GH_W[n];
  return (a * g) / PI;
}

double oracle_voigt_armstrong(double a, double v)
{
  if (v < 0.0) v = -v;
  if ((a < 1.0 && v < 4.0) || (a < 1.8 / (v + 1.0))) return voigt_k1(a, v);
  if (a < 2.5 && v < 4.0) return voigt_k2(a, v);
  return voigt_k3(a, v);
}

/* ---------------------------------------------------------- profiles -- */

static double wlambda_line(const NlteProblem *P, const double *L, int la)
{
  int nb = (int) L[NL_NBLUE], nl = (int) L[NL_NLAMBDA];
  const double *lam = P->lambda + nb;
  double Dw = CLIGHT / L[NL_LAMBDA0];
  if ((int) L[NL_SYMMETRIC]) Dw *= 2.0;
  double w;
  if (la == 0) w = 0.5 * (lam[1] - lam[0]);
  else if (la == nl - 1) w = 0.5 * (lam[la] - lam[la - 1]);
  else w = 0.5 * (lam[la + 1] - lam[la - 1]);
  return w * Dw;
}

static double wlambda_cont(const NlteProblem *P, const double *Cr, int la)
{
  int nb = (int) Cr[NC_NBLUE], nl = (int) Cr[NC_NLAMBDA];
  const double *lam = P->lambda + nb;
  if (la == 0) return 0.5 * (lam[1] - lam[0]);
  if (la == nl - 1) return 0.5 * (lam[la] - lam[la - 1]);
  return 0.5 * (lam[la + 1] - lam[la - 1]);
}

/* phi[line] is [Nlambda][2*nrays][ndep] (lamu = 2 (nrays la + mu) + to_obs),
   wphi [nline][ndep] holds the inverse normalisation (profile.c:199-364). */
void oracle_nlte_profiles(const NlteProblem *P, int nrays, const double *muz,
                          const double *wmu, double **phi, double *wphi)
{
  int nd = P->ndep;
  for (int kr = 0; kr < P->nline; kr++) {
    const double *L = P->lines + (long) kr * NL_NREC;
    int nl = (int) L[NL_NLAMBDA], nb = (int) L[NL_NBLUE];
    double lam0 = L[NL_LAMBDA0], cs = L[NL_CSHIFT], cf = L[NL_CFRAC];
    const double *ad = P->adamp + (long) kr * nd;
    double *wp = wphi + (long) kr * nd;
    for (int k = 0; k < nd; k++) wp[k] = 0.0;
    for (int la = 0; la < nl; la++) {
      double lam = P->lambda[nb + la];
      for (int mu = 0; mu < nrays; mu++) {
        double wlamu = wlambda_line(P, L, la) * 0.5 * wmu[mu];
        for (int to_obs = 0; to_obs <= 1; to_obs++) {
          double sign = to_obs ? 1.0 : -1.0;
          int lamu = 2 * (nrays * la + mu) + to_obs;
          double *ph = phi[kr] + (long) lamu * nd;
          for (int k = 0; k < nd; k++) {
            double vb = P->vbroad[k];
            double v = (lam - lam0 - cs) * CLIGHT / (vb * lam0);
            double vlos = P->moving ? muz[mu] * P->vel[k] / vb : 0.0;
            double vk = v + sign * vlos;
            double a = (int) L[NL_VOIGT] ? ad[k] : 0.0;
            ph[k] = oracle_voigt_armstrong(a, vk) * cf / (SQRTPI * vb);
            wp[k] += ph[k] * wlamu;
          }
        }
      }
    }
    for (int k = 0; k < nd; k++) wp[k] = 1.0 / wp[k];
  }
}

/* --------------------------------------------------------- linear algebra */

/* Crout LU with implicit pivoting and one step of iterative improvement
   (rh/ludcmp.c:36-177).  A is n x n row-major, overwritten. */
static int solve_linear_eq(int n, double *A, double *b)
{
  double Ac[64], bc[8], vv[8], res[8];
  int index[8];
  memcpy(Ac, A, sizeof(double) * n * n);
  memcpy(bc, b, sizeof(double) * n);
  for (int i = 0; i < n; i++) {
    double big = 0.0;
    for (int j = 0; j < n; j++) if (fabs(A[i * n + j]) > big) big = fabs(A[i * n + j]);
    if (big == 0.0) return -1;
    vv[i] = 1.0 / big;
  }
  for (int j = 0; j < n; j++) {
    int imax = 0;
    for (int i = 0; i < j; i++) {
      double sum = A[i * n + j];
      for (int k = 0; k < i; k++) sum -= A[i * n + k] * A[k * n + j];
      A[i * n + j] = sum;
    }
    double big = 0.0;
    for (int i = j; i < n; i++) {
      double sum = A[i * n + j];
      for (int k = 0; k < j; k++) sum -= A[i * n + k] * A[k * n + j];
      A[i * n + j] = sum;
      double dum = vv[i] * fabs(sum);
      if (dum >= big) { big = dum; imax = i; }
    }
    if (j != imax) {
      for (int k = 0; k < n; k++) {
        double t = A[imax * n + k]; A[imax * n + k] = A[j * n + k]; A[j * n + k] = t;
      }
      vv[imax] = vv[j];
    }
    index[j] = imax;
    if (A[j * n + j] == 0.0) A[j * n + j] = 1.0e-20;
    double dum = 1.0 / A[j * n + j];
    for (int i = j + 1; i < n; i++) A[i * n + j] *= dum;
  }
  for (int pass = 0; pass < 2; pass++) {
    double *x = pass ? res : b;
    if (pass) {
      for (int i = 0; i < n; i++) {
        res[i] = bc[i];
        for (int j = 0; j < n; j++) res[i] -= Ac[i * n + j] * b[j];
      }
    }
    int ii = -1;
    for (int i = 0; i < n; i++) {
      int ip = index[i];
      double sum = x[ip];
      x[ip] = x[i];
      if (ii >= 0) for (int j = ii; j < i; j++) sum -= A[i * n + j] * x[j];
      else if (sum) ii = i;
      x[i] = sum;
    }
    for (int i = n - 1; i >= 0; i--) {
      double sum = x[i];
      for (int j = i + 1; j < n; j++) sum -= A[i * n + j] * x[j];
      x[i] = sum / A[i * n + i];
    }
  }
  for (int i = 0; i < n; i++) b[i] += res[i];
  return 0;
}

/* --------------------------------------------------------- formal step -- */

typedef struct {
  int nact, type[NLTE_MAX_ACTIVE], kr[NLTE_MAX_ACTIVE], la[NLTE_MAX_ACTIVE];
  int i[NLTE_MAX_ACTIVE], j[NLTE_MAX_ACTIVE];
  int boundbound, polarized;
} ActiveSet;

static void active_set(const NlteProblem *P, int ns, ActiveSet *as)
{
  as->nact = 0;
  as->boundbound = 0;
  as->polarized = 0;
  for (int kr = 0; kr < P->ncont; kr++) {        /* continua first (sortlambda.c:290-335) */
    const double *Cr = P->cont + (long) kr * NC_NREC;
    int nb = (int) Cr[NC_NBLUE], nl = (int) Cr[NC_NLAMBDA];
    if (ns >= nb && ns < nb + nl && as->nact < NLTE_MAX_ACTIVE) {
      int n = as->nact++;
      as->type[n] = 1; as->kr[n] = kr; as->la[n] = ns - nb;
      as->i[n] = (int) Cr[NC_I]; as->j[n] = (int) Cr[NC_J];
    }
  }
  for (int kr = 0; kr < P->nline; kr++) {         /* then lines (sortlambda.c:336-372) */
    const double *L = P->lines + (long) kr * NL_NREC;
    int nb = (int) L[NL_NBLUE], nl = (int) L[NL_NLAMBDA];
    if (ns >= nb && ns < nb + nl && as->nact < NLTE_MAX_ACTIVE) {
      int n = as->nact++;
      as->type[n] = 0; as->kr[n] = kr; as->la[n] = ns - nb;
      as->i[n] = (int) L[NL_I]; as->j[n] = (int) L[NL_J];
      as->boundbound = 1;
      if ((int) L[NL_POLARIZED]) as->polarized = 1;
    }
  }
}

typedef struct {
  double *Vij, *gij, *wla;      /* [NLTE_MAX_ACTIVE][ndep] */
  double *chi_up, *chi_down, *Uji_down;   /* [nlevel][ndep] */
  double *eta_atom, *chi, *S, *I, *Psi, *Jdag, *Ieff;
} Work;

/* Opacity of the active set (opacity.c:64-300) for ray (mu, to_obs). */
static void active_opacity(const NlteProblem *P, const ActiveSet *as, int ns, int nrays,
                           int mu, int to_obs, double **phi, const double *wphi,
                           const double *n, Work *W, double *chi_act)
{
  int nd = P->ndep;
  const double hc = HPLANCK * CLIGHT, hc_4PI = hc / (4.0 * PI);
  const double twohc = 2.0 * hc / (NM_TO_M * NM_TO_M * NM_TO_M);
  const double hc_k = hc / (KBOLTZMANN * NM_TO_M);
  for (int k = 0; k < nd; k++) { chi_act[k] = 0.0; W->eta_atom[k] = 0.0; }
  for (int m = 0; m < as->nact; m++) {
    double *Vij = W->Vij + (long) m * nd, *gij = W->gij + (long) m * nd;
    double *wla = W->wla + (long) m * nd;
    int i = as->i[m], j = as->j[m], la = as->la[m];
    const double *ni = n + (long) i * nd, *nj = n + (long) j * nd;
    double twohnu3_c2;
    if (as->type[m] == 0) {
      const double *L = P->lines + (long) as->kr[m] * NL_NREC;
      int lamu = 2 * (nrays * la + mu) + to_obs;
      const double *ph = phi[as->kr[m]] + (long) lamu * nd;
      twohnu3_c2 = L[NL_AJI] / L[NL_BJI];
      double gijk = L[NL_BJI] / L[NL_BIJ];
      double Bijxhc_4PI = hc_4PI * L[NL_BIJ] * L[NL_ISOFRAC];
      double wl = wlambda_line(P, L, la);
      const double *wp = wphi + (long) as->kr[m] * nd;
      for (int k = 0; k < nd; k++) {
        gij[k] = gijk;
        Vij[k] = Bijxhc_4PI * ph[k];
        wla[k] = wl * wp[k] / hc_4PI;
      }
    } else {
      const double *Cr = P->cont + (long) as->kr[m] * NC_NREC;
      double lam = P->lambda[ns];
      twohnu3_c2 = twohc / (lam * lam * lam);
      double a = P->alpha[(long) Cr[NC_AOFF] + la];
      double wl = wlambda_cont(P, Cr, la);
      const double *nsi = P->nstar + (long) i * nd, *nsj = P->nstar + (long) j * nd;
      for (int k = 0; k < nd; k++) {
        Vij[k] = a;
        gij[k] = nsi[k] / nsj[k] * exp(-hc_k / (lam * P->T[k]));
        wla[k] = 4.0 * PI / HPLANCK * (wl / lam);
      }
    }
    for (int k = 0; k < nd; k++) {
      chi_act[k] += Vij[k] * (ni[k] - gij[k] * nj[k]);
      W->eta_atom[k] += twohnu3_c2 * gij[k] * Vij[k] * nj[k];
    }
  }
}

static double twohnu3_of(const NlteProblem *P, const ActiveSet *as, int m, int ns)
{
  if (as->type[m] == 0) {
    const double *L = P->lines + (long) as->kr[m] * NL_NREC;
    return L[NL_AJI] / L[NL_BJI];
  }
  double lam = P->lambda[ns];
  return 2.0 * HPLANCK * CLIGHT / (NM_TO_M * NM_TO_M * NM_TO_M) / (lam * lam * lam);
}

/* addtoCoupling (fillgamma.c:251-332) */
static void add_coupling(const NlteProblem *P, const ActiveSet *as, int ns,
                         const double *n, Work *W)
{
  int nd = P->ndep;
  for (int m = 0; m < as->nact; m++) {
    int i = as->i[m], j = as->j[m];
    for (int k = 0; k < nd; k++) {
      W->chi_up[(long) i * nd + k] = 0.0;
      W->chi_down[(long) j * nd + k] = 0.0;
      W->Uji_down[(long) j * nd + k] = 0.0;
    }
  }
  for (int m = 0; m < as->nact; m++) {
    int i = as->i[m], j = as->j[m];
    double t = twohnu3_of(P, as, m, ns);
    const double *Vij = W->Vij + (long) m * nd, *gij = W->gij + (long) m * nd;
    const double *wla = W->wla + (long) m * nd;
    for (int k = 0; k < nd; k++) {
      double chicc = Vij[k] * wla[k] * (n[(long) i * nd + k] - gij[k] * n[(long) j * nd + k]);
      W->chi_up[(long) i * nd + k] += chicc;
      W->chi_down[(long) j * nd + k] += chicc;
      W->Uji_down[(long) j * nd + k] += t * gij[k] * Vij[k];
    }
  }
}

/* addtoGamma (fillgamma.c:82-246); Psi already divided by chi. */
static void add_gamma(const NlteProblem *P, const ActiveSet *as, int ns, double wmu,
                      Work *W, double *Gamma)
{
  int nd = P->ndep, nl = P->nlevel;
  for (int k = 0; k < nd; k++) W->Ieff[k] = W->I[k] - W->Psi[k] * W->eta_atom[k];
  for (int m = 0; m < as->nact; m++) {
    int i = as->i[m], j = as->j[m];
    double t = twohnu3_of(P, as, m, ns);
    const double *Vij = W->Vij + (long) m * nd, *gij = W->gij + (long) m * nd;
    const double *wla = W->wla + (long) m * nd;
    double *Gij = Gamma + (long) (i * nl + j) * nd, *Gji = Gamma + (long) (j * nl + i) * nd;
    for (int k = 0; k < nd; k++) {
      double wlamu = Vij[k] * wla[k] * wmu;
      Gji[k] += W->Ieff[k] * wlamu;
      Gij[k] += (t + W->Ieff[k]) * gij[k] * wlamu;
    }
    for (int k = 0; k < nd; k++)
      Gij[k] -= W->chi_up[(long) i * nd + k] * W->Psi[k] * W->Uji_down[(long) j * nd + k] * wmu;
    for (int q = 0; q < as->nact; q++) {
      if (as->j[q] == i) {
        for (int k = 0; k < nd; k++)
          Gji[k] += W->chi_down[(long) j * nd + k] * W->Psi[k] * W->Uji_down[(long) i * nd + k] * wmu;
      }
    }
  }
}

/* addtoRates (fillgamma.c:375-461): R_ij += I V W wmu, R_ji += g (2 h nu^3 /
   c^2 + I) V W wmu, into rates [nline][2][ndep] followed by [ncont][2][ndep]. */
static void add_rates(const NlteProblem *P, const ActiveSet *as, int ns, double wmu,
                      const Work *W, double *rates)
{
  int nd = P->ndep;
  for (int m = 0; m < as->nact; m++) {
    double t = twohnu3_of(P, as, m, ns);
    long row = as->type[m] == 0 ? as->kr[m] : P->nline + as->kr[m];
    double *Rij = rates + 2 * row * nd, *Rji = Rij + nd;
    const double *Vij = W->Vij + (long) m * nd, *gij = W->gij + (long) m * nd;
    const double *wla = W->wla + (long) m * nd;
    for (int k = 0; k < nd; k++) {
      double wlamu = Vij[k] * wla[k] * wmu;
      Rij[k] += W->I[k] * wlamu;
      Rji[k] += gij[k] * (t + W->I[k]) * wlamu;
    }
  }
}

/* Formal() for one wavelength (formal.c:44-346).  J_new[ns] is replaced by
   the new mean intensity when update_J; Gamma accumulates when gamma != NULL;
   Iem[mu] receives the emergent intensity. */
static void formal_lambda(const NlteProblem *P, int ns, int nrays, const double *muz,
                          const double *wmu, double **phi, const double *wphi,
                          const double *n, const double *Jold, double *J_new, int update_J,
                          double *Gamma, Work *W, double *Iem, double *rates)
{
  int nd = P->ndep;
  ActiveSet as;
  active_set(P, ns, &as);
  const double *chi_c = P->chi_c + (long) ns * nd, *eta_c = P->eta_c + (long) ns * nd;
  const double *sca_c = P->sca_c + (long) ns * nd;
  double *chi_act = W->chi;  /* reused below */
  double lam = P->lambda[ns];
  double B0 = oracle_planck(P->T[nd - 2], lam), B1 = oracle_planck(P->T[nd - 1], lam);
  double *J = J_new + (long) ns * nd;
  for (int k = 0; k < nd; k++) W->Jdag[k] = Jold[(long) ns * nd + k];
  if (update_J) for (int k = 0; k < nd; k++) J[k] = 0.0;
  /* formal.c:92-101: a polarized active set or background, or a moving
     atmosphere with a line at this wavelength */
  int angle_dep = as.polarized || (P->bgline[ns] & 2) ||
                  (P->moving && (as.boundbound || (P->bgline[ns] & 1)));
  double *chi = (double *) malloc(nd * sizeof(double));
  if (angle_dep) {
    for (int mu = 0; mu < nrays; mu++) {
      double w = 0.5 * wmu[mu];
      for (int to_obs = 0; to_obs <= 1; to_obs++) {
        active_opacity(P, &as, ns, nrays, mu, to_obs, phi, wphi, n, W, chi_act);
        if (Gamma) add_coupling(P, &as, ns, n, W);
        for (int k = 0; k < nd; k++) {
          chi[k] = chi_act[k] + chi_c[k];
          W->S[k] = (W->eta_atom[k] + eta_c[k] + sca_c[k] * W->Jdag[k]) / chi[k];
        }
        oracle_scalar_bezier3(nd, P->height, 1.0 / muz[mu], chi, W->S, B0, B1, to_obs,
                              W->I, W->Psi);
        if (Gamma) {
          for (int k = 0; k < nd; k++) W->Psi[k] /= chi[k];
          add_gamma(P, &as, ns, w, W, Gamma);
        }
        if (update_J) for (int k = 0; k < nd; k++) J[k] += w * W->I[k];
        if (update_J && rates) add_rates(P, &as, ns, w, W, rates);
      }
      Iem[mu] = W->I[0];
    }
  } else {
    active_opacity(P, &as, ns, nrays, 0, 0, phi, wphi, n, W, chi_act);
    if (Gamma) add_coupling(P, &as, ns, n, W);
    for (int k = 0; k < nd; k++) {
      chi[k] = chi_act[k] + chi_c[k];
      W->S[k] = (W->eta_atom[k] + eta_c[k] + sca_c[k] * W->Jdag[k]) / chi[k];
    }
    for (int mu = 0; mu < nrays; mu++) {
      Iem[mu] = oracle_feautrier(nd, P->height, muz[mu], chi, W->S, B0, B1, W->I, W->Psi);
      if (Gamma) {
        for (int k = 0; k < nd; k++) W->Psi[k] /= chi[k];
        add_gamma(P, &as, ns, wmu[mu], W, Gamma);
      }
      if (update_J) for (int k = 0; k < nd; k++) J[k] += W->I[k] * wmu[mu];
      if (update_J && rates) add_rates(P, &as, ns, wmu[mu], W, rates);
    }
  }
  free(chi);
}

static void work_alloc(Work *W, int nd, int nl)
{
  W->Vij = calloc((long) NLTE_MAX_ACTIVE * nd, sizeof(double));
  W->gij = calloc((long) NLTE_MAX_ACTIVE * nd, sizeof(double));
  W->wla = calloc((long) NLTE_MAX_ACTIVE * nd, sizeof(double));
  W->chi_up = calloc((long) nl * nd, sizeof(double));
  W->chi_down = calloc((long) nl * nd, sizeof(double));
  W->Uji_down = calloc((long) nl * nd, sizeof(double));
  W->eta_atom = calloc(nd, sizeof(double));
  W->chi = calloc(nd, sizeof(double));
  W->S = calloc(nd, sizeof(double));
  W->I = calloc(nd, sizeof(double));
  W->Psi = calloc(nd, sizeof(double));
  W->Jdag = calloc(nd, sizeof(double));
  W->Ieff = calloc(nd, sizeof(double));
}

static void work_free(Work *W)
{
  free(W->Vij); free(W->gij); free(W->wla); free(W->chi_up); free(W->chi_down);
  free(W->Uji_down); free(W->eta_atom); free(W->chi); free(W->S); free(W->I);
  free(W->Psi); free(W->Jdag); free(W->Ieff);
}

static double **alloc_phi(const NlteProblem *P, int nrays)
{
  double **phi = malloc(sizeof(double *) * (P->nline > 0 ? P->nline : 1));
  for (int kr = 0; kr < P->nline; kr++) {
    int nl = (int) P->lines[(long) kr * NL_NREC + NL_NLAMBDA];
    phi[kr] = calloc((long) nl * 2 * nrays * P->ndep, sizeof(double));
  }
  return phi;
}

static void free_phi(const NlteProblem *P, double **phi)
{
  for (int kr = 0; kr < P->nline; kr++) free(phi[kr]);
  free(phi);
}

/* One pass over the spectrum: Gamma = C + radiative, J replaced, and, when
   rates is not NULL, the radiative rates of this pass (solveSpectrum,
   iterate.c:146-260, zeroes them first).  Gamma may be NULL (no operator). */
void oracle_nlte_spectrum_rates(const NlteProblem *P, const double *n, const double *Jold,
                                double *J_new, double *Gamma, double **phi,
                                const double *wphi, double *rates)
{
  int nd = P->ndep, nl = P->nlevel;
  Work W;
  work_alloc(&W, nd, nl);
  double Iem[64];
  if (Gamma) memcpy(Gamma, P->C, sizeof(double) * nl * nl * nd);
  if (rates) memset(rates, 0, sizeof(double) * 2 * (P->nline + P->ncont) * nd);
  for (int ns = 0; ns < P->nspect; ns++)
    formal_lambda(P, ns, P->nrays, P->muz, P->wmu, phi, wphi, n, Jold, J_new, 1, Gamma,
                  &W, Iem, rates);
  work_free(&W);
}

void oracle_nlte_spectrum(const NlteProblem *P, const double *n, const double *Jold,
                          double *J_new, double *Gamma, double **phi, const double *wphi)
{
  oracle_nlte_spectrum_rates(P, n, Jold, J_new, Gamma, phi, wphi, NULL);
}

/* statEquil (statequil.c:40-102) on n [nlevel][ndep] in place. */
int oracle_stat_equil(const NlteProblem *P, const double *Gamma, double *n)
{
  int nd = P->ndep, nl = P->nlevel, status = 0;
  double A[64], b[8];
  for (int k = 0; k < nd; k++) {
    int ie = 0;
    if (P->isum == -1) {
      double nmax = 0.0;
      for (int i = 0; i < nl; i++)
        if (n[(long) i * nd + k] > nmax) { nmax = n[(long) i * nd + k]; ie = i; }
    } else ie = P->isum;
    for (int i = 0; i < nl; i++)
      for (int j = 0; j < nl; j++) A[i * nl + j] = Gamma[(long) (i * nl + j) * nd + k];
    for (int i = 0; i < nl; i++) {
      double d = 0.0;
      A[i * nl + i] = 0.0;
      b[i] = 0.0;
      for (int j = 0; j < nl; j++) d += A[j * nl + i];
      A[i * nl + i] = -d;
    }
    b[ie] = P->ntotal[k];
    for (int j = 0; j < nl; j++) A[ie * nl + j] = 1.0;
    if (solve_linear_eq(nl, A, b)) status = -1;
    for (int i = 0; i < nl; i++) n[(long) i * nd + k] = b[i];
  }
  return status;
}

/* Ng (rh/accelerate.c:34-146) over the flattened populations. */
typedef struct {
  int N, Norder, Nperiod, Ndelay, count;
  double *prev;  /* [Norder+2][N] */
} Ng;

static void ng_init(Ng *g, int N, int delay, int order, int period, const double *sol)
{
  g->N = N; g->Norder = order; g->Nperiod = period;
  g->Ndelay = delay > order + 2 ? delay : order + 2;
  g->prev = calloc((long) (order + 2) * N, sizeof(double));
  memcpy(g->prev, sol, sizeof(double) * N);
  g->count = 1;
}

static int ng_accelerate(Ng *g, double *sol)
{
  int No = g->Norder, N = g->N;
  int i = g->count % (No + 2);
  memcpy(g->prev + (long) i * N, sol, sizeof(double) * N);
  g->count++;
  if (!(No > 0 && g->count >= g->Ndelay && !((g->count - g->Ndelay) % g->Nperiod)))
    return 0;
  double *Delta = malloc(sizeof(double) * (No + 1) * N);
  for (int q = 0; q <= No; q++) {
    int ip = (g->count - 1 - q) % (No + 2), ipp = (g->count - 2 - q) % (No + 2);
    for (int k = 0; k < N; k++)
      Delta[(long) q * N + k] = g->prev[(long) ip * N + k] - g->prev[(long) ipp * N + k];
  }
  double A[16] = {0}, b[4] = {0};
  for (int j = 0; j < No; j++) {
    for (int k = 0; k < N; k++) {
      double w = 1.0 / fabs(sol[k]);
      b[j] += w * Delta[k] * (Delta[k] - Delta[(long) (j + 1) * N + k]);
    }
    for (int q = 0; q < No; q++)
      for (int k = 0; k < N; k++) {
        double w = 1.0 / fabs(sol[k]);
        A[q * No + j] += w * (Delta[(long) (j + 1) * N + k] - Delta[k]) *
                         (Delta[(long) (q + 1) * N + k] - Delta[k]);
      }
  }
  solve_linear_eq(No, A, b);
  int i0 = (g->count - 1) % (No + 2);
  for (int q = 0; q < No; q++) {
    int ip = (g->count - 2 - q) % (No + 2);
    for (int k = 0; k < N; k++)
      sol[k] += b[q] * (g->prev[(long) ip * N + k] - g->prev[(long) i0 * N + k]);
  }
  memcpy(g->prev + (long) i0 * N, sol, sizeof(double) * N);
  free(Delta);
  return 1;
}

static double ng_maxchange(const Ng *g)
{
  if (g->count < 2) return 0.0;
  const double *old = g->prev + (long) ((g->count - 2) % (g->Norder + 2)) * g->N;
  const double *nw = g->prev + (long) ((g->count - 1) % (g->Norder + 2)) * g->N;
  double dmax = 0.0;
  for (int k = 0; k < g->N; k++)
    if (nw[k]) {
      double d = fabs((nw[k] - old[k]) / nw[k]);
      if (d > dmax) dmax = d;
    }
  return dmax;
}

/* Iterate (iterate.c:48-143): n (in/out) [nlevel][ndep], J (in/out)
   [nspect][ndep].  Returns the number of iterations; dpops[it] receives
   the convergence metric of each; rates (may be NULL) those of the last
   formal pass. */
int oracle_nlte_iterate_rates(const NlteProblem *P, double *n, double *J, double *dpops,
                              int *accelerated, double *rates)
{
  int nd = P->ndep, nl = P->nlevel;
  double **phi = alloc_phi(P, P->nrays);
  double *wphi = calloc((long) (P->nline > 0 ? P->nline : 1) * nd, sizeof(double));
  oracle_nlte_profiles(P, P->nrays, P->muz, P->wmu, phi, wphi);
  double *Gamma = malloc(sizeof(double) * nl * nl * nd);
  double *Jn = malloc(sizeof(double) * P->nspect * nd);
  Ng g;
  ng_init(&g, nl * nd, P->ng_delay, P->ng_order, P->ng_period, n);
  int niter = 1, done = 0;
  while (niter <= P->nmax_iter) {
    memcpy(Jn, J, sizeof(double) * P->nspect * nd);
    oracle_nlte_spectrum_rates(P, n, J, Jn, Gamma, phi, wphi, rates);
    memcpy(J, Jn, sizeof(double) * P->nspect * nd);
    oracle_stat_equil(P, Gamma, n);
    int acc = ng_accelerate(&g, n);
    double dp = ng_maxchange(&g);
    if (dpops) dpops[niter - 1] = dp;
    if (accelerated) accelerated[niter - 1] = acc;
    done = niter;
    if (dp < P->iter_limit) break;
    niter++;
  }
  free(g.prev); free(Gamma); free(Jn); free(wphi);
  free_phi(P, phi);
  return done;
}

int oracle_nlte_iterate(const NlteProblem *P, double *n, double *J, double *dpops,
                        int *accelerated)
{
  return oracle_nlte_iterate_rates(P, n, J, dpops, accelerated, NULL);
}

/* Emergent intensity at mu_out with the populations n and the fixed mean
   intensity J (pyrh_solveray.c:82-107: one ray, profiles recomputed,
   solveSpectrum without operator and without updating J). */
void oracle_nlte_emergent(const NlteProblem *P, double mu_out, const double *n,
                          const double *J, double *Iout)
{
  int nd = P->ndep;
  double muz[1] = {mu_out}, wmu[1] = {1.0};
  double **phi = alloc_phi(P, 1);
  double *wphi = calloc((long) (P->nline > 0 ? P->nline : 1) * nd, sizeof(double));
  oracle_nlte_profiles(P, 1, muz, wmu, phi, wphi);
  Work W;
  work_alloc(&W, nd, P->nlevel);
  double *Jdummy = malloc(sizeof(double) * P->nspect * nd);
  for (int ns = 0; ns < P->nspect; ns++) {
    double Iem[1];
    formal_lambda(P, ns, 1, muz, wmu, phi, wphi, n, J, Jdummy, 0, NULL, &W, Iem, NULL);
    Iout[ns] = Iem[0];
  }
  free(Jdummy);
  work_free(&W);
  free(wphi);
  free_phi(P, phi);
}
