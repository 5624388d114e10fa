/* rt_oracle.c -- CPU ORACLE (test infrastructure, never shipped or measured
 * as the product).  Plain-C, FP64 restatement of the reference's LTE
 * polarized synthesis hot path, used by tests/ to check the CUDA kernels and
 * by bench.py as the "port" CPU baseline.
 *
 * Parity pinned against the compiled reference (golden vectors in
 * tests/golden/, produced by tests/golden/make_golden.py from rhf1d()).
 *
 * Restated, in order of the data flow:
 *   humlicek_w      rh/voigt.c:381-419, rh/humlicek.c:28-118  (Humlicek 1982,
 *                   JQSRT 27, 437: four-region rational approximations of
 *                   W(z), z = a - i v)
 *   rlk_profile     rh/kurucz.c:729-827  (Doppler width, damping, Zeeman sums)
 *   rlk_opacity_at  rh/kurucz.c:511-724 and rh/background.c:469-546
 *   stokes_K        rh/stokesopac.c:28-87
 *   bezier3_coeffs  rh/bezier_aux.c:333-359
 *   cent_deriv      rh/bezier_aux.c:34-51 (Fritsch & Butland 1984)
 *   w3              rh/w3.c:44-63
 *   planck          rh/planck.c:38-63
 *   stokes_bezier3  rh/rhf1d/bezier_1D.c:52-300 (ray to the observer only:
 *                   the emergent Stokes vector does not depend on the other
 *                   direction, rh/rhf1d/formal.c:167-275)
 *   scalar_bezier3  rh/rhf1d/bezier_1D.c:306-541 (same ray; used when no
 *                   polarizable line covers the wavelength, formal.c:94-95,
 *                   and the wavelength is angle dependent, formal.c:96-101)
 *   feautrier       rh/rhf1d/feautrier.c:56-202 (wavelengths that are not
 *                   angle dependent: no line in window, or in a static
 *                   atmosphere no polarizable one, formal.c:284-304)
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "rt_oracle.h"
#include "nlte_oracle.h"

/* Physical constants as the reference defines them (rh/constant.h:28-68). */
#define CLIGHT      2.99792458E+08
#define HPLANCK     6.6260755E-34
#define KBOLTZMANN  1.380658E-23
#define AMU         1.6605402E-27
#define M_ELECTRON  9.1093897E-31
#define Q_ELECTRON  1.60217733E-19
#define NM_TO_M     1.0E-09
#define PI          3.14159265358979
#define SQRTPI      1.77245385090551
#define LARMOR      ((Q_ELECTRON / (4.0 * PI * M_ELECTRON)) * NM_TO_M)
#define Q_WING      20.0
#define MAX_GAUSS_DOPPLER 7.0
#define PLANCK_MAX_EXPONENT 150.0

/* ------------------------------------------------------------- Voigt -- */

typedef struct { double r, i; } cplx;

static inline cplx c_make(double r, double i) { cplx z = {r, i}; return z; }
static inline cplx c_add(cplx a, cplx b) { return c_make(a.r + b.r, a.i + b.i); }
static inline cplx c_addr(cplx a, double x) { return c_make(a.r + x, a.i); }
static inline cplx c_mul(cplx a, cplx b)
{ return c_make(a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r); }
static inline cplx c_scale(double s, cplx a) { return c_make(s * a.r, s * a.i); }
static inline cplx c_div(cplx a, cplx b)
{
  double d = b.r * b.r + b.i * b.i;
  return c_make((a.r * b.r + a.i * b.i) / d, (a.i * b.r - a.r * b.i) / d);
}
static inline cplx c_exp(cplx a)
{ double e = exp(a.r); return c_make(e * cos(a.i), e * sin(a.i)); }

/* Humlicek (1982) W4 rational approximations, coefficients as published. */
static const double HW3_A[5] = {0.5642236, 3.778987, 11.96482, 20.20933, 16.4955};
static const double HW3_B[5] = {6.699398, 21.69274, 39.27121, 38.82363, 16.4955};
static const double HW4_A[7] = {0.56419, 1.320522, 35.7668, 219.031, 1540.787,
                                3321.99, 36183.31};
static const double HW4_B[7] = {1.841439, 61.57037, 364.2191, 2186.181,
                                9022.228, 24322.84, 32066.6};

void oracle_humlicek(double a, double v, double *H, double *F)
{
  cplx t = c_make(a, -v), W;
  double s = fabs(v) + a;

  if (s >= 15.0) {                                   /* region I  */
    W = c_div(c_scale(0.5641896, t), c_addr(c_mul(t, t), 0.5));
  } else if (s >= 5.5) {                             /* region II */
    cplx u = c_mul(t, t);
    cplx num = c_mul(t, c_addr(c_scale(0.5641896, u), 1.410474));
    cplx den = c_addr(c_mul(u, c_addr(u, 3.0)), 0.75);
    W = c_div(num, den);
  } else if (a >= 0.195 * fabs(v) - 0.176) {         /* region III */
    cplx num = c_make(HW3_A[0], 0.0), den = c_addr(t, HW3_B[0]);
    for (int n = 1; n < 5; n++) {
      num = c_addr(c_mul(num, t), HW3_A[n]);
      den = c_addr(c_mul(den, t), HW3_B[n]);
    }
    W = c_div(num, den);
  } else {                                           /* region IV */
    cplx u = c_mul(t, c_scale(-1.0, t));
    cplx num = c_make(HW4_A[0], 0.0), den = c_addr(u, HW4_B[0]);
    for (int n = 1; n < 7; n++) {
      num = c_addr(c_mul(u, num), HW4_A[n]);
      den = c_addr(c_mul(u, den), HW4_B[n]);
    }
    cplx e = c_exp(c_scale(-1.0, u));
    cplx r = c_div(c_mul(t, num), den);
    W = c_make(e.r - r.r, e.i - r.i);
  }
  *H = W.r;
  if (F) *F = W.i;
}

/* --------------------------------------------------------- line profile -- */

/* Returns phi (Stokes I profile, normalised) and fills phiQUV / psiQUV for a
   polarizable line; rh/kurucz.c:729-827 with to_obs = TRUE. */
static double rlk_profile(const double *L, const double *zq, const double *zs,
                          const double *zw, int ncomp, const OracleDepth *d,
                          double lambda, int moving, double muz,
                          double *phiQUV, double *psiQUV, int magneto_optical)
{
  double vtherm = 2.0 * KBOLTZMANN / (AMU * L[RLK_WEIGHT]);
  double vbroad = sqrt(vtherm * d->T + d->vturb * d->vturb);
  double v = (lambda / L[RLK_LAMBDA0] - 1.0) * CLIGHT / vbroad;
  if (moving) v += muz * d->vel / vbroad;
  double sv = 1.0 / (SQRTPI * vbroad);

  phiQUV[0] = phiQUV[1] = phiQUV[2] = 0.0;
  psiQUV[0] = psiQUV[1] = psiQUV[2] = 0.0;

  if (L[RLK_GRAD] == 0.0) {
    double phi = (fabs(v) <= MAX_GAUSS_DOPPLER) ? exp(-v * v) : 0.0;
    return phi * sv;
  }
  double GvdW;
  int vdw = (int) L[RLK_VDWAALS];
  if (vdw == RLK_VDW_UNSOLD)       GvdW = L[RLK_CROSS] * pow(d->T, 0.3);
  else if (vdw == RLK_VDW_BARKLEM) GvdW = L[RLK_CROSS] * pow(d->T, (1.0 - L[RLK_ALPHA]) / 2.0);
  else                             GvdW = L[RLK_GVDWAALS];
  double adamp = (L[RLK_GRAD] + L[RLK_GSTARK] * d->ne + GvdW * (d->nHtot - d->np)) *
                 (L[RLK_LAMBDA0] * NM_TO_M) / (4.0 * PI * vbroad);

  if (!(int) L[RLK_POLARIZABLE]) {
    /* unpolarizable line: Armstrong's Voigt function, no Zeeman splitting
       (kurucz.c:824; the restatement of rh/voigt.c:126-243 is in
       nlte_oracle.c) */
    return oracle_voigt_armstrong(adamp, v) * sv;
  }
  double sin2g = 1.0 - d->cos_gamma * d->cos_gamma;
  double vB = (LARMOR * L[RLK_LAMBDA0]) * d->B / vbroad;
  double phs[3] = {0, 0, 0}, pss[3] = {0, 0, 0};   /* q = -1, 0, +1 */
  for (int c = 0; c < ncomp; c++) {
    double H, F;
    oracle_humlicek(adamp, v - zs[c] * vB, &H, &F);
    int q = (int) zq[c];
    phs[q + 1] += zw[c] * H;
    pss[q + 1] += zw[c] * F;
  }
  double phi_sigma = phs[2] + phs[0];
  double phi_delta = 0.5 * phs[1] - 0.25 * phi_sigma;
  double phi = (phi_delta * sin2g + 0.5 * phi_sigma) * sv;
  phiQUV[0] = phi_delta * sin2g * d->cos_2chi * sv;
  phiQUV[1] = phi_delta * sin2g * d->sin_2chi * sv;
  phiQUV[2] = 0.5 * (phs[2] - phs[0]) * d->cos_gamma * sv;
  if (magneto_optical) {
    double psi_sigma = pss[2] + pss[0];
    double psi_delta = 0.5 * pss[1] - 0.25 * psi_sigma;
    psiQUV[0] = psi_delta * sin2g * d->cos_2chi * sv;
    psiQUV[1] = psi_delta * sin2g * d->sin_2chi * sv;
    psiQUV[2] = 0.5 * (pss[2] - pss[0]) * d->cos_gamma * sv;
  }
  return phi;
}

/* Total LTE background record at one wavelength and depth:
   chi[4] (I,Q,U,V), eta[4], chip[3] (Q',U',V').  Returns flags
   bit0 = hasline, bit1 = ispolarized (rh/kurucz.c:533-724,
   rh/background.c:469-546; passive model-atom lines are not included). */
static int rlk_opacity_at(const OracleAtmos *A, const OracleLines *LN,
                          int k, double lambda, double *chi, double *eta,
                          double *chip)
{
  const double hc = HPLANCK * CLIGHT, hc_4PI = hc / (4.0 * PI);
  double dlamb_char = lambda * Q_WING * (LN->vmicro_char / CLIGHT);
  int flags = 0;
  double lc[4] = {0, 0, 0, 0}, le[4] = {0, 0, 0, 0}, lp[3] = {0, 0, 0};
  OracleDepth d;
  d.T = A->T[k]; d.ne = A->ne[k]; d.nHtot = A->nHtot[k]; d.np = A->np[k];
  d.vturb = A->vturb[k]; d.vel = A->vel[k]; d.B = A->B[k];
  double cg = cos(A->gamma_B[k]);
  if (A->muz == 1.0) {
    d.cos_gamma = cg;
    d.cos_2chi = cos(2.0 * A->chi_B[k]);
    d.sin_2chi = sin(2.0 * A->chi_B[k]);
  } else {                                  /* rh/rhf1d/project.c:60-75 */
    double mux = sqrt(1.0 - A->muz * A->muz), muy = 0.0;
    double csc = 1.0 / sqrt(1.0 - A->muz * A->muz);
    double sg = sin(A->gamma_B[k]);
    double bx = sg * cos(A->chi_B[k]), by = sg * sin(A->chi_B[k]), bz = cg;
    double b3 = mux * bx + muy * by + A->muz * bz;
    double b1 = csc * (bz - A->muz * b3);
    double b2 = csc * (muy * bx - mux * by);
    d.cos_gamma = b3;
    d.cos_2chi = (b1 * b1 - b2 * b2) / (1.0 - b3 * b3);
    d.sin_2chi = 2.0 * b1 * b2 / (1.0 - b3 * b3);
  }

  if (LN->nline > 0 &&
      !(lambda < LN->c[0 * RLK_NCONST + RLK_LAMBDA0] - dlamb_char ||
        lambda > LN->c[(LN->nline - 1) * RLK_NCONST + RLK_LAMBDA0] + dlamb_char)) {
    for (int n = 0; n < LN->nline; n++) {
      const double *L = LN->c + (long) n * RLK_NCONST;
      if (fabs(L[RLK_LAMBDA0] - lambda) > dlamb_char) continue;
      if (!(int) L[RLK_CONTRIBUTES]) continue;
      double hc_la = hc / (L[RLK_LAMBDA0] * NM_TO_M);
      double Bijhc_4PI = hc_4PI * L[RLK_BIJ] * L[RLK_ISOFRAC] * L[RLK_HFSFRAC] * L[RLK_GI];
      double twohnu3_c2 = L[RLK_AJI] / L[RLK_BJI];
      int pol = (int) L[RLK_POLARIZABLE];
      flags |= 1;
      if (pol) flags |= 2;
      const double *zq = LN->zeeman + ((long) n * 3 + 0) * LN->maxcomp;
      const double *zs = LN->zeeman + ((long) n * 3 + 1) * LN->maxcomp;
      const double *zw = LN->zeeman + ((long) n * 3 + 2) * LN->maxcomp;
      double pq[3], ps[3];
      double phi = rlk_profile(L, zq, zs, zw, pol ? LN->ncomp[n] : 0, &d,
                               lambda, LN->moving, A->muz, pq, ps,
                               LN->magneto_optical);
      if (phi) {
        double kT = 1.0 / (KBOLTZMANN * d.T);
        double nstage = A->line_pops[((long) n * 2 + 0) * A->ndep + k];
        double pf = A->line_pops[((long) n * 2 + 1) * A->ndep + k];
        double ni_gi = nstage * exp(-L[RLK_EI] * kT - pf);
        double nj_gj = ni_gi * exp(-hc_la * kT);
        double chi_l = Bijhc_4PI * (ni_gi - nj_gj);
        double eta_l = Bijhc_4PI * twohnu3_c2 * nj_gj;
        lc[0] += chi_l * phi;
        le[0] += eta_l * phi;
        if (pol && L[RLK_GRAD] != 0.0) {
          for (int s = 0; s < 3; s++) {
            lc[s + 1] += chi_l * pq[s];
            le[s + 1] += eta_l * pq[s];
          }
          if (LN->magneto_optical)
            for (int s = 0; s < 3; s++) lp[s] += chi_l * ps[s];
        }
      }
    }
  }
  for (int s = 0; s < 4; s++) { chi[s] = lc[s]; eta[s] = le[s]; }
  for (int s = 0; s < 3; s++) chip[s] = lp[s];
  return flags;
}

/* ------------------------------------------------------ solver helpers -- */

static double cent_deriv(double dsup, double dsdn, double up, double c, double dn)
{
  double fim1 = (c - up) / dsup, fi = (dn - c) / dsdn;
  if (fim1 * fi > 0.0) {
    double alpha = 0.333333333333333333333333 * (1.0 + dsdn / (dsdn + dsup));
    return (fim1 * fi) / ((1.0 - alpha) * fim1 + alpha * fi);
  }
  return 0.0;
}

static void bezier3_coeffs(double dt, double *alpha, double *beta, double *gamma,
                           double *theta, double *eps)
{
  double dt2 = dt * dt, dt3 = dt2 * dt;
  if (dt >= 5.e-2) {
    double e = exp(-dt);
    *eps = e;
    *alpha = (-6.0 + 6.0 * dt - 3.0 * dt2 + dt3 + 6.0 * e) / dt3;
    double r3 = 1.0 / dt3;
    *beta = (6.0 + (-6.0 - dt * (6.0 + dt * (3.0 + dt))) * e) * r3;
    *gamma = 3.0 * (6.0 + (-4.0 + dt) * dt - 2.0 * (3.0 + dt) * e) * r3;
    *theta = 3.0 * (e * (6.0 + dt2 + 4.0 * dt) + 2.0 * dt - 6.0) * r3;
  } else {
    double dt4 = dt2 * dt2;
    *eps = 1.0 - dt + 0.5 * dt2 - dt3 / 6.0 + dt4 / 24.0;
    *alpha = 0.25 * dt - 0.05 * dt2 + dt3 / 120.0 - dt4 / 840.0;
    *beta = 0.25 * dt - 0.20 * dt2 + dt3 / 12.0 - dt4 / 42.0;
    *gamma = 0.25 * dt - 0.10 * dt2 + dt3 * 0.025 - dt4 / 210.0;
    *theta = 0.25 * dt - 0.15 * dt2 + dt3 * 0.05 - dt4 / 84.0;
  }
}

static void w3(double dtau, double *w)
{
  if (dtau < 5.0E-4) {
    w[0] = dtau * (1.0 - 0.5 * dtau);
    double d2 = dtau * dtau;
    w[1] = d2 * (0.5 - dtau / 3.0);
    w[2] = d2 * dtau * (1.0 / 3.0 - 0.25 * dtau);
  } else if (dtau > 50.0) {
    w[1] = w[0] = 1.0;
    w[2] = 2.0;
  } else {
    double e = exp(-dtau);
    w[0] = 1.0 - e;
    w[1] = w[0] - dtau * e;
    w[2] = 2.0 * w[1] - dtau * dtau * e;
  }
}

double oracle_planck(double T, double lambda)
{
  double hc_kla = (HPLANCK * CLIGHT) / (KBOLTZMANN * NM_TO_M * lambda);
  double l = NM_TO_M * lambda;
  double twohnu3_c2 = (2.0 * HPLANCK * CLIGHT) / (l * l * l);
  double x = hc_kla / T;
  return (x <= PLANCK_MAX_EXPONENT) ? twohnu3_c2 / (exp(x) - 1.0) : 0.0;
}

/* K' of rh/stokesopac.c:28-87 from the total record at one depth. */
static void stokes_K(const double *chi4, const double *chip3, int mo, double K[4][4])
{
  memset(K, 0, 16 * sizeof(double));
  K[0][1] = chi4[1]; K[0][2] = chi4[2]; K[0][3] = chi4[3];
  if (mo) { K[1][2] = chip3[2]; K[1][3] = chip3[1]; K[2][3] = chip3[0]; }
  for (int j = 0; j < 3; j++)
    for (int i = j + 1; i < 4; i++) { K[j][i] /= chi4[0]; K[i][j] = K[j][i]; }
  if (mo) { K[1][3] *= -1.0; K[2][1] *= -1.0; K[3][2] *= -1.0; }
}

/* 4x4 inverse by cofactors, in float (the reference inverts Md in single
   precision, rh/rhf1d/bezier_1D.c:75,244) or in double. */
static void inv4_float(const double M[4][4], double R[4][4])
{
  float m[16], inv[16];
  for (int i = 0; i < 16; i++) m[i] = (float) M[i / 4][i % 4];
  inv[0] = m[5]*m[10]*m[15] - m[5]*m[11]*m[14] - m[9]*m[6]*m[15] + m[9]*m[7]*m[14] + m[13]*m[6]*m[11] - m[13]*m[7]*m[10];
  inv[4] = -m[4]*m[10]*m[15] + m[4]*m[11]*m[14] + m[8]*m[6]*m[15] - m[8]*m[7]*m[14] - m[12]*m[6]*m[11] + m[12]*m[7]*m[10];
  inv[8] = m[4]*m[9]*m[15] - m[4]*m[11]*m[13] - m[8]*m[5]*m[15] + m[8]*m[7]*m[13] + m[12]*m[5]*m[11] - m[12]*m[7]*m[9];
  inv[12] = -m[4]*m[9]*m[14] + m[4]*m[10]*m[13] + m[8]*m[5]*m[14] - m[8]*m[6]*m[13] - m[12]*m[5]*m[10] + m[12]*m[6]*m[9];
  inv[1] = -m[1]*m[10]*m[15] + m[1]*m[11]*m[14] + m[9]*m[2]*m[15] - m[9]*m[3]*m[14] - m[13]*m[2]*m[11] + m[13]*m[3]*m[10];
  inv[5] = m[0]*m[10]*m[15] - m[0]*m[11]*m[14] - m[8]*m[2]*m[15] + m[8]*m[3]*m[14] + m[12]*m[2]*m[11] - m[12]*m[3]*m[10];
  inv[9] = -m[0]*m[9]*m[15] + m[0]*m[11]*m[13] + m[8]*m[1]*m[15] - m[8]*m[3]*m[13] - m[12]*m[1]*m[11] + m[12]*m[3]*m[9];
  inv[13] = m[0]*m[9]*m[14] - m[0]*m[10]*m[13] - m[8]*m[1]*m[14] + m[8]*m[2]*m[13] + m[12]*m[1]*m[10] - m[12]*m[2]*m[9];
  inv[2] = m[1]*m[6]*m[15] - m[1]*m[7]*m[14] - m[5]*m[2]*m[15] + m[5]*m[3]*m[14] + m[13]*m[2]*m[7] - m[13]*m[3]*m[6];
  inv[6] = -m[0]*m[6]*m[15] + m[0]*m[7]*m[14] + m[4]*m[2]*m[15] - m[4]*m[3]*m[14] - m[12]*m[2]*m[7] + m[12]*m[3]*m[6];
  inv[10] = m[0]*m[5]*m[15] - m[0]*m[7]*m[13] - m[4]*m[1]*m[15] + m[4]*m[3]*m[13] + m[12]*m[1]*m[7] - m[12]*m[3]*m[5];
  inv[14] = -m[0]*m[5]*m[14] + m[0]*m[6]*m[13] + m[4]*m[1]*m[14] - m[4]*m[2]*m[13] - m[12]*m[1]*m[6] + m[12]*m[2]*m[5];
  inv[3] = -m[1]*m[6]*m[11] + m[1]*m[7]*m[10] + m[5]*m[2]*m[11] - m[5]*m[3]*m[10] - m[9]*m[2]*m[7] + m[9]*m[3]*m[6];
  inv[7] = m[0]*m[6]*m[11] - m[0]*m[7]*m[10] - m[4]*m[2]*m[11] + m[4]*m[3]*m[10] + m[8]*m[2]*m[7] - m[8]*m[3]*m[6];
  inv[11] = -m[0]*m[5]*m[11] + m[0]*m[7]*m[9] + m[4]*m[1]*m[11] - m[4]*m[3]*m[9] - m[8]*m[1]*m[7] + m[8]*m[3]*m[5];
  inv[15] = m[0]*m[5]*m[10] - m[0]*m[6]*m[9] - m[4]*m[1]*m[10] + m[4]*m[2]*m[9] + m[8]*m[1]*m[6] - m[8]*m[2]*m[5];
  float det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
  float rdet = 1.0f / det;
  for (int i = 0; i < 16; i++) R[i / 4][i % 4] = (double) (inv[i] * rdet);
}

static void inv4_double(const double M[4][4], double R[4][4])
{
  /* Gauss-Jordan with partial pivoting. */
  double a[4][8];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 8; j++) a[i][j] = (j < 4) ? M[i][j] : (j - 4 == i);
  for (int c = 0; c < 4; c++) {
    int p = c;
    for (int r = c + 1; r < 4; r++) if (fabs(a[r][c]) > fabs(a[p][c])) p = r;
    if (p != c) for (int j = 0; j < 8; j++) { double t = a[c][j]; a[c][j] = a[p][j]; a[p][j] = t; }
    double inv = 1.0 / a[c][c];
    for (int j = 0; j < 8; j++) a[c][j] *= inv;
    for (int r = 0; r < 4; r++) if (r != c) {
      double f = a[r][c];
      for (int j = 0; j < 8; j++) a[r][j] -= f * a[c][j];
    }
  }
  for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) R[i][j] = a[i][j + 4];
}

/* ------------------------------------------------------ formal solvers -- */

/* DELO-Bezier3 along the ray to the observer (k = Ndep-1 -> 0).
   chi[k]: total opacity; S[s][k]: Stokes source vector; K[k]: 4x4.
   Returns the emergent Stokes vector I0[4]. */
static void stokes_bezier3(int nd, const double *z, double imu, const double *chi,
                           double (*S)[4], double (*K)[4][4], double Bbot0,
                           double Bbot1, int md_float, double I0[4])
{
  const int dk = -1, k_start = nd - 1, k_end = 0;
  double Iup[4], Inew[4];
  double dtau_uw = 0.5 * imu * (chi[k_start] + chi[k_start + dk]) *
                   fabs(z[k_start] - z[k_start + dk]);
  /* THERMALIZED bottom boundary: Bnu[0] = B(T[Ndep-2]), Bnu[1] = B(T[Ndep-1]) */
  Iup[0] = Bbot1 - (Bbot0 - Bbot1) / dtau_uw;
  Iup[1] = Iup[2] = Iup[3] = 0.0;

  int k = k_start + dk;
  double dsup = fabs(z[k] - z[k - dk]) * imu;
  double dsdn = fabs(z[k + dk] - z[k]) * imu;
  double dchi_up = (chi[k] - chi[k - dk]) / dsup;
  double dchi_c = cent_deriv(dsup, dsdn, chi[k - dk], chi[k], chi[k + dk]);
  double c2 = fmax(chi[k] - (dsup / 3.0) * dchi_c, 0.0);
  double c1 = fmax(chi[k - dk] + (dsup / 3.0) * dchi_up, 0.0);
  dtau_uw = 0.25 * dsup * (chi[k] + chi[k - dk] + c1 + c2);

  double Ku[4][4], K0[4][4], Kd[4][4], dKu[4][4], dK0[4][4];
  double Su[4], S0[4], Sd[4], dSu[4], dS0[4];
  memcpy(Ku, K[k_start], sizeof(Ku));
  memcpy(K0, K[k_start + dk], sizeof(K0));
  memcpy(Su, S[k_start], sizeof(Su));
  memcpy(S0, S[k_start + dk], sizeof(S0));
  for (int n = 0; n < 4; n++) {
    dSu[n] = (S0[n] - Su[n]) / dtau_uw;
    for (int m = 0; m < 4; m++) dKu[n][m] = (K0[n][m] - Ku[n][m]) / dtau_uw;
  }

  for (k = k_start + dk; k != k_end; k += dk) {
    dsdn = fabs(z[k + dk] - z[k]) * imu;
    double dchi_dn;
    if (abs(k - k_end) > 1) {
      double dsdn2 = fabs(z[k + 2 * dk] - z[k + dk]) * imu;
      dchi_dn = cent_deriv(dsdn, dsdn2, chi[k], chi[k + dk], chi[k + 2 * dk]);
    } else
      dchi_dn = (chi[k + dk] - chi[k]) / dsdn;
    c2 = fmax(chi[k] + (dsdn / 3.0) * dchi_c, 0.0);
    c1 = fmax(chi[k + dk] - (dsdn / 3.0) * dchi_dn, 0.0);
    double dtau_dw = 0.25 * dsdn * (chi[k] + chi[k + dk] + c1 + c2);
    double dt = dtau_uw, dt03 = dt / 3.0;
    double alpha, beta, gamma, theta, eps;
    bezier3_coeffs(dt, &alpha, &beta, &gamma, &theta, &eps);

    memcpy(Kd, K[k + dk], sizeof(Kd));
    memcpy(Sd, S[k + dk], sizeof(Sd));
    for (int j = 0; j < 4; j++)
      for (int i = 0; i < 4; i++)
        dK0[j][i] = cent_deriv(dtau_uw, dtau_dw, Ku[j][i], K0[j][i], Kd[j][i]);
    for (int i = 0; i < 4; i++)
      dS0[i] = cent_deriv(dtau_uw, dtau_dw, Su[i], S0[i], Sd[i]);

    /* Ku.Ku and K0.K0; the reference's m4m forms c[j][i] = sum_k a[k][i] b[j][k]
       (rh/bezier_aux.c:88-99), i.e. (B A)[j][i], equal to A.A for A = B. */
    double KuKu[4][4], K0K0[4][4];
    for (int j = 0; j < 4; j++)
      for (int i = 0; i < 4; i++) {
        double s1 = 0.0, s2 = 0.0;
        for (int q = 0; q < 4; q++) {
          s1 += Ku[q][i] * Ku[j][q];
          s2 += K0[q][i] * K0[j][q];
        }
        KuKu[j][i] = s1; K0K0[j][i] = s2;
      }
    double Md[4][4], Ma[4][4], Mb[4][4], Mc[4][4];
    for (int j = 0; j < 4; j++)
      for (int i = 0; i < 4; i++) {
        double id = (i == j) ? 1.0 : 0.0;
        Md[j][i] = id + alpha * K0[j][i] - gamma *
                   -(dt03 * (K0K0[j][i] + dK0[j][i] + K0[j][i]) + K0[j][i]);
        Ma[j][i] = eps * id - beta * Ku[j][i] + theta *
                   (dt03 * (KuKu[j][i] + dKu[j][i] + Ku[j][i]) - Ku[j][i]);
        Mb[j][i] = beta * id + theta * (id - dt03 * Ku[j][i]);
        Mc[j][i] = alpha * id + gamma * (id + dt03 * K0[j][i]);
      }
    double V0[4];
    for (int i = 0; i < 4; i++) {
      double s = 0.0;
      for (int j = 0; j < 4; j++)
        s += Ma[i][j] * Iup[j] + Mb[i][j] * Su[j] + Mc[i][j] * S0[j];
      V0[i] = s + dt03 * (gamma * dS0[i] - theta * dSu[i]);
    }
    double R[4][4];
    if (md_float) inv4_float(Md, R); else inv4_double(Md, R);
    for (int i = 0; i < 4; i++) {
      double s = 0.0;
      for (int q = 0; q < 4; q++) s += R[i][q] * V0[q];
      Inew[i] = s;
    }
    memcpy(Iup, Inew, sizeof(Iup));
    memcpy(Su, S0, sizeof(Su)); memcpy(S0, Sd, sizeof(S0)); memcpy(dSu, dS0, sizeof(dSu));
    memcpy(Ku, K0, sizeof(Ku)); memcpy(K0, Kd, sizeof(K0)); memcpy(dKu, dK0, sizeof(dKu));
    dtau_uw = dtau_dw;
    dsup = dsdn;
    dchi_up = dchi_c;
    dchi_c = dchi_dn;
  }
  /* Linear last interval (rh/rhf1d/bezier_1D.c:266-299). */
  k = k_end;
  dtau_uw = 0.5 * imu * (chi[k] + chi[k - dk]) * fabs(z[k] - z[k - dk]);
  double w[3];
  w3(dtau_uw, w);
  double V0[4], A[4][4], Md[4][4], R[4][4];
  for (int n = 0; n < 4; n++) V0[n] = w[0] * S[k][n] + w[1] * -dSu[n];
  for (int n = 0; n < 4; n++) {
    for (int m = 0; m < 4; m++) {
      A[n][m] = -w[1] / dtau_uw * Ku[n][m];
      Md[n][m] = (w[0] - w[1] / dtau_uw) * K0[n][m];
    }
    A[n][n] = 1.0 - w[0];
    Md[n][n] = 1.0;
  }
  for (int n = 0; n < 4; n++)
    for (int m = 0; m < 4; m++) V0[n] += A[n][m] * Iup[m];
  if (md_float) inv4_float(Md, R); else inv4_double(Md, R);
  for (int i = 0; i < 4; i++) {
    double s = 0.0;
    for (int q = 0; q < 4; q++) s += R[i][q] * V0[q];
    I0[i] = s;
  }
}

/* Scalar Bezier3 along the ray to the observer; rh/rhf1d/bezier_1D.c:306-541.
   Optionally returns the diagonal operator Psi (not divided by chi). */
double oracle_scalar_bezier3(int nd, const double *z, double imu,
                             const double *chi, const double *S,
                             double Bbot0, double Bbot1, int to_obs,
                             double *Iout, double *Psi)
{
  int dk, k_start, k_end;
  if (to_obs) { dk = -1; k_start = nd - 1; k_end = 0; }
  else        { dk = 1;  k_start = 0; k_end = nd - 1; }
  double dtau_uw = 0.5 * imu * (chi[k_start] + chi[k_start + dk]) *
                   fabs(z[k_start] - z[k_start + dk]);
  double I_upw = to_obs ? Bbot1 - (Bbot0 - Bbot1) / dtau_uw : 0.0;
  if (Iout) Iout[k_start] = I_upw;
  if (Psi) Psi[k_start] = 0.0;
  int k = k_start + dk;
  double dsup = fabs(z[k] - z[k - dk]) * imu;
  double dsdn = fabs(z[k + dk] - z[k]) * imu;
  double dchi_up = (chi[k] - chi[k - dk]) / dsup;
  double dchi_c = cent_deriv(dsup, dsdn, chi[k - dk], chi[k], chi[k + dk]);
  double c1 = fmax(chi[k] - (dsup / 3.0) * dchi_c, 0.0);
  double c2 = fmax(chi[k - dk] + (dsup / 3.0) * dchi_up, 0.0);
  dtau_uw = dsup * (chi[k] + chi[k - dk] + c1 + c2) * 0.25;
  double dS_up = (S[k] - S[k - dk]) / dtau_uw;
  double dchi_dn = 0.0, dtau_dw = 0.0, dS_c = 0.0, Ik = I_upw;

  for (k = k_start + dk; k != k_end + dk; k += dk) {
    if (k != k_end) {
      dsdn = fabs(z[k + dk] - z[k]) * imu;
      if (abs(k - k_end) > 1) {
        double dsdn2 = fabs(z[k + 2 * dk] - z[k + dk]) * imu;
        dchi_dn = cent_deriv(dsdn, dsdn2, chi[k], chi[k + dk], chi[k + 2 * dk]);
      } else
        dchi_dn = (chi[k + dk] - chi[k]) / dsdn;
      c1 = fmax(chi[k] + (dsdn / 3.0) * dchi_c, 0.0);
      c2 = fmax(chi[k + dk] - (dsdn / 3.0) * dchi_dn, 0.0);
      dtau_dw = dsdn * (chi[k] + chi[k + dk] + c1 + c2) * 0.25;
      double dt03 = dtau_uw / 3.0;
      double alpha, beta, gamma, theta, eps;
      bezier3_coeffs(dtau_uw, &alpha, &beta, &gamma, &theta, &eps);
      dS_c = cent_deriv(dtau_uw, dtau_dw, S[k - dk], S[k], S[k + dk]);
      c1 = fmax(S[k] - dt03 * dS_c, 0.0);
      c2 = fmax(S[k - dk] + dt03 * dS_up, 0.0);
      Ik = I_upw * eps + alpha * S[k] + beta * S[k - dk] + gamma * c1 + theta * c2;
      if (Psi) Psi[k] = alpha + gamma;
    } else {
      dtau_uw = 0.5 * imu * (chi[k] + chi[k - dk]) * fabs(z[k] - z[k - dk]);
      double dS_uw = -(S[k] - S[k - dk]) / dtau_uw;
      double w[3];
      w3(dtau_uw, w);
      Ik = (1.0 - w[0]) * I_upw + w[0] * S[k] + w[1] * dS_uw;
      if (Psi) Psi[k] = w[0] - w[1] / dtau_uw;
    }
    if (Iout) Iout[k] = Ik;
    I_upw = Ik;
    dsup = dsdn;
    dchi_up = dchi_c;
    dchi_c = dchi_dn;
    dtau_uw = dtau_dw;
    dS_up = dS_c;
  }
  return Ik;
}

/* Second-order Feautrier solution for the ray mu with a ZERO top and a
   THERMALIZED bottom boundary; rh/rhf1d/feautrier.c:56-202 (STANDARD
   order).  Used for wavelengths without any line, where the reference's
   Formal() takes the angle-independent branch (rh/rhf1d/formal.c:285-310).
   Returns the emergent intensity; P and Psi (optional) receive the
   symmetric average and the diagonal operator. */
double oracle_feautrier(int nd, const double *z, double muz, const double *chi,
                        const double *S, double Bbot0, double Bbot1,
                        double *P, double *Psi)
{
  double *dtau = (double *) malloc(nd * sizeof(double));
  double *abc = (double *) malloc(nd * sizeof(double));
  double *A1 = (double *) malloc(nd * sizeof(double));
  double *C1 = (double *) malloc(nd * sizeof(double));
  double *F = (double *) malloc(nd * sizeof(double));
  double *G = (double *) malloc(nd * sizeof(double));
  double *zt = (double *) malloc(nd * sizeof(double));
  double *St = (double *) malloc(nd * sizeof(double));
  double *Pl = P ? P : (double *) malloc(nd * sizeof(double));
  double zmu = 0.5 / muz;
  for (int k = 0; k < nd - 1; k++)
    dtau[k] = zmu * (chi[k] + chi[k + 1]) * (z[k] - z[k + 1]);
  /* top: ZERO (r0 = h0 = 0, f0 = 1) */
  abc[0] = 1.0 + 2.0 / dtau[0];
  C1[0] = 2.0 / (dtau[0] * dtau[0]);
  St[0] = S[0];
  /* bottom: THERMALIZED (rN = 0, fN = 1) */
  double hN = Bbot1 - (Bbot0 - Bbot1) / dtau[nd - 2];
  abc[nd - 1] = 1.0 + 2.0 / dtau[nd - 2];
  A1[nd - 1] = 2.0 / (dtau[nd - 2] * dtau[nd - 2]);
  St[nd - 1] = S[nd - 1] + 2.0 * hN / dtau[nd - 2];
  for (int k = 1; k < nd - 1; k++) {
    double dmid = 0.5 * (dtau[k] + dtau[k - 1]);
    A1[k] = 1.0 / (dmid * dtau[k - 1]);
    C1[k] = 1.0 / (dmid * dtau[k]);
    abc[k] = 1.0;
    St[k] = S[k];
  }
  F[0] = abc[0] / C1[0];
  zt[0] = St[0] / (abc[0] + C1[0]);
  for (int k = 1; k < nd - 1; k++) {
    F[k] = (abc[k] + A1[k] * F[k - 1] / (1.0 + F[k - 1])) / C1[k];
    zt[k] = (St[k] + A1[k] * zt[k - 1]) / (C1[k] * (1.0 + F[k]));
  }
  Pl[nd - 1] = (St[nd - 1] + A1[nd - 1] * zt[nd - 2]) /
               (abc[nd - 1] + A1[nd - 1] * (F[nd - 2] / (1.0 + F[nd - 2])));
  for (int k = nd - 2; k >= 0; k--) Pl[k] = Pl[k + 1] / (1.0 + F[k]) + zt[k];
  if (Psi) {
    G[nd - 1] = abc[nd - 1] / A1[nd - 1];
    for (int k = nd - 2; k >= 1; k--)
      G[k] = (abc[k] + C1[k] * G[k + 1] / (1.0 + G[k + 1])) / A1[k];
    Psi[0] = 1.0 / (abc[0] + C1[0] * G[1] / (1.0 + G[1]));
    for (int k = 1; k < nd - 1; k++)
      Psi[k] = 1.0 / (abc[k] + A1[k] * F[k - 1] / (1.0 + F[k - 1]) +
                      C1[k] * G[k + 1] / (1.0 + G[k + 1]));
    Psi[nd - 1] = 1.0 / (abc[nd - 1] + A1[nd - 1] * F[nd - 2] / (1.0 + F[nd - 2]));
  }
  double Iplus = 2.0 * Pl[0];
  free(dtau); free(abc); free(A1); free(C1); free(F); free(G); free(zt); free(St);
  if (!P) free(Pl);
  return Iplus;
}

/* ------------------------------------------------------- batch driver -- */

int oracle_lte_opacity(const OracleAtmos *A, const OracleLines *LN, int k,
                       double lambda, double *chi4, double *eta4, double *chip3)
{
  return rlk_opacity_at(A, LN, k, lambda, chi4, eta4, chip3);
}

/* One atmosphere: emergent I,Q,U,V at every wavelength of the spectrum
   (out[4][nlam]).  chi_c/eta_c are [nlam][ndep].  Returns 0. */
int oracle_lte_synth(const OracleAtmos *A, const OracleLines *LN, int nlam,
                     const double *lam, const double *chi_c, const double *eta_c,
                     int md_float, double *out)
{
  int nd = A->ndep;
  double imu = 1.0 / A->muz;
  double *chi = (double *) malloc(nd * sizeof(double));
  double *Ss = (double *) malloc(nd * sizeof(double));
  double (*S)[4] = malloc(nd * sizeof(*S));
  double (*K)[4][4] = malloc(nd * sizeof(*K));
  double *chip = (double *) malloc(3 * nd * sizeof(double));
  for (int la = 0; la < nlam; la++) {
    double lambda = lam[la];
    int flags = 0;
    for (int k = 0; k < nd; k++) {
      double lc[4], le[4], lp[3];
      flags |= rlk_opacity_at(A, LN, k, lambda, lc, le, lp);
      double ct = chi_c[(long) la * nd + k] + lc[0];
      double et = eta_c[(long) la * nd + k] + le[0];
      chi[k] = ct;
      S[k][0] = et / ct;
      Ss[k] = et / ct;
      for (int s = 1; s < 4; s++) S[k][s] = le[s] / ct;
      double c4[4] = {ct, lc[1], lc[2], lc[3]};
      stokes_K(c4, lp, LN->magneto_optical, K[k]);
      for (int s = 0; s < 3; s++) chip[s * nd + k] = lp[s];
    }
    double B0 = oracle_planck(A->T[nd - 2], lambda);
    double B1 = oracle_planck(A->T[nd - 1], lambda);
    if ((flags & 2) && !LN->no_stokes) {
      double I0[4];
      stokes_bezier3(nd, A->height, imu, chi, S, K, B0, B1, md_float, I0);
      for (int s = 0; s < 4; s++) out[(long) s * nlam + la] = I0[s];
    } else {
      /* angle dependent (formal.c:96-101): a polarizable line in window, or
         any line in a moving atmosphere -- scalar Bezier3; otherwise the
         angle-independent Feautrier solution (formal.c:284-304) */
      if ((flags & 1) && ((flags & 2) || LN->moving))
        out[la] = oracle_scalar_bezier3(nd, A->height, imu, chi, Ss, B0, B1, 1, NULL, NULL);
      else
        out[la] = oracle_feautrier(nd, A->height, A->muz, chi, Ss, B0, B1, NULL, NULL);
      for (int s = 1; s < 4; s++) out[(long) s * nlam + la] = 0.0;
    }
  }
  free(chi); free(Ss); free(S); free(K); free(chip);
  return 0;
}

/* Many atmospheres with identical shapes, threaded over atmospheres.
   Arrays are [natm][...] with the same layout as oracle_lte_synth. */
int oracle_lte_synth_batch(int natm, int nthreads, const OracleAtmos *atms,
                           const OracleLines *LN, int nlam, const double *lam,
                           const double *chi_c, const double *eta_c,
                           int md_float, double *out)
{
#ifdef _OPENMP
  #pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int p = 0; p < natm; p++) {
    long plane = (long) nlam * atms[p].ndep;
    oracle_lte_synth(&atms[p], LN, nlam, lam, chi_c + p * plane,
                     eta_c + p * plane, md_float, out + (long) p * 4 * nlam);
  }
  (void) nthreads;
  return 0;
}
