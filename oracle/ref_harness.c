/* ref_harness.c -- TEST INFRASTRUCTURE, compiled only against the reference.
 *
 * Thin C harness linked together with the reference's own RH sources into
 * oracle/_ref/librh_ref.so (recipe: oracle/Makefile.ref).  It is used only to
 * generate golden vectors in tests/golden/ and never ships with the product.
 *
 *  harness_synth     wraps rhf1d() (rh/rhf1d/pyrh_compute1dray.c:112-389) and
 *                    copies the returned mySpectrum into caller buffers.
 *  harness_dump_lte  performs the same set-up sequence as rhf1d()
 *                    (pyrh_compute1dray.c:130-311) and writes the
 *                    intermediate quantities the formal-solution hot path
 *                    consumes (continuum, line constants, LTE stage densities,
 *                    height scale, Zeeman patterns, total background records)
 *                    as raw little-endian float64/int32 files into a directory.
 *  harness_dump_ltepops writes the element tables (partition functions,
 *                    ionisation potentials, abundances), LTEpops_elem() of
 *                    every element and Solve_ne() after the same set-up.
 *  harness_dump_chem writes ChemicalEquilibrium()'s inputs and results.
 *  harness_dump_nlte performs the whole rhf1d() sequence with one ACTIVE atom
 *                    and writes the converged populations, the collision
 *                    matrix, the wavelength grid and the emergent intensity.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#include "rh.h"
#include "atom.h"
#include "atmos.h"
#include "geometry.h"
#include "spectrum.h"
#include "background.h"
#include "inputs.h"
#include "constant.h"
#include "error.h"
#include "pyrh_compute1dray.h"

extern Atmosphere atmos;
extern Geometry geometry;
extern Spectrum spectrum;
extern InputData input;
extern CommandLine commandline;

void Linear(int Ntable, double *xtable, double *ytable, int N, double *x,
            double *y, bool_t hunt);
ZeemanMultiplet *RLKZeeman(RLK_Line *rlk);
void convertScales(Atmosphere *atmos, Geometry *geometry);
void getBoundary(Geometry *geometry);
void MULTIatmos(Atmosphere *atmos, Geometry *geometry, int Nabun,
                int *atomic_id, double *atomic_abundance);
void Bproject(void);
void Background(bool_t write_analyze_output, bool_t equilibria_only);

static int write_f64(const char *dir, const char *name, const double *x, long n)
{
  char path[1024];
  snprintf(path, sizeof(path), "%s/%s.f64", dir, name);
  FILE *fp = fopen(path, "wb");
  if (!fp) return -1;
  long w = (long) fwrite(x, sizeof(double), n, fp);
  fclose(fp);
  return (w == n) ? 0 : -1;
}

static int write_i32(const char *dir, const char *name, const int *x, long n)
{
  char path[1024];
  snprintf(path, sizeof(path), "%s/%s.i32", dir, name);
  FILE *fp = fopen(path, "wb");
  if (!fp) return -1;
  long w = (long) fwrite(x, sizeof(int), n, fp);
  fclose(fp);
  return (w == n) ? 0 : -1;
}

/* Calls rhf1d() on private copies of the nine atmosphere rows (rhf1d mutates
   its inputs in place, pyrh_compute1dray.c:263-270).  Returns the number of
   output wavelengths, or -1 if out_cap is too small.  atm is [9][Ndep]. */
int harness_synth(const char *cwd, double mu, int Ndep, const double *atm,
                  int atm_scale, int Nwave, const double *lam,
                  int out_cap, double *out_lam, double *sI, double *sQ,
                  double *sU, double *sV, int *stokes_flag)
{
  double *a = (double *) malloc(9 * Ndep * sizeof(double));
  double *w = (double *) malloc(Nwave * sizeof(double));
  memcpy(a, atm, 9 * Ndep * sizeof(double));
  memcpy(w, lam, Nwave * sizeof(double));

  mySpectrum s = rhf1d((char *) cwd, mu, Ndep,
                       a + 0 * Ndep, a + 1 * Ndep, a + 2 * Ndep, a + 3 * Ndep,
                       a + 4 * Ndep, a + 5 * Ndep, a + 6 * Ndep, a + 7 * Ndep,
                       a + 8 * Ndep, atm_scale, Nwave, w,
                       0, NULL, NULL, 0, NULL, NULL, 0, NULL, NULL,
                       0, NULL, NULL, 0, 0, 0, NULL);
  int n = s.nlw;
  if (n > out_cap) n = -1;
  else {
    for (int i = 0; i < n; i++) {
      out_lam[i] = s.lam[i];
      sI[i] = s.sI[i];
      sQ[i] = s.stokes ? s.sQ[i] : 0.0;
      sU[i] = s.stokes ? s.sU[i] : 0.0;
      sV[i] = s.stokes ? s.sV[i] : 0.0;
    }
    *stokes_flag = s.stokes;
  }
  free(s.lam); free(s.sI); free(s.sQ); free(s.sU); free(s.sV);
  free(a); free(w);
  return n;
}

/* harness_synth with log gf values overriding the line list's
   (loggf_ids: 0-based order of the lines in the list file,
   kurucz.c:250-260) and, with get_atomic_rfs, the reference's analytical
   d I / d log gf of those lines (pyrh_solveray.c:144-148), written to
   rfs[Nloggf][out_cap].  Stokes I only. */
int harness_synth_loggf(const char *cwd, double mu, int Ndep, const double *atm,
                        int Nwave, const double *lam, int Nloggf, const int *loggf_ids,
                        const double *loggf_values, int get_atomic_rfs, int out_cap,
                        double *out_lam, double *sI, double *rfs)
{
  double *a = (double *) malloc(9 * Ndep * sizeof(double));
  double *w = (double *) malloc(Nwave * sizeof(double));
  int *ids = (int *) malloc(Nloggf * sizeof(int));
  double *vals = (double *) malloc(Nloggf * sizeof(double));
  memcpy(a, atm, 9 * Ndep * sizeof(double));
  memcpy(w, lam, Nwave * sizeof(double));
  memcpy(ids, loggf_ids, Nloggf * sizeof(int));
  memcpy(vals, loggf_values, Nloggf * sizeof(double));

  mySpectrum s = rhf1d((char *) cwd, mu, Ndep,
                       a + 0 * Ndep, a + 1 * Ndep, a + 2 * Ndep, a + 3 * Ndep,
                       a + 4 * Ndep, a + 5 * Ndep, a + 6 * Ndep, a + 7 * Ndep,
                       a + 8 * Ndep, 0, Nwave, w,
                       0, NULL, NULL, Nloggf, ids, vals, 0, NULL, NULL,
                       0, NULL, NULL, get_atomic_rfs, 0, 0, NULL);
  int n = s.nlw;
  if (n > out_cap) n = -1;
  else {
    for (int i = 0; i < n; i++) {
      out_lam[i] = s.lam[i];
      sI[i] = s.sI[i];
      if (get_atomic_rfs)
        for (int p = 0; p < Nloggf; p++) rfs[(long) p * out_cap + i] = s.rfs[i][p];
    }
  }
  free(s.lam); free(s.sI); free(s.sQ); free(s.sU); free(s.sV);
  free(a); free(w); free(ids); free(vals);
  return n;
}

/* Set-up sequence of rhf1d() up to SortLambda() and getBoundary(), in the
   same order as pyrh_compute1dray.c:130-311, on private copies of the
   atmosphere rows and wavelengths (returned in *pa / *pw). */
static void lte_setup_ab(const char *cwd, double mu, int Ndep, const double *atm, int Nwave,
                         const double *lam, double **pa, double **pw, int Nabun, int *ab_id,
                         double *ab_val, int force_h_lte);

static void lte_setup(const char *cwd, double mu, int Ndep, const double *atm, int Nwave,
                      const double *lam, double **pa, double **pw)
{
  lte_setup_ab(cwd, mu, Ndep, atm, Nwave, lam, pa, pw, 0, NULL, NULL, 0);
}

/* lte_setup with abundance overrides (as rhf1d() passes compute1d's
   atomic_number / atomic_abundance to MULTIatmos) and, with force_h_lte,
   hydrogen in LTE as get_ne_from_nH() sets it before reading the atoms
   (rh/rhf1d/pyrh_hse.c:594). */
static void lte_setup_ab(const char *cwd, double mu, int Ndep, const double *atm, int Nwave,
                         const double *lam, double **pa, double **pw, int Nabun, int *ab_id,
                         double *ab_val, int force_h_lte)
{
  char tmp[512];
  double *a = (double *) malloc(9 * Ndep * sizeof(double));
  double *w = (double *) malloc(Nwave * sizeof(double));
  memcpy(a, atm, 9 * Ndep * sizeof(double));
  memcpy(w, lam, Nwave * sizeof(double));
  *pa = a;
  *pw = w;

  snprintf(commandline.keyword_input, sizeof(commandline.keyword_input),
           "%s/keyword.input", cwd);
  setOptions(1, NULL);
  readInput();
  input.verbose = FALSE;
  input.get_populations = FALSE;
  input.pyrhHSE = FALSE;
  input.get_atomic_rfs = FALSE;
  input.n_atomic_pars = 0;
  snprintf(tmp, sizeof(tmp), "%s/%s", cwd, input.atoms_input);
  strcpy(input.atoms_input, tmp);
  snprintf(tmp, sizeof(tmp), "%s/%s", cwd, input.molecules_input);
  strcpy(input.molecules_input, tmp);
  snprintf(tmp, sizeof(tmp), "%s/%s", cwd, input.KuruczData);
  strcpy(input.KuruczData, tmp);
  input.solve_ne = FALSE;
  spectrum.updateJ = TRUE;
  input.limit_memory = FALSE;
  input.solve_NLTE = FALSE;
  atmos.Nrlk = 0;
  geometry.Ndep = Ndep;

  if (force_h_lte) atmos.H_LTE = TRUE;
  MULTIatmos(&atmos, &geometry, Nabun, ab_id, ab_val);
  atmos.active_layer = -1;
  geometry.scale = TAU500;
  for (int k = 0; k < Ndep; k++) geometry.tau_ref[k] = POW10(a[k]);
  atmos.T = a + 1 * Ndep;
  atmos.ne = a + 2 * Ndep;
  geometry.vel = a + 3 * Ndep;
  atmos.vturb = a + 4 * Ndep;
  atmos.B = a + 5 * Ndep;
  atmos.gamma_B = a + 6 * Ndep;
  atmos.chi_B = a + 7 * Ndep;
  atmos.nHtot = a + 8 * Ndep;
  atmos.nH = matrix_double(atmos.NHydr, geometry.Ndep);
  atmos.Stokes = TRUE;
  atmos.moving = FALSE;
  for (int k = 0; k < Ndep; k++) {
    geometry.vel[k] *= KM_TO_M;
    atmos.vturb[k] *= KM_TO_M;
    atmos.ne[k] /= CUBE(CM_TO_M);
    atmos.nHtot[k] /= CUBE(CM_TO_M);
    atmos.B[k] /= 1e4;
  }
  for (int k = 0; k < Ndep; k++)
    if (fabs(geometry.vel[k]) >= atmos.vmacro_tresh) { atmos.moving = TRUE; break; }

  readAtomicModels();
  readMolecularModels();
  atmos.Nrays = geometry.Nrays = 1;
  geometry.muz[0] = mu;
  geometry.mux[0] = sqrt(1.0 - SQ(geometry.muz[0]));
  geometry.muy[0] = 0.0;
  geometry.wmu[0] = 1.0;
  Bproject();
  SortLambda(w, Nwave);
  getBoundary(&geometry);
}

/* Set-up sequence of rhf1d() up to convertScales(), in the same order as
   pyrh_compute1dray.c:130-311, followed by a dump of the hot-path inputs. */
int harness_dump_lte(const char *cwd, double mu, int Ndep, const double *atm,
                     int Nwave, const double *lam, const char *outdir)
{
  double *a, *w;
  lte_setup(cwd, mu, Ndep, atm, Nwave, lam, &a, &w);

  int Nspect = spectrum.Nspect, Nspace = atmos.Nspace;

  /* Pass 1: continuum only.  Background() reads the Kurucz list itself
     when none is loaded (background.c:288-293), so the list name is set to
     "none" for this pass (kurucz.c:140). */
  char kurucz_saved[MAX_LINE_SIZE];
  strcpy(kurucz_saved, input.KuruczData);
  strcpy(input.KuruczData, "none");
  atmos.Nrlk = 0;
  Background(FALSE, FALSE);
  strcpy(input.KuruczData, kurucz_saved);
  double *cont = (double *) malloc(3 * (long) Nspect * Nspace * sizeof(double));
  int *cflags = (int *) malloc(2 * Nspect * sizeof(int));
  for (int la = 0; la < Nspect; la++) {
    memcpy(cont + (0L * Nspect + la) * Nspace, spectrum.chi_c_lam[la], Nspace * sizeof(double));
    memcpy(cont + (1L * Nspect + la) * Nspace, spectrum.eta_c_lam[la], Nspace * sizeof(double));
    memcpy(cont + (2L * Nspect + la) * Nspace, spectrum.sca_c_lam[la], Nspace * sizeof(double));
    cflags[2 * la] = atmos.backgrflags[la].hasline;
    cflags[2 * la + 1] = atmos.backgrflags[la].ispolarized;
  }
  /* Pass 2: with the Kurucz lines, as rhf1d() runs it. */
  atmos.Nrlk = 0;
  Background(FALSE, FALSE);
  convertScales(&atmos, &geometry);

  double *tot_chi = (double *) malloc(4L * Nspect * Nspace * sizeof(double));
  double *tot_eta = (double *) malloc(4L * Nspect * Nspace * sizeof(double));
  double *tot_chip = (double *) calloc(3L * Nspect * Nspace, sizeof(double));
  int *tflags = (int *) malloc(2 * Nspect * sizeof(int));
  for (int la = 0; la < Nspect; la++) {
    int nrec = atmos.backgrflags[la].ispolarized ? 4 : 1;
    for (int i = 0; i < 4 * Nspace; i++) {
      tot_chi[(long) la * 4 * Nspace + i] = (i < nrec * Nspace) ? spectrum.chi_c_lam[la][i] : 0.0;
      tot_eta[(long) la * 4 * Nspace + i] = (i < nrec * Nspace) ? spectrum.eta_c_lam[la][i] : 0.0;
    }
    if (input.magneto_optical && atmos.backgrflags[la].ispolarized)
      memcpy(tot_chip + (long) la * 3 * Nspace, spectrum.chip_c_lam[la], 3 * Nspace * sizeof(double));
    tflags[2 * la] = atmos.backgrflags[la].hasline;
    tflags[2 * la + 1] = atmos.backgrflags[la].ispolarized;
  }

  write_f64(outdir, "lambda", spectrum.lambda, Nspect);
  write_f64(outdir, "cont", cont, 3L * Nspect * Nspace);
  write_i32(outdir, "cont_flags", cflags, 2 * Nspect);
  write_f64(outdir, "tot_chi", tot_chi, 4L * Nspect * Nspace);
  write_f64(outdir, "tot_eta", tot_eta, 4L * Nspect * Nspace);
  write_f64(outdir, "tot_chip", tot_chip, 3L * Nspect * Nspace);
  write_i32(outdir, "tot_flags", tflags, 2 * Nspect);
  write_f64(outdir, "height", geometry.height, Nspace);
  write_f64(outdir, "T", atmos.T, Nspace);
  write_f64(outdir, "ne", atmos.ne, Nspace);
  write_f64(outdir, "nHtot", atmos.nHtot, Nspace);
  write_f64(outdir, "vturb", atmos.vturb, Nspace);
  write_f64(outdir, "vel", geometry.vel, Nspace);
  write_f64(outdir, "B", atmos.B, Nspace);
  write_f64(outdir, "gamma_B", atmos.gamma_B, Nspace);
  write_f64(outdir, "chi_B", atmos.chi_B, Nspace);
  write_f64(outdir, "np", atmos.H->n[atmos.H->Nlevel - 1], Nspace);
  write_f64(outdir, "cos_gamma", atmos.cos_gamma[0], Nspace);
  write_f64(outdir, "cos_2chi", atmos.cos_2chi[0], Nspace);
  write_f64(outdir, "sin_2chi", atmos.sin_2chi[0], Nspace);

  /* Line constants (double[24] per line), Zeeman patterns and stage
     densities n[stage][k] with log partition function pf[k] as used in
     rlk_opacity (kurucz.c:662-677). */
  double *lc = (double *) calloc(24L * atmos.Nrlk, sizeof(double));
  double *lpop = (double *) calloc(2L * atmos.Nrlk * Nspace, sizeof(double));
  int maxcomp = 0;
  for (int n = 0; n < atmos.Nrlk; n++) {
    RLK_Line *r = &atmos.rlk_lines[n];
    if (r->polarizable && r->zm == NULL) r->zm = RLKZeeman(r);
    if (r->zm && r->zm->Ncomponent > maxcomp) maxcomp = r->zm->Ncomponent;
  }
  double *zm = (double *) calloc(3L * atmos.Nrlk * (maxcomp > 0 ? maxcomp : 1), sizeof(double));
  int *zn = (int *) calloc(atmos.Nrlk > 0 ? atmos.Nrlk : 1, sizeof(int));
  for (int n = 0; n < atmos.Nrlk; n++) {
    RLK_Line *r = &atmos.rlk_lines[n];
    Element *el = &atmos.elements[r->pt_index - 1];
    double *L = lc + 24L * n;
    L[0] = r->lambda0; L[1] = r->pt_index; L[2] = r->stage; L[3] = r->gi;
    L[4] = r->gj; L[5] = r->Ei; L[6] = r->Ej; L[7] = r->Aji; L[8] = r->Bji;
    L[9] = r->Bij; L[10] = r->Grad; L[11] = r->GStark; L[12] = r->GvdWaals;
    L[13] = r->vdwaals; L[14] = r->cross; L[15] = r->alpha;
    L[16] = r->isotope_frac; L[17] = r->hyperfine_frac; L[18] = r->polarizable;
    L[19] = el->weight; L[20] = (r->stage < el->Nstage - 1) && el->abundance_set;
    L[21] = r->gL_i; L[22] = r->gL_j; L[23] = (el->model != NULL);
    if (el->n == NULL) {
      el->n = matrix_double(el->Nstage, Nspace);
      LTEpops_elem(el);
    }
    double *pf = (double *) malloc(Nspace * sizeof(double));
    Linear(atmos.Npf, atmos.Tpf, el->pf[r->stage], Nspace, atmos.T, pf, TRUE);
    for (int k = 0; k < Nspace; k++) {
      lpop[(2L * n + 0) * Nspace + k] = el->n[r->stage][k];
      lpop[(2L * n + 1) * Nspace + k] = pf[k];
    }
    free(pf);
    if (r->zm) {
      zn[n] = r->zm->Ncomponent;
      for (int c = 0; c < r->zm->Ncomponent; c++) {
        zm[(3L * n + 0) * maxcomp + c] = r->zm->q[c];
        zm[(3L * n + 1) * maxcomp + c] = r->zm->shift[c];
        zm[(3L * n + 2) * maxcomp + c] = r->zm->strength[c];
      }
    }
  }
  write_f64(outdir, "line_const", lc, 24L * atmos.Nrlk);

  /* What the line-list reader takes besides the list: the element data of
     each line (weight, stages, abundance, abundance flag, ionisation
     potentials of the first four stages), hydrogen's and helium's weight
     and abundance, and the three Barklem tables as readBarklemTable parsed
     them (rows, columns, first effective quantum numbers, then cross and
     alpha, row-major). */
  double *eld = (double *) calloc(8L * (atmos.Nrlk > 0 ? atmos.Nrlk : 1), sizeof(double));
  for (int n = 0; n < atmos.Nrlk; n++) {
    Element *el = &atmos.elements[atmos.rlk_lines[n].pt_index - 1];
    double *E = eld + 8L * n;
    E[0] = el->weight; E[1] = el->Nstage; E[2] = el->abund; E[3] = el->abundance_set;
    for (int st = 0; st < 4; st++) E[4 + st] = (st < el->Nstage) ? el->ionpot[st] : 0.0;
  }
  write_f64(outdir, "rlk_element", eld, 8L * (atmos.Nrlk > 0 ? atmos.Nrlk : 1));
  free(eld);
  double hhe[4] = {atmos.elements[0].weight, atmos.elements[0].abund,
                   atmos.elements[1].weight, atmos.elements[1].abund};
  write_f64(outdir, "rlk_hhe", hhe, 4);
  {
    enum Barklemtype types[3] = {SP, PD, DF};
    const char *names[3] = {"barklem_sp", "barklem_pd", "barklem_df"};
    for (int t = 0; t < 3; t++) {
      Barklemstruct bs;
      if (!readBarklemTable(types[t], &bs)) continue;
      long n12 = (long) bs.N1 * bs.N2;
      double *tb = (double *) malloc((4 + 2 * n12) * sizeof(double));
      tb[0] = bs.N1; tb[1] = bs.N2; tb[2] = bs.neff1[0]; tb[3] = bs.neff2[0];
      for (long e = 0; e < n12; e++) {
        tb[4 + e] = bs.cross[0][e];
        tb[4 + n12 + e] = bs.alpha[0][e];
      }
      write_f64(outdir, names[t], tb, 4 + 2 * n12);
      free(tb);
    }
  }
  write_f64(outdir, "line_pops", lpop, 2L * atmos.Nrlk * Nspace);
  write_f64(outdir, "zeeman", zm, 3L * atmos.Nrlk * (maxcomp > 0 ? maxcomp : 1));
  write_i32(outdir, "zeeman_n", zn, atmos.Nrlk > 0 ? atmos.Nrlk : 1);

  int meta[8] = {Nspect, Nspace, atmos.Nrlk, maxcomp, input.magneto_optical,
                 atmos.moving, geometry.vboundary[TOP], geometry.vboundary[BOTTOM]};
  write_i32(outdir, "meta", meta, 8);
  double fmeta[4] = {atmos.vmicro_char, atmos.lambda_ref, mu, (double) input.StokesMode};
  write_f64(outdir, "fmeta", fmeta, 4);

  free(cont); free(cflags); free(tot_chi); free(tot_eta); free(tot_chip);
  free(tflags); free(lc); free(lpop); free(zm); free(zn);
  return Nspect;
}

/* Element tables, LTE stage populations and the electron density
   (readAbundance rh/abundance.c:72-220, LTEpops_elem rh/ltepops.c:116-166,
   Solve_ne and getfjk rh/solvene.c:55-198), after the set-up of rhf1d() with
   the abundance overrides and hydrogen in LTE, as get_ne_from_nH() runs it
   (rh/rhf1d/pyrh_hse.c:555-650).  Files:
     Tpf [Npf]; el_meta [Nelem][4] Nstage, abundance_set, abund, weight;
     el_pf [sum Nstage][Npf] (natural log for elements with an abundance);
     el_ionpot [sum Nstage] (J for elements with an abundance);
     T, ne, nHtot [Nspace] (SI);
     el_n [sum Nstage][Nspace] LTEpops_elem() of each element with an
       abundance at the atmosphere's own electron density (zeros otherwise);
     ne_solved [Nspace] Solve_ne(fromscratch = TRUE);
     ne_warm [Nspace] Solve_ne(fromscratch = FALSE), from the atmosphere's ne. */
void Solve_ne(double *ne, bool_t fromscratch);
void LTEpops_elem(Element *element);

int harness_dump_ltepops(const char *cwd, int Ndep, const double *atm, int Nabun,
                         int *ab_id, double *ab_val, const char *outdir)
{
  double *a, *w, lam500 = 500.0;
  lte_setup_ab(cwd, 1.0, Ndep, atm, 1, &lam500, &a, &w, Nabun, ab_id, ab_val, 1);
  int Nspace = atmos.Nspace, Nelem = atmos.Nelem, Npf = atmos.Npf, nst = 0;
  for (int n = 0; n < Nelem; n++) nst += atmos.elements[n].Nstage;
  double *meta = (double *) calloc(4L * Nelem, sizeof(double));
  double *pf = (double *) calloc((long) nst * Npf, sizeof(double));
  double *ion = (double *) calloc(nst, sizeof(double));
  double *pops = (double *) calloc((long) nst * Nspace, sizeof(double));
  long row = 0;
  for (int n = 0; n < Nelem; n++) {
    Element *el = &atmos.elements[n];
    meta[4 * n + 0] = el->Nstage;
    meta[4 * n + 1] = el->abundance_set;
    meta[4 * n + 2] = el->abund;
    meta[4 * n + 3] = el->weight;
    if (el->abundance_set) {
      if (el->n == NULL) el->n = matrix_double(el->Nstage, Nspace);
      LTEpops_elem(el);
    }
    for (int i = 0; i < el->Nstage; i++, row++) {
      memcpy(pf + row * Npf, el->pf[i], Npf * sizeof(double));
      ion[row] = el->ionpot[i];
      if (el->abundance_set) memcpy(pops + row * Nspace, el->n[i], Nspace * sizeof(double));
    }
  }
  double *ne1 = (double *) malloc(Nspace * sizeof(double));
  double *ne2 = (double *) malloc(Nspace * sizeof(double));
  memcpy(ne1, atmos.ne, Nspace * sizeof(double));
  memcpy(ne2, atmos.ne, Nspace * sizeof(double));
  Solve_ne(ne1, TRUE);
  Solve_ne(ne2, FALSE);
  write_f64(outdir, "Tpf", atmos.Tpf, Npf);
  write_f64(outdir, "el_meta", meta, 4L * Nelem);
  write_f64(outdir, "el_pf", pf, (long) nst * Npf);
  write_f64(outdir, "el_ionpot", ion, nst);
  write_f64(outdir, "T", atmos.T, Nspace);
  write_f64(outdir, "ne", atmos.ne, Nspace);
  write_f64(outdir, "nHtot", atmos.nHtot, Nspace);
  write_f64(outdir, "el_n", pops, (long) nst * Nspace);
  write_f64(outdir, "ne_solved", ne1, Nspace);
  write_f64(outdir, "ne_warm", ne2, Nspace);
  free(meta); free(pf); free(ion); free(pops); free(ne1); free(ne2);
  return Nspace;
}

#define PYRH_HARNESS_MAX_NUC 32
/* Chemical equilibrium (ChemicalEquilibrium, rh/chemequil.c:107-390) after
   the set-up of rhf1d() and the LTE populations of the atoms
   (SetLTEQuantities, rh/ltepops.c:224-249).  Files:
     T, ne, nHtot [Nspace] (SI);
     nuclei [Nnuclei] element index of each nucleus (elements bound in a
       molecule, in element order); nuc_model [Nnuclei] 1 if an atom model
       gives its neutral fraction;
     fn0 [Nnuclei][Nspace] the neutral fraction the equilibrium starts from
       (from the model's LTE populations, else from the element's partition
       functions, getfjk), as rh/chemequil.c:227-246 forms it;
     nmol [Nmolecule][Nspace], nHmin [Nspace] the results;
     ntot_model [Nnuclei][Nspace] the model atoms' total density afterwards
       (the nucleus' atomic density; zeros for nuclei without a model). */
void SetLTEQuantities(void);
void ChemicalEquilibrium(int NmaxIter, double iterLimit);
void getfjk(Element *element, double ne, int k, double *fjk, double *dfjk);

int harness_dump_chem(const char *cwd, int Ndep, const double *atm, const char *outdir)
{
  double *a, *w, lam500 = 500.0;
  lte_setup(cwd, 1.0, Ndep, atm, 1, &lam500, &a, &w);
  SetLTEQuantities();
  int Nspace = atmos.Nspace, nn = 0;
  int nuc[PYRH_HARNESS_MAX_NUC], model[PYRH_HARNESS_MAX_NUC];
  for (int i = 0; i < atmos.Nelem && nn < PYRH_HARNESS_MAX_NUC; i++)
    if (atmos.elements[i].Nmolecule > 0) {
      nuc[nn] = i;
      model[nn] = atmos.elements[i].model != NULL;
      nn++;
    }
  double *fn0 = (double *) calloc((long) nn * Nspace, sizeof(double));
  double fjk[16], dfjk[16];
  for (int i = 0; i < nn; i++) {
    Element *el = &atmos.elements[nuc[i]];
    Atom *atom = el->model;
    for (int k = 0; k < Nspace; k++) {
      if (atom == NULL) {
        getfjk(el, atmos.ne[k], k, fjk, dfjk);
        fn0[(long) i * Nspace + k] = fjk[0];
      } else {
        double s = 0.0;
        for (int j = 0; j < atom->Nlevel; j++) {
          if (atom->stage[j] > 0) break;
          if (atom->active && atom->initial_solution != OLD_POPULATIONS) s += atom->nstar[j][k];
          else s += atom->n[j][k];
        }
        fn0[(long) i * Nspace + k] = s / atom->ntotal[k];
      }
    }
  }
  ChemicalEquilibrium(N_MAX_CHEM_ITER, CHEM_ITER_LIMIT);
  double *nmol = (double *) malloc((long) atmos.Nmolecule * Nspace * sizeof(double));
  for (int m = 0; m < atmos.Nmolecule; m++)
    memcpy(nmol + (long) m * Nspace, atmos.molecules[m].n, Nspace * sizeof(double));
  double *ntot = (double *) calloc((long) nn * Nspace, sizeof(double));
  for (int i = 0; i < nn; i++)
    if (atmos.elements[nuc[i]].model)
      memcpy(ntot + (long) i * Nspace, atmos.elements[nuc[i]].model->ntotal, Nspace * sizeof(double));
  write_f64(outdir, "T", atmos.T, Nspace);
  write_f64(outdir, "ne", atmos.ne, Nspace);
  write_f64(outdir, "nHtot", atmos.nHtot, Nspace);
  write_i32(outdir, "nuclei", nuc, nn);
  write_i32(outdir, "nuc_model", model, nn);
  write_f64(outdir, "fn0", fn0, (long) nn * Nspace);
  write_f64(outdir, "nmol", nmol, (long) atmos.Nmolecule * Nspace);
  write_f64(outdir, "nHmin", atmos.nHmin, Nspace);
  write_f64(outdir, "ntot_model", ntot, (long) nn * Nspace);
  free(fn0); free(nmol); free(ntot);
  return atmos.Nmolecule;
}

/* ------------------------------------------------------------------ NLTE */

void Damping(AtomicLine *line, double *adamp);
double solveSpectrum(bool_t eval_operator, bool_t redistribute);
void statEquil(Atom *atom, int isum);
void initGammaAtom(Atom *atom);
void initSolution(bool_t pyrh_io_flag);
void initScatter(void);
void getProfiles(void);
void Iterate(int NmaxIter, double iterLimit);
void _solveray(double muz, mySpectrum *spec);

/* The background continuum of the LTE set-up (Background(), rh/background.c:
   139-631, without line lists: KURUCZ_DATA none, ALLOW_PASSIVE_BB FALSE),
   each of its processes evaluated alone at every wavelength, and what they
   read: the densities after the set-up and the atomic data.  Files:
     lambda [Nspect]; T, ne, nHmin, nH2, nOH, nCH [Nspace] (zeros where a
     molecule is absent, mol_present[3] says which is present);
     cont [3][Nspect][Nspace] chi_c, eta_c, sca_c as Background() stores them;
     comp [13][2][Nspect][Nspace]: per process (0 Thomson, 1 Hminus_bf,
       2 Hminus_ff, 3 OH_bf, 4 CH_bf, 5 Hydrogen_bf, 6 Hydrogen_ff,
       7 Rayleigh H, 8 Rayleigh He, 9 H2plus_ff, 10 Rayleigh_H2,
       11 H2minus_ff, 12 Metal_bf) its opacity and its emissivity (or its
       scattering opacity), zero where the routine reports no contribution;
     atoms_meta [Natom][4] Nlevel, Ncont, Nline, active; atoms_lev [sum
     Nlevel][3] E, g, stage; atoms_n, atoms_nstar [sum Nlevel][Nspace];
     atoms_cont [sum Ncont][8] i, j, lambda0, lambda[0], hydrogenic, alpha0,
     Nlambda, table offset; atoms_tab [sum Nlambda][2] lambda, alpha;
     atoms_line [sum Nline][5] i, j, lambda0, qwing, Aji; misc [4]
     vmicro_char, index of the He model (-1: none), index of H, Natom. */
int harness_dump_background(const char *cwd, double mu, int Ndep, const double *atm,
                            int Nwave, const double *lam, const char *outdir)
{
  double *a, *w;
  lte_setup(cwd, mu, Ndep, atm, Nwave, lam, &a, &w);
  int Nspect = spectrum.Nspect, Nspace = atmos.Nspace;
  strcpy(input.KuruczData, "none");
  atmos.Nrlk = 0;
  Background(FALSE, FALSE);

  double *cont = (double *) malloc(3L * Nspect * Nspace * sizeof(double));
  for (int la = 0; la < Nspect; la++) {
    memcpy(cont + (0L * Nspect + la) * Nspace, spectrum.chi_c_lam[la], Nspace * sizeof(double));
    memcpy(cont + (1L * Nspect + la) * Nspace, spectrum.eta_c_lam[la], Nspace * sizeof(double));
    memcpy(cont + (2L * Nspect + la) * Nspace, spectrum.sca_c_lam[la], Nspace * sizeof(double));
  }
  write_f64(outdir, "lambda", spectrum.lambda, Nspect);
  write_f64(outdir, "cont", cont, 3L * Nspect * Nspace);
  free(cont);

  /* each process alone (the routines keep their temperature indices from
     the Background() pass, which used the same temperatures) */
  const int NC = 13;
  double *comp = (double *) calloc((size_t) NC * 2 * Nspect * Nspace, sizeof(double));
  double *c1 = (double *) malloc(4L * Nspace * sizeof(double));
  double *c2 = (double *) malloc(4L * Nspace * sizeof(double));
  Atom *He = atmos.elements[1].model;
  for (int la = 0; la < Nspect; la++) {
    double lw = spectrum.lambda[la];
    for (int c = 0; c < NC; c++) {
      bool_t ok = FALSE, two = TRUE;
      for (int k = 0; k < Nspace; k++) c1[k] = c2[k] = 0.0;
      switch (c) {
        case 0: Thomson(c2); ok = TRUE; break;
        case 1: ok = Hminus_bf(lw, c1, c2); break;
        case 2: ok = Hminus_ff(lw, c1); two = FALSE; break;
        case 3: ok = OH_bf_opac(lw, c1, c2); break;
        case 4: ok = CH_bf_opac(lw, c1, c2); break;
        case 5: ok = Hydrogen_bf(lw, c1, c2); break;
        case 6: Hydrogen_ff(lw, c1); ok = TRUE; two = FALSE; break;
        case 7: ok = Rayleigh(lw, atmos.H, c2); break;
        case 8: ok = He ? Rayleigh(lw, He, c2) : FALSE; break;
        case 9: ok = H2plus_ff(lw, c1); two = FALSE; break;
        case 10: ok = Rayleigh_H2(lw, c2); break;
        case 11: ok = H2minus_ff(lw, c1); two = FALSE; break;
        case 12: ok = Metal_bf(lw, atmos.Natom - 1, atmos.atoms + 1, c1, c2); break;
      }
      if (!ok) continue;
      double *dst = comp + (((size_t) c * 2) * Nspect + la) * Nspace;
      memcpy(dst, c1, Nspace * sizeof(double));
      if (two) memcpy(dst + (size_t) Nspect * Nspace, c2, Nspace * sizeof(double));
    }
  }
  write_f64(outdir, "comp", comp, (long) NC * 2 * Nspect * Nspace);
  free(comp); free(c1); free(c2);

  /* densities */
  double *z = (double *) calloc(Nspace, sizeof(double));
  int mp[3] = {atmos.H2 != NULL, atmos.OH != NULL, atmos.CH != NULL};
  write_f64(outdir, "T", atmos.T, Nspace);
  write_f64(outdir, "ne", atmos.ne, Nspace);
  write_f64(outdir, "nHmin", atmos.nHmin, Nspace);
  write_f64(outdir, "nH2", atmos.H2 ? atmos.H2->n : z, Nspace);
  write_f64(outdir, "nOH", atmos.OH ? atmos.OH->n : z, Nspace);
  write_f64(outdir, "nCH", atmos.CH ? atmos.CH->n : z, Nspace);
  write_i32(outdir, "mol_present", mp, 3);
  free(z);

  /* atomic data */
  int Natom = atmos.Natom, nlev = 0, ncont = 0, nline = 0, ntab = 0;
  for (int m = 0; m < Natom; m++) {
    Atom *at = &atmos.atoms[m];
    nlev += at->Nlevel; ncont += at->Ncont; nline += at->Nline;
    for (int kr = 0; kr < at->Ncont; kr++) ntab += at->continuum[kr].Nlambda;
  }
  int *meta = (int *) malloc(4L * Natom * sizeof(int));
  double *lev = (double *) malloc(3L * nlev * sizeof(double));
  double *pn = (double *) malloc((long) nlev * Nspace * sizeof(double));
  double *pst = (double *) malloc((long) nlev * Nspace * sizeof(double));
  double *cr = (double *) malloc(8L * (ncont > 0 ? ncont : 1) * sizeof(double));
  double *tb = (double *) malloc(2L * (ntab > 0 ? ntab : 1) * sizeof(double));
  double *lr = (double *) malloc(5L * (nline > 0 ? nline : 1) * sizeof(double));
  int il = 0, ic = 0, it = 0, ik = 0, he_index = -1, h_index = -1;
  for (int m = 0; m < Natom; m++) {
    Atom *at = &atmos.atoms[m];
    if (at == He) he_index = m;
    if (at == atmos.H) h_index = m;
    meta[4 * m] = at->Nlevel; meta[4 * m + 1] = at->Ncont;
    meta[4 * m + 2] = at->Nline; meta[4 * m + 3] = at->active;
    for (int i = 0; i < at->Nlevel; i++, il++) {
      lev[3 * il] = at->E[i]; lev[3 * il + 1] = at->g[i]; lev[3 * il + 2] = at->stage[i];
      memcpy(pn + (long) il * Nspace, at->n[i], Nspace * sizeof(double));
      memcpy(pst + (long) il * Nspace, at->nstar[i], Nspace * sizeof(double));
    }
    for (int kr = 0; kr < at->Ncont; kr++, ic++) {
      AtomicContinuum *c = &at->continuum[kr];
      double *r = cr + 8L * ic;
      r[0] = c->i; r[1] = c->j; r[2] = c->lambda0; r[3] = c->lambda[0];
      r[4] = c->hydrogenic; r[5] = c->alpha0; r[6] = c->Nlambda; r[7] = it;
      for (int t = 0; t < c->Nlambda; t++, it++) {
        tb[2L * it] = c->lambda[t];
        tb[2L * it + 1] = c->alpha[t];
      }
    }
    for (int kr = 0; kr < at->Nline; kr++, ik++) {
      AtomicLine *l = &at->line[kr];
      double *r = lr + 5L * ik;
      r[0] = l->i; r[1] = l->j; r[2] = l->lambda0; r[3] = l->qwing; r[4] = l->Aji;
    }
  }
  write_i32(outdir, "atoms_meta", meta, 4L * Natom);
  write_f64(outdir, "atoms_lev", lev, 3L * nlev);
  write_f64(outdir, "atoms_n", pn, (long) nlev * Nspace);
  write_f64(outdir, "atoms_nstar", pst, (long) nlev * Nspace);
  write_f64(outdir, "atoms_cont", cr, 8L * ncont);
  write_f64(outdir, "atoms_tab", tb, 2L * ntab);
  write_f64(outdir, "atoms_line", lr, 5L * nline);
  double misc[4] = {atmos.vmicro_char, he_index, h_index, Natom};
  write_f64(outdir, "misc", misc, 4);
  free(meta); free(lev); free(pn); free(pst); free(cr); free(tb); free(lr);
  free(a); free(w);
  return Nspect;
}

/* Set-up of rhf1d() with an ACTIVE atom, up to initScatter()
   (pyrh_compute1dray.c:130-323). */
static void nlte_setup(const char *cwd, double mu, int Ndep, double *a, int Nwave,
                       double *w)
{
  char tmp[512];
  snprintf(commandline.keyword_input, sizeof(commandline.keyword_input),
           "%s/keyword.input", cwd);
  setOptions(1, NULL);
  readInput();
  input.verbose = FALSE;
  input.get_populations = FALSE;
  input.pyrhHSE = FALSE;
  input.get_atomic_rfs = FALSE;
  input.n_atomic_pars = 0;
  snprintf(tmp, sizeof(tmp), "%s/%s", cwd, input.atoms_input);
  strcpy(input.atoms_input, tmp);
  snprintf(tmp, sizeof(tmp), "%s/%s", cwd, input.molecules_input);
  strcpy(input.molecules_input, tmp);
  if (strcmp(input.KuruczData, "none")) {
    snprintf(tmp, sizeof(tmp), "%s/%s", cwd, input.KuruczData);
    strcpy(input.KuruczData, tmp);
  }
  input.solve_ne = FALSE;
  spectrum.updateJ = TRUE;
  input.limit_memory = FALSE;
  input.solve_NLTE = FALSE;
  atmos.Nrlk = 0;
  geometry.Ndep = Ndep;
  MULTIatmos(&atmos, &geometry, 0, NULL, NULL);
  atmos.active_layer = -1;
  geometry.scale = TAU500;
  for (int k = 0; k < Ndep; k++) geometry.tau_ref[k] = POW10(a[k]);
  atmos.T = a + 1 * Ndep;
  atmos.ne = a + 2 * Ndep;
  geometry.vel = a + 3 * Ndep;
  atmos.vturb = a + 4 * Ndep;
  atmos.B = a + 5 * Ndep;
  atmos.gamma_B = a + 6 * Ndep;
  atmos.chi_B = a + 7 * Ndep;
  atmos.nHtot = a + 8 * Ndep;
  atmos.nH = matrix_double(atmos.NHydr, geometry.Ndep);
  atmos.Stokes = TRUE;
  atmos.moving = FALSE;
  for (int k = 0; k < Ndep; k++) {
    geometry.vel[k] *= KM_TO_M;
    atmos.vturb[k] *= KM_TO_M;
    atmos.ne[k] /= CUBE(CM_TO_M);
    atmos.nHtot[k] /= CUBE(CM_TO_M);
    atmos.B[k] /= 1e4;
  }
  for (int k = 0; k < Ndep; k++)
    if (fabs(geometry.vel[k]) >= atmos.vmacro_tresh) { atmos.moving = TRUE; break; }
  readAtomicModels();
  readMolecularModels();
  for (int n = 0; n < atmos.Natom; n++)
    if (atmos.atoms[n].active) { input.solve_NLTE = TRUE; break; }
  if (atmos.Stokes) Bproject();
  SortLambda(w, Nwave);
  getBoundary(&geometry);
  Background(FALSE, FALSE);
  convertScales(&atmos, &geometry);
  if (input.solve_NLTE) getProfiles();
  initSolution(FALSE);
  if (input.solve_NLTE) initScatter();
}

static void dump_matrix(const char *dir, const char *name, double **m, int n1, int n2)
{
  double *buf = (double *) malloc((long) n1 * n2 * sizeof(double));
  for (int i = 0; i < n1; i++) memcpy(buf + (long) i * n2, m[i], n2 * sizeof(double));
  write_f64(dir, name, buf, (long) n1 * n2);
  free(buf);
}

/* mode 0: dump the set-up, run one iteration by hand (Gamma, J, statEquil)
   and dump it.  mode 1: run Iterate() and _solveray() and dump the
   converged populations and the emergent intensity. */
/* Radiative rates of the active atom as addtoRates left them
   (rh/fillgamma.c:375-461): <prefix>_line [Nline][2][Nspace] and
   <prefix>_cont [Ncont][2][Nspace], R_ij then R_ji. */
static void dump_rates(const char *outdir, const char *prefix, Atom *atom, int Nspace)
{
  char name[64];
  double *r = (double *) malloc(2L * (atom->Nline + atom->Ncont + 1) * Nspace * sizeof(double));
  for (int kr = 0; kr < atom->Nline; kr++) {
    memcpy(r + (2L * kr) * Nspace, atom->line[kr].Rij, Nspace * sizeof(double));
    memcpy(r + (2L * kr + 1) * Nspace, atom->line[kr].Rji, Nspace * sizeof(double));
  }
  snprintf(name, sizeof(name), "%s_line", prefix);
  write_f64(outdir, name, r, 2L * atom->Nline * Nspace);
  for (int kr = 0; kr < atom->Ncont; kr++) {
    memcpy(r + (2L * kr) * Nspace, atom->continuum[kr].Rij, Nspace * sizeof(double));
    memcpy(r + (2L * kr + 1) * Nspace, atom->continuum[kr].Rji, Nspace * sizeof(double));
  }
  snprintf(name, sizeof(name), "%s_cont", prefix);
  write_f64(outdir, name, r, 2L * atom->Ncont * Nspace);
  free(r);
}

int harness_nlte(const char *cwd, double mu, int Ndep, const double *atm, int Nwave,
                 const double *lam, const char *outdir, int mode)
{
  double *a = (double *) malloc(9 * Ndep * sizeof(double));
  double *w = (double *) malloc(Nwave * sizeof(double));
  memcpy(a, atm, 9 * Ndep * sizeof(double));
  memcpy(w, lam, Nwave * sizeof(double));
  nlte_setup(cwd, mu, Ndep, a, Nwave, w);
  if (atmos.Nactiveatom != 1) return -1;
  Atom *atom = atmos.activeatoms[0];
  int Nspect = spectrum.Nspect, Nspace = atmos.Nspace, Nl = atom->Nlevel;

  if (mode == 0) {
    int mi[16] = {Nspect, Nspace, atmos.Nrays, Nl, atom->Nline, atom->Ncont,
                  input.NmaxIter, input.Ngdelay, input.Ngorder, input.Ngperiod,
                  input.isum, input.NmaxScatter, atmos.moving,
                  geometry.vboundary[TOP], geometry.vboundary[BOTTOM], 0};
    write_i32(outdir, "meta", mi, 16);
    double mf[4] = {input.iterLimit, atmos.lambda_ref, mu, atmos.totalAbund};
    write_f64(outdir, "fmeta", mf, 4);
    write_f64(outdir, "lambda", spectrum.lambda, Nspect);
    write_f64(outdir, "muz", geometry.muz, atmos.Nrays);
    write_f64(outdir, "wmu", geometry.wmu, atmos.Nrays);
    write_f64(outdir, "T", atmos.T, Nspace);
    write_f64(outdir, "ne", atmos.ne, Nspace);
    write_f64(outdir, "nHtot", atmos.nHtot, Nspace);
    write_f64(outdir, "vel", geometry.vel, Nspace);
    write_f64(outdir, "vturb", atmos.vturb, Nspace);
    write_f64(outdir, "height", geometry.height, Nspace);
    double *bg = (double *) malloc(3L * Nspect * Nspace * sizeof(double));
    int *hl = (int *) malloc(Nspect * sizeof(int));
    for (int la = 0; la < Nspect; la++) {
      memcpy(bg + (0L * Nspect + la) * Nspace, spectrum.chi_c_lam[la], Nspace * sizeof(double));
      memcpy(bg + (1L * Nspect + la) * Nspace, spectrum.eta_c_lam[la], Nspace * sizeof(double));
      memcpy(bg + (2L * Nspect + la) * Nspace, spectrum.sca_c_lam[la], Nspace * sizeof(double));
      hl[la] = atmos.backgrflags[la].hasline | (atmos.backgrflags[la].ispolarized << 1);
    }
    write_f64(outdir, "background", bg, 3L * Nspect * Nspace);
    write_i32(outdir, "bgflags", hl, Nspect);
    free(bg); free(hl);
    dump_matrix(outdir, "J0", spectrum.J, Nspect, Nspace);
    write_f64(outdir, "g", atom->g, Nl);
    write_f64(outdir, "E", atom->E, Nl);
    write_i32(outdir, "stage", atom->stage, Nl);
    dump_matrix(outdir, "nstar", atom->nstar, Nl, Nspace);
    dump_matrix(outdir, "n0", atom->n, Nl, Nspace);
    write_f64(outdir, "ntotal", atom->ntotal, Nspace);
    dump_matrix(outdir, "C", atom->C, Nl * Nl, Nspace);
    write_f64(outdir, "vbroad", atom->vbroad, Nspace);
    /* lines: [i, j, lambda0, Aji, Bji, Bij, isotope_frac, Nblue, Nlambda,
               symmetric, Ncomponent, c_shift0, c_fraction0, Voigt, PRD,
               polarized]; polarized: the line makes the active set
               polarized (containsPolarized, rh/opacity.c:574-589) */
    double *lr = (double *) calloc(16L * atom->Nline, sizeof(double));
    double *ad = (double *) calloc((long) atom->Nline * Nspace, sizeof(double));
    double *wp = (double *) calloc((long) atom->Nline * Nspace, sizeof(double));
    double *ph = (double *) calloc((long) atom->Nline * 5 * 2 * atmos.Nrays * Nspace, sizeof(double));
    int *phla = (int *) calloc(atom->Nline * 5, sizeof(int));
    for (int kr = 0; kr < atom->Nline; kr++) {
      AtomicLine *l = &atom->line[kr];
      double *r = lr + 16L * kr;
      r[0] = l->i; r[1] = l->j; r[2] = l->lambda0; r[3] = l->Aji; r[4] = l->Bji;
      r[5] = l->Bij; r[6] = l->isotope_frac; r[7] = l->Nblue; r[8] = l->Nlambda;
      r[9] = l->symmetric; r[10] = l->Ncomponent;
      r[11] = l->Ncomponent > 0 ? l->c_shift[0] : 0.0;
      r[12] = l->Ncomponent > 0 ? l->c_fraction[0] : 1.0;
      r[13] = l->Voigt; r[14] = l->PRD;
      r[15] = atmos.Stokes && input.StokesMode != FIELD_FREE && l->polarizable;
      if (l->Voigt) Damping(l, ad + (long) kr * Nspace);
      memcpy(wp + (long) kr * Nspace, l->wphi, Nspace * sizeof(double));
      int sel[5] = {0, l->Nlambda / 4, l->Nlambda / 2, (3 * l->Nlambda) / 4, l->Nlambda - 1};
      /* the profile is stored per (lambda, ray, direction) only where it
         depends on the angle (rh/profile.c:154-170); otherwise one row per
         lambda serves every ray and direction */
      int angle_dep = atmos.moving || (l->polarizable && input.StokesMode > FIELD_FREE);
      for (int s = 0; s < 5; s++) {
        phla[kr * 5 + s] = sel[s];
        for (int q = 0; q < 2 * atmos.Nrays; q++) {
          int lamu = angle_dep ? 2 * atmos.Nrays * sel[s] + q : sel[s];
          memcpy(ph + (((long) kr * 5 + s) * 2 * atmos.Nrays + q) * Nspace, l->phi[lamu],
                 Nspace * sizeof(double));
        }
      }
    }
    write_f64(outdir, "lines", lr, 16L * atom->Nline);
    write_f64(outdir, "adamp", ad, (long) atom->Nline * Nspace);
    write_f64(outdir, "wphi", wp, (long) atom->Nline * Nspace);
    write_f64(outdir, "phi_sample", ph, (long) atom->Nline * 5 * 2 * atmos.Nrays * Nspace);
    write_i32(outdir, "phi_sample_la", phla, atom->Nline * 5);
    free(lr); free(ad); free(wp); free(ph); free(phla);
    /* continua: [i, j, Nblue, Nlambda, lambda0, hydrogenic] + alpha */
    int na = 0;
    for (int kr = 0; kr < atom->Ncont; kr++) na += atom->continuum[kr].Nlambda;
    double *cr = (double *) calloc(8L * atom->Ncont, sizeof(double));
    double *al = (double *) calloc(na > 0 ? na : 1, sizeof(double));
    int off = 0;
    for (int kr = 0; kr < atom->Ncont; kr++) {
      AtomicContinuum *c = &atom->continuum[kr];
      double *r = cr + 8L * kr;
      r[0] = c->i; r[1] = c->j; r[2] = c->Nblue; r[3] = c->Nlambda; r[4] = c->lambda0;
      r[5] = c->hydrogenic; r[6] = off;
      memcpy(al + off, c->alpha, c->Nlambda * sizeof(double));
      off += c->Nlambda;
    }
    write_f64(outdir, "continua", cr, 8L * atom->Ncont);
    write_f64(outdir, "alpha", al, na > 0 ? na : 1);
    free(cr); free(al);

    /* one iteration by hand: Gamma = C + radiative (Iterate, iterate.c:86-97) */
    initGammaAtom(atom);
    solveSpectrum(TRUE, FALSE);
    dump_matrix(outdir, "Gamma1", atom->Gamma, Nl * Nl, Nspace);
    dump_matrix(outdir, "J1", spectrum.J, Nspect, Nspace);
    dump_rates(outdir, "R1", atom, Nspace);
    statEquil(atom, input.isum);
    dump_matrix(outdir, "n1", atom->n, Nl, Nspace);
  } else {
    Iterate(input.NmaxIter, input.iterLimit);
    dump_matrix(outdir, "n_final", atom->n, Nl, Nspace);
    dump_rates(outdir, "R_final", atom, Nspace);
    dump_matrix(outdir, "J_final", spectrum.J, Nspect, Nspace);
    mySpectrum spec;
    spec.nlw = spectrum.Nspect;
    spec.Nrays = atmos.Nrays;
    _solveray(mu, &spec);
    write_f64(outdir, "lam_out", spec.lam, spec.nlw);
    write_f64(outdir, "I_out", spec.sI, spec.nlw);
    int mo[2] = {spec.nlw, 0};
    write_i32(outdir, "out_meta", mo, 2);
  }
  return Nspect;
}
