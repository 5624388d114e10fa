/* pyrh_gb300.h -- C ABI of the GB300 radiative-transfer hot path.
 *
 * Drop-in boundary for the polarized LTE synthesis that the reference runs
 * per atmosphere through rhf1d() (rh/rhf1d/pyrh_compute1dray.h:26-36, bound
 * to Python by pyrh.compute1d, pyrh.pyx:537-668).  The synthesis takes the
 * set-up that rhf1d() does before its hot loop -- LTE stage densities,
 * background continuum, tau500 -> height -- as arrays, from the caller or
 * from the set-up entry points further down (readers of the input files,
 * element tables, LTE populations, n_e, chemical equilibrium, background,
 * depth scales, hydrostatic equilibrium); it runs, on one GB300:
 *   - the Kurucz-line Zeeman/Voigt opacity of rlk_opacity()/RLKProfile()
 *     (rh/kurucz.c:511-827, Humlicek 1982 Voigt, rh/humlicek.c:28-118),
 *   - the formal solution of Formal() (rh/rhf1d/formal.c:44-346): DELO-Bezier3
 *     Stokes (rh/rhf1d/bezier_1D.c:52-300) where a polarizable line covers the
 *     wavelength, the scalar Bezier3 solver (bezier_1D.c:306-541) for NO_STOKES
 *     and where only unpolarizable lines cover it, and the Feautrier solver
 *     (rh/rhf1d/feautrier.c:56-202) where no line covers it -- or, in a static
 *     atmosphere (cfg->moving = 0), no polarizable line (formal.c:96-101),
 * for many atmospheres (pixels) at once.  Only the ray towards the observer
 * is solved: the emergent Stokes vector does not depend on the other
 * direction that Formal() also integrates in LTE.
 *
 * Conventions
 *   - All pointers in pyrh_lte_batch and pyrh_line are DEVICE pointers
 *     (caller-owned, cudaMalloc'd) unless a function says otherwise.
 *   - Units are SI, as the reference holds them after pyrh_compute1dray.c:
 *     263-270: height [m], T [K], ne/nHtot/np [m^-3], v [m/s], B [T],
 *     angles [rad], wavelengths [nm, vacuum].
 *   - Inputs are never modified (the reference mutates its inputs in place
 *     during a call, pyrh_compute1dray.c:263-270,351-357; this library does not).
 *   - Every entry point returns a pyrh_status; none calls exit().
 */
#ifndef PYRH_GB300_H
#define PYRH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PYRH_OK = 0,
  PYRH_ERR_ARG = 1,          /* bad shape, count, pointer or option */
  PYRH_ERR_UNSUPPORTED = 2,  /* input outside what the kernels implement */
  PYRH_ERR_CUDA = 3,         /* a CUDA runtime call failed */
  PYRH_ERR_NONCONVERGED = 4, /* iteration limit reached before convergence */
  PYRH_ERR_SINGULAR = 5,     /* singular rate matrix */
  PYRH_ERR_TIMEOUT = 6       /* device-side iteration budget exhausted */
} pyrh_status;

typedef enum { PYRH_FP64 = 0, PYRH_FP32 = 1 } pyrh_precision;

/* STOKES_MODE of keyword.input (rh/inputs.h): FULL_STOKES solves I,Q,U,V with
   DELO-Bezier3; NO_STOKES solves I with the scalar Bezier3 solver (Zeeman
   broadened profile, formal.c:94-95,225-235). */
typedef enum { PYRH_NO_STOKES = 0, PYRH_FULL_STOKES = 3 } pyrh_stokes_mode;

/* enum vdWaals of the reference (rh/atom.h:31). */
typedef enum {
  PYRH_VDW_UNSOLD = 0, PYRH_VDW_RIDDER = 1, PYRH_VDW_BARKLEM = 2, PYRH_VDW_KURUCZ = 3
} pyrh_vdw;

#define PYRH_MAX_LINES      16
#define PYRH_MAX_COMPONENTS 32   /* Zeeman components per line */
#define PYRH_MAX_DEPTH      512

/* One Kurucz (RLK) line after readKuruczLines()/RLKZeeman() have derived its
   constants; the fields of RLK_Line (rh/atom.h:156-167) that the opacity uses. */
typedef struct {
  double lambda0;          /* vacuum line centre [nm] */
  double Ei;               /* lower level energy [J] */
  double gi;               /* lower level statistical weight */
  double Aji, Bji, Bij;    /* Einstein coefficients (SI, per unit frequency) */
  double Grad, GStark, GvdWaals;   /* [s^-1], [m^3 s^-1], [m^3 s^-1] */
  double cross, alpha;     /* Unsold / Barklem cross-section parameters */
  double isotope_frac, hyperfine_frac;
  double weight;           /* element atomic weight [amu] */
  int32_t vdwaals;         /* pyrh_vdw */
  int32_t contributes;     /* element abundance set and stage < Nstage-1
                              (kurucz.c:614) and not covered by a model atom */
  int32_t polarizable;     /* kurucz.c:296,384-387 */
  int32_t ncomp;           /* Zeeman components (RLKZeeman, kurucz.c:832-920) */
  int32_t comp_q[PYRH_MAX_COMPONENTS];        /* Ml - Mu in {-1, 0, 1} */
  double  comp_shift[PYRH_MAX_COMPONENTS];    /* gLl*Ml - gLu*Mu */
  double  comp_strength[PYRH_MAX_COMPONENTS]; /* normalised per q */
} pyrh_line;

/* Temperature derivatives of the set-up quantities, for response functions
   and gradients that follow the temperature through the set-up.  The
   reference's response functions are finite differences of its whole
   synthesis (rh/rhf1d/rf_ray.c:205-293): every perturbed temperature re-runs
   Background() (continuum, LTE stage densities, proton density) and
   convertScales() (the height scale from tau_500,
   rh/rhf1d/multiatmos.c:126-138), so its temperature response includes how
   those inputs move with T.  Given these derivatives, pyrh_lte_rf,
   pyrh_lte_chi2_grad and pyrh_lte_stokes_vjp add the same terms.  Each
   pointer may be NULL, which holds that input fixed.  The set-up is local in
   depth: every derivative is with respect to the temperature of the same
   depth, except the interval lengths, which depend on the temperatures at
   both ends of their interval.  Device pointers, laid out like the batch
   arrays they differentiate. */
typedef struct {
  const void *dchi_c;          /* d chi_c / dT: layout and type of chi_c */
  const void *deta_c;          /* d eta_c / dT */
  const double *dline_pops;    /* [nline][2][sum ndep]: d n_stage/dT, d ln U/dT */
  const double *dnp;           /* [sum ndep]: d n_p / dT */
  const double *dlen_up;       /* [sum ndep]: entry k >= 1 of an atmosphere,
                                  d|height[k] - height[k-1]| / dT[k-1] */
  const double *dlen_dn;       /* [sum ndep]: entry k >= 1,
                                  d|height[k] - height[k-1]| / dT[k] */
} pyrh_lte_setup_dT;

/* A batch of atmospheres with possibly uneven depth and wavelength counts.
   Atmosphere p owns depths [depth_off[p], depth_off[p] + ndep[p]) of every
   per-depth array, wavelengths [lam_off[p], lam_off[p] + nlam[p]) of lambda,
   continuum entries [cont_off[p], cont_off[p] + ndep[p]*nlam[p]) laid out
   [depth][lambda] (lambda fastest), and output entries
   [4*lam_off[p], 4*lam_off[p] + 4*nlam[p]) laid out [stokes][lambda]. */
typedef struct {
  int32_t natm;
  int32_t max_ndep;            /* host value: max over ndep[] */
  int32_t max_nlam;            /* host value: max over nlam[] */
  int64_t total_depth;         /* host value: length of the per-depth arrays */
  const int32_t *ndep;         /* [natm] (3 <= ndep <= PYRH_MAX_DEPTH) */
  const int64_t *depth_off;    /* [natm] */
  const int32_t *nlam;         /* [natm] */
  const int64_t *lam_off;      /* [natm] */
  const int64_t *cont_off;     /* [natm] */
  const double *lambda;        /* [sum nlam] vacuum wavelength [nm] */
  const double *height, *T, *ne, *nHtot, *np, *vturb, *vlos, *B, *gamma_B, *chi_B;
  const double *line_pops;     /* [nline][2][sum ndep]: n[stage] [m^-3] and
                                  ln U(T) of the line's ionisation stage,
                                  as used in kurucz.c:662-677 */
  const void *chi_c;           /* continuum opacity [m^-1] (float or double,
                                  following the precision) */
  const void *eta_c;           /* continuum emissivity [W m^-3 Hz^-1 sr^-1] */
  const pyrh_lte_setup_dT *setup_dT;  /* optional HOST pointer (NULL: the
                                  set-up is held fixed); read only by the
                                  response-function entry points */
} pyrh_lte_batch;

typedef struct {
  int32_t precision;           /* pyrh_precision: FP32 also selects float
                                  chi_c/eta_c/output */
  int32_t stokes_mode;         /* pyrh_stokes_mode */
  int32_t magneto_optical;     /* MAGNETO_OPTICAL */
  int32_t moving;              /* atmos.moving (pyrh_compute1dray.c:272-278) */
  double  mu;                  /* cosine of the ray to the observer */
  double  vmicro_char;         /* VMICRO_CHAR [m/s]: line window 20 v/c */
  int32_t block_lambda;        /* wavelengths per block; 0 = tuned default */
  int32_t persistent_blocks;   /* 0: one block per (atmosphere, wavelength
                                  tile); > 0: at most this many blocks, each
                                  looping over tiles */
} pyrh_lte_config;

/* Emergent Stokes vectors for a batch; replaces the per-atmosphere hot loop
   of rhf1d() -> Iterate() -> solveSpectrum() -> Formal() with the background
   line opacity of Background() -> rlk_opacity() (background.c:519-546).
   stokes_out: [4 * sum nlam], float or double following the precision.
   lines: device array of nline pyrh_line.  stream: a cudaStream_t or NULL. */
pyrh_status pyrh_lte_stokes(const pyrh_lte_batch *batch, const pyrh_line *lines,
                            int32_t nline, const pyrh_lte_config *cfg,
                            void *stokes_out, void *stream);

/* Validates a HOST copy of a line table (component counts and q values,
   sort order, polarizable lines only where a Voigt profile is needed).
   pyrh_lte_stokes does not read its device table back to check it. */
pyrh_status pyrh_check_lines(const pyrh_line *host_lines, int32_t nline,
                             int32_t stokes_mode);

/* Same computation with HOST inputs and outputs: copies the batch to the
   device, runs pyrh_lte_stokes and copies the Stokes vectors back, all
   inside the call (the shape of a compute1d()-style call,
   pyrh.pyx:621-642).  When the atmospheres' depths, wavelengths, continuum
   and spectra follow one another in memory, the batch is uploaded in chunks
   of atmospheres (about 128 MB of continuum each, after a lead chunk of an
   eighth of that, so that the first launch waits for little), each
   synthesised on a second internal stream while the next uploads, and its
   spectra copied back on a third; pyrh_last_launch_count() then reports one
   launch per chunk.  Host
   buffers in page-locked memory let the copies run at full speed.  Device
   buffers are cached between calls with the same or smaller sizes.  Not
   re-entrant (one internal workspace). */
pyrh_status pyrh_lte_stokes_host(const pyrh_lte_batch *host_batch,
                                 const pyrh_line *host_lines, int32_t nline,
                                 const pyrh_lte_config *cfg, void *host_stokes_out);

/* A launch plan for one resident batch: pyrh_lte_plan_create times every
   wavelength tile (block_lambda, multiples of 32 up to 256 and up to the
   batch's widest spectrum) on the caller's buffers, keeps the fastest, and
   records one launch of pyrh_lte_stokes with it as a CUDA graph bound to
   those buffers (batch arrays, lines, stokes_out).  pyrh_lte_plan_launch
   replays the graph on any stream; the buffers' contents may change between
   launches, their addresses and the batch shape may not.  cfg->block_lambda
   is ignored (tuned); cfg->persistent_blocks is kept.  stream: a
   cudaStream_t (NULL uses an internal stream for the tuning launches and
   the capture).  The reference has no counterpart: it makes one call per
   atmosphere. */
typedef struct pyrh_lte_plan_s *pyrh_lte_plan;
pyrh_status pyrh_lte_plan_create(const pyrh_lte_batch *batch, const pyrh_line *lines,
                                 int32_t nline, const pyrh_lte_config *cfg, void *stokes_out,
                                 void *stream, pyrh_lte_plan *plan_out);
pyrh_status pyrh_lte_plan_launch(pyrh_lte_plan plan, void *stream);
/* The tuned tile and its measured time per launch [ms]. */
int32_t pyrh_lte_plan_block(pyrh_lte_plan plan);
double pyrh_lte_plan_ms(pyrh_lte_plan plan);
void pyrh_lte_plan_destroy(pyrh_lte_plan plan);

/* ------------------------------------------------------- response functions
 * Depth-resolved response functions of the emergent Stokes vector of
 * pyrh_lte_stokes to the atmosphere at every depth, and the gradient of a
 * weighted chi^2, by a hand-written adjoint of the DELO-Bezier3 recurrence
 * and of the Zeeman/Voigt opacity.  The reference computes the same
 * derivatives by finite differences of whole syntheses (rh/rhf1d/
 * rf_ray.c:205-293, perturbing T, v, v_turb, B, gamma, chi per depth); its
 * only analytical response functions are for log gf (rh/rhf1d/
 * bezier_1D.c:416-490).  Parameters, in this order and in the units of
 * pyrh_lte_batch: T [K], v_los [m/s], v_mic [m/s], B [T], gamma_B [rad],
 * chi_B [rad].  The continuum (chi_c, eta_c), stage densities and the
 * height scale are held fixed unless batch->setup_dT gives their
 * temperature derivatives (then T follows them, as the reference's finite
 * differences re-run its set-up).  Each wavelength is solved, and
 * differentiated, with the reference's solver for it: DELO-Bezier3 where a
 * polarizable line covers it (FULL_STOKES), scalar Bezier3 for NO_STOKES or
 * where only unpolarizable lines cover it, Feautrier where no line does (in
 * a static atmosphere also where no polarizable line does).
 * Without magneto-optical terms only.  cfg->block_lambda (0: 128) is the
 * wavelength tile of one work item: up to 256 in FP32, 128 in FP64. */
#define PYRH_RF_NPARAM    6
#define PYRH_RF_MAX_DEPTH 160

/* rf_out (float or double following the precision): for atmosphere p,
   entries [24 * cont_off[p], 24 * (cont_off[p] + ndep[p] * nlam[p])) laid
   out [stokes][param][depth][lambda] (lambda fastest): dS_s(lambda)/dx(k).
   rf_loggf_out (optional, NULL to skip): dS_s(lambda)/d log10(gf) of every
   line, entries [4 * nline * lam_off[p], 4 * nline * (lam_off[p] + nlam[p]))
   laid out [line][stokes][lambda] -- the atomic-parameter response functions
   of compute1d(..., get_atomic_rfs=True) (pyrh.pyx:537-668), there for
   Stokes I of NO_STOKES syntheses only.
   stokes_out receives the emergent Stokes vectors as for pyrh_lte_stokes. */
pyrh_status pyrh_lte_rf(const pyrh_lte_batch *batch, const pyrh_line *lines, int32_t nline,
                        const pyrh_lte_config *cfg, void *stokes_out, void *rf_out,
                        void *rf_loggf_out, void *stream);

/* chi2[p] = sum over lambda and s of weights * (S_s(lambda) - obs)^2, with
   obs and weights laid out like stokes_out; grad_out is [6][total_depth]
   (d chi2[p] / d x(k) at param * total_depth + depth_off[p] + k);
   grad_loggf_out (optional) is [natm][nline], d chi2[p] / d log10(gf_l).
   The outputs are overwritten. */
pyrh_status pyrh_lte_chi2_grad(const pyrh_lte_batch *batch, const pyrh_line *lines,
                               int32_t nline, const pyrh_lte_config *cfg, const void *obs,
                               const void *weights, void *stokes_out, void *chi2_out,
                               void *grad_out, void *grad_loggf_out, void *stream);

/* Vector-Jacobian product: grad_out[x * total_depth + depth_off[p] + k] =
   sum over lambda and s of dL_dstokes * dS_s(lambda)/dx(k), with dL_dstokes
   laid out like stokes_out (the adjoint a reverse-mode framework calls with
   the upstream gradient); grad_loggf_out (optional) [natm][nline] as for
   pyrh_lte_chi2_grad.  The outputs are overwritten. */
pyrh_status pyrh_lte_stokes_vjp(const pyrh_lte_batch *batch, const pyrh_line *lines,
                                int32_t nline, const pyrh_lte_config *cfg,
                                const void *dL_dstokes, void *stokes_out, void *grad_out,
                                void *grad_loggf_out, void *stream);

/* ------------------------------------------------------------------ NLTE
 * MALI lambda iteration for one active atom per atmosphere, replacing the
 * reference's Iterate() (rh/iterate.c:48-143) with its solveSpectrum() /
 * Formal() passes (profiles, rh/profile.c:67-371; opacity, rh/opacity.c:
 * 64-300; Gamma and cross-coupling, rh/fillgamma.c:82-332), statEquil()
 * (rh/statequil.c:40-102, LU of rh/ludcmp.c:36-177), Ng acceleration
 * (rh/accelerate.c:34-146) and MaxChange() (rh/maxchange.c:32-50), and the
 * emergent intensity of _solveray() (rh/rhf1d/pyrh_solveray.c:82-150).
 * The caller supplies the state that the reference's set-up leaves behind
 * (LTE populations, collision matrix, background, damping, cross-sections).
 * The formal solution is the scalar one of STOKES_MODE = NO_STOKES: with
 * FULL_STOKES the reference solves for I, Q, U, V wherever a polarizable
 * line is in window (formal.c:92-101), which this entry does not.  A
 * wavelength takes scalar Bezier3 in both directions of every ray where it
 * is angle dependent -- a polarized line in its active set or a polarized
 * background (even in a static atmosphere: the reference always sets
 * atmos.Stokes, pyrh_compute1dray.c:85, and only FIELD_FREE makes a set
 * unpolarized, opacity.c:574-589), or, in a moving atmosphere, any line --
 * and Feautrier once per ray otherwise (formal.c:92-101, 284-310).
 */
#define PYRH_NLTE_MAX_LEVELS  8
#define PYRH_NLTE_MAX_ACTIVE  16   /* transitions active at one wavelength */
#define PYRH_NLTE_MAX_RAYS    8
#define PYRH_NLTE_MAX_DEPTH   160
#define PYRH_NLTE_MAX_NG      4

/* One radiative transition of the active atom of one atmosphere. */
typedef struct {
  int32_t type;          /* 0 = bound-bound line, 1 = bound-free continuum */
  int32_t i, j;          /* lower and upper level */
  int32_t nblue;         /* first spectrum index (rh/sortlambda.c:296-355) */
  int32_t nlambda;       /* number of spectrum points covered */
  int32_t symmetric;     /* line->symmetric (getlambda.c:194) */
  int32_t voigt;         /* line->Voigt (damping used) */
  int32_t line_index;    /* row of adamp for lines */
  int32_t polarized;     /* lines: line->polarizable with STOKES_MODE other than
                            FIELD_FREE: its wavelengths are angle dependent
                            (containsPolarized, opacity.c:574-589) */
  int32_t reserved;      /* 0 */
  int64_t phi_off;       /* line profile block offset in the workspace */
  int64_t alpha_off;     /* continua: first cross-section in alpha[] */
  double lambda0, Aji, Bji, Bij, isotope_frac, c_shift, c_fraction;
} pyrh_nlte_transition;

/* A batch of atmospheres, each with the same number of atomic levels and
   its own depth grid, spectrum and transition table.  Arrays indexed by
   depth use depth_off[p] + k; spectral arrays lam_off[p] + la; per
   (lambda, depth) arrays cont_off[p] + k*nspect[p] + la (lambda fastest);
   per (level, depth) arrays (i*total_depth + depth_off[p] + k); the rate
   matrix C ((i*nlevel + j)*total_depth + depth_off[p] + k). */
typedef struct {
  int32_t natm, nlevel, max_ndep, max_nspect, max_nline;
  int64_t total_depth, total_lambda, total_cont;
  const int32_t *ndep, *nspect, *ntrans;          /* [natm] */
  const int64_t *depth_off, *lam_off, *cont_off, *trans_off, *adamp_off;  /* [natm] */
  const double *lambda;                           /* [total_lambda] nm */
  const double *height, *T, *vel, *vbroad, *ntotal;   /* [total_depth] SI */
  const double *nstar;                            /* [nlevel][total_depth] */
  const double *C;                                /* [nlevel^2][total_depth] */
  const double *chi_c, *eta_c, *sca_c;            /* [total_cont] */
  const int32_t *bgline;                          /* [total_lambda]: backgrflags,
                                  bit 0 hasline (a background line covers
                                  the wavelength: angle dependent with
                                  cfg->moving), bit 1 ispolarized (angle
                                  dependent; formal.c:92-101).  Background
                                  lines enter through chi_c/eta_c, Stokes I
                                  only (the I, Q, U, V solve of FULL_STOKES
                                  is outside this entry) */
  const pyrh_nlte_transition *trans;              /* [sum ntrans] */
  const double *alpha;                            /* continuum cross-sections */
  const double *adamp;                            /* [sum nline*ndep] */
  double *n;        /* [nlevel][total_depth]: start populations, then result */
  double *J;        /* [total_cont]: start mean intensity, then the last one */
  /* Optional (NULL: not kept): the radiative rates of every transition
     after its atmosphere's last formal solution, as addtoRates leaves them
     (rh/fillgamma.c:375-461; zeroed before each formal solution,
     rh/iterate.c:178): R_ij in slot 2t and R_ji in slot 2t + 1 of
     transition t (the atmosphere's table order), [2 max_ntrans][total_depth],
     s^-1.  max_ntrans >= every ntrans[p]; read only with rates. */
  int32_t max_ntrans;
  double *rates;
} pyrh_nlte_batch;

typedef struct {
  int32_t precision;      /* formal solution: PYRH_FP64 or PYRH_FP32; rates,
                             LU, Ng and convergence are always FP64 */
  int32_t nrays;
  double  muz[PYRH_NLTE_MAX_RAYS], wmu[PYRH_NLTE_MAX_RAYS];
  int32_t moving;         /* atmos.moving */
  int32_t isum;           /* I_SUM (-1: eliminate the most populated level) */
  int32_t ng_order, ng_delay, ng_period;
  int32_t nmax_iter;
  double  iter_limit;
} pyrh_nlte_config;

/* Bytes of device workspace pyrh_nlte_solve / pyrh_nlte_emergent need:
   the line profiles (phi_elems values: sum over atmospheres and lines of
   nlambda * 2 * nrays * ndep, addressed by the transitions' phi_off), their
   normalisation, a second mean-intensity buffer, the rate matrices, the Ng
   history and per-atmosphere iteration state. */
size_t pyrh_nlte_workspace_bytes(const pyrh_nlte_batch *batch, const pyrh_nlte_config *cfg,
                                 int64_t phi_elems);

/* Solves the batch; iterations[p] (device, int32) and dpops[p] (device,
   double) receive each atmosphere's iteration count and last convergence
   metric.  Returns PYRH_ERR_NONCONVERGED if an atmosphere reached nmax_iter
   above iter_limit. */
pyrh_status pyrh_nlte_solve(const pyrh_nlte_batch *batch, const pyrh_nlte_config *cfg,
                            void *workspace, size_t workspace_bytes,
                            int32_t *iterations, double *dpops, void *stream);

/* Emergent intensity at mu_out for every spectrum point with the batch's
   populations n and mean intensity J (pyrh_solveray.c:82-150); I_out is
   [total_lambda] (FP64). */
pyrh_status pyrh_nlte_emergent(const pyrh_nlte_batch *batch, const pyrh_nlte_config *cfg,
                               double mu_out, void *workspace, size_t workspace_bytes,
                               double *I_out, void *stream);

/* Size of the device array that pyrh_nlte_solve_static uses as scratch. */
#define PYRH_NLTE_STATIC_SCRATCH_BYTES (32u * 1024u * 1024u)

/* pyrh_nlte_solve for callers that cannot allocate device memory (their
   device memory belongs to another component's pool, their host forbids
   device allocation after start-up, or an allocation's implicit
   synchronisation is not acceptable).  No counterpart exists in the
   reference; it is the same solve as pyrh_nlte_solve with the workspace
   replaced by a fixed array of PYRH_NLTE_STATIC_SCRATCH_BYTES in device
   memory that every GPU loading this library holds until the process exits.
   phi_elems is the line-profile size of the batch (as for
   pyrh_nlte_workspace_bytes); batches whose scratch does not fit, or with
   more than 256 atmospheres, are rejected with PYRH_ERR_ARG.  The call
   allocates nothing.  Every call looks up the array's device address in
   the current context (cudaGetSymbolAddress, with the caller's device
   current) instead of keeping it from an earlier call, so a cudaDeviceReset
   or another context on the same device between calls is safe; the first
   call on a device also loads this library's device code there if that has
   not happened yet, so make that first call before any stream capture.
   Nothing in the array has to start at zero: the call clears its error
   word and its flags, and every kernel writes the rest (or zeroes it)
   before reading it, so each call may find the previous call's contents
   there.  All calls share the one array: calls
   that overlap on the GPU (other streams, other host threads) race on it. */
pyrh_status pyrh_nlte_solve_static(const pyrh_nlte_batch *batch, const pyrh_nlte_config *cfg,
                                   int64_t phi_elems, int32_t *iterations, double *dpops,
                                   void *stream);

/* ====================================================================
 * Host-side set-up (no device work): the RH model atom, the wavelength
 * grids of its transitions, the global wavelength grid and the output
 * index.  These restate the reference's set-up so that a caller can build
 * pyrh_nlte_batch wavelength tables (lambda, transition nblue / nlambda,
 * continuum cross-sections) from the *.atom file and keyword values the
 * reference reads, with bit-identical grids and integer ranges.
 * ==================================================================== */
#define PYRH_ATOM_MAX_LEVELS      64
#define PYRH_ATOM_MAX_LINES       128
#define PYRH_ATOM_MAX_CONT        64
#define PYRH_ATOM_MAX_COMPONENTS  8
#define PYRH_ATOM_MAX_TABLE       4096   /* explicit continuum table rows */
#define PYRH_ATOM_MAX_COLL        512    /* tabulated collision records */
#define PYRH_ATOM_MAX_COLLVALS    8192   /* their temperatures and values */
#define PYRH_ATOM_LABEL           20

typedef enum {
  PYRH_ATOM_VDW_UNSOLD = 0, PYRH_ATOM_VDW_RIDDER_RENSBERGEN = 1, PYRH_ATOM_VDW_BARKLEM = 2
} pyrh_atom_vdw;

typedef enum {
  PYRH_COLL_OMEGA = 0, PYRH_COLL_CE = 1, PYRH_COLL_CI = 2, PYRH_COLL_CP = 3, PYRH_COLL_CH = 4,
  PYRH_COLL_CH0 = 5, PYRH_COLL_CHP = 6, PYRH_COLL_CR = 7
} pyrh_coll_type;

typedef struct {
  double E;              /* J (from E_cm * h c / cm, readatom.c:204) */
  double E_cm;           /* as read, cm^-1 */
  double g;
  int32_t stage, abo_level;
  char label[PYRH_ATOM_LABEL + 4];
} pyrh_atom_level;

typedef struct {
  int32_t i, j;                  /* lower, upper level */
  int32_t nlambda;               /* as read */
  int32_t symmetric;             /* no ASYMM keyword */
  int32_t voigt, prd, vdwaals, ncomponent;
  double f, lambda0;             /* oscillator strength; vacuum nm */
  double Aji, Bji, Bij;
  double qcore, qwing;
  double cvdw[4], Grad, cStark, g_lande_eff;
  double c_shift[PYRH_ATOM_MAX_COMPONENTS], c_fraction[PYRH_ATOM_MAX_COMPONENTS];
} pyrh_atom_line;

typedef struct {
  int32_t i, j, nlambda, hydrogenic;
  double alpha0, lambda0, lambda_min;   /* m^2, vacuum nm, nm */
  int64_t table_off;                    /* explicit: rows in table_lambda/alpha */
} pyrh_atom_cont;

typedef struct {
  int32_t type, i, j, ntemp;
  int32_t temp_off, value_off;          /* into coll_values */
} pyrh_atom_coll;

typedef struct {
  char id[4];
  int32_t nlevel, nline, ncont, nfixed, ntable, ncoll, ncoll_values;
  pyrh_atom_level level[PYRH_ATOM_MAX_LEVELS];
  pyrh_atom_line line[PYRH_ATOM_MAX_LINES];
  pyrh_atom_cont cont[PYRH_ATOM_MAX_CONT];
  double table_lambda[PYRH_ATOM_MAX_TABLE], table_alpha[PYRH_ATOM_MAX_TABLE];
  pyrh_atom_coll coll[PYRH_ATOM_MAX_COLL];
  double coll_values[PYRH_ATOM_MAX_COLLVALS];
} pyrh_atom;

/* Keyword values the grids depend on. */
typedef struct {
  double vmicro_char;    /* m/s (VMICRO_CHAR, km/s in keyword.input) */
  double B_char;         /* T (B_STRENGTH_CHAR) */
  int32_t moving;        /* atmos.moving */
  int32_t stokes;        /* atmos.Stokes (pyrh sets it TRUE in every mode) */
} pyrh_grid_config;

/* Parses the text of an RH .atom file (replaces readAtom, rh/readatom.c:
   62-470): levels, bound-bound and bound-free transitions, and the
   tabulated collision records (TEMP, OMEGA, CE, CI, CP, CH, CH0, CH+, CR).
   Returns PYRH_ERR_UNSUPPORTED for other collision types or beyond the
   PYRH_ATOM_MAX_* limits. */
pyrh_status pyrh_atom_read(const char *text, pyrh_atom *atom);

/* Effective Lande factor of line kr (effectiveLande, rh/zeeman.c:106-125)
   and whether it is polarizable for an active atom (readatom.c:347-366):
   1 yes, 0 no, -1 a composite line that would be (an error there). */
double pyrh_atom_lande_eff(const pyrh_atom *atom, int32_t kr);
int32_t pyrh_atom_line_polarizable(const pyrh_atom *atom, int32_t kr, int32_t stokes);

/* Wavelength grid of line kr (getLambda, rh/getlambda.c:44-162) and of
   continuum kr (getLambdaCont, rh/getlambda.c:166-180, or its explicit
   table).  With lam NULL only the point count is returned; -1 on error. */
int32_t pyrh_line_grid(const pyrh_atom *atom, int32_t kr, const pyrh_grid_config *cfg,
                       double *lam, int32_t cap);
int32_t pyrh_cont_grid(const pyrh_atom *atom, int32_t kr, double *lam, int32_t cap);

/* Global wavelength grid (SortLambda, rh/sortlambda.c:42-420): lambda_ref
   (if > 0), the caller's wavelengths and the transition grids (ngrid
   grids, concatenated in grids[], grid_n points each), sorted ascending
   and with duplicates removed (a value is kept only if strictly larger
   than the previous one).  wave_inds[i] is the grid index of wave[i] (the
   reference's spectrum.wave_inds), nblue[g] / nlambda[g] the index range
   of grid g between its first and last wavelength, every grid point in
   between included (what the NLTE batch expects in its transitions). */
pyrh_status pyrh_sort_lambda(const double *wave, int32_t nwave, double lambda_ref,
                             const double *grids, const int32_t *grid_n, int32_t ngrid,
                             double *lam, int32_t cap, int32_t *nspect, int32_t *wave_inds,
                             int32_t *nblue, int32_t *nlambda);

/* Indices of the output wavelengths: every grid point except the one equal
   to lambda_ref (pyrh_solveray.c:115-156, which assumes it is present;
   PYRH_ERR_ARG here when it is not). */
pyrh_status pyrh_output_index(const double *lam, int32_t nspect, double lambda_ref,
                              int32_t *idx, int32_t *nout);

/* Hydrogenic bound-free cross-section of continuum kr on the wavelengths
   lam[0..n-1] (sortlambda.c:331-344 with Gaunt_bf, rh/hydrogen.c:269-281). */
double pyrh_gaunt_bf(double lambda, double n_eff, int32_t charge);
pyrh_status pyrh_cont_alpha(const pyrh_atom *atom, int32_t kr, const double *lam, int32_t n,
                            double *alpha);

/* Kurucz line list (readKuruczLines, rh/kurucz.c:121-430): one pyrh_line per
   record of the list text (fixed columns of the RLK format; the air
   wavelength converted to vacuum, gf to Aji/Bji/Bij, damping constants,
   isotope and hyperfine fractions), with the van der Waals cross-section
   from ABO coefficients in the record, Barklem's tables (getBarklemcross,
   rh/barklem.c:139-197) or Unsold's formula (getUnsoldcross,
   rh/kurucz.c:985-1020), and the Zeeman pattern of polarizable lines
   (RLKZeeman, rh/kurucz.c:832-920).  The element data that the reference
   reads from its abundance and partition-function files come from the
   caller, indexed by atomic number - 1 (hydrogen and helium at least). */
#define PYRH_ELEM_MAX_STAGES 4

typedef struct {
  double weight;                     /* amu */
  double abund;                      /* number abundance relative to hydrogen */
  int32_t nstage;                    /* ionisation stages with data */
  int32_t abundance_set;
  double ionpot[PYRH_ELEM_MAX_STAGES];   /* J */
} pyrh_element;

typedef struct {
  int32_t n1, n2;                    /* rows (lower level neff), columns (upper) */
  double neff1_0, neff2_0;           /* first effective quantum numbers; step 0.1 */
  const double *cross, *alpha;       /* [n1][n2] */
} pyrh_barklem_table;

typedef struct {
  int32_t stokes;                    /* atmos.Stokes (pyrh: always TRUE) */
  int32_t ls_lande;                  /* LS_LANDE */
  const pyrh_element *elements;
  int32_t nelem;
  const pyrh_barklem_table *barklem[3];   /* s-p, p-d, d-f tables or NULL */
  int32_t nloggf;                    /* log gf overrides by record index */
  const int32_t *loggf_ids;
  const double *loggf_values;
} pyrh_kurucz_config;

/* What a record gives beyond pyrh_line (for callers and tests). */
typedef struct {
  int32_t pt_index, stage;
  double gj, Ej, gL_i, gL_j;
} pyrh_kurucz_extra;

/* Parses a Barklem table file (readBarklemTable, rh/barklem.c:61-135; type
   0 = s-p, 1 = p-d, 2 = d-f) into caller arrays of n1 x n2 values and
   fills `table` to point at them. */
pyrh_status pyrh_barklem_parse(const char *text, int32_t type, double *cross, double *alpha,
                               pyrh_barklem_table *table);
pyrh_status pyrh_kurucz_read(const char *text, const pyrh_kurucz_config *cfg, pyrh_line *lines,
                             pyrh_kurucz_extra *extra, int32_t cap, int32_t *nline);

/* Per-depth NLTE set-up of a batch for one model atom, on the device (one
   thread per depth point): LTE populations (LTEpops, rh/ltepops.c:33-109),
   the collision rate matrix (CollisionRate, rh/collision.c:450-700: OMEGA,
   CE, CI, CP, CH, CH0, CH+ records on their TEMP grids, with the reference's
   cubic spline, rh/spline.c, or linear interpolation for two points) and the
   Doppler widths (readatom.c:178-186).  Arrays are device memory indexed by
   depth point like pyrh_nlte_batch (per level [nlevel][total_depth], per
   level pair [nlevel^2][total_depth]); the outputs are what that batch takes
   as nstar, C and vbroad. */
typedef struct {
  int64_t total_depth;
  const double *T, *ne, *ntotal, *vturb;   /* [total_depth] SI; ntotal = abundance * nHtot */
  const double *nh0, *np;                 /* neutral hydrogen ground level and protons,
                                             for CP, CH, CH0, CH+ records (else NULL) */
  double *nstar;                          /* [nlevel][total_depth] */
  double *C;                              /* [nlevel^2][total_depth] */
  double *vbroad;                         /* [total_depth] or NULL */
} pyrh_nlte_setup_batch;

size_t pyrh_nlte_setup_workspace_bytes(const pyrh_atom *atom);
pyrh_status pyrh_nlte_setup(const pyrh_atom *atom, double weight_amu,
                            const pyrh_nlte_setup_batch *batch, void *workspace,
                            size_t workspace_bytes, void *stream);

/* ---------------------------------------------------- background continuum --
 * The angle-independent background opacity, emissivity and scattering
 * opacity of Background() (rh/background.c:329-460; replaces the per-call
 * host pass of the reference's set-up, rhf1d() -> Background()): Thomson
 * (rh/thomson.c:35), H- bound-free and free-free (rh/hydrogen.c:310-615),
 * OH and CH bound-free (rh/ohchbf.c:53-691), hydrogen bound-free and
 * free-free (rh/hydrogen.c:151-305), Rayleigh scattering by H and He
 * (rh/rayleigh.c:33-100), H + H+ free-free, H2 Rayleigh and H2- free-free
 * (rh/hydrogen.c:621-995), bound-free of the passive metals
 * (rh/metal.c:71-171), with the optional fudge factors of compute1d
 * (background.c:365-455).  Line opacities (Kurucz lists, passive
 * bound-bound) are not part of it.  FP64.
 *
 * The model holds the atomic data every atmosphere shares; the batch holds
 * each atmosphere's temperatures, densities and wavelengths.  Outputs are in
 * the continuum layout of pyrh_lte_batch / pyrh_nlte_batch
 * (cont_off[p] + k * nspect[p] + la). */
#define PYRH_BG_MAX_DEPTH 512     /* depth points of one atmosphere */

/* A bound-free continuum: hydrogenic, alpha0 (lambda / lambda0)^3 g(lambda)
   / gbf0 with Seaton's Gaunt factor g(lambda, n_eff, charge) (hydrogen.c:269,
   metal.c:128-137; for hydrogen alpha0 = sigma0 n_eff, gbf0 = 1, charge =
   stage + 1, hydrogen.c:183-200), or the natural cubic spline of a table
   (spline.c); it adds where lambda_min <= lambda <= lambda0. */
typedef struct {
  int32_t hydrogenic;       /* 1 hydrogenic, 0 table */
  int32_t ntab;             /* table points (ascending lambda) at tab_off */
  int32_t n_i, n_j;         /* rows of pops: populations of the lower / upper level */
  int32_t nstar_i, nstar_j; /* rows of pops: their LTE populations */
  int64_t tab_off;          /* first point in tab_lambda / tab_alpha / tab_m2 */
  double lambda0, lambda_min;   /* nm */
  double alpha0, n_eff, charge, gbf0;
} pyrh_bg_continuum;

/* A bound-bound transition from the ground level of a Rayleigh scatterer
   (rayleigh.c:60-90): it adds f (lambda0^2 / (lambda^2 - lambda0^2))^2 where
   lambda > lambda_red = lambda0 (1 + qwing vmicro_char / c), with
   f = Aji (g_j / g_0) (lambda0 [m])^2 / C. */
typedef struct {
  double lambda0, lambda_red, f;
  int32_t scatterer;        /* 0 hydrogen, 1 helium */
  int32_t reserved;
} pyrh_bg_rayleigh_line;

typedef struct {
  int32_t ncont_h;          /* hydrogen's continua, first in cont (not used
                               when h_active: an active hydrogen adds its own) */
  int32_t ncont_metal;      /* then the passive metals' in the reference's atom order */
  const pyrh_bg_continuum *cont;                 /* device */
  const double *tab_lambda, *tab_alpha;          /* device, the tables of cont */
  double *tab_m2;           /* device, [ntab_total + 34]: spline second derivatives,
                               filled by pyrh_background_prepare */
  float *tab_f32;           /* device, [3][ntab_total]: tab_lambda, tab_alpha and tab_m2
                               in FP32, filled by pyrh_background_prepare for FP32
                               batches (NULL: FP64 batches only) */
  int64_t ntab_total;
  int32_t nray;
  const pyrh_bg_rayleigh_line *ray;              /* device */
  double ray_limit[2];      /* per scatterer: the shortest lambda_red of its ground lines */
  int32_t ray_pop[2];       /* per scatterer: row of pops holding its ground level (-1: none) */
  int32_t pop_nh0, pop_np;  /* rows of pops: hydrogen ground level, protons */
  int32_t npop;             /* rows of pops every index above stays below */
  int32_t nonlte;           /* 1 if a metal continuum's n rows are not its n* rows
                               (populations other than the LTE ones); checked by
                               pyrh_background_prepare */
  int32_t h_active;
  int32_t has_h2, has_oh, has_ch;   /* molecules present (atmos.H2, OH, CH) */
  int32_t add_scatter;      /* chi_c includes the scattering opacity (NLTE set-up) */
  int32_t nfudge;           /* optional fudge: 0 or the table length */
  const double *fudge_lambda;   /* device [nfudge] nm, ascending */
  const double *fudge;          /* device [3][nfudge]: H-minus, scattering, metals */
} pyrh_bg_model;

typedef struct {
  int32_t natm, max_nspect, max_ndep;   /* max_ndep <= PYRH_BG_MAX_DEPTH */
  int32_t precision;        /* pyrh_precision of the outputs and of the depth loop
                               (the wavelength terms are FP64 either way) */
  int64_t total_depth;
  const int32_t *ndep, *nspect;                    /* [natm] */
  const int64_t *depth_off, *lam_off, *cont_off;   /* [natm] */
  const double *lambda;                            /* [total_lambda] nm */
  const double *T, *ne, *nHmin, *nH2, *nOH, *nCH;  /* [total_depth] K, m^-3 (nH2 / nOH
                                                      / nCH only where present) */
  const void *pops;         /* [npop][total_depth] the level populations the model's rows
                               name, double or float following precision */
  void *chi_c, *eta_c, *sca_c;                     /* [total_cont] out, double or float */
} pyrh_bg_batch;

/* Once per model (and again if it changes): checks every row and table
   index against npop and ntab_total and the nonlte flag against the rows,
   and puts the spline second derivatives of every tabulated continuum and
   of the H- bound-free table into model->tab_m2 (and the FP32 copies into
   tab_f32).  pyrh_background takes only a model that passed it;
   PYRH_ERR_UNSUPPORTED there when max_ndep needs more shared memory than a
   block has (more than about 1300 depths in FP64). */
pyrh_status pyrh_background_prepare(const pyrh_bg_model *model, void *stream);
/* The background of every atmosphere and wavelength of the batch. */
pyrh_status pyrh_background(const pyrh_bg_model *model, const pyrh_bg_batch *batch,
                            void *stream);

/* -------------------------------------- element tables and LTE populations --
 * The element data of the reference's abundance and partition-function files
 * (readAbundance, rh/abundance.c:72-220), and on the device, one thread per
 * depth point: the LTE ionisation-stage populations (LTEpops_elem,
 * rh/ltepops.c:116-166), the stage density and log partition function each
 * Kurucz line reads (rlk_opacity, rh/kurucz.c:662-677: the line_pops input
 * of pyrh_lte_batch) and the electron density (Solve_ne with getfjk,
 * rh/solvene.c:55-198, as pyrh's get_ne_from_nH runs it,
 * rh/rhf1d/pyrh_hse.c:555-650: hydrogen in LTE, every element's stage
 * fractions from its partition functions).  Elements are indexed by atomic
 * number - 1 (the reference's table of 99 elements, rh/atomweights.h). */
#define PYRH_NELEM 99
#define PYRH_PF_MAX_STAGES 8     /* stages of one element in the tables */

typedef struct {
  int32_t nelem;                /* PYRH_NELEM */
  int32_t npf;                  /* temperatures of the partition-function grid */
  const double *Tpf;            /* [npf] K, ascending */
  const double *abund;          /* [nelem] number abundance relative to hydrogen */
  const int32_t *nstage;        /* [nelem] stages (<= PYRH_PF_MAX_STAGES) */
  const int32_t *stage_off;     /* [nelem] first row of the element in lnpf and ionpot */
  const double *lnpf;           /* [sum nstage][npf] ln U of each stage */
  const double *ionpot;         /* [sum nstage] ionisation potential of each stage, J */
} pyrh_elem_tables;

/* Abundances from the text of an abundance file (readAbundance,
   abundance.c:97-176): "ID value" records, '#' comments; the value of the
   n-th record (1-based, comments not counted) is replaced by ab_val[i] where
   ab_id[i] == n (compute1d's atomic_number / atomic_abundance); a hydrogen
   value of 12.0 means the values are log10 + 12; metallicity (dex) scales
   every element but hydrogen.  abund and abundance_set are [PYRH_NELEM]. */
pyrh_status pyrh_abundance_parse(const char *text, int32_t nabun, const int32_t *ab_id,
                                 const double *ab_val, double metallicity, double *abund,
                                 int32_t *abundance_set);
/* atmos.totalAbund and atmos.wght_per_H (abundance.c:168-221): the sums, in
   element order over the elements with an abundance, of the abundances and
   of abundance x atomic weight [amu] (the reference's weight table). */
pyrh_status pyrh_abundance_totals(const double *abund, const int32_t *abundance_set,
                                  double *total_abund, double *wght_per_H);
/* Element index (atomic number - 1) of a model atom's ID as readAtom matches
   it (readatom.c:109-126); -1 if no element matches. */
int32_t pyrh_element_index(const char *id);
/* The partition-function file (XDR: Npf, Tpf[Npf], then per element its
   atomic number, Nstage, U[Nstage][Npf] and ionisation potentials in cm^-1;
   abundance.c:151-220).  With lnpf == NULL only *npf and *nrows (sum of
   nstage) are set.  Otherwise Tpf [npf], nstage and stage_off [PYRH_NELEM],
   lnpf [nrows][npf] and ionpot [nrows] are filled; for elements with
   abundance_set the partition functions become ln U and the potentials J, as
   the reference converts them (the others keep the file's values). */
pyrh_status pyrh_pf_parse(const unsigned char *bytes, size_t nbytes,
                          const int32_t *abundance_set, int32_t *npf, int32_t *nrows,
                          double *Tpf, int32_t *nstage, int32_t *stage_off, double *lnpf,
                          double *ionpot);

/* The device arrays below are [npoint] (one value per depth point of a
   batch); tables holds device pointers. */
/* Stage populations of the selected elements (LTEpops_elem at the given
   electron density): pops [sum over sel of nstage][npoint], the elements in
   the order of sel (a host array of element indices). */
pyrh_status pyrh_lte_stage_pops(const pyrh_elem_tables *tables, int64_t npoint,
                                const double *T, const double *ne, const double *nHtot,
                                int32_t nsel, const int32_t *sel, double *pops, void *stream);
/* line_pops [nline][2][npoint] of pyrh_lte_batch for lines of the given
   elements and stages (host arrays): the stage density n[stage] and
   ln U_stage(T) of each line's element at every depth point. */
pyrh_status pyrh_line_pops(const pyrh_elem_tables *tables, int64_t npoint, const double *T,
                           const double *ne, const double *nHtot, int32_t nline,
                           const int32_t *elem, const int32_t *stage, double *line_pops,
                           void *stream);
/* Electron density by Solve_ne's Newton iteration (at most 10 steps, to a
   relative change of 1e-2), from the values in ne (fromscratch 0), from
   hydrogen's ionisation alone with its partition function (1, Solve_ne) or
   with U = 1 (2, get_ne of rh/rhf1d/pyrh_background.c:459-540, which the
   hydrostatic equilibrium calls); ne is overwritten.  niter
   (device [npoint], or NULL) receives the steps taken, -1 where the
   iteration did not reach its limit (the reference warns and goes on). */
pyrh_status pyrh_solve_ne(const pyrh_elem_tables *tables, int64_t npoint, const double *T,
                          const double *nHtot, double *ne, int32_t fromscratch, int32_t *niter,
                          void *stream);

/* ------------------------------------------------------ chemical equilibrium --
 * Molecule files (readMolecule, rh/readmolecule.c:66-240: ID, charge,
 * constituents, dissociation energy, fit type, formation temperatures,
 * partition-function and equilibrium-constant fits) and, on the device with
 * one thread per depth point, the molecular equilibrium of
 * ChemicalEquilibrium (rh/chemequil.c:107-390): Newton iteration on the
 * nuclei's conservation and the molecules' Saha equations with H- in the
 * hydrogen balance, equilibrium constants by equilconstant
 * (rh/chemequil.c:456-535), Crout LU with one improvement (ludcmp.c),
 * stopping at a relative change of 1e-3 or after 10 steps
 * (rh/background.h:18-19). */
#define PYRH_MOL_MAX_ELEMENTS 4
#define PYRH_MOL_MAX_COEF 12
#define PYRH_CHEM_MAX_NUCLEI 8
#define PYRH_CHEM_MAX_MOLECULES 24

typedef enum {
  PYRH_FIT_KURUCZ_70 = 0, PYRH_FIT_KURUCZ_85 = 1, PYRH_FIT_SAUVAL_TATUM_84 = 2,
  PYRH_FIT_IRWIN_81 = 3, PYRH_FIT_TSUJI_73 = 4
} pyrh_mol_fit;

typedef struct {
  char id[16];
  int32_t charge;                               /* 0 or 1 */
  int32_t nelement;                             /* constituent elements */
  int32_t pt_index[PYRH_MOL_MAX_ELEMENTS];      /* element index (atomic number - 1) */
  int32_t pt_count[PYRH_MOL_MAX_ELEMENTS];      /* atoms of each */
  int32_t nnuclei;                              /* atoms in the molecule */
  int32_t fit;                                  /* pyrh_mol_fit */
  double ediss;                                 /* dissociation energy, J */
  double tmin, tmax;                            /* formation range, K */
  int32_t npf, neqc;
  double pf_coef[PYRH_MOL_MAX_COEF];            /* in the reference's storage order */
  double eqc_coef[PYRH_MOL_MAX_COEF];
} pyrh_molecule;

/* Parses the text of one molecule file; constituents must be elements with
   abundance_set ([PYRH_NELEM]). */
pyrh_status pyrh_molecule_read(const char *text, const int32_t *abundance_set,
                               pyrh_molecule *molecule);

/* Chemical equilibrium at npoint depth points for the molecules mol[nmol]
   (host array; the first must be H2, as the reference requires).  The
   nuclei are the elements bound in some molecule, in element order
   (hydrogen first); fn0_model (host array [PYRH_NELEM] of device pointers,
   or NULL) gives, for an element with an atom model, the neutral fraction of
   its LTE populations at every point; elements without one take theirs
   from the tables' partition functions (getfjk).  Outputs (device):
   nmol [nmol][npoint] molecule densities, nHmin [npoint], nnuc
   [nnuclei][npoint] the nuclei's atomic densities afterwards (a model atom's
   populations scale by nnuc / its total), niter [npoint] steps taken (-1:
   not converged; may be NULL). */
pyrh_status pyrh_chem_equil(const pyrh_elem_tables *tables, const pyrh_molecule *mol,
                            int32_t nmol, int64_t npoint, const double *T, const double *ne,
                            const double *nHtot, const double *const *fn0_model, double *nmol_out,
                            double *nHmin, double *nnuc, int32_t *niter, void *stream);

/* ------------------------------------- passive atoms, equilibria, depth scales --
 * The model atoms of a run's atoms.input, all passive (LTE), as the
 * background and the equilibria read them: levels of every atom as rows of
 * one population array [level][npoint] (device), atoms in the list's order. */
#define PYRH_MAX_PASSIVE_ATOMS 24

typedef struct {
  int32_t natom;
  int32_t elem[PYRH_MAX_PASSIVE_ATOMS];         /* element index of each model atom */
  int32_t lev_off[PYRH_MAX_PASSIVE_ATOMS + 1];  /* its levels are rows lev_off[m] ..
                                                   lev_off[m+1]-1 of the populations */
  const double *E, *g;                          /* device [lev_off[natom]]: J, statistical weight */
  const int32_t *stage;                         /* device [lev_off[natom]] */
} pyrh_passive_atoms;

/* The equilibria of Background() (background.c:155-170 with SOLVE_NE NONE)
   at npoint depth points for the given electron density: every atom's LTE
   populations (LTEpops without Debye lowering, rh/ltepops.c:33-109), the
   chemical equilibrium of the molecules (pyrh_chem_equil) from the model
   atoms' neutral fractions, and the populations of the atoms bound in
   molecules scaled by the share of their nuclei left atomic
   (chemequil.c:219-238, 330-339).  Outputs (device): pops [nlevel][npoint],
   nmol [nmol][npoint], nHmin [npoint]. */
pyrh_status pyrh_equilibria(const pyrh_elem_tables *tables, const pyrh_molecule *mol,
                            int32_t nmol, const pyrh_passive_atoms *atoms, int64_t npoint,
                            const double *T, const double *ne, const double *nHtot, double *pops,
                            double *nmol_out, double *nHmin, void *stream);

/* The depth scales of convertScales (rh/rhf1d/multiatmos.c:100-177) for
   natm atmospheres from the continuum opacity at the reference wavelength:
   given log10 tau_ref (scale 0), log10 column mass [g cm^-2] (1) or height
   [km] (2) -- converted as the reference does, pyrh_compute1dray.c:229-245 --
   the other two follow by the trapezoid rule, and on the tau and
   column-mass scales the heights are shifted to zero where tau_ref = 1. */
typedef struct {
  int32_t natm, ndep;    /* ndep >= 2 */
  int32_t scale;         /* 0 tau_ref, 1 column mass, 2 height */
  double gravity;        /* m s^-2 */
  double total_abund, wght_per_H;
  /* device arrays [ndep][natm] */
  const double *scale_in;        /* the given scale, in the reference's input units */
  const double *T, *ne, *nHtot;  /* K, m^-3 */
  const double *chi_ref;         /* continuum opacity at lambda_ref, m^-1 */
  double *tau_ref, *cmass, *height;   /* out: 1, kg m^-2, m */
} pyrh_scales_batch;

pyrh_status pyrh_convert_scales(const pyrh_scales_batch *batch, void *stream);

/* -------------------------------------------------- hydrostatic equilibrium --
 * pyrh's hse() (rh/rhf1d/pyrh_hse.c:67-399, pyrh.pyx:427-487) for a batch of
 * atmospheres with the same number of depth points, all on the device.  Layer
 * by layer from the top, each atmosphere iterates until its hydrogen density
 * changes by at most eta_limit (relative) or nmax_iter passes are done; a
 * pass takes the electron density (get_ne: Solve_ne from hydrogen's
 * ionisation with U = 1), the equilibria (pyrh_equilibria), the continuum
 * opacity at 500 nm (pyrh_Background, rh/rhf1d/pyrh_background.c:144-457:
 * the background without the metals' bound-free continua, scattering
 * included), and the gas pressure by the trapezoid in log tau500 (or in
 * height) and from it the hydrogen density. */
typedef struct {
  double gravity;        /* m s^-2 (MULTIatmos: 10^4.4 cm s^-2) */
  double total_abund;    /* atmos.totalAbund (pyrh_abundance_totals) */
  double wght_per_H;     /* atmos.wght_per_H, amu */
  int32_t scale;         /* 0: log10 tau500, 2: height in km (the reference's
                            column-mass branch leaves its pressure step unset) */
  int32_t nmax_iter;     /* NMAX_HSE_ITER, 50 */
  double eta_limit;      /* 1e-2 */
} pyrh_hse_config;

typedef struct {
  int32_t natm, ndep;    /* natm <= 65535 per call */
  /* device arrays [ndep][natm], depth point k of atmosphere a at k * natm + a */
  const double *scale;   /* log10 tau500 or height [km] */
  const double *T;       /* K */
  const double *pg_top;  /* device [natm]: gas pressure of the top layer, Pa */
  double *ne, *nHtot;    /* out, m^-3 */
  double *rho, *pg;      /* out, kg m^-3 and Pa */
  double *opacity;       /* out or NULL: the 500 nm opacity of each layer, m^-1 */
  int32_t *niter;        /* out or NULL: passes per layer (-1: nmax_iter reached first) */
} pyrh_hse_batch;

/* bg: a model prepared by pyrh_background_prepare whose population rows are
   the atoms' levels (npop == atoms->lev_off[natom]; FP64); mol: as for
   pyrh_chem_equil, with H2 / OH / CH (when present) giving the background's
   molecule densities. */
pyrh_status pyrh_hse(const pyrh_elem_tables *tables, const pyrh_molecule *mol, int32_t nmol,
                     const pyrh_bg_model *bg, const pyrh_passive_atoms *atoms,
                     const pyrh_hse_config *cfg, const pyrh_hse_batch *batch, void *stream);

/* Number of kernel launches the last pyrh_lte_stokes / pyrh_nlte_* call issued. */
int32_t pyrh_last_launch_count(void);

/* Library version string and the text of the last error on this thread. */
const char *pyrh_version(void);
const char *pyrh_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* PYRH_GB300_H */
