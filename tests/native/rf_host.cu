// rf_host.cu -- TEST HARNESS: evaluates the response-function math of
// pyrh_gb300/csrc/lte_rf.cuh on the CPU for one atmosphere, in the same
// order as the GPU kernel (per-depth quantities and their derivatives in the
// working precision; forward sweep on the values; reverse sweep; reverse-mode
// contraction through the opacity at each handed-over depth), so the adjoint
// can be compared with finite differences of the CPU oracle and with the
// GPU.  rf_eval works in FP64, rf_eval_f32 in FP32; rf_eval_jac is rf_eval
// with the opacity derivatives taken in forward mode instead (six dual
// directions through every sum, local_q_jac), an independent check of the
// reverse-mode contraction.
// Built by tests/conftest.py (rf_harness) with nvcc, host code only.
#include <stdint.h>
#include <string.h>

#include "../../include/pyrh_gb300.h"
#include "../../pyrh_gb300/csrc/lte_rf.cuh"

using namespace pyrh;

// Optional temperature derivatives of the set-up (null members: held fixed);
// layouts as rf_eval_t's inputs ([nlam][nd], [nline][2][nd], [nd]).
// STOKES_MODE of the next evaluations (PYRH_FULL_STOKES or PYRH_NO_STOKES)
static int g_stokes_mode = PYRH_FULL_STOKES;
extern "C" void rf_set_stokes_mode(int mode) { g_stokes_mode = mode; }
// atmos.moving: 0 for a static atmosphere (line shifts ignored, and
// Feautrier where no polarizable line covers the wavelength)
static int g_moving = 1;
extern "C" void rf_set_moving(int moving) { g_moving = moving; }

struct SetupDT {
  const double *dchi_c, *deta_c, *dline_pops, *dnp, *dlen_up, *dlen_dn;
};

template <typename R, bool JAC>
struct Emit {
  int nd;
  const double* T;
  double lm;
  double* rfl;
  int nline;
  const LineDepth<R>* ld;   // [line][depth] with stride PYRH_MAX_DEPTH_RF
  const GeoD<R>* geo;
  const R* dlam;
  unsigned inwin;
  const int* ncomp;
  const R *cs, *cw;
  const int* cq;
  const R *chi_c, *eta_c;   // [depth] at this wavelength
  const Tape<R>* tp;
  R* gf;                    // [4][PYRH_MAX_LINES] log gf accumulators
  const R *dchi_c, *deta_c; // [depth] at this wavelength, or nullptr
  const R *len_up, *len_dn; // [depth] d ds_k/dT_{k-1}, d ds_k/dT_k
  const ScalarAdj<R>* fa;    // no line in window: the Feautrier adjoint of the I seed
  void operator()(int k, const R* qb_in, const R* bpl_in, const R* sdn_in,
                  const R* sup_in) const {
    R qb[32], bpl[4], sdn[4], sup[4];
    for (int e = 0; e < 32; ++e) qb[e] = fa ? R(0) : qb_in[e];
    for (int s = 0; s < 4; ++s) {
      bpl[s] = fa ? R(0) : bpl_in[s];
      sdn[s] = fa ? R(0) : sdn_in[s];
      sup[s] = fa ? R(0) : sup_in[s];
    }
    if (fa) {
      qb[0] = fa->chib[k];
      qb[1] = fa->Sb[k];
      bpl[0] = (k == nd - 2) ? fa->B0b : (k == nd - 1) ? fa->B1b : R(0);
      sdn[0] = fa->dsb[k];
      sup[0] = (k + 1 < nd) ? fa->dsb[k + 1] : R(0);
    }
    R g[4][kNX];
    if (JAC) {
      R q[8], J[8][kNX];
      local_q_jac<R>(nline, ld + k, PYRH_MAX_DEPTH_RF, geo[k], dlam, inwin, ncomp, cs, cw, cq,
                     PYRH_MAX_COMPONENTS, chi_c[k], eta_c[k], q, J);
      for (int s = 0; s < 4; ++s)
        for (int x = 0; x < kNX; ++x) {
          g[s][x] = 0;
          for (int n = 0; n < 8; ++n) g[s][x] += qb[s * 8 + n] * J[n][x];
        }
      // continuum derivative terms as in local_q_vjp: dq/dchi_c, dq/deta_c
      const R ichi = R(1) / q[0];
      for (int s = 0; s < 4; ++s) {
        const R* a = qb + s * 8;
        R chib = a[0];
        for (int n = 1; n < 8; ++n) chib -= a[n] * q[n] * ichi;
        g[s][0] += chib * (dchi_c ? dchi_c[k] : R(0)) + a[1] * ichi * (deta_c ? deta_c[k] : R(0));
      }
    } else {
      for (int s = 0; s < 4; ++s)
        for (int x = 0; x < kNX; ++x) g[s][x] = 0;
      local_q_vjp<R, 4>(nline, ld + k, PYRH_MAX_DEPTH_RF, geo[k], dlam, inwin, ncomp, cs, cw, cq,
                        PYRH_MAX_COMPONENTS, tp->q[k], qb, g, gf, tp->z[k],
                        dchi_c ? dchi_c[k] : R(0), deta_c ? deta_c[k] : R(0));
    }
    const R dB = (k >= nd - 2) ? R(planck_dT(T[k], lm)) : R(0);
    const R ldn = len_dn[k], lup = (k + 1 < nd) ? len_up[k + 1] : R(0);
    for (int s = 0; s < 4; ++s)
      for (int x = 0; x < kNX; ++x)
        rfl[(s * kNX + x) * nd + k] =
            double(g[s][x] + (x == 0 ? bpl[s] * dB + sdn[s] * ldn + sup[s] * lup : R(0)));
  }
};

// atmosphere arrays SI [nd]; line_pops [nline][2][nd]; lines: pyrh_line[nline];
// chi_c, eta_c [nlam][nd]; out: stokes [nlam][4], rf [nlam][4][6][nd],
// rf_gf [nlam][4][nline] (dS/dlog10 gf; the forward-mode variant leaves it 0)
template <typename R, bool JAC>
static int rf_eval_t(int nd, const double* height, const double* T, const double* ne,
                     const double* nHtot, const double* np, const double* vturb,
                     const double* vel, const double* B, const double* gam, const double* chb,
                     const double* line_pops, int nline, const pyrh_line* lines, int nlam,
                     const double* lam, const double* chi_c, const double* eta_c, double mu,
                     double vmicro_char, double* stokes, double* rf, double* rf_gf,
                     const SetupDT& dT) {
  if (nd < 3 || nd > PYRH_MAX_DEPTH_RF || nline > PYRH_MAX_LINES) return -1;
  static LineDepth<R> ld[PYRH_MAX_LINES][PYRH_MAX_DEPTH_RF];
  static GeoD<R> geo[PYRH_MAX_DEPTH_RF];
  static Tape<R> tape;
  int ncomp[PYRH_MAX_LINES], cq[PYRH_MAX_LINES * PYRH_MAX_COMPONENTS];
  R cs[PYRH_MAX_LINES * PYRH_MAX_COMPONENTS], cw[PYRH_MAX_LINES * PYRH_MAX_COMPONENTS];
  for (int l = 0; l < nline; ++l) {
    const pyrh_line& L = lines[l];
    LineConstD c = {L.lambda0, L.Ei, L.gi, L.Aji, L.Bji, L.Bij, L.Grad, L.GStark, L.GvdWaals,
                    L.cross, L.alpha, L.isotope_frac, L.hyperfine_frac, L.weight, L.vdwaals};
    ncomp[l] = L.polarizable ? L.ncomp : kArmstrong;
    for (int m = 0; m < PYRH_MAX_COMPONENTS; ++m) {
      cq[l * PYRH_MAX_COMPONENTS + m] = L.comp_q[m];
      cs[l * PYRH_MAX_COMPONENTS + m] = R(L.comp_shift[m]);
      cw[l * PYRH_MAX_COMPONENTS + m] = R(L.comp_strength[m]);
    }
    for (int k = 0; k < nd; ++k)
      ld[l][k] = line_depth<R>(c, R(T[k]), R(vel[k]), R(vturb[k]), R(B[k]), R(ne[k]), R(nHtot[k]),
                               R(np[k]), R(line_pops[(l * 2 + 0) * nd + k]),
                               R(line_pops[(l * 2 + 1) * nd + k]), R(mu), g_moving != 0,
                               dT.dline_pops ? R(dT.dline_pops[(l * 2 + 0) * nd + k]) : R(0),
                               dT.dline_pops ? R(dT.dline_pops[(l * 2 + 1) * nd + k]) : R(0),
                               dT.dnp ? R(dT.dnp[k]) : R(0));
  }
  for (int k = 0; k < nd; ++k) geo[k] = geometry_d<R>(R(gam[k]), R(chb[k]), R(mu));
  R ds[PYRH_MAX_DEPTH_RF];
  ds[0] = 0;
  for (int k = 1; k < nd; ++k) ds[k] = R(fabs(height[k] - height[k - 1]) / mu);
  R lup[PYRH_MAX_DEPTH_RF], ldn[PYRH_MAX_DEPTH_RF];
  for (int k = 0; k < nd; ++k) {
    lup[k] = (k >= 1 && dT.dlen_up) ? R(dT.dlen_up[k] / mu) : R(0);
    ldn[k] = (k >= 1 && dT.dlen_dn) ? R(dT.dlen_dn[k] / mu) : R(0);
  }
  R cc[PYRH_MAX_DEPTH_RF], ec[PYRH_MAX_DEPTH_RF], dcc[PYRH_MAX_DEPTH_RF], dec[PYRH_MAX_DEPTH_RF];
  for (int la = 0; la < nlam; ++la) {
    const double lm = lam[la];
    const double dlc = lm * kQ_WING * (vmicro_char / kCLIGHT);
    unsigned inwin = 0;
    bool pol = false, anypol = false;
    R dlam[PYRH_MAX_LINES];
    for (int l = 0; l < nline; ++l) {
      dlam[l] = R(lm - lines[l].lambda0);
      if (fabs(lines[l].lambda0 - lm) <= dlc && lines[l].contributes) {
        inwin |= 1u << l;
        pol |= lines[l].polarizable != 0 && g_stokes_mode == PYRH_FULL_STOKES;
        anypol |= lines[l].polarizable != 0;
      }
    }
    double* rfl = rf + (int64_t)la * 4 * kNX * nd;
    memset(rfl, 0, sizeof(double) * 4 * kNX * nd);
    double* gfl = rf_gf + (int64_t)la * 4 * nline;
    for (int e = 0; e < 4 * nline; ++e) gfl[e] = 0.0;
    for (int k = 0; k < nd; ++k) {
      cc[k] = R(chi_c[(int64_t)la * nd + k]);
      ec[k] = R(eta_c[(int64_t)la * nd + k]);
      dcc[k] = dT.dchi_c ? R(dT.dchi_c[(int64_t)la * nd + k]) : R(0);
      dec[k] = dT.deta_c ? R(dT.deta_c[(int64_t)la * nd + k]) : R(0);
    }
    auto qop = [&](int k, R* q) {
      local_q<R, true>(nline, &ld[0][k], PYRH_MAX_DEPTH_RF, geo[k], dlam, inwin, ncomp, cs, cw, cq,
                       PYRH_MAX_COMPONENTS, cc[k], ec[k], q, tape.z[k]);
    };
    const double B0 = planck(T[nd - 2], lm), B1 = planck(T[nd - 1], lm);
    R out[4];
    delo_forward<R>(tape, ds, nd, B0, B1, out, qop);
    // the reference's solver: Feautrier without a line in window, scalar
    // Bezier3 when no line in window is polarizable, DELO-Bezier3 otherwise
    static FeautTape<R> ft;
    static ScalarTape<R> sbt;
    static ScalarAdj<R> fadj;
    const bool feaut = inwin == 0u || (!anypol && !g_moving);
    if (feaut) {
      out[0] = feautrier_fwd<R>(tape, ds, nd, B0, B1, ft);
      feautrier_vjp<R>(tape, ds, nd, B0, B1, ft, R(1), fadj);
    } else if (!pol) {
      out[0] = scalar_bezier_fwd<R>(tape, ds, nd, B0, B1, sbt);
      scalar_bezier_vjp<R>(tape, ds, nd, B0, B1, sbt, R(1), fadj);
    }
    if (!pol) out[1] = out[2] = out[3] = R(0);
    for (int s = 0; s < 4; ++s) stokes[la * 4 + s] = double(out[s]);
    const R one = pol ? R(1) : R(0);
    const R seed[4][4] = {{one, 0, 0, 0}, {0, one, 0, 0}, {0, 0, one, 0}, {0, 0, 0, one}};
    R gfa[4 * PYRH_MAX_LINES];
    for (int e = 0; e < 4 * PYRH_MAX_LINES; ++e) gfa[e] = R(0);
    Emit<R, JAC> emit{nd, T, lm, rfl, nline, &ld[0][0], geo, dlam, inwin, ncomp, cs, cw, cq, cc, ec,
                      &tape, gfa, dcc, dec, lup, ldn, pol ? nullptr : &fadj};
    delo_reverse_stream<R, 4>(tape, ds, nd, B0, B1, seed, emit);
    for (int s = 0; s < 4; ++s)
      for (int l = 0; l < nline; ++l) gfl[s * nline + l] = double(gfa[s * PYRH_MAX_LINES + l]);
  }
  return 0;
}

#define RF_ARGS                                                                              \
  int nd, const double *height, const double *T, const double *ne, const double *nHtot,       \
      const double *np, const double *vturb, const double *vel, const double *B,              \
      const double *gam, const double *chb, const double *line_pops, int nline,               \
      const pyrh_line *lines, int nlam, const double *lam, const double *chi_c,               \
      const double *eta_c, double mu, double vmicro_char, double *stokes, double *rf,        \
      double *rf_gf
#define RF_PASS                                                                              \
  nd, height, T, ne, nHtot, np, vturb, vel, B, gam, chb, line_pops, nline, lines, nlam, lam,  \
      chi_c, eta_c, mu, vmicro_char, stokes, rf, rf_gf

#define DT_ARGS                                                                              \
  const double *dchi_c, const double *deta_c, const double *dline_pops, const double *dnp,    \
      const double *dlen_up, const double *dlen_dn
#define DT_PASS SetupDT{dchi_c, deta_c, dline_pops, dnp, dlen_up, dlen_dn}

extern "C" int rf_eval(RF_ARGS) { return rf_eval_t<double, false>(RF_PASS, SetupDT{}); }
extern "C" int rf_eval_f32(RF_ARGS) { return rf_eval_t<float, false>(RF_PASS, SetupDT{}); }
extern "C" int rf_eval_jac(RF_ARGS) { return rf_eval_t<double, true>(RF_PASS, SetupDT{}); }
// the same with the set-up's temperature derivatives (any of them NULL)
extern "C" int rf_eval_dT(RF_ARGS, DT_ARGS) { return rf_eval_t<double, false>(RF_PASS, DT_PASS); }
extern "C" int rf_eval_f32_dT(RF_ARGS, DT_ARGS) {
  return rf_eval_t<float, false>(RF_PASS, DT_PASS);
}
extern "C" int rf_eval_jac_dT(RF_ARGS, DT_ARGS) { return rf_eval_t<double, true>(RF_PASS, DT_PASS); }
