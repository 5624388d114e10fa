// rf_host.cu -- TEST HARNESS: evaluates the response-function math of
// pyrh_gb300/csrc/lte_rf.cuh on the CPU in FP64 for one atmosphere, so the
// adjoint can be compared with finite differences of the CPU oracle.
// Built by tests/test_rf_host.py with nvcc (host code only).
#include <stdint.h>
#include <string.h>

#define PYRH_MAX_DEPTH_RF 160
#include "../../include/pyrh_gb300.h"
#include "../../pyrh_gb300/csrc/lte_rf.cuh"

using namespace pyrh;

static Tape<double> g_tape;
static double g_qb[PYRH_MAX_DEPTH_RF][4][8];
static double g_J[PYRH_MAX_DEPTH_RF][8][kNX];

// atmosphere arrays SI [nd]; line_pops [nline][2][nd]; lines: pyrh_line[nline];
// chi_c, eta_c [nlam][nd]; out: stokes [nlam][4], rf [nlam][4][6][nd]
extern "C" int rf_eval(int nd, const double* height, const double* T, const double* ne,
                       const double* nHtot, const double* np, const double* vturb,
                       const double* vel, const double* B, const double* gam, const double* chb,
                       const double* line_pops, int nline, const pyrh_line* lines, int nlam,
                       const double* lam, const double* chi_c, const double* eta_c, double mu,
                       double vmicro_char, double* stokes, double* rf) {
  if (nd > PYRH_MAX_DEPTH_RF || nline > PYRH_MAX_LINES) return -1;
  static LineDepth<double> ld[PYRH_MAX_LINES][PYRH_MAX_DEPTH_RF];
  static GeoD<double> geo[PYRH_MAX_DEPTH_RF];
  int ncomp[PYRH_MAX_LINES], cq[PYRH_MAX_LINES * PYRH_MAX_COMPONENTS];
  double cs[PYRH_MAX_LINES * PYRH_MAX_COMPONENTS], cw[PYRH_MAX_LINES * PYRH_MAX_COMPONENTS];
  for (int l = 0; l < nline; ++l) {
    const pyrh_line& L = lines[l];
    LineConstD c = {L.lambda0, L.Ei, L.gi, L.Aji, L.Bji, L.Bij, L.Grad, L.GStark, L.GvdWaals,
                    L.cross, L.alpha, L.isotope_frac, L.hyperfine_frac, L.weight, L.vdwaals};
    ncomp[l] = L.polarizable ? L.ncomp : 0;
    for (int m = 0; m < PYRH_MAX_COMPONENTS; ++m) {
      cq[l * PYRH_MAX_COMPONENTS + m] = L.comp_q[m];
      cs[l * PYRH_MAX_COMPONENTS + m] = L.comp_shift[m];
      cw[l * PYRH_MAX_COMPONENTS + m] = L.comp_strength[m];
    }
    for (int k = 0; k < nd; ++k)
      ld[l][k] = line_depth<double>(c, T[k], vel[k], vturb[k], B[k], ne[k], nHtot[k], np[k],
                                    line_pops[(l * 2 + 0) * nd + k], line_pops[(l * 2 + 1) * nd + k],
                                    mu, true);
  }
  for (int k = 0; k < nd; ++k) geo[k] = geometry_d<double>(gam[k], chb[k], mu);
  double ds[PYRH_MAX_DEPTH_RF];
  ds[0] = 0;
  for (int k = 1; k < nd; ++k) ds[k] = fabs(height[k] - height[k - 1]) / mu;
  for (int la = 0; la < nlam; ++la) {
    const double lm = lam[la];
    const double dlc = lm * kQ_WING * (vmicro_char / kCLIGHT);
    unsigned inwin = 0;
    bool pol = false;
    double dlam[PYRH_MAX_LINES];
    for (int l = 0; l < nline; ++l) {
      dlam[l] = lm - lines[l].lambda0;
      if (fabs(lines[l].lambda0 - lm) <= dlc && lines[l].contributes) {
        inwin |= 1u << l;
        pol |= lines[l].polarizable != 0;
      }
    }
    double* rfl = rf + (int64_t)la * 4 * kNX * nd;
    memset(rfl, 0, sizeof(double) * 4 * kNX * nd);
    if (!pol) { for (int s = 0; s < 4; ++s) stokes[la * 4 + s] = 0.0; continue; }
    LineDepth<double> ldk[PYRH_MAX_LINES];
    for (int k = 0; k < nd; ++k) {
      for (int l = 0; l < nline; ++l) ldk[l] = ld[l][k];
      local_q_jac<double>(nline, ldk, geo[k], dlam, inwin, ncomp, cs, cw, cq, PYRH_MAX_COMPONENTS,
                          chi_c[(int64_t)la * nd + k], eta_c[(int64_t)la * nd + k], g_tape.q[k],
                          g_J[k]);
    }
    const double B0 = planck(T[nd - 2], lm), B1 = planck(T[nd - 1], lm);
    double out[4];
    delo_forward<double>(g_tape, ds, nd, B0, B1, out);
    for (int s = 0; s < 4; ++s) stokes[la * 4 + s] = out[s];
    double seed[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    double Bb[4][2];
    delo_reverse<double, 4>(g_tape, ds, nd, B0, B1, seed, g_qb, Bb);
    for (int s = 0; s < 4; ++s)
      for (int k = 0; k < nd; ++k)
        for (int x = 0; x < kNX; ++x) {
          double v = 0.0;
          for (int n = 0; n < 8; ++n) v += g_qb[k][s][n] * g_J[k][n][x];
          if (x == 0 && k == nd - 2) v += Bb[s][0] * planck_dT(T[k], lm);
          if (x == 0 && k == nd - 1) v += Bb[s][1] * planck_dT(T[k], lm);
          rfl[(s * kNX + x) * nd + k] = v;
        }
  }
  return 0;
}
