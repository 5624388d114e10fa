// background.cu -- the angle-independent background continuum of the
// reference's Background() (rh/background.c:329-460) on the GPU, FP64.
//
// One thread owns one (atmosphere, wavelength): it evaluates everything
// that depends on the wavelength alone once -- the H- bound-free spline
// (hydrogen.c:310-365), the fractional wavelength indices of the free-free
// and OH / CH tables, the hydrogen cross-sections (hydrogen.c:183-200), the
// Rayleigh cross-sections (rayleigh.c:60-90, hydrogen.c:960-980), the
// Gaunt factor's wavelength term and the cross-section of every metal
// continuum that covers the wavelength (metal.c:120-140) -- and then walks
// down the atmosphere, adding the processes at each depth in the order of
// background.c:341-460 and writing chi_c, eta_c and sca_c (consecutive
// threads hold consecutive wavelengths, so the stores coalesce).  What
// depends on the depth alone (the fractional temperature indices of the
// tables, the electron pressure) is computed once per block in shared
// memory: a block's threads share one atmosphere.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pyrh_gb300.h"
#include "background_tables.h"
#include "rt_device.cuh"

namespace pyrh {
void set_error(const char* fmt, ...);
void set_launches(int n);

namespace {

// rh/constant.h:28-52 (those rt_device.cuh does not hold)
constexpr double kEPSILON_0 = 8.854187817E-12;
constexpr double kE_RYDBERG = 2.1798741E-18;
constexpr double kEV = 1.60217733E-19;
constexpr double kTHETA0 = 5.03974756E+03;
constexpr double kCM_TO_M = 1.0E-02;
constexpr double kMICRON_TO_NM = 1.0E+03;
constexpr double kMEGABARN_TO_M2 = 1.0E-22;
constexpr double kLG10 = 2.30258509299404568402;
constexpr double kRAYLEIGH_H2_LIMIT = 121.57;   // hydrogen.c:938

__device__ const double kHmBfLam[] = {PYRH_BG_HMIN_BF_LAMBDA};
__device__ const double kHmBfAlpha[] = {PYRH_BG_HMIN_BF_ALPHA};
__device__ const double kHmFfLam[] = {PYRH_BG_HMIN_FF_LAMBDA};
__device__ const double kHmFfTheta[] = {PYRH_BG_HMIN_FF_THETA};
__device__ const double kHmFfKappa[] = {PYRH_BG_HMIN_FF_KAPPA};
__device__ const double kJohnA[] = {PYRH_BG_HMIN_FF_LONG_A};
__device__ const double kJohnB[] = {PYRH_BG_HMIN_FF_LONG_B};
__device__ const double kJohnC[] = {PYRH_BG_HMIN_FF_LONG_C};
__device__ const double kJohnD[] = {PYRH_BG_HMIN_FF_LONG_D};
__device__ const double kJohnE[] = {PYRH_BG_HMIN_FF_LONG_E};
__device__ const double kJohnF[] = {PYRH_BG_HMIN_FF_LONG_F};
__device__ const double kH2mLam[] = {PYRH_BG_H2MIN_FF_LAMBDA};
__device__ const double kH2mTheta[] = {PYRH_BG_H2MIN_FF_THETA};
__device__ const double kH2mKappa[] = {PYRH_BG_H2MIN_FF_KAPPA};
__device__ const double kH2pLam[] = {PYRH_BG_H2PLUS_FF_LAMBDA};
__device__ const double kH2pTemp[] = {PYRH_BG_H2PLUS_FF_TEMP};
__device__ const double kH2pKappa[] = {PYRH_BG_H2PLUS_FF_KAPPA};
__device__ const double kRH2Coef[] = {PYRH_BG_RAYLEIGH_H2_COEF};
__device__ const double kRH2Lam[] = {PYRH_BG_RAYLEIGH_H2_LAMBDA};
__device__ const double kRH2Sigma[] = {PYRH_BG_RAYLEIGH_H2_SIGMA};
__device__ const double kOHTemp[] = {PYRH_BG_OH_BF_TEMP};
__device__ const double kOHEv[] = {PYRH_BG_OH_BF_EV};
__device__ const double kOHSig[] = {PYRH_BG_OH_BF_LOGSIGMA};
__device__ const double kCHTemp[] = {PYRH_BG_CH_BF_TEMP};
__device__ const double kCHEv[] = {PYRH_BG_CH_BF_EV};
__device__ const double kCHSig[] = {PYRH_BG_CH_BF_LOGSIGMA};

// FP32 copies of the tables the depth loop interpolates
__device__ const float kHmFfKappaF[] = {PYRH_BG_HMIN_FF_KAPPA};
__device__ const float kH2mKappaF[] = {PYRH_BG_H2MIN_FF_KAPPA};
__device__ const float kH2pKappaF[] = {PYRH_BG_H2PLUS_FF_KAPPA};
__device__ const float kOHSigF[] = {PYRH_BG_OH_BF_LOGSIGMA};
__device__ const float kCHSigF[] = {PYRH_BG_CH_BF_LOGSIGMA};

template <typename R> struct DepthTables;
template <> struct DepthTables<double> {
  __device__ static const double* hmff() { return kHmFfKappa; }
  __device__ static const double* h2m() { return kH2mKappa; }
  __device__ static const double* h2p() { return kH2pKappa; }
  __device__ static const double* oh() { return kOHSig; }
  __device__ static const double* ch() { return kCHSig; }
};
template <> struct DepthTables<float> {
  __device__ static const float* hmff() { return kHmFfKappaF; }
  __device__ static const float* h2m() { return kH2mKappaF; }
  __device__ static const float* h2p() { return kH2pKappaF; }
  __device__ static const float* oh() { return kOHSigF; }
  __device__ static const float* ch() { return kCHSigF; }
};

constexpr int kHmBfN = PYRH_BG_HMIN_BF_LAMBDA_N;
constexpr int kHmFfNL = PYRH_BG_HMIN_FF_LAMBDA_N, kHmFfNT = PYRH_BG_HMIN_FF_THETA_N;
constexpr int kH2mNL = PYRH_BG_H2MIN_FF_LAMBDA_N, kH2mNT = PYRH_BG_H2MIN_FF_THETA_N;
constexpr int kH2pNL = PYRH_BG_H2PLUS_FF_LAMBDA_N, kH2pNT = PYRH_BG_H2PLUS_FF_TEMP_N;
constexpr int kRH2N = PYRH_BG_RAYLEIGH_H2_LAMBDA_N;
constexpr int kOHNT = PYRH_BG_OH_BF_TEMP_N, kOHNE = PYRH_BG_OH_BF_EV_N;
constexpr int kCHNT = PYRH_BG_CH_BF_TEMP_N, kCHNE = PYRH_BG_CH_BF_EV_N;
constexpr int kMaxHCont = 16;        // hydrogen continua evaluated per wavelength
constexpr int kBlock = 128;          // wavelengths per block

static_assert(PYRH_BG_HMIN_BF_ALPHA_N == kHmBfN, "H- bound-free table");
static_assert(PYRH_BG_HMIN_FF_KAPPA_N == kHmFfNL * kHmFfNT, "H- free-free table");
static_assert(PYRH_BG_H2MIN_FF_KAPPA_N == kH2mNL * kH2mNT, "H2- free-free table");
static_assert(PYRH_BG_H2PLUS_FF_KAPPA_N == kH2pNL * kH2pNT, "H2+ free-free table");
static_assert(PYRH_BG_OH_BF_LOGSIGMA_N == kOHNT * kOHNE, "OH table");
static_assert(PYRH_BG_CH_BF_LOGSIGMA_N == kCHNT * kCHNE, "CH table");

// Bracket j with t[j] <= x < t[j + 1] of an ascending table (what Hunt and
// Locate give, rh/hunt.c), by bisection.
__device__ __forceinline__ int bracket(const double* t, int n, double x) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (hi + lo) >> 1;
    if (x >= t[mid]) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Fractional index of x in an ascending table, held at the ends
// (hydrogen.c:497-508).
__device__ __forceinline__ double frac_index(const double* t, int n, double x) {
  if (x <= t[0]) return 0.0;
  if (x >= t[n - 1]) return (double)(n - 1);
  const int j = bracket(t, n, x);
  return j + (x - t[j]) / (t[j + 1] - t[j]);
}

// hydrogen.c:998-1020: f[j * ncol + i] at the fractional indices (x, y), in
// the working precision of the depth loop (the table's entries converted as
// they are read).
template <typename R>
__device__ __forceinline__ R bilinear_r(int ncol, int nrow, const R* f, R x, R y) {
  const int i = (int)x;
  const R fx = x - R(i);
  const int i1 = (i == ncol - 1) ? i : i + 1;
  const int j = (int)y;
  const R fy = y - R(j);
  const int j1 = (j == nrow - 1) ? j : j + 1;
  return (R(1) - fx) * (R(1) - fy) * f[j * ncol + i] + fx * (R(1) - fy) * f[j * ncol + i1] +
         (R(1) - fx) * fy * f[j1 * ncol + i] + fx * fy * f[j1 * ncol + i1];
}

// Seaton's bound-free Gaunt factor (hydrogen.c:269-283).
__device__ __forceinline__ double gaunt_bf(double lam, double n_eff, double charge) {
  const double x = ((kHPLANCK * kCLIGHT) / (lam * kNM_TO_M)) / (kE_RYDBERG * (charge * charge));
  const double x3 = pow(x, 0.33333333);
  const double nsqx = 1.0 / ((n_eff * n_eff) * x);
  return 1.0 + 0.1728 * x3 * (1.0 - 2.0 * nsqx) -
         0.0496 * (x3 * x3) * (1.0 - (1.0 - nsqx) * 0.66666667 * nsqx);
}

// The same in the working precision (the metal continua's cross-sections,
// evaluated per atmosphere).
template <typename R>
__device__ __forceinline__ R gaunt_bf_r(R lam, R n_eff, R charge) {
  if constexpr (sizeof(R) == 8) {
    return gaunt_bf(lam, n_eff, charge);
  } else {
    const float x = (float(kHPLANCK * kCLIGHT / kNM_TO_M / kE_RYDBERG) / lam) / (charge * charge);
    const float x3 = powf(x, 0.33333333f);
    const float nsqx = 1.0f / ((n_eff * n_eff) * x);
    return 1.0f + 0.1728f * x3 * (1.0f - 2.0f * nsqx) -
           0.0496f * (x3 * x3) * (1.0f - (1.0f - nsqx) * 0.66666667f * nsqx);
  }
}

template <typename R>
__device__ __forceinline__ int bracket_r(const R* t, int n, R x) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (hi + lo) >> 1;
    if (x >= t[mid]) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <typename R>
__device__ __forceinline__ R spline_eval_r(const R* x, const R* y, const R* M, int n, R v) {
  if (v <= x[0]) return y[0];
  if (v >= x[n - 1]) return y[n - 1];
  const int j = bracket_r<R>(x, n, v);
  const R hj = x[j + 1] - x[j];
  const R fx = (v - x[j]) / hj;
  const R fx1 = R(1) - fx;
  return fx1 * y[j] + fx * y[j + 1] +
         (fx1 * (fx1 * fx1 - R(1)) * M[j] + fx * (fx * fx - R(1)) * M[j + 1]) * (hj * hj) / R(6);
}

// Natural cubic spline through (x, y) with second derivatives M (spline.c).
__device__ __forceinline__ double spline_eval(const double* x, const double* y, const double* M,
                                              int n, double v) {
  if (v <= x[0]) return y[0];
  if (v >= x[n - 1]) return y[n - 1];
  const int j = bracket(x, n, v);
  const double hj = x[j + 1] - x[j];
  const double fx = (v - x[j]) / hj;
  const double fx1 = 1 - fx;
  return fx1 * y[j] + fx * y[j + 1] +
         (fx1 * (fx1 * fx1 - 1) * M[j] + fx * (fx * fx - 1) * M[j + 1]) * (hj * hj) / 6.0;
}

// Cross-section of a metal continuum at lambda (metal.c:126-140).
template <typename R>
__device__ __forceinline__ R metal_alpha(const pyrh_bg_model& m, const pyrh_bg_continuum& C,
                                         double lam) {
  if constexpr (sizeof(R) == 8) {
    if (C.hydrogenic) {
      const double r = lam / C.lambda0;
      return C.alpha0 * (r * r * r) * gaunt_bf(lam, C.n_eff, C.charge) / C.gbf0;
    }
    return spline_eval(m.tab_lambda + C.tab_off, m.tab_alpha + C.tab_off, m.tab_m2 + C.tab_off,
                       C.ntab, lam);
  } else {
    const float l = (float)lam;
    if (C.hydrogenic) {
      const float r = l / (float)C.lambda0;
      return (float)C.alpha0 * (r * r * r) * gaunt_bf_r<float>(l, (float)C.n_eff, (float)C.charge) /
             (float)C.gbf0;
    }
    const int64_t N = m.ntab_total;
    return spline_eval_r<float>(m.tab_f32 + C.tab_off, m.tab_f32 + N + C.tab_off,
                                m.tab_f32 + 2 * N + C.tab_off, C.ntab, l);
  }
}

// linear.c:22-51 for one value of an ascending table.
__device__ __forceinline__ double linear(const double* xt, const double* yt, int n, double v) {
  if (v <= xt[0]) return yt[0];
  if (v >= xt[n - 1]) return yt[n - 1];
  const int j = bracket(xt, n, v);
  const double fx = (xt[j + 1] - v) / (xt[j + 1] - xt[j]);
  return fx * yt[j] + (1 - fx) * yt[j + 1];
}

// Second derivatives of the natural cubic spline through n points
// (spline.c:38-66), u as scratch.
__device__ void spline_coef(const double* x, const double* y, int n, double* M, double* u) {
  double hj = x[1] - x[0];
  double D = (y[1] - y[0]) / hj;
  M[0] = 0.0;   // holds q
  u[0] = 0.0;
  for (int j = 1; j < n - 1; ++j) {
    const double hj1 = x[j + 1] - x[j];
    const double mu = hj / (hj + hj1);
    const double D1 = (y[j + 1] - y[j]) / hj1;
    const double p = mu * M[j - 1] + 2;
    M[j] = (mu - 1) / p;
    u[j] = ((D1 - D) * 6 / (hj + hj1) - mu * u[j - 1]) / p;
    hj = hj1;
    D = D1;
  }
  M[n - 1] = 0.0;
  for (int j = n - 2; j >= 0; --j) M[j] = M[j] * M[j + 1] + u[j];
}

// One thread per tabulated continuum, and the H- bound-free table last.
__global__ void bg_spline_kernel(pyrh_bg_model m) {
  const int ncont = m.ncont_h + m.ncont_metal;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  double u[64];
  if (c < ncont) {
    const pyrh_bg_continuum C = m.cont[c];
    if (C.hydrogenic || C.ntab < 2 || C.ntab > 64) return;
    spline_coef(m.tab_lambda + C.tab_off, m.tab_alpha + C.tab_off, C.ntab,
                m.tab_m2 + C.tab_off, u);
    if (m.tab_f32)
      for (int i = 0; i < C.ntab; ++i) {
        const int64_t o = C.tab_off + i;
        m.tab_f32[o] = (float)m.tab_lambda[o];
        m.tab_f32[m.ntab_total + o] = (float)m.tab_alpha[o];
        m.tab_f32[2 * m.ntab_total + o] = (float)m.tab_m2[o];
      }
  } else if (c == ncont) {
    spline_coef(kHmBfLam, kHmBfAlpha, kHmBfN, m.tab_m2 + m.ntab_total, u);
  }
}

// What depends on the depth alone, staged per block (a block's threads
// share one atmosphere): [kDepthFields][max_ndep] in the working precision.
enum DepthField {
  kInvT, kNe, kPe, kNHmin, kNH0, kNp, kNH2, kNOH, kNCH, kRay0, kRay1, kSqrtTheta, kT,
  kHffDepth,                      // sigma_ff / sqrt(T) ne np (hydrogen.c:251-256)
  kFHmTheta, kFH2mTheta, kFH2pTemp,  // fractional table indices
  kFOHt, kFCHt,                      // OH / CH temperature index, -1 outside the table
  kDepthFields
};

// FP32 keeps its products inside its range: sigma_ff / sqrt(T) ne np (up to
// ~1e39 in deep layers) is staged times kFfScale and nu^3 divided by it, and
// John's constant k theta0 1e-32 (~7e-52) is split across the two densities.
template <typename R>
constexpr double kFfScale = sizeof(R) == 4 ? 1.0E-30 : 1.0;

template <typename R>
__device__ __forceinline__ R dexp(R x) { return exp(x); }
template <>
__device__ __forceinline__ float dexp<float>(float x) { return expf(x); }

// Opacity and emissivity of a wavelength's bound-free continua at one depth
// (hydrogen.c:205-212, metal.c:147-153): sum alpha (1 - e^-x) n_i and
// 2 h nu^3 / c^2 (n*_i / n*_j) e^-x alpha n_j, the LTE entries as one sum
// of alpha n_i.
template <typename R>
__device__ __forceinline__ void continuum_sums(const pyrh_bg_model& m, const R* P, int64_t td,
                                               int64_t d, const int* row, const R* alpha, int n,
                                               R omex, R twex, R& chi, R& eta) {
  R s = R(0), c = R(0), e = R(0);
  for (int q = 0; q < n; ++q) {
    const int r = row[q];
    if (r >= 0) {
      s += alpha[q] * P[(int64_t)r * td + d];
    } else {
      const pyrh_bg_continuum& C = m.cont[-1 - r];
      const R gn = P[(int64_t)C.nstar_i * td + d] / P[(int64_t)C.nstar_j * td + d] *
                   P[(int64_t)C.n_j * td + d];
      c += alpha[q] * P[(int64_t)C.n_i * td + d];
      e += alpha[q] * gn;
    }
  }
  chi = (s + c) * omex;
  eta = twex * (s + e);
}

// Everything that depends on the wavelength alone (FP64, kept in the
// working precision), evaluated once per thread and wavelength.
template <typename R>
struct LambdaTerms {
  bool hmbf, hm_long, oh, ch, ray[2], h2p, rh2, h2m;
  R hck, tw, a_hm, john[6], li_hm, ei_oh, ei_ch, nu3, x3ff, yT, sig_ray[2], li_h2p, sig_rh2,
      li_h2m, hf, sf, mf;
  int nh;
  // Each covered continuum is one entry (cross-section, row): row >= 0 names
  // the lower level's population row of a continuum whose populations are
  // the LTE ones (n = n*: its emissivity 2 h nu^3 / c^2 (n*_i / n*_j) e^-x
  // alpha n_j is 2 h nu^3 / c^2 e^-x alpha n_i), row < 0 the continuum
  // -1 - row of any other.
  int hc_row[kMaxHCont];
  R hc_sig[kMaxHCont];
  __device__ void init(const pyrh_bg_model& m, double lam, double sigma_T) {
    const double hc_kla = (kHPLANCK * kCLIGHT) / (kKBOLTZMANN * kNM_TO_M * lam);
    const double lm = kNM_TO_M * lam;
    const double twohnu3_c2 = (2.0 * kHPLANCK * kCLIGHT) / (lm * lm * lm);
    hck = R(hc_kla);
    tw = R(twohnu3_c2);
    // H- bound-free (hydrogen.c:336-345)
    hmbf = lam > kHmBfLam[0] && lam < kHmBfLam[kHmBfN - 1];
    a_hm = hmbf ? R(spline_eval(kHmBfLam, kHmBfAlpha, m.tab_m2 + m.ntab_total, kHmBfN, lam) *
                    1.0E-21)
                : R(0);
    // H- free-free: the table's wavelength index, or John's coefficients
    hm_long = lam >= kHmFfLam[kHmFfNL - 1];
    for (int n = 0; n < 6; ++n) john[n] = R(0);
    li_hm = R(0);
    if (hm_long) {
      const double lmu = lam / kMICRON_TO_NM, linv = 1.0 / lmu;
      for (int n = 1; n < 6; ++n)
        john[n] = R((lmu * lmu) * kJohnA[n] + kJohnB[n] +
                    linv * (kJohnC[n] + linv * (kJohnD[n] + linv * (kJohnE[n] + linv * kJohnF[n]))));
    } else {
      const int j = bracket(kHmFfLam, kHmFfNL, lam);
      li_hm = R(j + (lam - kHmFfLam[j]) / (kHmFfLam[j + 1] - kHmFfLam[j]));
    }
    // OH and CH (ohchbf.c:360-366)
    const double Eev = (kHPLANCK * kCLIGHT) / (lam * kNM_TO_M) / kEV;
    oh = m.has_oh && !(Eev < kOHEv[0] || Eev > kOHEv[kOHNE - 1]);
    ch = m.has_ch && !(Eev < kCHEv[0] || Eev > kCHEv[kCHNE - 1]);
    ei_oh = oh ? R(frac_index(kOHEv, kOHNE, Eev)) : R(0);
    ei_ch = ch ? R(frac_index(kCHEv, kCHNE, Eev)) : R(0);
    // hydrogen bound-free: cross-sections of the continua covering lambda
    nh = 0;
    if (!m.h_active)
      for (int c = 0; c < m.ncont_h && nh < kMaxHCont; ++c) {
        const pyrh_bg_continuum& C = m.cont[c];
        if (lam <= C.lambda0 && lam >= C.lambda_min) {
          const double r = lam / C.lambda0;
          hc_row[nh] = (C.n_i == C.nstar_i && C.n_j == C.nstar_j) ? C.n_i : -1 - c;
          hc_sig[nh] = R(C.alpha0 * gaunt_bf(lam, C.n_eff, C.charge) * (r * r * r));
          ++nh;
        }
      }
    // hydrogen free-free (hydrogen.c:241-256): wavelength terms
    const double lc = (lam * kNM_TO_M) / kCLIGHT;
    nu3 = R(lc * lc * lc / kFfScale<R>);
    x3ff = R(pow(((kHPLANCK * kCLIGHT) / (lam * kNM_TO_M)) / kE_RYDBERG, 0.33333333));
    yT = R((2.0 * lam * kNM_TO_M * kKBOLTZMANN) / (kHPLANCK * kCLIGHT));   // y = yT T
    // Rayleigh by hydrogen and helium (rayleigh.c:60-90)
    {
      double fomega[2] = {0.0, 0.0};
      for (int s = 0; s < 2; ++s) ray[s] = m.ray_pop[s] >= 0 && lam > m.ray_limit[s];
      for (int r = 0; r < m.nray; ++r) {
        const pyrh_bg_rayleigh_line& L = m.ray[r];
        const int s = L.scatterer;
        if (s < 0 || s > 1 || !ray[s] || !(lam > L.lambda_red)) continue;
        const double q = lam / L.lambda0;
        const double lambda2 = 1.0 / (q * q - 1.0);
        fomega[s] += L.f * (lambda2 * lambda2);
      }
      for (int s = 0; s < 2; ++s) sig_ray[s] = R(sigma_T * fomega[s]);
    }
    // H + H+ free-free, H2 Rayleigh, H2- free-free
    h2p = lam < kH2pLam[kH2pNL - 1];
    li_h2p = R(0);
    if (h2p) {
      const int j = bracket(kH2pLam, kH2pNL, lam);
      li_h2p = R(j + (lam - kH2pLam[j]) / (kH2pLam[j + 1] - kH2pLam[j]));
    }
    rh2 = m.has_h2 && lam >= kRAYLEIGH_H2_LIMIT;
    sig_rh2 = R(0);
    if (rh2) {
      double s2;
      if (lam <= kRH2Lam[kRH2N - 1]) {
        s2 = linear(kRH2Lam, kRH2Sigma, kRH2N, lam);
      } else {
        const double l2 = 1.0 / (lam * lam);
        s2 = (kRH2Coef[0] + (kRH2Coef[1] + kRH2Coef[2] * l2) * l2) * (l2 * l2);
      }
      sig_rh2 = R(s2 * kMEGABARN_TO_M2);
    }
    h2m = m.has_h2 && lam < kH2mLam[kH2mNL - 1];
    li_h2m = R(0);
    if (h2m) {
      const int j = bracket(kH2mLam, kH2mNL, lam);
      li_h2m = R(j + (lam - kH2mLam[j]) / (kH2mLam[j + 1] - kH2mLam[j]));
    }
    hf = sf = mf = R(1);
    if (m.nfudge > 1) {
      hf = R(linear(m.fudge_lambda, m.fudge, m.nfudge, lam));
      sf = R(linear(m.fudge_lambda, m.fudge + m.nfudge, m.nfudge, lam));
      mf = R(linear(m.fudge_lambda, m.fudge + 2 * m.nfudge, m.nfudge, lam));
    }
  }
};

// Atmospheres per block, at most: the wavelength terms are evaluated once
// for the group when its atmospheres share the wavelength (the usual
// batch); small batches take smaller groups so that every SM has blocks.
constexpr int kGroup = 8;

// Shared memory of a block: the depth fields, then the metal continua's
// per-depth sums [nacc][max_ndep][blockDim] (nacc 1, or 3 with non-LTE
// continua): each thread adds its wavelength's continua into its own
// column, one continuum at a time, so the cross-sections are evaluated once
// per atmosphere and wavelength and never stored.
template <typename R>
__host__ __device__ inline size_t bg_smem_bytes(int max_ndep, int block, int nonlte) {
  return sizeof(R) * (size_t)max_ndep * (kDepthFields + (size_t)(nonlte ? 3 : 1) * block);
}

template <typename R>
__global__ void __launch_bounds__(kBlock)
bg_kernel(pyrh_bg_model m, pyrh_bg_batch b, int group) {
  extern __shared__ __align__(16) unsigned char bg_smem[];
  R* ds = reinterpret_cast<R*>(bg_smem);
  const int MD = b.max_ndep;
  const int64_t td = b.total_depth;
  const R* P = static_cast<const R*>(b.pops);
  const double sigma_T = 8.0 * kPI / 3.0 *
                         pow(kQ_ELECTRON / (sqrt(4.0 * kPI * kEPSILON_0) *
                                            (sqrt(kM_ELECTRON) * kCLIGHT)), 4);
  const double C0 = (kQ_ELECTRON * kQ_ELECTRON) / (4.0 * kPI * kEPSILON_0) / sqrt(kM_ELECTRON);
  const double sigma_ff = 4.0 / 3.0 * sqrt(2.0 * kPI / (3.0 * kKBOLTZMANN)) * (C0 * C0 * C0) /
                          (kHPLANCK * kCLIGHT);
  const R sT = R(sigma_T);
  const int bd = blockDim.x, tid = threadIdx.x;
  const int la = blockIdx.x * bd + tid;
  R* acc_s = ds + kDepthFields * MD;       // sum of alpha n_i of the LTE continua
  R* acc_c = acc_s + (size_t)MD * bd;      // non-LTE: sum of alpha n_i
  R* acc_e = acc_c + (size_t)MD * bd;      // non-LTE: sum of alpha (n*_i / n*_j) n_j
  LambdaTerms<R> t;
  double lam_have = -1.0;
  R* chi_o = static_cast<R*>(b.chi_c);
  R* eta_o = static_cast<R*>(b.eta_c);
  R* sca_o = static_cast<R*>(b.sca_c);
  auto D = [&](int f, int k) { return ds[f * MD + k]; };
  for (int pi = 0; pi < group; ++pi) {
    const int p = blockIdx.y * group + pi;
    if (p >= b.natm) break;                              // uniform in the block
    const int nd = b.ndep[p], ns = b.nspect[p];
    if ((int)blockIdx.x * bd >= ns || nd > MD) continue;   // uniform in the block
    const int64_t doff = b.depth_off[p], coff = b.cont_off[p];
    __syncthreads();                                     // the previous atmosphere's reads
    for (int k = threadIdx.x; k < nd; k += blockDim.x) {
      const int64_t d = doff + k;
      const double T = b.T[d], ne = b.ne[d];
      const double nh0 = P[(int64_t)m.pop_nh0 * td + d], np = P[(int64_t)m.pop_np * td + d];
      auto put = [&](int f, double v) { ds[f * MD + k] = R(v); };
      put(kInvT, 1.0 / T);
      put(kT, T);
      put(kNe, ne);
      put(kPe, ne * kKBOLTZMANN * T);
      put(kNHmin, b.nHmin[d]);
      put(kNH0, nh0);
      put(kNp, np);
      put(kNH2, m.has_h2 ? b.nH2[d] : 0.0);
      put(kNOH, m.has_oh ? b.nOH[d] : 0.0);
      put(kNCH, m.has_ch ? b.nCH[d] : 0.0);
      put(kRay0, m.ray_pop[0] >= 0 ? (double)P[(int64_t)m.ray_pop[0] * td + d] : 0.0);
      put(kRay1, m.ray_pop[1] >= 0 ? (double)P[(int64_t)m.ray_pop[1] * td + d] : 0.0);
      put(kSqrtTheta, sqrt(kTHETA0 / T));
      put(kHffDepth, sigma_ff / sqrt(T) * ne * np * kFfScale<R>);
      put(kFHmTheta, frac_index(kHmFfTheta, kHmFfNT, kTHETA0 / T));
      put(kFH2mTheta, frac_index(kH2mTheta, kH2mNT, kTHETA0 / T));
      put(kFH2pTemp, frac_index(kH2pTemp, kH2pNT, T));
      put(kFOHt, (T < kOHTemp[0] || T > kOHTemp[kOHNT - 1]) ? -1.0 : frac_index(kOHTemp, kOHNT, T));
      put(kFCHt, (T < kCHTemp[0] || T > kCHTemp[kCHNT - 1]) ? -1.0 : frac_index(kCHTemp, kCHNT, T));
    }
    __syncthreads();
    if (la >= ns) continue;
    const double lam = b.lambda[b.lam_off[p] + la];
    if (!(lam == lam_have)) {
      t.init(m, lam, sigma_T);
      lam_have = lam;
    }
    // metals (metal.c:103-153): per-depth sums of the continua covering lambda
    for (int k = 0; k < nd; ++k) acc_s[k * bd + tid] = R(0);
    if (m.nonlte)
      for (int k = 0; k < nd; ++k) acc_c[k * bd + tid] = acc_e[k * bd + tid] = R(0);
    bool any_metal = false;
    for (int c = m.ncont_h; c < m.ncont_h + m.ncont_metal; ++c) {
      const pyrh_bg_continuum& C = m.cont[c];
      if (!(lam <= C.lambda0 && lam >= C.lambda_min)) continue;
      any_metal = true;
      const R a = metal_alpha<R>(m, C, lam);
      if (C.n_i == C.nstar_i && C.n_j == C.nstar_j) {
        const R* pi = P + (int64_t)C.n_i * td + doff;
        for (int k = 0; k < nd; ++k) acc_s[k * bd + tid] += a * pi[k];
      } else {
        const R* pi = P + (int64_t)C.n_i * td + doff;
        const R* pj = P + (int64_t)C.n_j * td + doff;
        const R* si = P + (int64_t)C.nstar_i * td + doff;
        const R* sj = P + (int64_t)C.nstar_j * td + doff;
        for (int k = 0; k < nd; ++k) {
          acc_c[k * bd + tid] += a * pi[k];
          acc_e[k * bd + tid] += a * (si[k] / sj[k] * pj[k]);
        }
      }
    }

    // --- down the atmosphere
    for (int k = 0; k < nd; ++k) {
      const int64_t d = doff + k;
      const R xT = t.hck * D(kInvT, k);
      const R ex = dexp<R>(-xT);
      const R omex = R(1) - ex;
      // planck.c:38-63 from the same exponential: 2 h nu^3 / c^2 e^-x / (1 - e^-x)
      const R B = (xT <= R(150)) ? t.tw * ex / omex : R(0);
      const R pe = D(kPe, k), nH0 = D(kNH0, k), ne = D(kNe, k);
      R chi = R(0), eta = R(0);
      R sca = ne * sT;
      if (t.hmbf) {
        const R nm = D(kNHmin, k);
        chi += nm * omex * t.a_hm;
        eta += nm * t.tw * ex * t.a_hm;
      }
      {
        R cff;
        if (t.hm_long) {
          R s = R(0), tn = R(1);
          const R st = D(kSqrtTheta, k);
          for (int n = 1; n < 6; ++n) {
            tn *= st;
            s += tn * t.john[n];
          }
          if constexpr (sizeof(R) == 8)
            cff = s * (nH0 * (ne * R(kKBOLTZMANN * kTHETA0 * 1.0E-32)));
          else
            cff = s * ((nH0 * R(1.0E-26)) * (ne * R(kKBOLTZMANN * kTHETA0 * 1.0E-6)));
        } else {
          const R kap = bilinear_r<R>(kHmFfNT, kHmFfNL, DepthTables<R>::hmff(), D(kFHmTheta, k),
                                      t.li_hm);
          cff = (nH0 * R(1.0E-29)) * pe * kap;
        }
        chi += cff;
        eta += cff * B;
      }
      chi *= t.hf;
      eta *= t.hf;
      if (t.oh && D(kFOHt, k) >= R(0)) {
        const R kap = dexp<R>(R(kLG10) * bilinear_r<R>(kOHNT, kOHNE, DepthTables<R>::oh(),
                                                       D(kFOHt, k), t.ei_oh)) *
                      R(kCM_TO_M * kCM_TO_M);
        const R n = D(kNOH, k);
        chi += n * omex * kap;
        eta += n * t.tw * ex * kap;
      }
      if (t.ch && D(kFCHt, k) >= R(0)) {
        const R kap = dexp<R>(R(kLG10) * bilinear_r<R>(kCHNT, kCHNE, DepthTables<R>::ch(),
                                                       D(kFCHt, k), t.ei_ch)) *
                      R(kCM_TO_M * kCM_TO_M);
        const R n = D(kNCH, k);
        chi += n * omex * kap;
        eta += n * t.tw * ex * kap;
      }
      if (t.nh > 0) {
        R cb, eb;
        continuum_sums<R>(m, P, td, d, t.hc_row, t.hc_sig, t.nh, omex, t.tw * ex, cb, eb);
        chi += cb;
        eta += eb;
      }
      {
        // Seaton's free-free Gaunt factor at charge 1 (hydrogen.c:286-304)
        const R y = t.yT * D(kT, k);
        R g = R(1) + R(0.1728) * t.x3ff * (R(1) + y) -
              R(0.0496) * (t.x3ff * t.x3ff) * (R(1) + (R(1) + y) * R(0.33333333) * y);
        g = g > R(1) ? g : R(1);
        const R cff = D(kHffDepth, k) * t.nu3 * omex * g;
        chi += cff;
        eta += cff * B;
      }
      if (t.ray[0]) sca += t.sig_ray[0] * D(kRay0, k);
      if (t.ray[1]) sca += t.sig_ray[1] * D(kRay1, k);
      if (t.h2p) {
        const R kap = bilinear_r<R>(kH2pNT, kH2pNL, DepthTables<R>::h2p(), D(kFH2pTemp, k),
                                    t.li_h2p);
        const R cff = (nH0 * R(1.0E-29)) * (D(kNp, k) * R(1.0E-20)) * kap;
        chi += cff;
        eta += cff * B;
      }
      if (t.rh2) sca += t.sig_rh2 * D(kNH2, k);
      if (t.h2m) {
        const R nh2 = D(kNH2, k);
        R cff = R(0);
        if (nh2 > R(0))
          cff = (nh2 * R(1.0E-29)) * pe *
                bilinear_r<R>(kH2mNT, kH2mNL, DepthTables<R>::h2m(), D(kFH2mTheta, k), t.li_h2m);
        chi += cff;
        eta += cff * B;
      }
      if (any_metal) {
        const R sl = acc_s[k * bd + tid];
        const R cm = m.nonlte ? sl + acc_c[k * bd + tid] : sl;
        const R em = m.nonlte ? sl + acc_e[k * bd + tid] : sl;
        chi += cm * omex * t.mf;
        eta += t.tw * ex * em * t.mf;
      }
      sca *= t.sf;
      if (m.add_scatter) chi += sca;
      const int64_t o = coff + (int64_t)k * ns + la;
      chi_o[o] = chi;
      eta_o[o] = eta;
      sca_o[o] = sca;
    }
  }
}

}  // namespace
}  // namespace pyrh

extern "C" {

pyrh_status pyrh_background_prepare(const pyrh_bg_model* model, void* stream) {
  pyrh::set_launches(0);
  if (!model || !model->tab_m2 || (model->ncont_h + model->ncont_metal > 0 && !model->cont) ||
      model->ncont_h < 0 || model->ncont_metal < 0 || model->ncont_h > pyrh::kMaxHCont) {
    pyrh::set_error("background model: NULL arrays or hydrogen continua beyond %d",
                    pyrh::kMaxHCont);
    return PYRH_ERR_ARG;
  }
  const int ncont = model->ncont_h + model->ncont_metal;
  // rows, tables and the nonlte flag, from a host copy of the continua
  if (ncont > 0) {
    pyrh_bg_continuum* hc = new pyrh_bg_continuum[ncont];
    cudaError_t e = cudaMemcpy(hc, model->cont, sizeof(pyrh_bg_continuum) * ncont,
                               cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      delete[] hc;
      pyrh::set_error("background model: %s", cudaGetErrorString(e));
      return PYRH_ERR_CUDA;
    }
    bool bad_tab = false, bad_row = false, nonlte = false;
    auto row_ok = [&](int32_t r) { return r >= 0 && r < model->npop; };
    for (int c = 0; c < ncont; ++c) {
      const pyrh_bg_continuum& C = hc[c];
      if (!row_ok(C.n_i) || !row_ok(C.n_j) || !row_ok(C.nstar_i) || !row_ok(C.nstar_j))
        bad_row = true;
      if (!C.hydrogenic && (C.ntab < 2 || C.ntab > 64 || C.tab_off < 0 ||
                            C.tab_off + C.ntab > model->ntab_total))
        bad_tab = true;
      if (c < model->ncont_h) continue;
      if (C.n_i != C.nstar_i || C.n_j != C.nstar_j) nonlte = true;
    }
    delete[] hc;
    if (nonlte && !model->nonlte) {
      pyrh::set_error("background model: non-LTE metal continua with nonlte = 0");
      return PYRH_ERR_ARG;
    }
    if (bad_row || bad_tab) {
      pyrh::set_error(bad_row ? "background model: a population row outside [0, npop)"
                              : "background model: a table with fewer than 2 or more than 64 "
                                "points, or outside ntab_total");
      return PYRH_ERR_ARG;
    }
  }
  const int n = ncont + 1;
  pyrh::bg_spline_kernel<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(*model);
  cudaError_t e = cudaGetLastError();
  pyrh::set_launches(1);
  if (e != cudaSuccess) {
    pyrh::set_error("background prepare: %s", cudaGetErrorString(e));
    return PYRH_ERR_CUDA;
  }
  return PYRH_OK;
}

pyrh_status pyrh_background(const pyrh_bg_model* model, const pyrh_bg_batch* b, void* stream) {
  pyrh::set_launches(0);
  if (!model || !b || b->natm < 1 || b->max_nspect < 1 || !b->ndep || !b->nspect ||
      (b->precision != PYRH_FP32 && b->precision != PYRH_FP64) ||
      !b->depth_off || !b->lam_off || !b->cont_off || !b->lambda || !b->T || !b->ne ||
      !b->nHmin || !b->pops || !b->chi_c || !b->eta_c || !b->sca_c ||
      (model->has_h2 && !b->nH2) || (model->has_oh && !b->nOH) || (model->has_ch && !b->nCH)) {
    pyrh::set_error("background batch: NULL array or empty batch");
    return PYRH_ERR_ARG;
  }
  if (b->natm > 65535) {
    pyrh::set_error("background batch: %d atmospheres (limit 65535 per call)", b->natm);
    return PYRH_ERR_ARG;
  }
  if (b->max_ndep < 1 || b->max_ndep > PYRH_BG_MAX_DEPTH) {
    pyrh::set_error("background batch: max_ndep %d outside [1, %d]", b->max_ndep,
                    PYRH_BG_MAX_DEPTH);
    return PYRH_ERR_ARG;
  }
  auto row_ok = [&](int32_t r) { return r >= 0 && r < model->npop; };
  if (!row_ok(model->pop_nh0) || !row_ok(model->pop_np) ||
      (model->ray_pop[0] >= model->npop) || (model->ray_pop[1] >= model->npop) ||
      (model->nray > 0 && !model->ray) || (model->nfudge > 1 && (!model->fudge_lambda || !model->fudge))) {
    pyrh::set_error("background model: a population row outside [0, npop) or a NULL table");
    return PYRH_ERR_ARG;
  }
  // the widest block (of 32 to 128 threads) whose sums fit the shared memory
  const bool f32 = b->precision == PYRH_FP32;
  if (f32 && !model->tab_f32) {
    pyrh::set_error("background: an FP32 batch needs model->tab_f32");
    return PYRH_ERR_ARG;
  }
  auto smem_of = [&](int bs) {
    return f32 ? pyrh::bg_smem_bytes<float>(b->max_ndep, bs, model->nonlte)
               : pyrh::bg_smem_bytes<double>(b->max_ndep, bs, model->nonlte);
  };
  int bs = pyrh::kBlock;
  while (bs > 32 && smem_of(bs) > 160 * 1024) bs -= 32;
  const size_t smem = smem_of(bs);
  if (smem > 220 * 1024) {
    pyrh::set_error("background: %d depths need %zu B of shared memory", b->max_ndep, smem);
    return PYRH_ERR_UNSUPPORTED;
  }
  const int ntile = (b->max_nspect + bs - 1) / bs;
  int dev = 0, nsm = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int group = (int)(((int64_t)b->natm * ntile) / (4 * (int64_t)nsm));
  group = group < 1 ? 1 : (group > pyrh::kGroup ? pyrh::kGroup : group);
  dim3 g(ntile, (b->natm + group - 1) / group);
  cudaError_t ea;
  if (f32) {
    ea = cudaFuncSetAttribute(pyrh::bg_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem);
    if (ea == cudaSuccess)
      pyrh::bg_kernel<float><<<g, bs, smem, (cudaStream_t)stream>>>(*model, *b, group);
  } else {
    ea = cudaFuncSetAttribute(pyrh::bg_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem);
    if (ea == cudaSuccess)
      pyrh::bg_kernel<double><<<g, bs, smem, (cudaStream_t)stream>>>(*model, *b, group);
  }
  if (ea != cudaSuccess) {
    pyrh::set_error("background: %s", cudaGetErrorString(ea));
    return PYRH_ERR_CUDA;
  }
  cudaError_t e = cudaGetLastError();
  pyrh::set_launches(1);
  if (e != cudaSuccess) {
    pyrh::set_error("background: %s", cudaGetErrorString(e));
    return PYRH_ERR_CUDA;
  }
  return PYRH_OK;
}

}  // extern "C"
