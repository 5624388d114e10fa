// rt_device.cuh -- device building blocks of the formal solution.
//
// Restates, for FP64 and FP32 evaluation on sm_103a:
//   humlicek        rh/voigt.c:381-419, rh/humlicek.c:28-118 (Humlicek 1982,
//                   JQSRT 27, 437; W(z) for z = a - i v in four regions)
//   cent_deriv      rh/bezier_aux.c:34-51 (Fritsch & Butland 1984)
//   bezier3_coeffs  rh/bezier_aux.c:333-359; the FP32 form evaluates the
//                   closed expressions only for dt >= 1.5 and a Taylor
//                   series below, because the closed form cancels
//                   catastrophically in single precision for small dt
//   w3              rh/w3.c:44-63 (always FP64)
//   planck          rh/planck.c:38-63 (always FP64)
#pragma once

#include <cuda_runtime.h>
#include <math.h>

// Functions here are host-and-device so the same math is unit-testable on
// the CPU (FP64); single-precision hardware intrinsics are device-only.
#define PYRH_HD __host__ __device__ __forceinline__

namespace pyrh {

// Physical constants with the values of the reference (rh/constant.h:28-68).
constexpr double kCLIGHT = 2.99792458E+08;
constexpr double kHPLANCK = 6.6260755E-34;
constexpr double kKBOLTZMANN = 1.380658E-23;
constexpr double kAMU = 1.6605402E-27;
constexpr double kM_ELECTRON = 9.1093897E-31;
constexpr double kQ_ELECTRON = 1.60217733E-19;
constexpr double kNM_TO_M = 1.0E-09;
constexpr double kPI = 3.14159265358979;
constexpr double kSQRTPI = 1.77245385090551;
constexpr double kLARMOR = (kQ_ELECTRON / (4.0 * kPI * kM_ELECTRON)) * kNM_TO_M;
constexpr double kQ_WING = 20.0;
constexpr double kMAX_GAUSS_DOPPLER = 7.0;

template <typename R> struct Cx { R r, i; };

template <typename R>
PYRH_HD Cx<R> cmul(Cx<R> a, Cx<R> b) {
  return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r};
}
// Division: IEEE in FP64; in FP32 the fast reciprocal-based division
// (__fdividef, 2 ulp), which the FP32 accuracy budget (1e-4) allows.
PYRH_HD double fdiv(double a, double b) { return a / b; }

// A hint that moves the cache line of p (generic address: local memory or a
// global array) into L1; nothing on the host.
PYRH_HD void prefetch_l1(const void* p) {
#ifdef __CUDA_ARCH__
  asm volatile("prefetch.L1 [%0];" ::"l"(p));
#else
  (void)p;
#endif
}
PYRH_HD float fdiv(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdividef(a, b);
#else
  return a / b;
#endif
}

template <typename R>
PYRH_HD Cx<R> cdiv(Cx<R> a, Cx<R> b) {
  R inv = fdiv(R(1), b.r * b.r + b.i * b.i);
  return {(a.r * b.r + a.i * b.i) * inv, (a.i * b.r - a.r * b.i) * inv};
}

PYRH_HD double dev_exp(double x) { return exp(x); }
PYRH_HD float dev_exp(float x) {
#ifdef __CUDA_ARCH__
  return __expf(x);
#else
  return expf(x);
#endif
}
PYRH_HD void dev_sincos(double x, double* s, double* c) {
#ifdef __CUDA_ARCH__
  sincos(x, s, c);
#else
  *s = ::sin(x);
  *c = ::cos(x);
#endif
}
// |x| <= 2 a |v| stays below ~11 in Humlicek region IV; the hardware sine /
// cosine keeps an absolute error near 1e-6 there, far inside the budget.
PYRH_HD void dev_sincos(float x, float* s, float* c) {
#ifdef __CUDA_ARCH__
  __sincosf(x, s, c);
#else
  *s = ::sinf(x);
  *c = ::cosf(x);
#endif
}

// Humlicek W4: returns H = Re W, F = Im W for t = a - i v.
template <typename R>
PYRH_HD void humlicek(R a, R v, R& H, R& F) {
  const Cx<R> t = {a, -v};
  const R s = fabs(v) + a;
  Cx<R> W;
  if (s >= R(15.0)) {
    Cx<R> num = {R(0.5641896) * t.r, R(0.5641896) * t.i};
    Cx<R> den = cmul(t, t);
    den.r += R(0.5);
    W = cdiv(num, den);
  } else if (s >= R(5.5)) {
    Cx<R> u = cmul(t, t);
    Cx<R> num = {R(0.5641896) * u.r + R(1.410474), R(0.5641896) * u.i};
    num = cmul(t, num);
    Cx<R> den = {u.r + R(3.0), u.i};
    den = cmul(u, den);
    den.r += R(0.75);
    W = cdiv(num, den);
  } else if (a >= R(0.195) * fabs(v) - R(0.176)) {
    Cx<R> num = {R(0.5642236), R(0)};
    Cx<R> den = {t.r + R(6.699398), t.i};
    num = cmul(num, t); num.r += R(3.778987);
    den = cmul(den, t); den.r += R(21.69274);
    num = cmul(num, t); num.r += R(11.96482);
    den = cmul(den, t); den.r += R(39.27121);
    num = cmul(num, t); num.r += R(20.20933);
    den = cmul(den, t); den.r += R(38.82363);
    num = cmul(num, t); num.r += R(16.4955);
    den = cmul(den, t); den.r += R(16.4955);
    W = cdiv(num, den);
  } else {
    // u = -t^2
    Cx<R> u = {-(t.r * t.r - t.i * t.i), -(R(2) * t.r * t.i)};
    Cx<R> num = {R(0.56419), R(0)};
    Cx<R> den = {u.r + R(1.841439), u.i};
    num = cmul(u, num); num.r += R(1.320522);
    den = cmul(u, den); den.r += R(61.57037);
    num = cmul(u, num); num.r += R(35.7668);
    den = cmul(u, den); den.r += R(364.2191);
    num = cmul(u, num); num.r += R(219.031);
    den = cmul(u, den); den.r += R(2186.181);
    num = cmul(u, num); num.r += R(1540.787);
    den = cmul(u, den); den.r += R(9022.228);
    num = cmul(u, num); num.r += R(3321.99);
    den = cmul(u, den); den.r += R(24322.84);
    num = cmul(u, num); num.r += R(36183.31);
    den = cmul(u, den); den.r += R(32066.6);
    R e = dev_exp(-u.r), sn, cs;
    dev_sincos(-u.i, &sn, &cs);
    Cx<R> r = cdiv(cmul(t, num), den);
    W = {e * cs - r.r, e * sn - r.i};
  }
  H = W.r;
  F = W.i;
}

template <typename R>
PYRH_HD R cent_deriv(R dsup, R dsdn, R up, R c, R dn) {
  R fim1 = fdiv(c - up, dsup), fi = fdiv(dn - c, dsdn);
  if (fim1 * fi > R(0)) {
    R alpha = R(0.333333333333333333333333) * (R(1) + fdiv(dsdn, dsdn + dsup));
    return fdiv(fim1 * fi, (R(1) - alpha) * fim1 + alpha * fi);
  }
  return R(0);
}

// cent_deriv with the path lengths' reciprocals and the weight alpha
// precomputed (shared by all entries of one depth).
template <typename R>
PYRH_HD R cent_deriv_w(R rdsup, R rdsdn, R alpha, R up, R c, R dn) {
  R fim1 = (c - up) * rdsup, fi = (dn - c) * rdsdn;
  if (fim1 * fi > R(0)) return fdiv(fim1 * fi, (R(1) - alpha) * fim1 + alpha * fi);
  return R(0);
}

struct BezierW { double a, b, g, t, e; };

// Reference branches (FP64 mode).
PYRH_HD void bezier3_coeffs(double dt, double& alpha, double& beta,
                                               double& gamma, double& theta, double& eps) {
  double dt2 = dt * dt, dt3 = dt2 * dt;
  if (dt >= 5.e-2) {
    double e = exp(-dt);
    eps = e;
    alpha = (-6.0 + 6.0 * dt - 3.0 * dt2 + dt3 + 6.0 * e) / dt3;
    double r3 = 1.0 / dt3;
    beta = (6.0 + (-6.0 - dt * (6.0 + dt * (3.0 + dt))) * e) * r3;
    gamma = 3.0 * (6.0 + (-4.0 + dt) * dt - 2.0 * (3.0 + dt) * e) * r3;
    theta = 3.0 * (e * (6.0 + dt2 + 4.0 * dt) + 2.0 * dt - 6.0) * r3;
  } else {
    double dt4 = dt2 * dt2;
    eps = 1.0 - dt + 0.5 * dt2 - dt3 / 6.0 + dt4 / 24.0;
    alpha = 0.25 * dt - 0.05 * dt2 + dt3 / 120.0 - dt4 / 840.0;
    beta = 0.25 * dt - 0.20 * dt2 + dt3 / 12.0 - dt4 / 42.0;
    gamma = 0.25 * dt - 0.10 * dt2 + dt3 * 0.025 - dt4 / 210.0;
    theta = 0.25 * dt - 0.15 * dt2 + dt3 * 0.05 - dt4 / 84.0;
  }
}

// FP32 mode: Taylor series (x^1..x^11) of the same weights for dt < 1.5,
// the closed form above it; the series coefficients are the exact Taylor
// coefficients of the closed forms (alternating tails of exp(-x)).
PYRH_HD float horner11(float x, const float* c) {
  float s = c[10];
#pragma unroll
  for (int i = 9; i >= 0; --i) s = fmaf(s, x, c[i]);
  return s * x;
}

PYRH_HD void bezier3_coeffs(float dt, float& alpha, float& beta,
                                               float& gamma, float& theta, float& eps) {
  eps = expf(-dt);
  if (dt >= 1.5f) {
    float dt2 = dt * dt, dt3 = dt2 * dt, r3 = 1.0f / dt3;
    alpha = (-6.0f + 6.0f * dt - 3.0f * dt2 + dt3 + 6.0f * eps) * r3;
    beta = (6.0f + (-6.0f - dt * (6.0f + dt * (3.0f + dt))) * eps) * r3;
    gamma = 3.0f * (6.0f + (-4.0f + dt) * dt - 2.0f * (3.0f + dt) * eps) * r3;
    theta = 3.0f * (eps * (6.0f + dt2 + 4.0f * dt) + 2.0f * dt - 6.0f) * r3;
  } else {
    const float ca[11] = {0.25f, -0.05f, 8.333333333e-3f, -1.190476190e-3f, 1.488095238e-4f,
                          -1.653439153e-5f, 1.653439153e-6f, -1.503126503e-7f,
                          1.252605419e-8f, -9.635426302e-10f, 6.882447359e-11f};
    const float cb[11] = {0.25f, -0.2f, 8.333333333e-2f, -2.380952381e-2f, 5.208333333e-3f,
                          -9.259259259e-4f, 1.388888889e-4f, -1.803751804e-5f,
                          2.066798942e-6f, -2.119793786e-7f, 1.968379945e-8f};
    const float cg[11] = {0.25f, -0.1f, 0.025f, -4.761904762e-3f, 7.440476190e-4f,
                          -9.920634921e-5f, 1.157407407e-5f, -1.202501203e-6f,
                          1.127344877e-7f, -9.635426302e-9f, 7.570692095e-10f};
    const float ct[11] = {0.25f, -0.15f, 0.05f, -1.190476190e-2f, 2.232142857e-3f,
                          -3.472222222e-4f, 4.629629630e-5f, -5.411255411e-6f,
                          5.636724387e-7f, -5.299484466e-8f, 4.542415257e-9f};
    alpha = horner11(dt, ca);
    beta = horner11(dt, cb);
    gamma = horner11(dt, cg);
    theta = horner11(dt, ct);
  }
}

PYRH_HD void w3(double dtau, double* w) {
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

PYRH_HD double planck(double T, double lambda) {
  double hc_kla = (kHPLANCK * kCLIGHT) / (kKBOLTZMANN * kNM_TO_M * lambda);
  double l = kNM_TO_M * lambda;
  double twohnu3_c2 = (2.0 * kHPLANCK * kCLIGHT) / (l * l * l);
  double x = hc_kla / T;
  return (x <= 150.0) ? twohnu3_c2 / (exp(x) - 1.0) : 0.0;
}

// The same in single precision (the FP32 synthesis kernel's boundary
// condition); exp(x) overflows float above x = 88, where B is far below the
// smallest emissivity of a float continuum, so the cut is at 80.
PYRH_HD float planck_f(float T, double lambda) {
  const float hc_kla = float((kHPLANCK * kCLIGHT) / (kKBOLTZMANN * kNM_TO_M)) / float(lambda);
  const float l = float(lambda);
  const float twohnu3_c2 = float(2.0 * kHPLANCK * kCLIGHT / (kNM_TO_M * kNM_TO_M * kNM_TO_M)) / (l * l * l);
  const float x = hc_kla / T;
  return (x <= 80.0f) ? twohnu3_c2 / (expf(x) - 1.0f) : 0.0f;
}

// Solve M x = b for a 4x4 system by LU without pivoting (the DELO-Bezier
// matrices are unit-diagonal-dominated; the reference inverts them by
// cofactors, rh/bezier_aux.c:133-329).  All indices are compile-time.
template <typename R>
PYRH_HD void solve4(R M[4][4], const R b[4], R x[4]) {
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    R inv = R(1) / M[c][c];
#pragma unroll
    for (int r = c + 1; r < 4; ++r) {
      R f = M[r][c] * inv;
      M[r][c] = f;
#pragma unroll
      for (int j = c + 1; j < 4; ++j) M[r][j] -= f * M[c][j];
    }
  }
  R y[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    R s = b[r];
#pragma unroll
    for (int j = 0; j < r; ++j) s -= M[r][j] * y[j];
    y[r] = s;
  }
#pragma unroll
  for (int r = 3; r >= 0; --r) {
    R s = y[r];
#pragma unroll
    for (int j = r + 1; j < 4; ++j) s -= M[r][j] * x[j];
    x[r] = s / M[r][r];
  }
}

}  // namespace pyrh
