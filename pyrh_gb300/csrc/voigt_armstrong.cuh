// voigt_armstrong.cuh -- Armstrong's (1967) Voigt function H(a, v) as the
// reference evaluates it (rh/voigt.c:126-243): the Dawson-function series
// for small a and v, and 10-point Gauss-Hermite quadratures elsewhere.  The
// NLTE line profiles use it in FP64 (profile.c:67-371); the LTE synthesis
// uses it, in the working precision, for Kurucz lines that are not
// polarizable (kurucz.c:824); the response-function code instantiates it on
// a two-direction dual number (Dual2 below) for dH/da and dH/dv, the exact
// derivative of this approximation branch by branch.  Tables in this file
// are per translation unit.
#pragma once

#include "rt_device.cuh"

namespace pyrh {

// ------------------------------------------------------- Armstrong Voigt --
// Chebyshev coefficients of Dawson(5x) in odd T_{2n+1}(x) on [0,1] and the
// 20-point Gauss-Hermite rule (positive half), both from their definitions.
#define PYRH_ARMSTRONG_DAWSON { \
    0.1999999999972224, -0.18400000000299979, 0.15583999999650247, -0.12166400000439881, \
    0.087708159994039123, -0.058514124808690643, 0.036215730162391359, -0.020849765439803627, \
    0.011196011634627011, -0.0056231896167108913, 0.0026487634172264554, -0.0011732670757704463, \
    0.00048995199780883401, -0.00019336308015277829, 7.2287744678832942e-05, -2.565551249788587e-05, \
    8.6620736840759859e-06, -2.7876379719252641e-06, 8.5668736268524721e-07, -2.5184337837693224e-07, \
    7.0936022149218665e-08, -1.917322572749502e-08, 4.9801256466357896e-09, -1.2447733996061773e-09, \
    2.9977766411656295e-10, -6.9644956269250685e-11, 1.5626242538020159e-11, -3.3896879080452118e-12, \
    7.1161574262122503e-13, -1.4472012169242576e-13, 2.8536768232975401e-14, -5.4606927155058021e-15, \
    1.0148769468261627e-15, -1.8333259200975614e-16}
#define PYRH_ARMSTRONG_GH_T { \
    0.24534070830090124, 0.73747372854539439, 1.2340762153953231, 1.7385377121165861, \
    2.2549740020892757, 2.7888060584281305, 3.3478545673832163, 3.9447640401156252, \
    4.6036824495507442, 5.3874808900112328}
#define PYRH_ARMSTRONG_GH_W { \
    0.46224366960061009, 0.28667550536283415, 0.10901720602002329, 0.024810520887463643, \
    0.0032437733422378567, 0.00022833863601635365, 7.8025564785320599e-06, \
    1.0860693707692782e-07, 4.3993409922731747e-10, 2.2293936455341447e-13}
// -2 / n of the series in a (n = 2..50), formed by the compiler: the same
// correctly rounded quotients a division in the loop gives.
#define PYRH_ARM_N2(n) (-2.0 / (n))
#define PYRH_ARMSTRONG_NEG2N { 0.0, 0.0, \
    PYRH_ARM_N2(2), PYRH_ARM_N2(3), PYRH_ARM_N2(4), PYRH_ARM_N2(5), PYRH_ARM_N2(6), \
    PYRH_ARM_N2(7), PYRH_ARM_N2(8), PYRH_ARM_N2(9), PYRH_ARM_N2(10), PYRH_ARM_N2(11), \
    PYRH_ARM_N2(12), PYRH_ARM_N2(13), PYRH_ARM_N2(14), PYRH_ARM_N2(15), PYRH_ARM_N2(16), \
    PYRH_ARM_N2(17), PYRH_ARM_N2(18), PYRH_ARM_N2(19), PYRH_ARM_N2(20), PYRH_ARM_N2(21), \
    PYRH_ARM_N2(22), PYRH_ARM_N2(23), PYRH_ARM_N2(24), PYRH_ARM_N2(25), PYRH_ARM_N2(26), \
    PYRH_ARM_N2(27), PYRH_ARM_N2(28), PYRH_ARM_N2(29), PYRH_ARM_N2(30), PYRH_ARM_N2(31), \
    PYRH_ARM_N2(32), PYRH_ARM_N2(33), PYRH_ARM_N2(34), PYRH_ARM_N2(35), PYRH_ARM_N2(36), \
    PYRH_ARM_N2(37), PYRH_ARM_N2(38), PYRH_ARM_N2(39), PYRH_ARM_N2(40), PYRH_ARM_N2(41), \
    PYRH_ARM_N2(42), PYRH_ARM_N2(43), PYRH_ARM_N2(44), PYRH_ARM_N2(45), PYRH_ARM_N2(46), \
    PYRH_ARM_N2(47), PYRH_ARM_N2(48), PYRH_ARM_N2(49), PYRH_ARM_N2(50)}
static __constant__ double kArmNeg2N[51] = PYRH_ARMSTRONG_NEG2N;
static const double kArmNeg2NHost[51] = PYRH_ARMSTRONG_NEG2N;
static __constant__ double kDawsonCheb[34] = PYRH_ARMSTRONG_DAWSON;
static __constant__ double kGhT[10] = PYRH_ARMSTRONG_GH_T;
static __constant__ double kGhW[10] = PYRH_ARMSTRONG_GH_W;
static const double kDawsonChebHost[34] = PYRH_ARMSTRONG_DAWSON;
static const double kGhTHost[10] = PYRH_ARMSTRONG_GH_T;
static const double kGhWHost[10] = PYRH_ARMSTRONG_GH_W;

// the tables from the side that runs the code
PYRH_HD double arm_dawson(int n) {
#ifdef __CUDA_ARCH__
  return kDawsonCheb[n];
#else
  return kDawsonChebHost[n];
#endif
}
PYRH_HD double arm_ght(int n) {
#ifdef __CUDA_ARCH__
  return kGhT[n];
#else
  return kGhTHost[n];
#endif
}
PYRH_HD double arm_neg2n(int n) {
#ifdef __CUDA_ARCH__
  return kArmNeg2N[n];
#else
  return kArmNeg2NHost[n];
#endif
}

// The series' stopping test |g / funct| <= 1e-8 (voigt.c).  In FP64 it is
// decided by a product where the quotient is clearly on one side and by
// the division itself only within 1e-12 of the limit, so every decision is
// the division's (FP64 divisions dominated the profile kernel's time); in
// other precisions and for dual numbers the division is kept as written.
template <typename R>
PYRH_HD bool arm_series_done(const R& g, const R& funct) {
  return fabs(g / funct) <= R(1.0e-8);
}
template <>
PYRH_HD bool arm_series_done<double>(const double& g, const double& funct) {
  const double ag = fabs(g), lim = 1.0e-8 * fabs(funct);
  if (ag < lim * (1.0 - 1.0e-12)) return true;
  if (ag > lim * (1.0 + 1.0e-12)) return false;
  return fabs(g / funct) <= 1.0e-8;
}

// -2 / n: from the table in FP64 (the same value), divided otherwise.
template <typename R>
PYRH_HD R arm_m2n(int n) { return R(-2) / R(n); }
template <>
PYRH_HD double arm_m2n<double>(int n) { return arm_neg2n(n); }

PYRH_HD double arm_ghw(int n) {
#ifdef __CUDA_ARCH__
  return kGhW[n];
#else
  return kGhWHost[n];
#endif
}




// A value with its derivatives along two directions (a and v here), for
// voigt_armstrong_t<Dual2<R>>.  In its own namespace so that argument-
// dependent lookup finds these functions for Dual2 arguments while plain
// names inside pyrh keep resolving to the standard math functions.
namespace ad {
template <typename R>
struct Dual2 {
  R x, d0, d1;
  PYRH_HD Dual2() : x(0), d0(0), d1(0) {}
  PYRH_HD Dual2(double c) : x(R(c)), d0(0), d1(0) {}
  PYRH_HD Dual2(float c) : x(R(c)), d0(0), d1(0) {}
  PYRH_HD Dual2(int c) : x(R(c)), d0(0), d1(0) {}
  PYRH_HD Dual2(R x_, R a, R b) : x(x_), d0(a), d1(b) {}
};
template <typename R>
PYRH_HD Dual2<R> operator+(const Dual2<R>& a, const Dual2<R>& b) {
  return {a.x + b.x, a.d0 + b.d0, a.d1 + b.d1};
}
template <typename R>
PYRH_HD Dual2<R> operator-(const Dual2<R>& a, const Dual2<R>& b) {
  return {a.x - b.x, a.d0 - b.d0, a.d1 - b.d1};
}
template <typename R>
PYRH_HD Dual2<R> operator-(const Dual2<R>& a) {
  return {-a.x, -a.d0, -a.d1};
}
template <typename R>
PYRH_HD Dual2<R> operator*(const Dual2<R>& a, const Dual2<R>& b) {
  return {a.x * b.x, a.d0 * b.x + a.x * b.d0, a.d1 * b.x + a.x * b.d1};
}
template <typename R>
PYRH_HD Dual2<R> operator/(const Dual2<R>& a, const Dual2<R>& b) {
  const R q = a.x / b.x;
  return {q, (a.d0 - q * b.d0) / b.x, (a.d1 - q * b.d1) / b.x};
}
template <typename R>
PYRH_HD Dual2<R>& operator+=(Dual2<R>& a, const Dual2<R>& b) {
  a = a + b;
  return a;
}
template <typename R>
PYRH_HD Dual2<R>& operator*=(Dual2<R>& a, const Dual2<R>& b) {
  a = a * b;
  return a;
}
template <typename R> PYRH_HD bool operator<(const Dual2<R>& a, const Dual2<R>& b) { return a.x < b.x; }
template <typename R> PYRH_HD bool operator>(const Dual2<R>& a, const Dual2<R>& b) { return a.x > b.x; }
template <typename R> PYRH_HD bool operator<=(const Dual2<R>& a, const Dual2<R>& b) { return a.x <= b.x; }
template <typename R>
PYRH_HD Dual2<R> exp(const Dual2<R>& a) {
  const R e = ::exp(a.x);
  return {e, e * a.d0, e * a.d1};
}
template <typename R>
PYRH_HD Dual2<R> cos(const Dual2<R>& a) {
  const R s = -::sin(a.x);
  return {::cos(a.x), s * a.d0, s * a.d1};
}
template <typename R>
PYRH_HD Dual2<R> atan(const Dual2<R>& a) {
  const R f = R(1) / (R(1) + a.x * a.x);
  return {::atan(a.x), f * a.d0, f * a.d1};
}
template <typename R>
PYRH_HD Dual2<R> log(const Dual2<R>& a) {
  const R f = R(1) / a.x;
  return {::log(a.x), f * a.d0, f * a.d1};
}
template <typename R>
PYRH_HD Dual2<R> fabs(const Dual2<R>& a) {
  return a.x < R(0) ? -a : a;
}
}  // namespace ad

// Out of line on the device: a long routine that only lines which are not
// polarizable reach; inlined at each call site it would bloat the hot
// kernels' code (and their compile time) for nothing.
#ifdef __CUDA_ARCH__
#define PYRH_VOIGT_FN __host__ __device__ __noinline__
#else
#define PYRH_VOIGT_FN inline
#endif

// SP: for profiles stored in single precision (R = double): the Gaussian
// factor exp(a^2 - v^2) cos(2 v a) in FP32 where a < 0.1 (the exponent's
// rounding to float put back to first order) and the Dawson Chebyshev sum
// cut after the 24 terms whose coefficients exceed 1e-10.  Over a in
// [1e-4, 1], v in [0, 200] H moves by at most 2e-7 of itself (3 roundings
// of a float); the FP64 divisions and transcendentals this saves set the
// time of the profile set-up.
template <typename R, bool SP = false>
PYRH_VOIGT_FN R voigt_armstrong_t(R a, R v) {
  if (v < R(0)) v = -v;
  if ((a < R(1) && v < R(4)) || (a < R(1.8) / (v + R(1)))) {
    const R a2 = a * a, v2 = v * v;
    R u1 = R(0);
    if (!((v2 - a2) > R(70))) {
      bool sp = false;
      if constexpr (SP) {
        if (a < R(0.1)) {
          const R x = a2 - v2;
          const float xf = float(x);
          u1 = R(expf(xf)) * (R(1) + (x - R(xf))) * R(cosf(float(R(2) * v * a)));
          sp = true;
        }
      }
      if (!sp) u1 = R(exp(a2 - v2) * cos(R(2) * v * a));
    }
    R dn01, dn02;
    if (v > R(5)) {
      const R r = R(1) / v2;
      dn01 = -r * (R(0.5) + r * (R(0.75) + r * (R(1.875) + r * (R(6.5625) + r * (R(29.53125) +
             r * (R(1162.4218) + r * R(1055.7421)))))));
      dn02 = (R(1) - dn01) / (R(2) * v);
    } else {
      R b1 = R(0), b2 = R(0), b = R(0);
      const R x = v / R(5), coef = R(4) * x * x - R(2);
      for (int n = SP ? 23 : 33; n >= 0; --n) {
        b = coef * b1 - b2 + R(arm_dawson(n));
        b2 = b1;
        b1 = b;
      }
      dn02 = x * (b - b2);
      dn01 = R(1) - R(2) * v * dn02;
    }
    R funct = a * dn01;
    if (a > R(1.0e-8)) {
      R q = R(1), an = a;
      for (int n = 2; n <= 50; ++n) {
        const R dn = (v * dn01 + dn02) * arm_m2n<R>(n);
        dn02 = dn01;
        dn01 = dn;
        if (n % 2) {
          q = -q;
          an *= a2;
          const R g = dn * an;
          funct += q * g;
          if (arm_series_done<R>(g, funct)) return u1 - R(1.12837917) * funct;
        }
      }
    }
    return u1 - R(1.12837917) * funct;
  }
  if (a < R(2.5) && v < R(4)) {
    R g = R(0);
    const R a2 = a * a;
    for (int n = 0; n < 10; ++n) {
      const R t = R(arm_ght(n)), r = t - v, s = t + v;
      g += (R(4) * t * t - R(2)) *
           (r * atan(r / a) + s * atan(s / a) - R(0.5) * a * (log(a2 + r * r) + log(a2 + s * s))) *
           R(arm_ghw(n));
    }
    return g / R(kPI);
  }
  R g = R(0);
  const R a2 = a * a;
  for (int n = 0; n < 10; ++n) {
    const R t = R(arm_ght(n));
    g += (R(1) / ((v - t) * (v - t) + a2) + R(1) / ((v + t) * (v + t) + a2)) * R(arm_ghw(n));
  }
  return (a * g) / R(kPI);
}


__device__ __forceinline__ double voigt_armstrong(double a, double v) {
  return voigt_armstrong_t<double>(a, v);
}

// H(a, v) with dH/da and dH/dv
template <typename R>
PYRH_VOIGT_FN R voigt_armstrong_d(R a, R v, R& dHda, R& dHdv) {
  const ad::Dual2<R> r = voigt_armstrong_t<ad::Dual2<R>>(ad::Dual2<R>(a, R(1), R(0)),
                                                          ad::Dual2<R>(v, R(0), R(1)));
  dHda = r.d0;
  dHdv = r.d1;
  return r.x;
}

}  // namespace pyrh
