// lte_rf.cuh -- response functions of the polarized LTE synthesis.
//
// Depth-resolved response functions dS_s(lambda)/dx(k) of the emergent
// Stokes vector to x = (T, v_los, v_mic, B, gamma, chi) at every depth, and
// the gradient of a weighted chi^2, for the same path as lte_stokes.cu
// (DELO-Bezier3 without magneto-optical terms, ray to the observer).
//
// Method, per (atmosphere, wavelength):
//  1. forward sweep of the DELO-Bezier3 recurrence (bezier_1D.c:52-300),
//     recording the per-depth optical quantities q_k = (chi, S_I..S_V,
//     K'_Q, K'_U, K'_V) and the per-step state on a thread-private tape;
//  2. hand-written reverse (adjoint) sweep of that recurrence, giving
//     dS_s(0)/dq_k for every depth (seeds: the four Stokes outputs, or the
//     chi^2 weights);
//  3. q_k depends only on the parameters of depth k, so the local Jacobian
//     dq_k/dx_k (forward-mode dual numbers through the Zeeman/Voigt opacity
//     of kurucz.c:729-827 and the line strength of kurucz.c:638-680, with
//     the exact derivative of each Humlicek region) closes the chain.
// The reference has no analytical response functions for these parameters;
// its definition is finite differences of the whole synthesis
// (rf_ray.c:205-293), which re-runs the set-up for every perturbation.  The
// set-up's outputs are inputs here (continuum chi_c and eta_c, stage
// densities, proton density, path lengths); where the caller passes their
// temperature derivatives (pyrh_lte_setup_dT) the temperature response
// carries them too: the continuum terms through dL/dchi_c and dL/deta_c
// (local_q_vjp), the populations through the line quantities (line_depth),
// and the path lengths through their own adjoints in the reverse sweep.
// Without them the set-up is held fixed.
#pragma once

#include "../../include/pyrh_gb300.h"
#include "rt_device.cuh"
#include "voigt_armstrong.cuh"

#ifndef PYRH_MAX_DEPTH_RF
#define PYRH_MAX_DEPTH_RF PYRH_RF_MAX_DEPTH
#endif

namespace pyrh {

constexpr int kNX = 6;  // T, v_los, v_mic, B, gamma, chi
// Zeeman component count that marks a line which is not polarizable: its
// profile is Armstrong's Voigt function H(a, v), Stokes I only (kurucz.c:824)
constexpr int kArmstrong = -1;

// ------------------------------------------------------------- duals -----
template <typename R>
struct D6 {
  R v;
  R d[kNX];
};

template <typename R>
PYRH_HD D6<R> dconst(R v) {
  D6<R> r;
  r.v = v;
  for (int i = 0; i < kNX; ++i) r.d[i] = R(0);
  return r;
}
template <typename R>
PYRH_HD D6<R> dvar(R v, int i) {
  D6<R> r = dconst(v);
  r.d[i] = R(1);
  return r;
}
template <typename R>
PYRH_HD D6<R> operator+(const D6<R>& a, const D6<R>& b) {
  D6<R> r;
  r.v = a.v + b.v;
  for (int i = 0; i < kNX; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <typename R>
PYRH_HD D6<R> operator-(const D6<R>& a, const D6<R>& b) {
  D6<R> r;
  r.v = a.v - b.v;
  for (int i = 0; i < kNX; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <typename R>
PYRH_HD D6<R> operator*(const D6<R>& a, const D6<R>& b) {
  D6<R> r;
  r.v = a.v * b.v;
  for (int i = 0; i < kNX; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <typename R>
PYRH_HD D6<R> operator*(R s, const D6<R>& a) {
  D6<R> r;
  r.v = s * a.v;
  for (int i = 0; i < kNX; ++i) r.d[i] = s * a.d[i];
  return r;
}
template <typename R>
PYRH_HD D6<R> operator/(const D6<R>& a, const D6<R>& b) {
  D6<R> r;
  const R ib = R(1) / b.v;
  r.v = a.v * ib;
  for (int i = 0; i < kNX; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <typename R>
PYRH_HD D6<R> dsqrt(const D6<R>& a) {
  D6<R> r;
  r.v = sqrt(a.v);
  const R h = R(0.5) / r.v;
  for (int i = 0; i < kNX; ++i) r.d[i] = h * a.d[i];
  return r;
}
template <typename R>
PYRH_HD D6<R> dexp(const D6<R>& a) {
  D6<R> r;
  r.v = exp(a.v);
  for (int i = 0; i < kNX; ++i) r.d[i] = r.v * a.d[i];
  return r;
}
template <typename R>
PYRH_HD D6<R> dpow(const D6<R>& a, R p) {
  D6<R> r;
  r.v = pow(a.v, p);
  const R f = p * r.v / a.v;
  for (int i = 0; i < kNX; ++i) r.d[i] = f * a.d[i];
  return r;
}
template <typename R>
PYRH_HD D6<R> dcos(const D6<R>& a) {
  D6<R> r;
  r.v = cos(a.v);
  const R f = -sin(a.v);
  for (int i = 0; i < kNX; ++i) r.d[i] = f * a.d[i];
  return r;
}
template <typename R>
PYRH_HD D6<R> dsin(const D6<R>& a) {
  D6<R> r;
  r.v = sin(a.v);
  const R f = cos(a.v);
  for (int i = 0; i < kNX; ++i) r.d[i] = f * a.d[i];
  return r;
}

// ---------------------------------------------- Humlicek with derivative --
// W(t) and dW/dt for t = a - i v, differentiating each region's rational
// approximation exactly (so the derivative is that of the forward model).
// Derivatives of the rational forms as (P' - W Q') / Q with W = P / Q
// already known: one complex division, and no Q^2, whose |Q^2|^2 would
// overflow single precision near |v| = 5.5 (|Q|^2 reaches 1e21 there).
template <typename R>
PYRH_HD void humlicek_d(R a, R v, Cx<R>& W, Cx<R>& dW) {
  const Cx<R> t = {a, -v};
  const R s = fabs(v) + a;
  if (s >= R(15.0)) {
    // W = c t / (t^2 + 1/2);  W' = c (1/2 - t^2) / (t^2 + 1/2)^2
    const R c0 = R(0.5641896);
    Cx<R> t2 = cmul(t, t);
    Cx<R> den = {t2.r + R(0.5), t2.i};
    W = cdiv(Cx<R>{c0 * t.r, c0 * t.i}, den);
    dW = cdiv(cdiv(Cx<R>{c0 * (R(0.5) - t2.r), -c0 * t2.i}, den), den);
  } else if (s >= R(5.5)) {
    // W = t (c1 u + c2) / (u (u + 3) + 3/4), u = t^2
    const R c1 = R(0.5641896), c2 = R(1.410474);
    Cx<R> u = cmul(t, t);
    Cx<R> g = {c1 * u.r + c2, c1 * u.i};
    Cx<R> N = cmul(t, g);
    Cx<R> dN = {g.r + R(2) * c1 * u.r, g.i + R(2) * c1 * u.i};  // g + t * c1 * 2t
    Cx<R> D = cmul(u, Cx<R>{u.r + R(3), u.i});
    D.r += R(0.75);
    Cx<R> dD = cmul(Cx<R>{R(2) * u.r + R(3), R(2) * u.i}, Cx<R>{R(2) * t.r, R(2) * t.i});
    W = cdiv(N, D);
    // (N/D)' = (N' - W D') / D
    const Cx<R> wd = cmul(W, dD);
    dW = cdiv(Cx<R>{dN.r - wd.r, dN.i - wd.i}, D);
  } else if (a >= R(0.195) * fabs(v) - R(0.176)) {
    const R A[5] = {R(0.5642236), R(3.778987), R(11.96482), R(20.20933), R(16.4955)};
    const R B[5] = {R(6.699398), R(21.69274), R(39.27121), R(38.82363), R(16.4955)};
    Cx<R> P = {A[0], R(0)}, dP = {R(0), R(0)};
    Cx<R> Q = {t.r + B[0], t.i}, dQ = {R(1), R(0)};
    for (int n = 1; n < 5; ++n) {
      dP = cmul(dP, t); dP.r += P.r; dP.i += P.i;
      P = cmul(P, t); P.r += A[n];
      dQ = cmul(dQ, t); dQ.r += Q.r; dQ.i += Q.i;
      Q = cmul(Q, t); Q.r += B[n];
    }
    W = cdiv(P, Q);
    const Cx<R> wq = cmul(W, dQ);
    dW = cdiv(Cx<R>{dP.r - wq.r, dP.i - wq.i}, Q);
  } else {
    // W = exp(t^2) - t P(u) / Q(u), u = -t^2
    const R A[7] = {R(0.56419), R(1.320522), R(35.7668), R(219.031), R(1540.787), R(3321.99), R(36183.31)};
    const R B[7] = {R(1.841439), R(61.57037), R(364.2191), R(2186.181), R(9022.228), R(24322.84), R(32066.6)};
    Cx<R> u = {-(t.r * t.r - t.i * t.i), -(R(2) * t.r * t.i)};
    Cx<R> P = {A[0], R(0)}, dP = {R(0), R(0)};           // derivatives w.r.t. u
    Cx<R> Q = {u.r + B[0], u.i}, dQ = {R(1), R(0)};
    for (int n = 1; n < 7; ++n) {
      dP = cmul(dP, u); dP.r += P.r; dP.i += P.i;
      P = cmul(u, P); P.r += A[n];
      dQ = cmul(dQ, u); dQ.r += Q.r; dQ.i += Q.i;
      Q = cmul(u, Q); Q.r += B[n];
    }
    R e = dev_exp(-u.r), sn, cs;
    dev_sincos(-u.i, &sn, &cs);
    Cx<R> E = {e * cs, e * sn};                             // exp(t^2)
    Cx<R> r = cdiv(P, Q);
    Cx<R> tr = cmul(t, r);
    W = {E.r - tr.r, E.i - tr.i};
    // d/dt [t P/Q] = P/Q + t (P' - r Q')/Q * du/dt,  du/dt = -2t
    const Cx<R> rq = cmul(r, dQ);
    Cx<R> dr = cdiv(Cx<R>{dP.r - rq.r, dP.i - rq.i}, Q);
    Cx<R> tdr = cmul(cmul(t, dr), Cx<R>{R(-2) * t.r, R(-2) * t.i});
    Cx<R> dE = cmul(E, Cx<R>{R(2) * t.r, R(2) * t.i});
    dW = {dE.r - r.r - tdr.r, dE.i - r.i - tdr.i};
  }
}

// ------------------------------------------- per-(line, depth) quantities --
// Value and derivatives w.r.t. (T, v_los, v_mic, B, gamma, chi) of the
// line quantities of one depth (kurucz.c:638-680, 745-783), stored compactly:
// every one of them depends on T and v_mic (through the Doppler width, the
// damping and the LTE strength); besides those, only the velocity shift
// depends on v_los and only the Zeeman splitting on B, and none on the
// field angles.  So a field keeps its value and two derivatives (DC), and
// the two single-parameter derivatives are stored once: 20 numbers instead
// of six full duals (42), which is what the shared-memory tables of the
// response-function kernel hold per (line, depth).
template <typename R>
struct DC {
  R v, dT, dvt;
};

template <typename R>
struct LineDepth {
  DC<R> inv_vb, vshift, adamp, vB, chil, etal;
  R dvsh_dvel;   // d vshift / d v_los
  R dvB_dB;      // d vB / d B
  bool gauss;    // Grad == 0
};

// The full dual of a stored field (slot `extra` gets `dx`).
template <typename R>
PYRH_HD D6<R> expand(const DC<R>& c, int extra = -1, R dx = R(0)) {
  D6<R> r = dconst(c.v);
  r.d[0] = c.dT;
  r.d[2] = c.dvt;
  if (extra >= 0) r.d[extra] = dx;
  return r;
}

template <typename R>
PYRH_HD DC<R> compact(const D6<R>& a) {
  return DC<R>{a.v, a.d[0], a.d[2]};
}

struct LineConstD {
  double lambda0, Ei, gi, Aji, Bji, Bij, Grad, GStark, GvdWaals, cross, alpha, isotope_frac,
      hyperfine_frac, weight;
  int vdwaals;
};

// dn_dT, dlnU_dT, dnp_dT: derivatives of the set-up's stage density, log
// partition function and proton density with respect to the temperature of
// the same depth (zero: held fixed).  The reference's finite-difference
// response functions re-run the LTE populations for every perturbed T
// (rf_ray.c:257-283 -> Background() -> LTEpops), so its temperature
// response carries these terms.
template <typename R>
PYRH_HD LineDepth<R> line_depth(const LineConstD& L, R T, R vel, R vturb, R B, R ne, R nHtot,
                                R np, R nstage, R lnU, R muz, bool moving, R dn_dT = R(0),
                                R dlnU_dT = R(0), R dnp_dT = R(0)) {
  const D6<R> dT = dvar(T, 0), dv = dvar(vel, 1), dvt = dvar(vturb, 2), dB = dvar(B, 3);
  D6<R> nst = dconst(nstage), lnUd = dconst(lnU), npd = dconst(np);
  nst.d[0] = dn_dT;
  lnUd.d[0] = dlnU_dT;
  npd.d[0] = dnp_dT;
  const R vtherm = R(2.0 * kKBOLTZMANN / (kAMU * L.weight));
  const D6<R> vb = dsqrt(vtherm * dT + dvt * dvt);
  const D6<R> one = dconst(R(1));
  const D6<R> inv_vb = R(kCLIGHT / L.lambda0) * (one / vb);
  const D6<R> vshift = moving ? muz * (dv / vb) : dconst(R(0));
  const D6<R> sv = R(1.0 / kSQRTPI) * (one / vb);
  const bool gauss = (L.Grad == 0.0);
  D6<R> adamp;
  if (!gauss) {
    D6<R> GvdW;
    if (L.vdwaals == 0) GvdW = R(L.cross) * dpow(dT, R(0.3));
    else if (L.vdwaals == 2) GvdW = R(L.cross) * dpow(dT, R((1.0 - L.alpha) / 2.0));
    else GvdW = dconst(R(L.GvdWaals));
    const D6<R> G = dconst(R(L.Grad + L.GStark * ne)) + (dconst(nHtot) - npd) * GvdW;
    adamp = R(L.lambda0 * kNM_TO_M / (4.0 * kPI)) * (G / vb);
  } else {
    adamp = dconst(R(-1));
  }
  const D6<R> vBd = R(kLARMOR * L.lambda0) * (dB / vb);
  const R hc = R(kHPLANCK * kCLIGHT);
  const R hc_la = R(kHPLANCK * kCLIGHT / (L.lambda0 * kNM_TO_M));
  const R B4 = R(kHPLANCK * kCLIGHT / (4.0 * kPI) * L.Bij * L.isotope_frac * L.hyperfine_frac * L.gi);
  const R tw = R(L.Aji / L.Bji);
  const D6<R> kT = one / (R(kKBOLTZMANN) * dT);
  const D6<R> ni = nst * dexp(dconst(R(0)) - lnUd - R(L.Ei) * kT);
  const D6<R> nj = ni * dexp(dconst(R(0)) - hc_la * kT);
  LineDepth<R> o;
  o.inv_vb = compact(inv_vb);
  o.vshift = compact(vshift);
  o.adamp = compact(adamp);
  o.vB = compact(vBd);
  o.chil = compact((B4 * (ni - nj)) * sv);
  o.etal = compact(((B4 * tw) * nj) * sv);
  o.dvsh_dvel = vshift.d[1];
  o.dvB_dB = vBd.d[3];
  o.gauss = gauss;
  (void)hc;
  return o;
}

// Projected field geometry (project.c:38-79) with derivatives w.r.t. gamma
// (slot 4) and chi (slot 5): sin^2(g) cos(2c), sin^2(g) sin(2c), cos(g), sin^2(g).
template <typename R>
struct GeoD {
  D6<R> gQ, gU, gV, s2g;
};

template <typename R>
PYRH_HD GeoD<R> geometry_d(R gam, R chb, R muz) {
  const D6<R> g = dvar(gam, 4), c = dvar(chb, 5);
  D6<R> cg, c2c, s2c;
  if (muz == R(1)) {
    cg = dcos(g);
    c2c = dcos(R(2) * c);
    s2c = dsin(R(2) * c);
  } else {
    const R mux = sqrt(R(1) - muz * muz), csc = R(1) / sqrt(R(1) - muz * muz);
    const D6<R> sg = dsin(g);
    const D6<R> bx = sg * dcos(c), by = sg * dsin(c), bz = dcos(g);
    const D6<R> b3 = mux * bx + muz * bz;
    const D6<R> b1 = csc * (bz - muz * b3);
    const D6<R> b2 = (-csc * mux) * by;
    const D6<R> den = dconst(R(1)) - b3 * b3;
    cg = b3;
    c2c = (b1 * b1 - b2 * b2) / den;
    s2c = (R(2) * (b1 * b2)) / den;
  }
  GeoD<R> o;
  o.s2g = dconst(R(1)) - cg * cg;
  o.gQ = o.s2g * c2c;
  o.gU = o.s2g * s2c;
  o.gV = cg;
  return o;
}

// Local optical quantities q = (chi, S0..S3, k1..k3) and their Jacobian
// dq/dx at one depth for one wavelength (kurucz.c:669-715, formal.c:178-208,
// stokesopac.c:47-79), MAGNETO_OPTICAL off.  comp_* are the Zeeman tables
// of each line (q index 0..2 for Ml - Mu = -1, 0, +1).
// Line l's quantities at this depth are ld[l * ld_stride].
template <typename R>
PYRH_HD void local_q_jac(int nline, const LineDepth<R>* ld, int ld_stride, const GeoD<R>& geo,
                         const R* dlam, unsigned inwin, const int* ncomp, const R* cshift,
                         const R* cweight, const int* cq, int maxcomp, R chi_c, R eta_c, R q[8],
                         R J[8][kNX]) {
  D6<R> cI = dconst(R(0)), cQ = cI, cU = cI, cV = cI, eI = cI, eQ = cI, eU = cI, eV = cI;
  for (int l = 0; l < nline; ++l) {
    if (!((inwin >> l) & 1u)) continue;
    const LineDepth<R>& Ls = ld[l * ld_stride];
    struct {
      D6<R> inv_vb, vshift, adamp, vB, chil, etal;
    } L = {expand(Ls.inv_vb), expand(Ls.vshift, 1, Ls.dvsh_dvel), expand(Ls.adamp),
           expand(Ls.vB, 3, Ls.dvB_dB), expand(Ls.chil), expand(Ls.etal)};
    const D6<R> v = dlam[l] * L.inv_vb + L.vshift;
    if (Ls.gauss) {
      const D6<R> phi = (fabs(v.v) <= R(kMAX_GAUSS_DOPPLER)) ? dexp(dconst(R(0)) - v * v) : dconst(R(0));
      cI = cI + L.chil * phi;
      eI = eI + L.etal * phi;
      continue;
    }
    if (ncomp[l] == kArmstrong) {
      R dHda, dHdv;
      D6<R> H;
      H.v = voigt_armstrong_d<R>(L.adamp.v, v.v, dHda, dHdv);
      for (int i = 0; i < kNX; ++i) H.d[i] = dHda * L.adamp.d[i] + dHdv * v.d[i];
      cI = cI + L.chil * H;
      eI = eI + L.etal * H;
      continue;
    }
    D6<R> ph[3] = {dconst(R(0)), dconst(R(0)), dconst(R(0))};
    for (int c = 0; c < ncomp[l]; ++c) {
      const R sh = cshift[l * maxcomp + c], w = cweight[l * maxcomp + c];
      Cx<R> W, dW;
      const R vv = v.v - sh * L.vB.v;
      humlicek_d<R>(L.adamp.v, vv, W, dW);
      // t = a - i (v - sh vB): dt = da - i (dv - sh dvB); dH = Re(W' dt)
      D6<R> H;
      H.v = W.r;
      for (int i = 0; i < kNX; ++i) {
        const R dre = L.adamp.d[i], dim = -(v.d[i] - sh * L.vB.d[i]);
        H.d[i] = dW.r * dre - dW.i * dim;
      }
      const int qi = cq[l * maxcomp + c] + 1;
      ph[qi < 0 ? 0 : (qi > 2 ? 2 : qi)] = ph[qi < 0 ? 0 : (qi > 2 ? 2 : qi)] + w * H;
    }
    const D6<R> sig = ph[2] + ph[0];
    const D6<R> del = R(0.5) * ph[1] - R(0.25) * sig;
    const D6<R> phiI = del * geo.s2g + R(0.5) * sig;
    const D6<R> phiQ = del * geo.gQ, phiU = del * geo.gU, phiV = R(0.5) * ((ph[2] - ph[0]) * geo.gV);
    cI = cI + L.chil * phiI; eI = eI + L.etal * phiI;
    cQ = cQ + L.chil * phiQ; eQ = eQ + L.etal * phiQ;
    cU = cU + L.chil * phiU; eU = eU + L.etal * phiU;
    cV = cV + L.chil * phiV; eV = eV + L.etal * phiV;
  }
  const D6<R> chi = dconst(chi_c) + cI;
  const D6<R> out[8] = {chi,
                        (dconst(eta_c) + eI) / chi, eQ / chi, eU / chi, eV / chi,
                        cQ / chi, cU / chi, cV / chi};
  for (int n = 0; n < 8; ++n) {
    q[n] = out[n].v;
    for (int i = 0; i < kNX; ++i) J[n][i] = out[n].d[i];
  }
}

// Lines whose Zeeman profile sums are kept per depth (on the tape) for the
// reverse sweep: the first kZLines lines inside their windows at a
// wavelength, in list order.  Per line kZ values: the three profile sums
// ph_q = sum_{c in q} w_c H(x_c) (q = sigma-, pi, sigma+) and their
// derivatives with respect to the damping a, the reduced frequency x and the
// Zeeman splitting v_B:  sum w Re W',  sum w Im W',  -sum w sh Im W'
// (W' = dW/dt, t = a - i x; dH/da = Re W', dH/dx = Im W').  Gaussian lines
// keep phi and dphi/dx in the first two slots, lines that are not
// polarizable H, dH/da and dH/dv of Armstrong's function in the first three.
constexpr int kZLines = 2;
constexpr int kZ = 12;

// q of one depth (the forward sweep): the same sums as local_q_jac on the
// value parts, with the single-precision fast Humlicek where R is float.
// With SUMS, the Humlicek derivative is evaluated as well and the profile
// sums of the first kZLines in-window lines are stored in z.
// UP = false leaves out the branch for lines that are not polarizable (for
// blocks without them; see lte_rf_kernel.cuh).
// Out of line on the device: the forward sweep calls it from four sites
// (three boundary depths and the loop), and one copy of its body instead of
// four keeps the adjoint kernel's instructions in cache.  Measured on the
// chi^2 gradient of 4096 atmospheres x 224 wavelengths: 29.4 -> 26.5 ms
// (full response functions 59.1 -> 55.8 ms); taking the reverse-sweep
// contraction (local_q_vjp) out of line as well measured slower.
#ifdef __CUDA_ARCH__
#define PYRH_OUTLINE __host__ __device__ __noinline__
#else
#define PYRH_OUTLINE inline
#endif
template <typename R, bool SUMS = false, bool UP = true>
PYRH_OUTLINE void local_q(int nline, const LineDepth<R>* ld, int ld_stride, const GeoD<R>& geo,
                     const R* dlam, unsigned inwin, const int* ncomp, const R* cshift,
                     const R* cweight, const int* cq, int maxcomp, R chi_c, R eta_c, R q[8],
                     R (*z)[kZ] = nullptr) {
  R cI = 0, cQ = 0, cU = 0, cV = 0, eI = 0, eQ = 0, eU = 0, eV = 0;
  int slot = 0;
  for (int l = 0; l < nline; ++l) {
    if (!((inwin >> l) & 1u)) continue;
    const LineDepth<R>& L = ld[l * ld_stride];
    const R v = dlam[l] * L.inv_vb.v + L.vshift.v;
    const bool keep = SUMS && slot < kZLines;
    if (L.gauss) {
      const R phi = (fabs(v) <= R(kMAX_GAUSS_DOPPLER)) ? dev_exp(-v * v) : R(0);
      cI += L.chil.v * phi;
      eI += L.etal.v * phi;
      if (keep) {
        z[slot][0] = phi;
        z[slot][1] = R(-2) * v * phi;
      }
      slot += SUMS ? 1 : 0;
      continue;
    }
    if (UP && ncomp[l] == kArmstrong) {
      R H;
      if (SUMS) {
        R dHda, dHdv;
        H = voigt_armstrong_d<R>(L.adamp.v, v, dHda, dHdv);
        if (keep) {
          z[slot][0] = H;
          z[slot][1] = dHda;
          z[slot][2] = dHdv;
        }
      } else {
        H = voigt_armstrong_t<R>(L.adamp.v, v);
      }
      cI += L.chil.v * H;
      eI += L.etal.v * H;
      slot += SUMS ? 1 : 0;
      continue;
    }
    R ph[3] = {0, 0, 0}, pa[3] = {0, 0, 0}, px[3] = {0, 0, 0}, pv[3] = {0, 0, 0};
    for (int c = 0; c < ncomp[l]; ++c) {
      const R sh = cshift[l * maxcomp + c], w = cweight[l * maxcomp + c];
      const int qi0 = cq[l * maxcomp + c] + 1;
      const int qi = qi0 < 0 ? 0 : (qi0 > 2 ? 2 : qi0);
      if (SUMS) {
        Cx<R> W, dW;
        humlicek_d<R>(L.adamp.v, v - sh * L.vB.v, W, dW);
        ph[qi] += w * W.r;
        pa[qi] += w * dW.r;
        px[qi] += w * dW.i;
        pv[qi] -= w * sh * dW.i;
      } else {
        R H, F;
        humlicek<R>(L.adamp.v, v - sh * L.vB.v, H, F);
        ph[qi] += w * H;
      }
    }
    if (keep)
      for (int g = 0; g < 3; ++g) {
        z[slot][g] = ph[g];
        z[slot][3 + g] = pa[g];
        z[slot][6 + g] = px[g];
        z[slot][9 + g] = pv[g];
      }
    slot += SUMS ? 1 : 0;
    const R sig = ph[2] + ph[0];
    const R del = R(0.5) * ph[1] - R(0.25) * sig;
    const R phiI = del * geo.s2g.v + R(0.5) * sig;
    const R phiQ = del * geo.gQ.v, phiU = del * geo.gU.v, phiV = R(0.5) * ((ph[2] - ph[0]) * geo.gV.v);
    cI += L.chil.v * phiI; eI += L.etal.v * phiI;
    cQ += L.chil.v * phiQ; eQ += L.etal.v * phiQ;
    cU += L.chil.v * phiU; eU += L.etal.v * phiU;
    cV += L.chil.v * phiV; eV += L.etal.v * phiV;
  }
  const R chi = chi_c + cI;
  const R rchi = fdiv(R(1), chi);
  q[0] = chi;
  q[1] = (eta_c + eI) * rchi;
  q[2] = eQ * rchi;
  q[3] = eU * rchi;
  q[4] = eV * rchi;
  q[5] = cQ * rchi;
  q[6] = cU * rchi;
  q[7] = cV * rchi;
}

// Reverse-mode contraction of the local opacity: for NS adjoint vectors
// qb[s][8] = dL_s/dq (q as in local_q_jac), accumulates
// out[s][x] += sum_n qb[s][n] dq_n/dx for the six parameters of this depth.
// Instead of carrying six derivative directions through every profile sum
// (local_q_jac), the adjoints run backwards from q through the line sums and
// the Zeeman components to the per-line primitives (a, v, v_B, chi_l, eta_l)
// and the field geometry, and only those are multiplied by their
// derivatives with respect to the parameters (the .d parts of LineDepth and
// GeoD).  q holds the forward values of this depth (the tape).
// With gf != nullptr, also accumulates gf[s * PYRH_MAX_LINES + l] += dL_s /
// d log10(gf_l) of this depth: the line's opacity and emissivity are both
// proportional to its gf (kurucz.c:638-680), so the derivative is
// ln 10 (chi_l-bar chi_l + eta_l-bar eta_l).
// With z (the profile sums local_q<R, true> stored for this depth), the
// first kZLines in-window lines take their profile sums and derivatives from
// z instead of re-evaluating the Zeeman components.
// dchic_dT, detac_dT: temperature derivatives of the continuum opacity and
// emissivity of this (depth, wavelength) from the set-up (zero: held fixed).
template <typename R, int NS, bool UP = true>
PYRH_HD void local_q_vjp(int nline, const LineDepth<R>* ld, int ld_stride, const GeoD<R>& geo,
                         const R* dlam, unsigned inwin, const int* ncomp, const R* cshift,
                         const R* cweight, const int* cq, int maxcomp, const R q[8],
                         const R* qb, R out[NS][kNX], R* gf = nullptr,
                         const R (*z)[kZ] = nullptr, R dchic_dT = R(0), R detac_dT = R(0)) {
  int slot = 0;
  const R ichi = fdiv(R(1), q[0]);
  R eb[NS][4], cb[NS][4];
  R gb[NS][4];   // adjoints of s2g, gQ, gU, gV
  for (int s = 0; s < NS; ++s) {
    const R* a = qb + s * 8;
    R chib = a[0];
    for (int n = 1; n < 8; ++n) chib -= a[n] * q[n] * ichi;
    cb[s][0] = chib;
    for (int j = 0; j < 3; ++j) cb[s][j + 1] = a[5 + j] * ichi;
    for (int j = 0; j < 4; ++j) eb[s][j] = a[1 + j] * ichi;
    for (int j = 0; j < 4; ++j) gb[s][j] = R(0);
  }
  for (int l = 0; l < nline; ++l) {
    if (!((inwin >> l) & 1u)) continue;
    const LineDepth<R>& L = ld[l * ld_stride];
    const R v = dlam[l] * L.inv_vb.v + L.vshift.v;
    const R* zl = (z && slot < kZLines) ? z[slot] : nullptr;
    ++slot;
    R ab[NS], vb[NS], vBb[NS], chilb[NS], etalb[NS];
    if (L.gauss) {
      const R phi = zl ? zl[0] : ((fabs(v) <= R(kMAX_GAUSS_DOPPLER)) ? dev_exp(-v * v) : R(0));
      const R dphi = zl ? zl[1] : R(-2) * v * phi;
      for (int s = 0; s < NS; ++s) {
        const R phib = cb[s][0] * L.chil.v + eb[s][0] * L.etal.v;
        chilb[s] = cb[s][0] * phi;
        etalb[s] = eb[s][0] * phi;
        vb[s] = phib * dphi;
        ab[s] = vBb[s] = R(0);
      }
    } else if (UP && ncomp[l] == kArmstrong) {
      R H, dHda, dHdv;
      if (zl) {
        H = zl[0];
        dHda = zl[1];
        dHdv = zl[2];
      } else {
        H = voigt_armstrong_d<R>(L.adamp.v, v, dHda, dHdv);
      }
      for (int s = 0; s < NS; ++s) {
        const R phib = cb[s][0] * L.chil.v + eb[s][0] * L.etal.v;
        chilb[s] = cb[s][0] * H;
        etalb[s] = eb[s][0] * H;
        ab[s] = phib * dHda;
        vb[s] = phib * dHdv;
        vBb[s] = R(0);
      }
    } else {
      R phb[NS][3];
      for (int s = 0; s < NS; ++s) {
        R fI = cb[s][0] * L.chil.v + eb[s][0] * L.etal.v;
        R fQ = cb[s][1] * L.chil.v + eb[s][1] * L.etal.v;
        R fU = cb[s][2] * L.chil.v + eb[s][2] * L.etal.v;
        R fV = cb[s][3] * L.chil.v + eb[s][3] * L.etal.v;
        const R delb = fI * geo.s2g.v + fQ * geo.gQ.v + fU * geo.gU.v;
        const R sigb = R(0.5) * fI - R(0.25) * delb;
        phb[s][1] = R(0.5) * delb;
        phb[s][2] = sigb + R(0.5) * fV * geo.gV.v;
        phb[s][0] = sigb - R(0.5) * fV * geo.gV.v;
        ab[s] = vb[s] = vBb[s] = R(0);
      }
      R ph[3] = {0, 0, 0};
      if (zl) {
        for (int g = 0; g < 3; ++g) {
          ph[g] = zl[g];
          for (int s = 0; s < NS; ++s) {
            ab[s] += phb[s][g] * zl[3 + g];
            vb[s] += phb[s][g] * zl[6 + g];
            vBb[s] += phb[s][g] * zl[9 + g];
          }
        }
      } else {
        for (int c = 0; c < ncomp[l]; ++c) {
          const R sh = cshift[l * maxcomp + c], w = cweight[l * maxcomp + c];
          Cx<R> W, dW;
          humlicek_d<R>(L.adamp.v, v - sh * L.vB.v, W, dW);
          const int qi0 = cq[l * maxcomp + c] + 1;
          const int qi = qi0 < 0 ? 0 : (qi0 > 2 ? 2 : qi0);
          ph[qi] += w * W.r;
          for (int s = 0; s < NS; ++s) {
            const R hb = w * phb[s][qi];
            const R xb = hb * dW.i;   // dH/dx = Im W' (t = a - i x)
            ab[s] += hb * dW.r;       // dH/da = Re W'
            vb[s] += xb;
            vBb[s] -= sh * xb;
          }
        }
      }
      const R sig = ph[2] + ph[0];
      const R del = R(0.5) * ph[1] - R(0.25) * sig;
      const R phiI = del * geo.s2g.v + R(0.5) * sig;
      const R phiQ = del * geo.gQ.v, phiU = del * geo.gU.v;
      const R dV = R(0.5) * (ph[2] - ph[0]);
      const R phiV = dV * geo.gV.v;
      for (int s = 0; s < NS; ++s) {
        chilb[s] = cb[s][0] * phiI + cb[s][1] * phiQ + cb[s][2] * phiU + cb[s][3] * phiV;
        etalb[s] = eb[s][0] * phiI + eb[s][1] * phiQ + eb[s][2] * phiU + eb[s][3] * phiV;
        const R fI = cb[s][0] * L.chil.v + eb[s][0] * L.etal.v;
        const R fQ = cb[s][1] * L.chil.v + eb[s][1] * L.etal.v;
        const R fU = cb[s][2] * L.chil.v + eb[s][2] * L.etal.v;
        const R fV = cb[s][3] * L.chil.v + eb[s][3] * L.etal.v;
        gb[s][0] += fI * del;
        gb[s][1] += fQ * del;
        gb[s][2] += fU * del;
        gb[s][3] += fV * dV;
      }
    }
    // the line quantities depend on T and v_mic (slots 0 and 2), the shift
    // also on v_los (1) and the splitting also on B (3)
    for (int s = 0; s < NS; ++s) {
      out[s][0] += ab[s] * L.adamp.dT + vb[s] * (dlam[l] * L.inv_vb.dT + L.vshift.dT) +
                   vBb[s] * L.vB.dT + chilb[s] * L.chil.dT + etalb[s] * L.etal.dT;
      out[s][2] += ab[s] * L.adamp.dvt + vb[s] * (dlam[l] * L.inv_vb.dvt + L.vshift.dvt) +
                   vBb[s] * L.vB.dvt + chilb[s] * L.chil.dvt + etalb[s] * L.etal.dvt;
      out[s][1] += vb[s] * L.dvsh_dvel;
      out[s][3] += vBb[s] * L.dvB_dB;
    }
    if (gf)
      for (int s = 0; s < NS; ++s)
        gf[s * PYRH_MAX_LINES + l] +=
            R(2.302585092994045684) * (chilb[s] * L.chil.v + etalb[s] * L.etal.v);
  }
  for (int s = 0; s < NS; ++s)
    for (int x = 0; x < kNX; ++x)
      out[s][x] += gb[s][0] * geo.s2g.d[x] + gb[s][1] * geo.gQ.d[x] + gb[s][2] * geo.gU.d[x] +
                   gb[s][3] * geo.gV.d[x];
  // continuum: chi = chi_c + lines and S = (eta_c + lines) / chi, so
  // dL/dchi_c = cb[s][0] and dL/deta_c = eb[s][0]
  for (int s = 0; s < NS; ++s) out[s][0] += cb[s][0] * dchic_dT + eb[s][0] * detac_dT;
}

// ------------------------------------------------- coefficient derivatives --
template <typename R>
PYRH_HD void bezier3_coeffs_d(R dt, R c[5], R dc[5]) {
  // c = (alpha, beta, gamma, theta, eps), dc = d/d(dt)
  bezier3_coeffs(dt, c[0], c[1], c[2], c[3], c[4]);
  const R thr = sizeof(R) == 8 ? R(5.e-2) : R(1.5);
  if (dt >= thr) {
    const R e = c[4], t = dt, rt = fdiv(R(1), t), rt3 = rt * rt * rt;
    dc[0] = (R(6) - R(6) * t + R(3) * t * t - R(6) * e) * rt3 - R(3) * c[0] * rt;
    dc[1] = e - R(3) * c[1] * rt;
    dc[2] = R(3) * (R(-4) + R(2) * t + (R(4) + R(2) * t) * e) * rt3 - R(3) * c[2] * rt;
    dc[3] = R(3) * (e * (R(-2) - R(2) * t - t * t) + R(2)) * rt3 - R(3) * c[3] * rt;
    dc[4] = -e;
  } else if (sizeof(R) == 8) {
    const R t = dt, t2 = t * t, t3 = t2 * t;
    dc[4] = R(-1) + t - R(0.5) * t2 + t3 / R(6);
    dc[0] = R(0.25) - R(0.1) * t + t2 / R(40) - t3 / R(210);
    dc[1] = R(0.25) - R(0.4) * t + t2 / R(4) - R(2) * t3 / R(21);
    dc[2] = R(0.25) - R(0.2) * t + R(0.075) * t2 - R(4) * t3 / R(210);
    dc[3] = R(0.25) - R(0.3) * t + R(0.15) * t2 - t3 / R(21);
  } else {
    // derivative of the 11-term series of the single-precision form
    const R ca[11] = {R(0.25), R(-0.05), R(8.333333333e-3), R(-1.190476190e-3), R(1.488095238e-4),
                      R(-1.653439153e-5), R(1.653439153e-6), R(-1.503126503e-7),
                      R(1.252605419e-8), R(-9.635426302e-10), R(6.882447359e-11)};
    const R cb[11] = {R(0.25), R(-0.2), R(8.333333333e-2), R(-2.380952381e-2), R(5.208333333e-3),
                      R(-9.259259259e-4), R(1.388888889e-4), R(-1.803751804e-5),
                      R(2.066798942e-6), R(-2.119793786e-7), R(1.968379945e-8)};
    const R cg[11] = {R(0.25), R(-0.1), R(0.025), R(-4.761904762e-3), R(7.440476190e-4),
                      R(-9.920634921e-5), R(1.157407407e-5), R(-1.202501203e-6),
                      R(1.127344877e-7), R(-9.635426302e-9), R(7.570692095e-10)};
    const R ct[11] = {R(0.25), R(-0.15), R(0.05), R(-1.190476190e-2), R(2.232142857e-3),
                      R(-3.472222222e-4), R(4.629629630e-5), R(-5.411255411e-6),
                      R(5.636724387e-7), R(-5.299484466e-8), R(4.542415257e-9)};
    const R* cs[4] = {ca, cb, cg, ct};
    for (int m = 0; m < 4; ++m) {
      R s = R(11) * cs[m][10];
      for (int i = 9; i >= 0; --i) s = s * dt + R(i + 1) * cs[m][i];
      dc[m] = s;
    }
    dc[4] = -c[4];
  }
}

// --------------------------------------------------------- cent_deriv VJP --
// w = cent_deriv(dsup, dsdn, a, b, c); accumulates adjoints of all five args.
// The quantities that depend only on the two intervals are computed once per
// interval pair (CdW) and shared by the entries of one depth.
template <typename R>
struct CdW {
  R rsup, rsdn, al, dal_dsup, dal_dsdn;
};

template <typename R>
PYRH_HD CdW<R> cd_weights(R dsup, R dsdn) {
  CdW<R> w;
  w.rsup = fdiv(R(1), dsup);
  w.rsdn = fdiv(R(1), dsdn);
  const R rs = fdiv(R(1), dsdn + dsup);
  const R third = R(0.333333333333333333333333);
  w.al = third * (R(1) + dsdn * rs);
  w.dal_dsdn = third * dsup * rs * rs;
  w.dal_dsup = -third * dsdn * rs * rs;
  return w;
}

template <typename R>
PYRH_HD void cent_deriv_vjp(const CdW<R>& w, R a, R b, R c, R wbar, R& dsupb, R& dsdnb, R& ab,
                            R& bb, R& cb) {
  const R fim1 = (b - a) * w.rsup, fi = (c - b) * w.rsdn;
  if (!(fim1 * fi > R(0)) || wbar == R(0)) return;
  const R D = (R(1) - w.al) * fim1 + w.al * fi, N = fim1 * fi;
  const R rD = fdiv(R(1), D);
  const R Nb = wbar * rD, Db = -Nb * N * rD;
  const R f1b = Nb * fi + Db * (R(1) - w.al);
  const R f2b = Nb * fim1 + Db * w.al;
  const R alb = Db * (fi - fim1);
  dsdnb += alb * w.dal_dsdn;
  dsupb += alb * w.dal_dsup;
  ab -= f1b * w.rsup;
  bb += f1b * w.rsup - f2b * w.rsdn;
  cb += f2b * w.rsdn;
  dsupb -= f1b * fim1 * w.rsup;
  dsdnb -= f2b * fi * w.rsdn;
}

// ----------------------------------------------------------- DELO step ---
// Structured DELO-Bezier3 step without magneto-optical terms (see
// delo_step in lte_stokes.cu).  k vectors hold (K'_Q, K'_U, K'_V).
template <typename R>
struct StepIn {
  R al, be, ga, th, ep, dt03;
  R ku[3], k0[3], dku[3], dk0[3];
  R Su[4], S0[4], dSu[4], dS0[4];
  R Iu[4];
};

template <typename R>
PYRH_HD void md_solve(R c, const R b[3], const R k0[3], const R V[4], R x[4]) {
  const R sig = R(1) + c * (k0[0] * k0[0] + k0[1] * k0[1] + k0[2] * k0[2]);
  const R f = fdiv(c, sig);
  const R kb = k0[0] * b[0] + k0[1] * b[1] + k0[2] * b[2];
  const R kv = k0[0] * V[1] + k0[1] * V[2] + k0[2] * V[3];
  R w[3], z[3];
  for (int j = 0; j < 3; ++j) {
    w[j] = b[j] - f * kb * k0[j];
    z[j] = V[j + 1] - f * kv * k0[j];
  }
  const R x0 = fdiv(V[0] - (b[0] * z[0] + b[1] * z[1] + b[2] * z[2]),
                    sig - (b[0] * w[0] + b[1] * w[1] + b[2] * w[2]));
  x[0] = x0;
  for (int j = 0; j < 3; ++j) x[j + 1] = z[j] - x0 * w[j];
}

template <typename R>
PYRH_HD void step_fwd(const StepIn<R>& s, R x[4], R V[4], R b[3], R& c) {
  c = s.ga * s.dt03;
  const R pK = s.al + s.ga * (R(1) + s.dt03);
  const R ca = s.th * s.dt03, pa = -s.be - s.th + s.th * s.dt03;
  const R bt = s.be + s.th, ag = s.al + s.ga, tdt = s.th * s.dt03, gdt = s.ga * s.dt03;
  const R kuIv = s.ku[0] * s.Iu[1] + s.ku[1] * s.Iu[2] + s.ku[2] * s.Iu[3];
  const R ku2 = s.ku[0] * s.ku[0] + s.ku[1] * s.ku[1] + s.ku[2] * s.ku[2];
  R h[3];
  for (int j = 0; j < 3; ++j) h[j] = pa * s.ku[j] + ca * s.dku[j];
  V[0] = (s.ep + ca * ku2) * s.Iu[0] + h[0] * s.Iu[1] + h[1] * s.Iu[2] + h[2] * s.Iu[3] +
         bt * s.Su[0] - tdt * (s.ku[0] * s.Su[1] + s.ku[1] * s.Su[2] + s.ku[2] * s.Su[3]) +
         ag * s.S0[0] + gdt * (s.k0[0] * s.S0[1] + s.k0[1] * s.S0[2] + s.k0[2] * s.S0[3]) +
         s.dt03 * (s.ga * s.dS0[0] - s.th * s.dSu[0]);
  for (int j = 0; j < 3; ++j)
    V[j + 1] = h[j] * s.Iu[0] + s.ep * s.Iu[j + 1] + ca * s.ku[j] * kuIv - tdt * s.ku[j] * s.Su[0] +
               bt * s.Su[j + 1] + gdt * s.k0[j] * s.S0[0] + ag * s.S0[j + 1] +
               s.dt03 * (s.ga * s.dS0[j + 1] - s.th * s.dSu[j + 1]);
  for (int j = 0; j < 3; ++j) b[j] = pK * s.k0[j] + c * s.dk0[j];
  md_solve(c, b, s.k0, V, x);
}

// Reverse of step_fwd: given xb = dL/dx, accumulate into sb (same layout).
// x, b and c are the step's forward results (step_fwd).
template <typename R>
PYRH_HD void step_vjp(const StepIn<R>& s, const R x[4], const R b[3], R c, const R xb[4],
                      StepIn<R>& sb) {
  const R pK = s.al + s.ga * (R(1) + s.dt03);
  const R ca = s.th * s.dt03, pa = -s.be - s.th + s.th * s.dt03;
  const R bt = s.be + s.th, ag = s.al + s.ga, tdt = s.th * s.dt03, gdt = s.ga * s.dt03;
  // Md is symmetric: Vb = Md^-1 xb
  R Vb[4];
  md_solve(c, b, s.k0, xb, Vb);
  // Md entries: Md00 = 1 + c|k0|^2, Md0j = Mdj0 = b_j, Mdij = d_ij + c k0_i k0_j
  const R xk = x[1] * s.k0[0] + x[2] * s.k0[1] + x[3] * s.k0[2];
  const R vk = Vb[1] * s.k0[0] + Vb[2] * s.k0[1] + Vb[3] * s.k0[2];
  const R k02 = s.k0[0] * s.k0[0] + s.k0[1] * s.k0[1] + s.k0[2] * s.k0[2];
  const R sigb = -Vb[0] * x[0];
  R cb = -vk * xk + sigb * k02, bb[3], k0b[3];
  for (int j = 0; j < 3; ++j) {
    bb[j] = -(Vb[0] * x[j + 1] + Vb[j + 1] * x[0]);
    k0b[j] = -c * (Vb[j + 1] * xk + vk * x[j + 1]) + sigb * R(2) * c * s.k0[j];
  }
  R pKb = 0, cab = 0, pab = 0, btb = 0, agb = 0, tdtb = 0, gdtb = 0;
  for (int j = 0; j < 3; ++j) {
    pKb += bb[j] * s.k0[j];
    k0b[j] += pK * bb[j];
    cb += bb[j] * s.dk0[j];
    sb.dk0[j] += c * bb[j];
  }
  // V0
  const R ku2 = s.ku[0] * s.ku[0] + s.ku[1] * s.ku[1] + s.ku[2] * s.ku[2];
  const R kuIv = s.ku[0] * s.Iu[1] + s.ku[1] * s.Iu[2] + s.ku[2] * s.Iu[3];
  const R kuSv = s.ku[0] * s.Su[1] + s.ku[1] * s.Su[2] + s.ku[2] * s.Su[3];
  const R k0S0v = s.k0[0] * s.S0[1] + s.k0[1] * s.S0[2] + s.k0[2] * s.S0[3];
  R hb[3] = {0, 0, 0}, h[3];
  for (int j = 0; j < 3; ++j) h[j] = pa * s.ku[j] + ca * s.dku[j];
  {
    const R v = Vb[0];
    sb.ep += v * s.Iu[0];
    cab += v * ku2 * s.Iu[0];
    for (int j = 0; j < 3; ++j) sb.ku[j] += v * ca * s.Iu[0] * R(2) * s.ku[j];
    sb.Iu[0] += v * (s.ep + ca * ku2);
    for (int j = 0; j < 3; ++j) { hb[j] += v * s.Iu[j + 1]; sb.Iu[j + 1] += v * h[j]; }
    btb += v * s.Su[0]; sb.Su[0] += v * bt;
    tdtb -= v * kuSv;
    for (int j = 0; j < 3; ++j) { sb.ku[j] -= v * tdt * s.Su[j + 1]; sb.Su[j + 1] -= v * tdt * s.ku[j]; }
    agb += v * s.S0[0]; sb.S0[0] += v * ag;
    gdtb += v * k0S0v;
    for (int j = 0; j < 3; ++j) { k0b[j] += v * gdt * s.S0[j + 1]; sb.S0[j + 1] += v * gdt * s.k0[j]; }
    sb.dt03 += v * (s.ga * s.dS0[0] - s.th * s.dSu[0]);
    sb.ga += v * s.dt03 * s.dS0[0]; sb.dS0[0] += v * s.dt03 * s.ga;
    sb.th -= v * s.dt03 * s.dSu[0]; sb.dSu[0] -= v * s.dt03 * s.th;
  }
  for (int j = 0; j < 3; ++j) {
    const R v = Vb[j + 1];
    hb[j] += v * s.Iu[0]; sb.Iu[0] += v * h[j];
    sb.ep += v * s.Iu[j + 1]; sb.Iu[j + 1] += v * s.ep;
    cab += v * s.ku[j] * kuIv;
    sb.ku[j] += v * ca * kuIv;
    for (int m = 0; m < 3; ++m) {
      sb.ku[m] += v * ca * s.ku[j] * s.Iu[m + 1];
      sb.Iu[m + 1] += v * ca * s.ku[j] * s.ku[m];
    }
    tdtb -= v * s.ku[j] * s.Su[0]; sb.ku[j] -= v * tdt * s.Su[0]; sb.Su[0] -= v * tdt * s.ku[j];
    btb += v * s.Su[j + 1]; sb.Su[j + 1] += v * bt;
    gdtb += v * s.k0[j] * s.S0[0]; k0b[j] += v * gdt * s.S0[0]; sb.S0[0] += v * gdt * s.k0[j];
    agb += v * s.S0[j + 1]; sb.S0[j + 1] += v * ag;
    sb.dt03 += v * (s.ga * s.dS0[j + 1] - s.th * s.dSu[j + 1]);
    sb.ga += v * s.dt03 * s.dS0[j + 1]; sb.dS0[j + 1] += v * s.dt03 * s.ga;
    sb.th -= v * s.dt03 * s.dSu[j + 1]; sb.dSu[j + 1] -= v * s.dt03 * s.th;
  }
  for (int j = 0; j < 3; ++j) {
    pab += hb[j] * s.ku[j]; sb.ku[j] += hb[j] * pa;
    cab += hb[j] * s.dku[j]; sb.dku[j] += hb[j] * ca;
    sb.k0[j] += k0b[j];
  }
  // scalars back to the coefficients
  sb.ga += cb * s.dt03; sb.dt03 += cb * s.ga;
  sb.al += pKb; sb.ga += pKb * (R(1) + s.dt03); sb.dt03 += pKb * s.ga;
  sb.th += cab * s.dt03; sb.dt03 += cab * s.th;
  sb.be -= pab; sb.th += pab * (s.dt03 - R(1)); sb.dt03 += pab * s.th;
  sb.be += btb; sb.th += btb;
  sb.al += agb; sb.ga += agb;
  sb.th += tdtb * s.dt03; sb.dt03 += tdtb * s.th;
  sb.ga += gdtb * s.dt03; sb.dt03 += gdtb * s.ga;
}

// ------------------------------------------------------ forward with tape --
template <typename R>
struct Tape {
  R q[PYRH_MAX_DEPTH_RF][8];   // chi, S[4], k[3] per depth
  R I[PYRH_MAX_DEPTH_RF][4];   // I_k
  R T[PYRH_MAX_DEPTH_RF];      // dtau_uw of step k (T_k), and T[0] = dtau_dw of step 1
  R dchi[PYRH_MAX_DEPTH_RF];   // dchi_c used by step k (dchi_dn of step k+1)
  R dS0[PYRH_MAX_DEPTH_RF][4]; // dS0_k (dSu of step k-1); index nd-1 holds the initial dSu
  R dK0[PYRH_MAX_DEPTH_RF][3];
  R dchi_up0;                  // initial dchi_up
  R z[PYRH_MAX_DEPTH_RF][kZLines][kZ];   // profile sums of local_q<R, true>
};

// Forward DELO-Bezier3 sweep from the bottom boundary to the surface
// (bezier_1D.c:52-300), writing the tape.  qop(k, q) returns the optical
// quantities of depth k; they are computed once, two depths ahead of the
// step that first needs them, kept in a three-depth register window and
// written to the tape (never read back here).
template <typename R, typename QOp>
PYRH_HD void delo_forward(Tape<R>& tp, const R* ds, int nd, double B0, double B1, R out[4],
                          const QOp& qop) {
  const int N = nd;
  R qa[8], qb[8], qc[8];   // depths k+1, k, k-1 of the step being taken
  qop(N - 1, qa);
  qop(N - 2, qb);
  qop(N - 3, qc);
  for (int n = 0; n < 8; ++n) {
    tp.q[N - 1][n] = qa[n];
    tp.q[N - 2][n] = qb[n];
    tp.q[N - 3][n] = qc[n];
  }
  const double dtau0 = 0.5 * ((double)qa[0] + (double)qb[0]) * (double)ds[N - 1];
  R Iu[4] = {R(B1 - (B0 - B1) / dtau0), R(0), R(0), R(0)};
  for (int n = 0; n < 4; ++n) tp.I[N - 1][n] = Iu[n];
  R dSu[4], dKu[3], dchi_c, Tk;
  {
    const int k = N - 2;
    const R dsup = ds[k + 1], dsdn = ds[k];
    const R cu = qa[0], cc = qb[0], cd = qc[0];
    const R dchi_up = fdiv(cc - cu, dsup);
    dchi_c = cent_deriv<R>(dsup, dsdn, cu, cc, cd);
    const R c2 = fmax(cc - (dsup / R(3)) * dchi_c, R(0));
    const R c1 = fmax(cu + (dsup / R(3)) * dchi_up, R(0));
    Tk = R(0.25) * dsup * (cc + cu + c1 + c2);
    tp.T[k] = Tk;
    tp.dchi[k] = dchi_c;
    tp.dchi_up0 = dchi_up;
    for (int n = 0; n < 4; ++n) dSu[n] = tp.dS0[N - 1][n] = (qb[1 + n] - qa[1 + n]) / Tk;
    for (int n = 0; n < 3; ++n) dKu[n] = tp.dK0[N - 1][n] = (qb[5 + n] - qa[5 + n]) / Tk;
  }
  for (int k = N - 2; k >= 1; --k) {
    // q[k-2] enters this step's chi derivative and the next step's window
    R qd[8];
    if (k > 1) {
      qop(k - 2, qd);
      for (int n = 0; n < 8; ++n) tp.q[k - 2][n] = qd[n];
    }
    const R dsdn = ds[k];
    const R dchi_dn = (k > 1) ? cent_deriv<R>(dsdn, ds[k - 1], qb[0], qc[0], qd[0])
                              : fdiv(qc[0] - qb[0], dsdn);
    const R c2 = fmax(qb[0] + (dsdn / R(3)) * dchi_c, R(0));
    const R c1 = fmax(qc[0] - (dsdn / R(3)) * dchi_dn, R(0));
    const R Tdw = R(0.25) * dsdn * (qb[0] + qc[0] + c1 + c2);
    tp.T[k - 1] = Tdw;
    tp.dchi[k - 1] = dchi_dn;
    StepIn<R> st;
    R cf[5];
    bezier3_coeffs(Tk, cf[0], cf[1], cf[2], cf[3], cf[4]);
    st.al = cf[0]; st.be = cf[1]; st.ga = cf[2]; st.th = cf[3]; st.ep = cf[4];
    st.dt03 = Tk / R(3);
    for (int n = 0; n < 3; ++n) {
      st.ku[n] = qa[5 + n];
      st.k0[n] = qb[5 + n];
      st.dku[n] = dKu[n];
      st.dk0[n] = cent_deriv<R>(Tk, Tdw, qa[5 + n], qb[5 + n], qc[5 + n]);
      tp.dK0[k][n] = st.dk0[n];
    }
    for (int n = 0; n < 4; ++n) {
      st.Su[n] = qa[1 + n];
      st.S0[n] = qb[1 + n];
      st.dSu[n] = dSu[n];
      st.dS0[n] = cent_deriv<R>(Tk, Tdw, qa[1 + n], qb[1 + n], qc[1 + n]);
      tp.dS0[k][n] = st.dS0[n];
      st.Iu[n] = Iu[n];
    }
    R x[4], V[4], bv[3], c;
    step_fwd(st, x, V, bv, c);
    for (int n = 0; n < 4; ++n) tp.I[k][n] = Iu[n] = x[n];
    for (int n = 0; n < 4; ++n) dSu[n] = st.dS0[n];
    for (int n = 0; n < 3; ++n) dKu[n] = st.dk0[n];
    dchi_c = dchi_dn;
    Tk = Tdw;
    for (int n = 0; n < 8; ++n) {
      qa[n] = qb[n];
      qb[n] = qc[n];
      if (k > 1) qc[n] = qd[n];
    }
  }
  // last interval: now qa = q[1], qb = q[0]
  const double dtau = 0.5 * ((double)qb[0] + (double)qa[0]) * (double)ds[1];
  double w[3];
  w3(dtau, w);
  const R w0 = R(w[0]), w1 = R(w[1]), wd = R(w[1] / dtau);
  const R* ku = &qa[5];
  const R* k0 = &qb[5];
  R V[4];
  V[0] = w0 * qb[1] - w1 * dSu[0] + (R(1) - w0) * Iu[0] -
         wd * (ku[0] * Iu[1] + ku[1] * Iu[2] + ku[2] * Iu[3]);
  for (int j = 0; j < 3; ++j)
    V[j + 1] = w0 * qb[2 + j] - w1 * dSu[j + 1] + (R(1) - w0) * Iu[j + 1] - wd * ku[j] * Iu[0];
  const R g = w0 - wd;
  const R bv[3] = {g * k0[0], g * k0[1], g * k0[2]};
  const R x0 = fdiv(V[0] - (bv[0] * V[1] + bv[1] * V[2] + bv[2] * V[3]),
                    R(1) - (bv[0] * bv[0] + bv[1] * bv[1] + bv[2] * bv[2]));
  out[0] = x0;
  for (int j = 0; j < 3; ++j) out[j + 1] = V[j + 1] - x0 * bv[j];
  for (int n = 0; n < 4; ++n) tp.I[0][n] = out[n];
}

// w3 derivatives (w3.c:44-63)
PYRH_HD void w3_d(double dtau, double w[3], double dw[2]) {
  w3(dtau, w);
  if (dtau < 5.0E-4) {
    dw[0] = 1.0 - dtau;
    dw[1] = dtau - dtau * dtau;
  } else if (dtau > 50.0) {
    dw[0] = dw[1] = 0.0;
  } else {
    const double e = exp(-dtau);
    dw[0] = e;
    dw[1] = dtau * e;
  }
}

// The tape entries that reverse step k+1 reads first (and the profile sums
// of depth k-1, which the emit after that step contracts): requested during
// step k so that they arrive while it computes.  Local memory is laid out
// word by word across the 32 threads of a warp, so one request per word.
// Chi^2 gradient of 4096 atmospheres x 224 wavelengths: 26.5 -> 25.4 ms;
// adding L2 requests three steps ahead measured slower (27.6 ms).
template <typename R>
PYRH_HD void prefetch_step(const Tape<R>& tp, int k, int N) {
  const auto pf = [](const void* p) { prefetch_l1(p); };
  const int k1 = k + 1 < N ? k + 1 : N - 1, k2 = k + 2 < N ? k + 2 : N - 1;
  pf(&tp.T[k1]);
  pf(&tp.dchi[k1]);
  for (int n = 0; n < 8; ++n) pf(&tp.q[k2][n]);
  for (int n = 0; n < 4; ++n) {
    pf(&tp.I[k2][n]);
    pf(&tp.dS0[k2][n]);
  }
  for (int n = 0; n < 3; ++n) pf(&tp.dK0[k2][n]);
  if (k >= 1)
    for (int j = 0; j < kZLines; ++j)
      for (int n = 0; n < kZ; ++n) pf(&tp.z[k - 1][j][n]);
}

// Reverse (adjoint) sweep of delo_forward for NS seeds (seed[s][4] =
// dL_s/dI_0).  dL/dq_j is handed to emit(j, qb_j, bpl, sdn, sup) as soon as
// no later step can add to it (step k reaches depths k-2 .. k+1), so only
// four depths of adjoints are live at a time instead of all of them.  qb_j
// is R[NS][8]; bpl[s] is dL_s/dB for the Planck function of depth j
// (non-zero only for the two bottom depths, whose temperatures set the
// boundary condition I = B1 - (B0 - B1)/dtau); sdn[s] and sup[s] are dL_s/d
// ds_j and dL_s/d ds_{j+1}, the adjoints of the path lengths of the two
// intervals that meet at depth j (zero where there is none), final by the
// time depth j is handed over.  The steps are shared by the seeds.
template <typename R, int NS, typename Emit>
PYRH_HD void delo_reverse_stream(const Tape<R>& tp, const R* ds, int nd, double B0, double B1,
                                 const R seed[NS][4], Emit&& emit) {
  const int N = nd;
  // Adjoints of the four live depths, named by their place relative to the
  // step being reversed (k+1, k, k-1, k-2) and rotated after each step, so
  // every index is known at compile time and the arrays stay in registers.
  R qu[NS][8], qc[NS][8], qd[NS][8], qdd[NS][8];
  for (int s = 0; s < NS; ++s)
    for (int n = 0; n < 8; ++n) qu[s][n] = qc[s][n] = qd[s][n] = qdd[s][n] = R(0);
  R zero_b[NS];
  for (int s = 0; s < NS; ++s) zero_b[s] = R(0);
  R Ib[NS][4], dSb[NS][4], dKb[NS][3], dchib[NS], Tb[NS];
  // path-length adjoints of the intervals ending at depths k, k-1, k-2 of
  // the step being reversed (ds_k, ds_{k-1}, ds_{k-2}), rotated like qc..qdd
  R sc[NS], sd[NS], sdd[NS];
  for (int s = 0; s < NS; ++s) sc[s] = sd[s] = sdd[s] = R(0);
  // ---- last interval ----
  {
    const double dtau = 0.5 * ((double)tp.q[0][0] + (double)tp.q[1][0]) * (double)ds[1];
    double w[3], dw[2];
    w3_d(dtau, w, dw);
    const R w0 = R(w[0]), w1 = R(w[1]), wd = R(w[1] / dtau);
    const R* ku = &tp.q[1][5];
    const R* k0 = &tp.q[0][5];
    const R* dSu = tp.dS0[1];
    const R* I1 = tp.I[1];
    R V[4];
    V[0] = w0 * tp.q[0][1] - w1 * dSu[0] + (R(1) - w0) * I1[0] -
           wd * (ku[0] * I1[1] + ku[1] * I1[2] + ku[2] * I1[3]);
    for (int j = 0; j < 3; ++j)
      V[j + 1] = w0 * tp.q[0][2 + j] - w1 * dSu[j + 1] + (R(1) - w0) * I1[j + 1] - wd * ku[j] * I1[0];
    const R g = w0 - wd;
    const R bv[3] = {g * k0[0], g * k0[1], g * k0[2]};
    const R Dn = R(1) - (bv[0] * bv[0] + bv[1] * bv[1] + bv[2] * bv[2]);
    const R x0 = (V[0] - (bv[0] * V[1] + bv[1] * V[2] + bv[2] * V[3])) / Dn;
    R(&q0)[NS][8] = qd;   // depth 0 is k-1 of the first step
    R(&q1)[NS][8] = qc;   // depth 1 is its k
    for (int s = 0; s < NS; ++s) {
      R Vb[4] = {0, 0, 0, 0}, bb[3] = {0, 0, 0};
      R x0b = seed[s][0];
      for (int j = 0; j < 3; ++j) {
        Vb[j + 1] += seed[s][j + 1];
        x0b -= bv[j] * seed[s][j + 1];
        bb[j] -= x0 * seed[s][j + 1];
      }
      Vb[0] += x0b / Dn;
      for (int j = 0; j < 3; ++j) {
        Vb[j + 1] -= x0b / Dn * bv[j];
        bb[j] -= x0b / Dn * V[j + 1];
      }
      const R Dnb = -x0b * x0 / Dn;
      for (int j = 0; j < 3; ++j) bb[j] += Dnb * R(-2) * bv[j];
      R gb = 0, w0b = 0, w1b = 0, wdb = 0;
      for (int j = 0; j < 3; ++j) { gb += bb[j] * k0[j]; q0[s][5 + j] += g * bb[j]; }
      w0b += gb; wdb -= gb;
      for (int n = 0; n < 4; ++n) { Ib[s][n] = R(0); dSb[s][n] = R(0); }
      w0b += Vb[0] * (tp.q[0][1] - I1[0]);
      q0[s][1] += Vb[0] * w0;
      dSb[s][0] -= Vb[0] * w1;
      w1b -= Vb[0] * dSu[0];
      Ib[s][0] += Vb[0] * (R(1) - w0);
      wdb -= Vb[0] * (ku[0] * I1[1] + ku[1] * I1[2] + ku[2] * I1[3]);
      for (int j = 0; j < 3; ++j) {
        q1[s][5 + j] -= Vb[0] * wd * I1[j + 1];
        Ib[s][j + 1] -= Vb[0] * wd * ku[j];
      }
      for (int j = 0; j < 3; ++j) {
        const R v = Vb[j + 1];
        w0b += v * (tp.q[0][2 + j] - I1[j + 1]);
        q0[s][2 + j] += v * w0;
        dSb[s][j + 1] -= v * w1;
        w1b -= v * dSu[j + 1];
        Ib[s][j + 1] += v * (R(1) - w0);
        wdb -= v * ku[j] * I1[0];
        q1[s][5 + j] -= v * wd * I1[0];
        Ib[s][0] -= v * wd * ku[j];
      }
      w1b += wdb / R(dtau);
      const double dtb = (double)w0b * dw[0] + (double)w1b * dw[1] - (double)wdb * w[1] / (dtau * dtau);
      q0[s][0] += R(0.5 * (double)ds[1] * dtb);
      q1[s][0] += R(0.5 * (double)ds[1] * dtb);
      sc[s] = R(0.5 * ((double)tp.q[0][0] + (double)tp.q[1][0]) * dtb);   // ds_1
      for (int n = 0; n < 3; ++n) dKb[s][n] = R(0);
      dchib[s] = R(0);
      Tb[s] = R(0);
    }
  }
  // ---- steps k = 1 .. N-2 (reverse order of the forward sweep) ----
  for (int k = 1; k <= N - 2; ++k) {
    prefetch_step(tp, k, N);
    const R Tk = tp.T[k], Tdw = tp.T[k - 1];
    StepIn<R> st;
    R cf[5], dcf[5];
    bezier3_coeffs_d(Tk, cf, dcf);
    st.al = cf[0]; st.be = cf[1]; st.ga = cf[2]; st.th = cf[3]; st.ep = cf[4];
    st.dt03 = Tk / R(3);
    const int kup = (k + 1 == N - 1) ? N - 1 : k + 1;
    for (int n = 0; n < 3; ++n) {
      st.ku[n] = tp.q[k + 1][5 + n]; st.k0[n] = tp.q[k][5 + n];
      st.dku[n] = tp.dK0[kup][n]; st.dk0[n] = tp.dK0[k][n];
    }
    for (int n = 0; n < 4; ++n) {
      st.Su[n] = tp.q[k + 1][1 + n]; st.S0[n] = tp.q[k][1 + n];
      st.dSu[n] = tp.dS0[kup][n]; st.dS0[n] = tp.dS0[k][n];
      st.Iu[n] = tp.I[k + 1][n];
    }
    // the step's solution is I_k on the tape; b and c of its matrix are cheap
    const R c = st.ga * st.dt03, pK = st.al + st.ga * (R(1) + st.dt03);
    R bvec[3];
    for (int n = 0; n < 3; ++n) bvec[n] = pK * st.k0[n] + c * st.dk0[n];
    const R* x = tp.I[k];
    const R dsdn = ds[k];
    const R rdsdn = fdiv(R(1), dsdn);
    const CdW<R> wT = cd_weights<R>(Tk, Tdw);
    CdW<R> wchi;
    if (k > 1) wchi = cd_weights<R>(dsdn, ds[k - 1]);
    const R dchi_c = tp.dchi[k], dchi_dn = tp.dchi[k - 1];
    const bool c2pos = tp.q[k][0] + (dsdn / R(3)) * dchi_c > R(0);
    const bool c1pos = tp.q[k - 1][0] - (dsdn / R(3)) * dchi_dn > R(0);
    for (int s = 0; s < NS; ++s) {
      StepIn<R> sb;
      sb.al = sb.be = sb.ga = sb.th = sb.ep = sb.dt03 = R(0);
      for (int n = 0; n < 3; ++n) sb.ku[n] = sb.k0[n] = sb.dku[n] = sb.dk0[n] = R(0);
      for (int n = 0; n < 4; ++n) sb.Su[n] = sb.S0[n] = sb.dSu[n] = sb.dS0[n] = sb.Iu[n] = R(0);
      step_vjp(st, x, bvec, c, Ib[s], sb);
      for (int n = 0; n < 4; ++n) sb.dS0[n] += dSb[s][n];
      for (int n = 0; n < 3; ++n) sb.dk0[n] += dKb[s][n];
      R Tkb = R(0), Tdwb = Tb[s];
      for (int n = 0; n < 3; ++n)
        cent_deriv_vjp<R>(wT, tp.q[k + 1][5 + n], tp.q[k][5 + n], tp.q[k - 1][5 + n], sb.dk0[n],
                          Tkb, Tdwb, qu[s][5 + n], qc[s][5 + n], qd[s][5 + n]);
      for (int n = 0; n < 4; ++n)
        cent_deriv_vjp<R>(wT, tp.q[k + 1][1 + n], tp.q[k][1 + n], tp.q[k - 1][1 + n], sb.dS0[n],
                          Tkb, Tdwb, qu[s][1 + n], qc[s][1 + n], qd[s][1 + n]);
      Tkb += sb.al * dcf[0] + sb.be * dcf[1] + sb.ga * dcf[2] + sb.th * dcf[3] + sb.ep * dcf[4] +
             sb.dt03 / R(3);
      for (int n = 0; n < 3; ++n) { qu[s][5 + n] += sb.ku[n]; qc[s][5 + n] += sb.k0[n]; }
      for (int n = 0; n < 4; ++n) { qu[s][1 + n] += sb.Su[n]; qc[s][1 + n] += sb.S0[n]; }
      R dchi_cb = R(0), dchi_dnb = dchib[s];
      {
        // Tdw = ds_k/4 (chi_k + chi_{k-1} + c1 + c2), c2 = chi_k + ds_k/3
        // dchi_c, c1 = chi_{k-1} - ds_k/3 dchi_dn (each clipped at zero)
        const R a = R(0.25) * dsdn * Tdwb;
        qc[s][0] += a;
        qd[s][0] += a;
        sc[s] += Tdwb * Tdw * rdsdn;
        if (c2pos) { qc[s][0] += a; dchi_cb += (dsdn / R(3)) * a; sc[s] += a * dchi_c / R(3); }
        if (c1pos) { qd[s][0] += a; dchi_dnb -= (dsdn / R(3)) * a; sc[s] -= a * dchi_dn / R(3); }
      }
      if (k > 1) {
        cent_deriv_vjp<R>(wchi, tp.q[k][0], tp.q[k - 1][0], tp.q[k - 2][0], dchi_dnb, sc[s], sd[s],
                          qc[s][0], qd[s][0], qdd[s][0]);
      } else {
        qd[s][0] += dchi_dnb * rdsdn;
        qc[s][0] -= dchi_dnb * rdsdn;
        sc[s] -= dchi_dnb * dchi_dn * rdsdn;
      }
      for (int n = 0; n < 4; ++n) { Ib[s][n] = sb.Iu[n]; dSb[s][n] = sb.dSu[n]; }
      for (int n = 0; n < 3; ++n) dKb[s][n] = sb.dku[n];
      dchib[s] = dchi_cb;
      Tb[s] = Tkb;
    }
    // depth k-2 received its last term from this step's chi derivative, and
    // ds_{k-1} its last from this step's
    if (k >= 2) emit(k - 2, &qdd[0][0], zero_b, sdd, sd);
    // rotate: depth k+2 (first reached by the next step) starts at zero
    for (int s = 0; s < NS; ++s) {
      for (int n = 0; n < 8; ++n) {
        qdd[s][n] = qd[s][n];
        qd[s][n] = qc[s][n];
        qc[s][n] = qu[s][n];
        qu[s][n] = R(0);
      }
      sdd[s] = sd[s];
      sd[s] = sc[s];
      sc[s] = R(0);
    }
  }
  // ---- initial values (k = N-2 set-up and the bottom boundary) ----
  R bpl[2][NS];
  {
    const int k = N - 2;
    const R T = tp.T[k];
    const R dsup = ds[k + 1], dsdn = ds[k];
    const R cu = tp.q[k + 1][0], cc = tp.q[k][0];
    const R dchi_c = tp.dchi[k], dchi_up = tp.dchi_up0;
    const double dtau0 = 0.5 * ((double)tp.q[N - 1][0] + (double)tp.q[N - 2][0]) * (double)ds[N - 1];
    // after the last rotation depth N-1 is in qc, N-2 in qd and N-3 in qdd;
    // this set-up step reaches exactly those three (eu, ec, ed below)
    R(&eu)[NS][8] = qc;
    R(&ec)[NS][8] = qd;
    R(&ed)[NS][8] = qdd;
    // and the path lengths ds_{N-1} in sc, ds_{N-2} in sd, ds_{N-3} in sdd
    for (int s = 0; s < NS; ++s) {
      for (int n = 0; n < 4; ++n) {
        ec[s][1 + n] += dSb[s][n] / T;
        eu[s][1 + n] -= dSb[s][n] / T;
        Tb[s] -= dSb[s][n] * tp.dS0[N - 1][n] / T;
      }
      for (int n = 0; n < 3; ++n) {
        ec[s][5 + n] += dKb[s][n] / T;
        eu[s][5 + n] -= dKb[s][n] / T;
        Tb[s] -= dKb[s][n] * tp.dK0[N - 1][n] / T;
      }
      const R a = R(0.25) * dsup * Tb[s];
      ec[s][0] += a;
      eu[s][0] += a;
      sc[s] += Tb[s] * T / dsup;
      R dchi_cb = dchib[s], dchi_upb = R(0);
      if (cc - (dsup / R(3)) * dchi_c > R(0)) {
        ec[s][0] += a;
        dchi_cb -= (dsup / R(3)) * a;
        sc[s] -= a * dchi_c / R(3);
      }
      if (cu + (dsup / R(3)) * dchi_up > R(0)) {
        eu[s][0] += a;
        dchi_upb += (dsup / R(3)) * a;
        sc[s] += a * dchi_up / R(3);
      }
      ec[s][0] += dchi_upb / dsup;
      eu[s][0] -= dchi_upb / dsup;
      sc[s] -= dchi_upb * dchi_up / dsup;
      cent_deriv_vjp<R>(cd_weights<R>(dsup, dsdn), cu, cc, tp.q[k - 1][0], dchi_cb, sc[s], sd[s],
                        eu[s][0], ec[s][0], ed[s][0]);
      const double ib = (double)Ib[s][0];
      bpl[1][s] = R(ib * (1.0 + 1.0 / dtau0));
      bpl[0][s] = R(-ib / dtau0);
      const double dtb = ib * (B0 - B1) / (dtau0 * dtau0);
      eu[s][0] += R(0.5 * (double)ds[N - 1] * dtb);
      ec[s][0] += R(0.5 * (double)ds[N - 1] * dtb);
      sc[s] += R(0.5 * ((double)tp.q[N - 1][0] + (double)tp.q[N - 2][0]) * dtb);
    }
  }
  emit(N - 3, &qdd[0][0], zero_b, sdd, sd);
  emit(N - 2, &qd[0][0], bpl[0], sd, sc);
  emit(N - 1, &qc[0][0], bpl[1], sc, zero_b);
}

// ------------------------------------------ Feautrier (no line in window) --
// Where no line is inside its window the reference solves the unpolarized
// transfer equation with second-order Feautrier (rh/rhf1d/feautrier.c:56-202,
// ZERO top and THERMALIZED bottom), not DELO-Bezier3; the two differ by
// ~3e-3 of I there.  feautrier_fwd repeats the synthesis kernel's one-pass
// bottom-up elimination (solve_feautrier in lte_stokes.cu) on the optical
// quantities the forward sweep taped (chi = q[0], S = q[1]) and keeps its
// recurrence (G_k, y_k, dtau_k); feautrier_vjp runs the adjoint of that
// elimination top-down and returns dL/dchi_k, dL/dS_k, dL/d ds_k (path
// lengths) and dL/dB of the two bottom Planck values, for dL/dI_0 = Ib.
template <typename R>
struct FeautTape {
  R G[PYRH_MAX_DEPTH_RF], y[PYRH_MAX_DEPTH_RF], dtau[PYRH_MAX_DEPTH_RF];
};

// Adjoints a scalar (Stokes I only) solver hands to the per-depth
// contraction: dL/dchi_k, dL/dS_k, dL/d ds_k and the two Planck values.
template <typename R>
struct ScalarAdj {
  R chib[PYRH_MAX_DEPTH_RF], Sb[PYRH_MAX_DEPTH_RF], dsb[PYRH_MAX_DEPTH_RF];
  R B0b, B1b;
};

// Out of line on the device: it runs once per thread at most, and keeping
// it out of the kernel body keeps that body's instruction footprint small.
#ifdef __CUDA_ARCH__
#define PYRH_COLD __host__ __device__ __noinline__
#else
#define PYRH_COLD inline
#endif

template <typename R>
PYRH_COLD R feautrier_fwd(const Tape<R>& tp, const R* ds, int N, double B0, double B1,
                          FeautTape<R>& ft) {
  for (int k = 0; k < N - 1; ++k)
    ft.dtau[k] = R(0.5) * (tp.q[k][0] + tp.q[k + 1][0]) * ds[k + 1];
  R dtb = ft.dtau[N - 2];
  const R hN = R(B1 - (B0 - B1) / (double)dtb);
  const R abcN = R(1) + R(2) / dtb;
  const R A1N = R(2) / (dtb * dtb);
  R G = abcN / A1N;
  R y = (tp.q[N - 1][1] + R(2) * hN / dtb) / (abcN + A1N);
  ft.G[N - 1] = G;
  ft.y[N - 1] = y;
  for (int k = N - 2; k >= 1; --k) {
    const R dta = ft.dtau[k - 1];
    dtb = ft.dtau[k];
    const R dmid = R(0.5) * (dtb + dta);
    const R A1 = R(1) / (dmid * dta), C1 = R(1) / (dmid * dtb);
    const R Gn = (R(1) + C1 * G / (R(1) + G)) / A1;
    y = (tp.q[k][1] + C1 * y) / (A1 * (R(1) + Gn));
    G = Gn;
    ft.G[k] = G;
    ft.y[k] = y;
  }
  const R dt0 = ft.dtau[0];
  const R abc0 = R(1) + R(2) / dt0, C10 = R(2) / (dt0 * dt0);
  const R P0 = (tp.q[0][1] + C10 * y) / (abc0 + C10 * G / (R(1) + G));
  return R(2) * P0;
}

template <typename R>
PYRH_COLD void feautrier_vjp(const Tape<R>& tp, const R* ds, int N, double B0, double B1,
                             const FeautTape<R>& ft, R Ib, ScalarAdj<R>& fa) {
  R dtb_adj[PYRH_MAX_DEPTH_RF];
  for (int k = 0; k < N; ++k) fa.chib[k] = fa.Sb[k] = fa.dsb[k] = dtb_adj[k] = R(0);
  // top row: P0 = (S_0 + C10 y_1) / (abc0 + C10 g(G_1)), g(G) = G / (1 + G)
  R Gb, yb;
  {
    const R dt0 = ft.dtau[0], G1 = ft.G[1], y1 = ft.y[1];
    const R abc0 = R(1) + R(2) / dt0, C10 = R(2) / (dt0 * dt0);
    const R g1 = G1 / (R(1) + G1);
    const R den = abc0 + C10 * g1;
    const R P0 = (tp.q[0][1] + C10 * y1) / den;
    const R P0b = R(2) * Ib;
    const R numb = P0b / den, denb = -P0b * P0 / den;
    fa.Sb[0] += numb;
    const R C10b = numb * y1 + denb * g1;
    yb = numb * C10;
    Gb = denb * C10 / ((R(1) + G1) * (R(1) + G1));
    dtb_adj[0] += denb * (-R(2) / (dt0 * dt0)) + C10b * (-R(4) / (dt0 * dt0 * dt0));
  }
  // interior rows, top-down: step k made (G_k, y_k) from (G_{k+1}, y_{k+1})
  for (int k = 1; k <= N - 2; ++k) {
    const R dta = ft.dtau[k - 1], dtb = ft.dtau[k];
    const R dmid = R(0.5) * (dtb + dta);
    const R A1 = R(1) / (dmid * dta), C1 = R(1) / (dmid * dtb);
    const R Gk = ft.G[k], yk = ft.y[k], G = ft.G[k + 1], y = ft.y[k + 1];
    const R g = G / (R(1) + G);
    const R D = A1 * (R(1) + Gk);
    const R Nb = yb / D, Db = -yb * yk / D;
    fa.Sb[k] += Nb;
    R C1b = Nb * y;
    const R ynb = Nb * C1;
    R A1b = Db * (R(1) + Gk);
    const R Gkb = Gb + Db * A1;
    const R Mb = Gkb / A1;
    A1b -= Gkb * Gk / A1;
    C1b += Mb * g;
    const R Gnb = Mb * C1 / ((R(1) + G) * (R(1) + G));
    const R dmidb = -(A1b * A1 + C1b * C1) / dmid;
    dtb_adj[k - 1] += -A1b * A1 / dta + R(0.5) * dmidb;
    dtb_adj[k] += -C1b * C1 / dtb + R(0.5) * dmidb;
    Gb = Gnb;
    yb = ynb;
  }
  // bottom row: G = abcN / A1N, y = (S + 2 hN / dtb) / (abcN + A1N)
  {
    const R dtb = ft.dtau[N - 2];
    const double hNd = B1 - (B0 - B1) / (double)dtb;
    const R hN = R(hNd);
    const R abcN = R(1) + R(2) / dtb, A1N = R(2) / (dtb * dtb);
    const R den = abcN + A1N;
    const R y = ft.y[N - 1], G = ft.G[N - 1];
    const R numb = yb / den, denb = -yb * y / den;
    fa.Sb[N - 1] += numb;
    const R hNb = numb * R(2) / dtb;
    R dtbb = numb * (-R(2) * hN / (dtb * dtb));
    const R abcNb = denb + Gb / A1N, A1Nb = denb - Gb * G / A1N;
    dtbb += abcNb * (-R(2) / (dtb * dtb)) + A1Nb * (-R(4) / (dtb * dtb * dtb));
    fa.B1b = R((double)hNb * (1.0 + 1.0 / (double)dtb));
    fa.B0b = R(-(double)hNb / (double)dtb);
    dtbb += R((double)hNb * (B0 - B1) / ((double)dtb * (double)dtb));
    dtb_adj[N - 2] += dtbb;
  }
  // dtau_k = (chi_k + chi_{k+1}) ds_{k+1} / 2
  for (int k = 0; k < N - 1; ++k) {
    const R a = R(0.5) * dtb_adj[k];
    fa.chib[k] += a * ds[k + 1];
    fa.chib[k + 1] += a * ds[k + 1];
    fa.dsb[k + 1] += a * (tp.q[k][0] + tp.q[k + 1][0]);
  }
}

// ------------------------------- scalar Bezier3 (unpolarized lines only) --
// Where lines are inside their windows but none of them is polarizable the
// reference solves with scalar Bezier3 (Piecewise_Bezier3_1D,
// bezier_1D.c:306-541): clipped control points on S, a one-sided slope at
// the bottom and in the last interval; it differs from DELO-Bezier3 with
// K' = 0 by ~2e-3 of I.  Its optical-depth intervals T_k and centred chi
// derivatives are the ones delo_forward tapes, so the forward pass here
// reruns only the S recurrence (as solve_scalar in lte_stokes.cu) and keeps
// I_k; scalar_bezier_vjp runs its adjoint, then dtau_vjp turns the interval
// adjoints into dL/dchi_k and dL/d ds_k.
template <typename R>
struct ScalarTape {
  R I[PYRH_MAX_DEPTH_RF];
};

// Adjoint of the intervals T_k = ds_{k+1} (chi_k + chi_{k+1} + c1 + c2) / 4
// of delo_forward (clipped chi control points from the centred derivatives
// tp.dchi) for given dL/dT_k (k = 0 .. N-2).
template <typename R>
PYRH_COLD void dtau_vjp(const Tape<R>& tp, const R* ds, int N, const R* Tb, R* chib, R* dsb) {
  R dchib[PYRH_MAX_DEPTH_RF];
  for (int k = 0; k < N; ++k) dchib[k] = R(0);
  for (int k = 0; k <= N - 3; ++k) {      // made by step k+1 as its lower interval
    const R dsd = ds[k + 1], a = R(0.25) * dsd * Tb[k];
    chib[k + 1] += a;
    chib[k] += a;
    dsb[k + 1] += Tb[k] * tp.T[k] / dsd;
    if (tp.q[k + 1][0] + (dsd / R(3)) * tp.dchi[k + 1] > R(0)) {
      chib[k + 1] += a;
      dchib[k + 1] += (dsd / R(3)) * a;
      dsb[k + 1] += a * tp.dchi[k + 1] / R(3);
    }
    if (tp.q[k][0] - (dsd / R(3)) * tp.dchi[k] > R(0)) {
      chib[k] += a;
      dchib[k] -= (dsd / R(3)) * a;
      dsb[k + 1] -= a * tp.dchi[k] / R(3);
    }
  }
  {                                       // the first interval, k = N-2
    const int k = N - 2;
    const R dsu = ds[N - 1], a = R(0.25) * dsu * Tb[k];
    const R dchi_up = tp.dchi_up0;
    R dchi_upb = R(0);
    chib[k] += a;
    chib[k + 1] += a;
    dsb[N - 1] += Tb[k] * tp.T[k] / dsu;
    if (tp.q[k][0] - (dsu / R(3)) * tp.dchi[k] > R(0)) {
      chib[k] += a;
      dchib[k] -= (dsu / R(3)) * a;
      dsb[N - 1] -= a * tp.dchi[k] / R(3);
    }
    if (tp.q[k + 1][0] + (dsu / R(3)) * dchi_up > R(0)) {
      chib[k + 1] += a;
      dchi_upb += (dsu / R(3)) * a;
      dsb[N - 1] += a * dchi_up / R(3);
    }
    chib[k] += dchi_upb / dsu;
    chib[k + 1] -= dchi_upb / dsu;
    dsb[N - 1] -= dchi_upb * dchi_up / dsu;
  }
  // centred chi derivatives: depth k from ds_{k+1}, ds_k and chi_{k+1..k-1};
  // depth 0 one-sided
  for (int k = 1; k <= N - 2; ++k)
    cent_deriv_vjp<R>(cd_weights<R>(ds[k + 1], ds[k]), tp.q[k + 1][0], tp.q[k][0],
                      tp.q[k - 1][0], dchib[k], dsb[k + 1], dsb[k], chib[k + 1], chib[k],
                      chib[k - 1]);
  chib[0] += dchib[0] / ds[1];
  chib[1] -= dchib[0] / ds[1];
  dsb[1] -= dchib[0] * tp.dchi[0] / ds[1];
}

template <typename R>
PYRH_COLD R scalar_bezier_fwd(const Tape<R>& tp, const R* ds, int N, double B0, double B1,
                              ScalarTape<R>& st) {
  const double dtau0 = 0.5 * ((double)tp.q[N - 1][0] + (double)tp.q[N - 2][0]) * (double)ds[N - 1];
  R I = R(B1 - (B0 - B1) / dtau0);
  st.I[N - 1] = I;
  R dSup = (tp.q[N - 2][1] - tp.q[N - 1][1]) / tp.T[N - 2];
  for (int k = N - 2; k >= 1; --k) {
    const R Tk = tp.T[k], Tdw = tp.T[k - 1];
    const R Su = tp.q[k + 1][1], Sc = tp.q[k][1], Sd = tp.q[k - 1][1];
    R al, be, ga, th, ep;
    bezier3_coeffs(Tk, al, be, ga, th, ep);
    const R dt03 = Tk / R(3);
    const R dSc = cent_deriv<R>(Tk, Tdw, Su, Sc, Sd);
    const R c1 = fmax(Sc - dt03 * dSc, R(0)), c2 = fmax(Su + dt03 * dSup, R(0));
    I = I * ep + al * Sc + be * Su + ga * c1 + th * c2;
    st.I[k] = I;
    dSup = dSc;
  }
  const double dtau = 0.5 * ((double)tp.q[0][0] + (double)tp.q[1][0]) * (double)ds[1];
  double w[3];
  w3(dtau, w);
  const R dSuw = -(tp.q[0][1] - tp.q[1][1]) / R(dtau);
  return (R(1) - R(w[0])) * I + R(w[0]) * tp.q[0][1] + R(w[1]) * dSuw;
}

template <typename R>
PYRH_COLD void scalar_bezier_vjp(const Tape<R>& tp, const R* ds, int N, double B0, double B1,
                                 const ScalarTape<R>& st, R Ib, ScalarAdj<R>& fa) {
  R Tb[PYRH_MAX_DEPTH_RF], dSb[PYRH_MAX_DEPTH_RF];
  for (int k = 0; k < N; ++k) fa.chib[k] = fa.Sb[k] = fa.dsb[k] = Tb[k] = dSb[k] = R(0);
  // last interval: I_0 = (1 - w0) I_1 + w0 S_0 + w1 (S_1 - S_0) / dtau
  R Iub;
  {
    const double dtau = 0.5 * ((double)tp.q[0][0] + (double)tp.q[1][0]) * (double)ds[1];
    double w[3], dw[2];
    w3_d(dtau, w, dw);
    const R w0 = R(w[0]), w1 = R(w[1]);
    const R dSuw = -(tp.q[0][1] - tp.q[1][1]) / R(dtau);
    Iub = Ib * (R(1) - w0);
    fa.Sb[0] += Ib * w0;
    const R dSuwb = Ib * w1;
    fa.Sb[1] += dSuwb / R(dtau);
    fa.Sb[0] -= dSuwb / R(dtau);
    const double dtb = (double)(Ib * (tp.q[0][1] - st.I[1])) * dw[0] +
                       (double)(Ib * dSuw) * dw[1] - (double)dSuwb * (double)dSuw / dtau;
    fa.chib[0] += R(0.5 * (double)ds[1] * dtb);
    fa.chib[1] += R(0.5 * (double)ds[1] * dtb);
    fa.dsb[1] += R(0.5 * ((double)tp.q[0][0] + (double)tp.q[1][0]) * dtb);
  }
  // steps k = 1 .. N-2: I_k = I_{k+1} ep + al S_k + be S_{k+1} + ga c1 + th c2
  for (int k = 1; k <= N - 2; ++k) {
    const R Tk = tp.T[k], Tdw = tp.T[k - 1];
    const R Su = tp.q[k + 1][1], Sc = tp.q[k][1], Sd = tp.q[k - 1][1];
    R cf[5], dcf[5];
    bezier3_coeffs_d(Tk, cf, dcf);
    const R dt03 = Tk / R(3);
    const R dSc = cent_deriv<R>(Tk, Tdw, Su, Sc, Sd);
    const bool top = (k == N - 2);
    const R dSup = top ? (tp.q[N - 2][1] - tp.q[N - 1][1]) / Tk
                       : cent_deriv<R>(tp.T[k + 1], Tk, tp.q[k + 2][1], Su, Sc);
    const R c1 = fmax(Sc - dt03 * dSc, R(0)), c2 = fmax(Su + dt03 * dSup, R(0));
    R Tkb = Iub * (st.I[k + 1] * dcf[4] + Sc * dcf[0] + Su * dcf[1] + c1 * dcf[2] + c2 * dcf[3]);
    fa.Sb[k] += Iub * cf[0];
    fa.Sb[k + 1] += Iub * cf[1];
    const R c1b = Iub * cf[2], c2b = Iub * cf[3];
    if (Sc - dt03 * dSc > R(0)) {
      fa.Sb[k] += c1b;
      Tkb -= c1b * dSc / R(3);
      dSb[k] -= c1b * dt03;
    }
    if (Su + dt03 * dSup > R(0)) {
      fa.Sb[k + 1] += c2b;
      Tkb += c2b * dSup / R(3);
      const R dSupb = c2b * dt03;
      if (top) {
        fa.Sb[N - 2] += dSupb / Tk;
        fa.Sb[N - 1] -= dSupb / Tk;
        Tkb -= dSupb * dSup / Tk;
      } else {
        dSb[k + 1] += dSupb;
      }
    }
    // dS_k has all its terms now (this step's c1, the previous one's c2)
    cent_deriv_vjp<R>(cd_weights<R>(Tk, Tdw), Su, Sc, Sd, dSb[k], Tkb, Tb[k - 1], fa.Sb[k + 1],
                      fa.Sb[k], fa.Sb[k - 1]);
    Tb[k] += Tkb;
    Iub *= cf[4];
  }
  // bottom boundary I_{N-1} = B1 - (B0 - B1) / dtau0
  {
    const double dtau0 = 0.5 * ((double)tp.q[N - 1][0] + (double)tp.q[N - 2][0]) * (double)ds[N - 1];
    const double ib = (double)Iub;
    fa.B1b = R(ib * (1.0 + 1.0 / dtau0));
    fa.B0b = R(-ib / dtau0);
    const double dtb = ib * (B0 - B1) / (dtau0 * dtau0);
    fa.chib[N - 1] += R(0.5 * (double)ds[N - 1] * dtb);
    fa.chib[N - 2] += R(0.5 * (double)ds[N - 1] * dtb);
    fa.dsb[N - 1] += R(0.5 * ((double)tp.q[N - 1][0] + (double)tp.q[N - 2][0]) * dtb);
  }
  dtau_vjp<R>(tp, ds, N, Tb, fa.chib, fa.dsb);
}

// dB_nu/dT of planck() (planck.c:38-63)
PYRH_HD double planck_dT(double T, double lambda) {
  const double hc_kla = (kHPLANCK * kCLIGHT) / (kKBOLTZMANN * kNM_TO_M * lambda);
  const double x = hc_kla / T;
  if (x > 150.0) return 0.0;
  const double l = kNM_TO_M * lambda;
  const double twohnu3_c2 = (2.0 * kHPLANCK * kCLIGHT) / (l * l * l);
  const double ex = exp(x);
  return twohnu3_c2 * ex * x / (T * (ex - 1.0) * (ex - 1.0));
}

}  // namespace pyrh
