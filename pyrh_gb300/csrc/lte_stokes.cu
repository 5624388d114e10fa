// lte_stokes.cu -- fused Kurucz-line Zeeman opacity + formal solution.
//
// One thread owns one (atmosphere, wavelength) pair and integrates the ray
// towards the observer from the bottom boundary up, keeping the depth
// recurrence in registers.  A block works on one atmosphere and a tile of
// consecutive wavelengths (wavelength fastest in HBM, so the continuum loads
// of a warp coalesce).  Per block, everything that depends on depth and line
// but not on wavelength (Doppler width, damping, Zeeman splitting, LTE line
// strength, projected field geometry, path lengths) is computed once into
// shared memory and read back as warp broadcasts.  The grid is persistent:
// blocks loop over (atmosphere, tile) work items.
//
// Reference functions restated here (file:line in the reference tree):
//   rlk_opacity   rh/kurucz.c:511-724   (line window, LTE populations, sums)
//   RLKProfile    rh/kurucz.c:729-827   (v, damping, Zeeman components)
//   Bproject      rh/rhf1d/project.c:38-79
//   StokesK       rh/stokesopac.c:28-87
//   Formal        rh/rhf1d/formal.c:157-310 (solver choice per wavelength)
//   Piece_Stokes_Bezier3_1D  rh/rhf1d/bezier_1D.c:52-300
//   Piecewise_Bezier3_1D     rh/rhf1d/bezier_1D.c:306-541
//   Feautrier                rh/rhf1d/feautrier.c:56-202 (eliminated from the
//                            bottom up so the emergent value needs no storage)
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pyrh_gb300.h"
#include "rt_device.cuh"
#include "voigt_armstrong.cuh"
#include "lte_stokes.cuh"

namespace pyrh {

// Per-(line, depth) quantities in shared memory, field-major: [line][F][depth].
enum LineField { LF_INVVB = 0, LF_VSHIFT, LF_ADAMP, LF_VB, LF_CHI, LF_ETA, LF_N };
// Per-depth quantities: [G][depth].
enum GeoField { GF_DS = 0, GF_GQ, GF_GU, GF_GV, GF_SIN2G, GF_N };

template <typename R>
struct Smem {
  R* geo;        // [GF_N][maxd]
  R* lp;         // [nline][LF_N][maxd]
  R* cshift;     // [nline][PYRH_MAX_COMPONENTS]
  R* cweight;    // [nline][PYRH_MAX_COMPONENTS]
  int* cq;       // [nline][PYRH_MAX_COMPONENTS]
  double* lam0;  // [nline]
  int* meta;     // [nline][3]: ncomp, polarizable, contributes
  R* dlam;       // [nline][block]: lambda - lambda0 of each thread's wavelength
  float* lc;     // [nline][LC_N]: per-line constants of the FP32 set-up
  int maxd;
};

// Per-line constants of the single-precision set-up (phase 1 of the FP32
// kernel), formed in FP64 once per block.
enum LineConst {
  LC_VTH = 0,  // 2 k / (amu weight): v_D^2 = LC_VTH T + v_turb^2
  LC_CL0,      // c / lambda0
  LC_DAMP,     // lambda0 [m] / (4 pi)
  LC_LARM,     // Larmor constant x lambda0
  LC_XI,       // E_i / k
  LC_XIJ,      // h c / (lambda0 k)
  LC_BIJ,      // h c / (4 pi) B_ij x isotope and hyperfine fractions x g_i
  LC_BIJE,     // the same x A_ji / B_ji
  LC_GRAD, LC_GSTARK, LC_CROSS, LC_VDWX,  // damping: G_vdW = LC_CROSS T^LC_VDWX
  LC_N
};

template <typename R>
__device__ __forceinline__ Smem<R> carve(unsigned char* base, int nline, int maxd) {
  Smem<R> s;
  size_t off = 0;
  s.lam0 = reinterpret_cast<double*>(base + off); off += sizeof(double) * nline;
  s.geo = reinterpret_cast<R*>(base + off); off += sizeof(R) * GF_N * maxd;
  s.lp = reinterpret_cast<R*>(base + off); off += sizeof(R) * nline * LF_N * maxd;
  s.cshift = reinterpret_cast<R*>(base + off); off += sizeof(R) * nline * PYRH_MAX_COMPONENTS;
  s.cweight = reinterpret_cast<R*>(base + off); off += sizeof(R) * nline * PYRH_MAX_COMPONENTS;
  s.cq = reinterpret_cast<int*>(base + off); off += sizeof(int) * nline * PYRH_MAX_COMPONENTS;
  s.meta = reinterpret_cast<int*>(base + off); off += sizeof(int) * nline * 3;
  off = (off + sizeof(R) - 1) / sizeof(R) * sizeof(R);
  s.dlam = reinterpret_cast<R*>(base + off); off += sizeof(R) * nline * blockDim.x;
  s.lc = reinterpret_cast<float*>(base + off);
  s.maxd = maxd;
  return s;
}

// The per-thread line offsets live in shared memory ([line][thread], one
// bank per thread): as a runtime-indexed register array they took a stack
// frame and pushed the FP32 kernel into spills.  (The DELO window's opacity
// at four depths, 28 values in registers, also spills at the 64-register cap;
// a per-thread ring of it in shared memory removed those spills but measured
// slower: the spilled values are L1 hits, the ring's loads cost issue slots.)
template <typename R>
size_t smem_bytes(int nline, int maxd, int block) {
  return sizeof(double) * nline + sizeof(R) * GF_N * maxd + sizeof(R) * nline * LF_N * maxd +
         2 * sizeof(R) * nline * PYRH_MAX_COMPONENTS + sizeof(int) * nline * PYRH_MAX_COMPONENTS +
         sizeof(int) * nline * 3 + sizeof(R) + sizeof(R) * nline * block +
         sizeof(float) * nline * LC_N + 16;
}

struct Work {
  int p, la0, nd, nl;
  int64_t doff, loff, coff;
};

// Opacity of one wavelength at one depth: chi (total), S[4], K6 = (Q, U, V,
// Q', U', V') / chi.  Line sums are accumulated in list order and added to
// the continuum afterwards, as kurucz.c:593-715 and background.c:534-537 do.
// UP: the block has lines that are not polarizable (Armstrong's Voigt);
// blocks without them run an instantiation that does not contain that
// branch, whose call would otherwise add register spills to the hot loop.
template <typename R, bool MO, bool UP = false>
struct Opacity {
  const Smem<R>* sm;
  const R* chi_c;  // continuum base for this (atmosphere, wavelength): index k*nl
  const R* eta_c;
  int nl;
  int nline;
  unsigned inwin;  // bit l: line l inside its window at this wavelength
  const R* dlam;   // lambda - lambda0 of line l at dlam[l * stride]
  int stride;

  __device__ __forceinline__ void operator()(int k, R& chi, R S[4], R K6[6]) const {
    const int maxd = sm->maxd;
    R cI = 0, cQ = 0, cU = 0, cV = 0, eI = 0, eQ = 0, eU = 0, eV = 0;
    R pQ = 0, pU = 0, pV = 0;
    const R gQ = sm->geo[GF_GQ * maxd + k], gU = sm->geo[GF_GU * maxd + k];
    const R gV = sm->geo[GF_GV * maxd + k], s2g = sm->geo[GF_SIN2G * maxd + k];
    for (int l = 0; l < nline; ++l) {
      if (!((inwin >> l) & 1u)) continue;
      const R* lp = sm->lp + (size_t)l * LF_N * maxd;
      const R v = dlam[l * stride] * lp[LF_INVVB * maxd + k] + lp[LF_VSHIFT * maxd + k];
      const R a = lp[LF_ADAMP * maxd + k];
      const R chil = lp[LF_CHI * maxd + k], etal = lp[LF_ETA * maxd + k];
      if (a < R(0)) {  // Grad == 0: Doppler core only (kurucz.c:776-779)
        R phi = (fabs(v) <= R(kMAX_GAUSS_DOPPLER)) ? dev_exp(-v * v) : R(0);
        cI += chil * phi;
        eI += etal * phi;
        continue;
      }
      if (UP && !sm->meta[3 * l + 1]) {   // not polarizable: Armstrong's Voigt, I only (kurucz.c:824)
        const R phi = voigt_armstrong_t<R>(a, v);
        cI += chil * phi;
        eI += etal * phi;
        continue;
      }
      const R vB = lp[LF_VB * maxd + k];
      const int nc = sm->meta[3 * l + 0];
      const R* csh = sm->cshift + l * PYRH_MAX_COMPONENTS;
      const R* cw = sm->cweight + l * PYRH_MAX_COMPONENTS;
      const int* cq = sm->cq + l * PYRH_MAX_COMPONENTS;
      R ph[3] = {0, 0, 0}, ps[3] = {0, 0, 0};
      for (int c = 0; c < nc; ++c) {
        R H, F;
        humlicek<R>(a, v - csh[c] * vB, H, F);
        const int q = cq[c] + 1;
        const R w = cw[c];
        if (q == 0) { ph[0] += w * H; ps[0] += w * F; }
        else if (q == 1) { ph[1] += w * H; ps[1] += w * F; }
        else { ph[2] += w * H; ps[2] += w * F; }
      }
      const R sig = ph[2] + ph[0];
      const R del = R(0.5) * ph[1] - R(0.25) * sig;
      const R phiI = del * s2g + R(0.5) * sig;
      const R phiQ = del * gQ, phiU = del * gU, phiV = R(0.5) * (ph[2] - ph[0]) * gV;
      cI += chil * phiI; eI += etal * phiI;
      cQ += chil * phiQ; eQ += etal * phiQ;
      cU += chil * phiU; eU += etal * phiU;
      cV += chil * phiV; eV += etal * phiV;
      if (MO) {
        const R psig = ps[2] + ps[0];
        const R pdel = R(0.5) * ps[1] - R(0.25) * psig;
        pQ += chil * (pdel * gQ);
        pU += chil * (pdel * gU);
        pV += chil * (R(0.5) * (ps[2] - ps[0]) * gV);
      }
    }
    const size_t ci = (size_t)k * nl;
    chi = chi_c[ci] + cI;
    const R rchi = fdiv(R(1), chi);
    S[0] = (eta_c[ci] + eI) * rchi;
    S[1] = eQ * rchi;
    S[2] = eU * rchi;
    S[3] = eV * rchi;
    K6[0] = cQ * rchi; K6[1] = cU * rchi; K6[2] = cV * rchi;
    if (MO) { K6[3] = pQ * rchi; K6[4] = pU * rchi; K6[5] = pV * rchi; }
    else { K6[3] = K6[4] = K6[5] = R(0); }
  }
};

// K' of StokesK (stokesopac.c:47-86) from its six free parameters.
template <typename R, bool MO>
__device__ __forceinline__ void build_K(const R k6[6], R K[4][4]) {
  K[0][0] = 0;      K[0][1] = k6[0]; K[0][2] = k6[1]; K[0][3] = k6[2];
  K[1][0] = k6[0];  K[1][1] = 0;     K[2][2] = 0;     K[3][3] = 0;
  K[2][0] = k6[1];  K[3][0] = k6[2];
  if (MO) {
    K[1][2] = k6[5];  K[2][1] = -k6[5];
    K[1][3] = -k6[4]; K[3][1] = k6[4];
    K[2][3] = k6[3];  K[3][2] = -k6[3];
  } else {
    K[1][2] = K[2][1] = K[1][3] = K[3][1] = K[2][3] = K[3][2] = 0;
  }
}

// One DELO-Bezier3 step (bezier_1D.c:207-247): with the interval weights,
// the K' parameters and derivatives at the upwind (u) and central (0) points
// and the source vectors, returns the new Stokes vector in I (in place).
// Without magneto-optical terms K' has non-zeros only in row/column 0, so
//   Md = [[1 + c|k|^2, b^T], [b, I + c k k^T]],  c = gamma*dt/3,
// which is solved with the Schur complement of its 3x3 block and the
// Sherman-Morrison inverse of I + c k k^T (about 60 flops instead of a 4x4
// factorisation); the magneto-optical case keeps the general 4x4 algebra.
template <typename R, bool MO>
__device__ __forceinline__ void delo_step(R alpha, R beta, R gamma, R theta, R eps, R dt03,
                                          const R ku[6], const R k0[6], const R dku[6],
                                          const R dk0[6], const R Su[4], const R S0[4],
                                          const R dSu[4], const R dS0[4], R I[4]) {
  if (!MO) {
    const R c = gamma * dt03, pK = alpha + gamma * (R(1) + dt03);
    const R ca = theta * dt03, pa = -beta - theta + theta * dt03;
    const R bt = beta + theta, ag = alpha + gamma, tdt = theta * dt03, gdt = gamma * dt03;
    const R kuIv = ku[0] * I[1] + ku[1] * I[2] + ku[2] * I[3];
    const R ku2 = ku[0] * ku[0] + ku[1] * ku[1] + ku[2] * ku[2];
    R V[4];
    V[0] = (eps + ca * ku2) * I[0] + (pa * ku[0] + ca * dku[0]) * I[1] +
           (pa * ku[1] + ca * dku[1]) * I[2] + (pa * ku[2] + ca * dku[2]) * I[3] +
           bt * Su[0] - tdt * (ku[0] * Su[1] + ku[1] * Su[2] + ku[2] * Su[3]) + ag * S0[0] +
           gdt * (k0[0] * S0[1] + k0[1] * S0[2] + k0[2] * S0[3]) +
           dt03 * (gamma * dS0[0] - theta * dSu[0]);
#pragma unroll
    for (int j = 0; j < 3; ++j)
      V[j + 1] = (pa * ku[j] + ca * dku[j]) * I[0] + eps * I[j + 1] + ca * ku[j] * kuIv -
                 tdt * ku[j] * Su[0] + bt * Su[j + 1] + gdt * k0[j] * S0[0] + ag * S0[j + 1] +
                 dt03 * (gamma * dS0[j + 1] - theta * dSu[j + 1]);
    // solve Md x = V
    const R b0 = pK * k0[0] + c * dk0[0], b1 = pK * k0[1] + c * dk0[1], b2 = pK * k0[2] + c * dk0[2];
    const R sig = R(1) + c * (k0[0] * k0[0] + k0[1] * k0[1] + k0[2] * k0[2]);
    const R f = fdiv(c, sig);
    const R kb = k0[0] * b0 + k0[1] * b1 + k0[2] * b2;
    const R kv = k0[0] * V[1] + k0[1] * V[2] + k0[2] * V[3];
    const R w0 = b0 - f * kb * k0[0], w1 = b1 - f * kb * k0[1], w2 = b2 - f * kb * k0[2];
    const R z0 = V[1] - f * kv * k0[0], z1 = V[2] - f * kv * k0[1], z2 = V[3] - f * kv * k0[2];
    const R x0 = fdiv(V[0] - (b0 * z0 + b1 * z1 + b2 * z2), sig - (b0 * w0 + b1 * w1 + b2 * w2));
    I[0] = x0;
    I[1] = z0 - x0 * w0;
    I[2] = z1 - x0 * w1;
    I[3] = z2 - x0 * w2;
  } else {
    R Ku[4][4], K0[4][4], dKu[4][4], dK0[4][4];
    build_K<R, MO>(ku, Ku);
    build_K<R, MO>(k0, K0);
    build_K<R, MO>(dku, dKu);
    build_K<R, MO>(dk0, dK0);
    R Md[4][4], V0[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      R v = 0;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        R kk0 = 0, kku = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          kk0 += K0[j][q] * K0[q][i];
          kku += Ku[j][q] * Ku[q][i];
        }
        const R id = (i == j) ? R(1) : R(0);
        Md[j][i] = id + alpha * K0[j][i] + gamma * (dt03 * (kk0 + dK0[j][i] + K0[j][i]) + K0[j][i]);
        const R ma = eps * id - beta * Ku[j][i] + theta * (dt03 * (kku + dKu[j][i] + Ku[j][i]) - Ku[j][i]);
        const R mb = beta * id + theta * (id - dt03 * Ku[j][i]);
        const R mc = alpha * id + gamma * (id + dt03 * K0[j][i]);
        v += ma * I[i] + mb * Su[i] + mc * S0[i];
      }
      V0[j] = v + dt03 * (gamma * dS0[j] - theta * dSu[j]);
    }
    solve4<R>(Md, V0, I);
  }
}

// Linear last interval (bezier_1D.c:266-299).
template <typename R, bool MO>
__device__ __forceinline__ void delo_last(R w0, R w1, R wd, const R ku[6], const R k0[6],
                                          const R S0[4], const R dSu[4], R I[4], R out[4]) {
  if (!MO) {
    // A = (1-w0) I - wd Ku (off-diagonal); Md = I + (w0 - wd) K0 (off-diagonal)
    R V[4];
    V[0] = w0 * S0[0] - w1 * dSu[0] + (R(1) - w0) * I[0] -
           wd * (ku[0] * I[1] + ku[1] * I[2] + ku[2] * I[3]);
#pragma unroll
    for (int j = 0; j < 3; ++j)
      V[j + 1] = w0 * S0[j + 1] - w1 * dSu[j + 1] + (R(1) - w0) * I[j + 1] - wd * ku[j] * I[0];
    const R g = w0 - wd;
    const R b0 = g * k0[0], b1 = g * k0[1], b2 = g * k0[2];
    const R x0 = fdiv(V[0] - (b0 * V[1] + b1 * V[2] + b2 * V[3]),
                      R(1) - (b0 * b0 + b1 * b1 + b2 * b2));
    out[0] = x0;
    out[1] = V[1] - x0 * b0;
    out[2] = V[2] - x0 * b1;
    out[3] = V[3] - x0 * b2;
  } else {
    R Ku[4][4], K0[4][4], Md[4][4], V0[4];
    build_K<R, MO>(ku, Ku);
    build_K<R, MO>(k0, K0);
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      R v = w0 * S0[n] + w1 * -dSu[n];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const R A = (n == m) ? (R(1) - w0) : (-wd * Ku[n][m]);
        v += A * I[m];
        Md[n][m] = (n == m) ? R(1) : (w0 - wd) * K0[n][m];
      }
      V0[n] = v;
    }
    solve4<R>(Md, V0, out);
  }
}

// DELO-Bezier3 along the ray to the observer; bezier_1D.c:52-300 with
// to_obs = TRUE (k_start = Ndep-1, k_end = 0, dk = -1).
template <typename R, bool MO, bool UP>
__device__ void solve_stokes(const Opacity<R, MO, UP>& op, const R* ds, int nd, double B0,
                             double B1, R out[4]) {
  constexpr int NK = MO ? 6 : 3;
  // pipeline: u = k+1, c = k, d = k-1, dd = k-2
  R chi_u, chi_c, chi_d, chi_dd;
  R S_u[4], S_c[4], S_d[4], S_dd[4];
  R k_u[6], k_c[6], k_d[6], k_dd[6];
  op(nd - 1, chi_u, S_u, k_u);
  op(nd - 2, chi_c, S_c, k_c);
  op(nd - 3, chi_d, S_d, k_d);

  R I[4];
  {
    const double dtau0 = 0.5 * ((double)chi_u + (double)chi_c) * (double)ds[nd - 1];
    I[0] = R(B1 - (B0 - B1) / dtau0);
    I[1] = I[2] = I[3] = R(0);
  }
  int k = nd - 2;
  R dsup = ds[k + 1], dsdn = ds[k];
  R dchi_up = fdiv(chi_c - chi_u, dsup);
  R dchi_c = cent_deriv<R>(dsup, dsdn, chi_u, chi_c, chi_d);
  R c2 = fmax(chi_c - (dsup / R(3)) * dchi_c, R(0));
  R c1 = fmax(chi_u + (dsup / R(3)) * dchi_up, R(0));
  R dtau_uw = R(0.25) * dsup * (chi_c + chi_u + c1 + c2);
  R dSu[4], dKu6[6];
  {
    const R r = fdiv(R(1), dtau_uw);
#pragma unroll
    for (int n = 0; n < 4; ++n) dSu[n] = (S_c[n] - S_u[n]) * r;
#pragma unroll
    for (int n = 0; n < 6; ++n) dKu6[n] = (n < NK) ? (k_c[n] - k_u[n]) * r : R(0);
  }

  for (k = nd - 2; k >= 1; --k) {
    // downwind derivative of chi needs depth k-2
    R dchi_dn;
    dsdn = ds[k];
    if (k > 1) {
      op(k - 2, chi_dd, S_dd, k_dd);
      dchi_dn = cent_deriv<R>(dsdn, ds[k - 1], chi_c, chi_d, chi_dd);
    } else {
      dchi_dn = fdiv(chi_d - chi_c, dsdn);
    }
    c2 = fmax(chi_c + (dsdn / R(3)) * dchi_c, R(0));
    c1 = fmax(chi_d - (dsdn / R(3)) * dchi_dn, R(0));
    const R dtau_dw = R(0.25) * dsdn * (chi_c + chi_d + c1 + c2);
    const R dt = dtau_uw, dt03 = dt / R(3);
    R alpha, beta, gamma, theta, eps;
    bezier3_coeffs(dt, alpha, beta, gamma, theta, eps);

    // derivatives at the central point share 1/dtau and the weight
    const R rup = fdiv(R(1), dtau_uw), rdn = fdiv(R(1), dtau_dw);
    const R aw = R(0.333333333333333333333333) * (R(1) + fdiv(dtau_dw, dtau_dw + dtau_uw));
    R dK06[6], dS0[4];
#pragma unroll
    for (int n = 0; n < 6; ++n)
      dK06[n] = (n < NK) ? cent_deriv_w<R>(rup, rdn, aw, k_u[n], k_c[n], k_d[n]) : R(0);
#pragma unroll
    for (int n = 0; n < 4; ++n) dS0[n] = cent_deriv_w<R>(rup, rdn, aw, S_u[n], S_c[n], S_d[n]);

    delo_step<R, MO>(alpha, beta, gamma, theta, eps, dt03, k_u, k_c, dKu6, dK06, S_u, S_c, dSu,
                     dS0, I);

    // shift the window one depth up
#pragma unroll
    for (int n = 0; n < 4; ++n) { S_u[n] = S_c[n]; S_c[n] = S_d[n]; S_d[n] = S_dd[n]; dSu[n] = dS0[n]; }
#pragma unroll
    for (int n = 0; n < 6; ++n) { k_u[n] = k_c[n]; k_c[n] = k_d[n]; k_d[n] = k_dd[n]; dKu6[n] = dK06[n]; }
    chi_u = chi_c; chi_c = chi_d; chi_d = chi_dd;
    dtau_uw = dtau_dw;
    dchi_c = dchi_dn;
  }
  // chi_c/S_c/k_c = depth 0, chi_u/S_u/k_u = depth 1.
  const double dtau = 0.5 * ((double)chi_c + (double)chi_u) * (double)ds[1];
  double w[3];
  w3(dtau, w);
  delo_last<R, MO>(R(w[0]), R(w[1]), R(w[1] / dtau), k_u, k_c, S_c, dSu, I, out);
}

// Scalar Bezier3 along the ray to the observer (bezier_1D.c:306-541).
template <typename R, bool MO, bool UP>
__device__ R solve_scalar(const Opacity<R, MO, UP>& op, const R* ds, int nd, double B0, double B1) {
  R chi_u, chi_c, chi_d, chi_dd, S4[4], K6[6];
  R S_u, S_c, S_d, S_dd = 0;
  op(nd - 1, chi_u, S4, K6); S_u = S4[0];
  op(nd - 2, chi_c, S4, K6); S_c = S4[0];
  chi_d = chi_c; S_d = S_c;
  if (nd >= 3) { op(nd - 3, chi_d, S4, K6); S_d = S4[0]; }
  const double dtau0 = 0.5 * ((double)chi_u + (double)chi_c) * (double)ds[nd - 1];
  R I_upw = R(B1 - (B0 - B1) / dtau0);
  int k = nd - 2;
  R dsup = ds[k + 1], dsdn = (k >= 1) ? ds[k] : ds[k + 1];
  R dchi_up = (chi_c - chi_u) / dsup;
  R dchi_c = cent_deriv<R>(dsup, dsdn, chi_u, chi_c, chi_d);
  R c1 = fmax(chi_c - (dsup / R(3)) * dchi_c, R(0));
  R c2 = fmax(chi_u + (dsup / R(3)) * dchi_up, R(0));
  R dtau_uw = dsup * (chi_c + chi_u + c1 + c2) * R(0.25);
  R dS_up = (S_c - S_u) / dtau_uw;
  for (k = nd - 2; k >= 1; --k) {
    dsdn = ds[k];
    R dchi_dn;
    if (k > 1) {
      op(k - 2, chi_dd, S4, K6); S_dd = S4[0];
      dchi_dn = cent_deriv<R>(dsdn, ds[k - 1], chi_c, chi_d, chi_dd);
    } else {
      dchi_dn = (chi_d - chi_c) / dsdn;
    }
    c1 = fmax(chi_c + (dsdn / R(3)) * dchi_c, R(0));
    c2 = fmax(chi_d - (dsdn / R(3)) * dchi_dn, R(0));
    const R dtau_dw = dsdn * (chi_c + chi_d + c1 + c2) * R(0.25);
    const R dt03 = dtau_uw / R(3);
    R alpha, beta, gamma, theta, eps;
    bezier3_coeffs(dtau_uw, alpha, beta, gamma, theta, eps);
    const R dS_c = cent_deriv<R>(dtau_uw, dtau_dw, S_u, S_c, S_d);
    c1 = fmax(S_c - dt03 * dS_c, R(0));
    c2 = fmax(S_u + dt03 * dS_up, R(0));
    I_upw = I_upw * eps + alpha * S_c + beta * S_u + gamma * c1 + theta * c2;
    S_u = S_c; S_c = S_d; S_d = S_dd;
    chi_u = chi_c; chi_c = chi_d; chi_d = chi_dd;
    dchi_c = dchi_dn;
    dtau_uw = dtau_dw;
    dS_up = dS_c;
  }
  const double dtau = 0.5 * ((double)chi_c + (double)chi_u) * (double)ds[1];
  double w[3];
  w3(dtau, w);
  const R dS_uw = -(S_c - S_u) / R(dtau);
  return (R(1) - R(w[0])) * I_upw + R(w[0]) * S_c + R(w[1]) * dS_uw;
}

// Feautrier (feautrier.c:56-202, STANDARD order, ZERO top, THERMALIZED
// bottom), eliminated from the bottom up: P[k] = P[k-1]/(1+G[k]) + y[k].
template <typename R, bool MO, bool UP>
__device__ R solve_feautrier(const Opacity<R, MO, UP>& op, const R* ds, int nd, double B0, double B1) {
  R S4[4], K6[6];
  R chi_b, chi_a;                   // depths k+1 and k
  op(nd - 1, chi_b, S4, K6);
  R S_b = S4[0];
  op(nd - 2, chi_a, S4, K6);
  R S_a = S4[0];
  R dtau_b = R(0.5) * (chi_a + chi_b) * ds[nd - 1];        // dtau[nd-2]
  const R hN = R(B1 - (B0 - B1) / (double)dtau_b);
  const R abcN = R(1) + R(2) / dtau_b;
  const R A1N = R(2) / (dtau_b * dtau_b);
  R G = abcN / A1N;
  R y = (S_b + R(2) * hN / dtau_b) / (abcN + A1N);
  for (int k = nd - 2; k >= 1; --k) {
    R chi_n;
    op(k - 1, chi_n, S4, K6);
    const R S_n = S4[0];
    const R dtau_a = R(0.5) * (chi_n + chi_a) * ds[k];      // dtau[k-1]
    const R dmid = R(0.5) * (dtau_b + dtau_a);
    const R A1 = R(1) / (dmid * dtau_a), C1 = R(1) / (dmid * dtau_b);
    const R Gn = (R(1) + C1 * G / (R(1) + G)) / A1;
    y = (S_a + C1 * y) / (A1 * (R(1) + Gn));
    G = Gn;
    chi_a = chi_n; S_a = S_n; dtau_b = dtau_a;
  }
  // top row: abc[0] = 1 + 2/dtau[0], C1[0] = 2/dtau[0]^2
  const R abc0 = R(1) + R(2) / dtau_b, C10 = R(2) / (dtau_b * dtau_b);
  const R P0 = (S_a + C10 * y) / (abc0 + C10 * G / (R(1) + G));
  return R(2) * P0;
}

// Phase 2 of the synthesis kernel: one wavelength per thread, with the
// solver the reference picks for it (formal.c:94-95, 285-310).
template <typename R, bool MO, bool UP>
__device__ __forceinline__ void synth_wavelength(const LteArgs& args, const Smem<R>& sm, int p,
                                                 int la0, int nl, int nd, int nline,
                                                 int64_t doff) {
  const int la = la0 + threadIdx.x;
  if (la < nl) {
    const int64_t loff = args.lam_off[p];
    const double lam = args.lambda[loff + la];
    const double dlc = lam * kQ_WING * (args.vmicro_char / kCLIGHT);
    Opacity<R, MO, UP> op;
    op.sm = &sm;
    op.nl = nl;
    op.nline = nline;
    op.chi_c = static_cast<const R*>(args.chi_c) + args.cont_off[p] + la;
    op.eta_c = static_cast<const R*>(args.eta_c) + args.cont_off[p] + la;
    op.inwin = 0u;
    op.dlam = sm.dlam + threadIdx.x;
    op.stride = blockDim.x;
    bool pol = false;
    for (int l = 0; l < nline; ++l) {
      const double dl = lam - sm.lam0[l];
      sm.dlam[l * blockDim.x + threadIdx.x] = R(dl);
      if (fabs(sm.lam0[l] - lam) <= dlc && sm.meta[3 * l + 2]) {
        op.inwin |= 1u << l;
        pol |= (sm.meta[3 * l + 1] != 0);
      }
    }
    const double B0 = sizeof(R) == 4 ? (double)planck_f((float)args.T[doff + nd - 2], lam)
                                     : planck(args.T[doff + nd - 2], lam);
    const double B1 = sizeof(R) == 4 ? (double)planck_f((float)args.T[doff + nd - 1], lam)
                                     : planck(args.T[doff + nd - 1], lam);
    const R* ds = sm.geo + GF_DS * sm.maxd;
    R st[4] = {0, 0, 0, 0};
    // angle dependent (formal.c:96-101): a polarizable line in window, or
    // any line in a moving atmosphere; otherwise Feautrier (formal.c:284-304)
    if (op.inwin == 0u || (!pol && !args.moving)) {
      st[0] = solve_feautrier<R, MO, UP>(op, ds, nd, B0, B1);
    } else if (pol && args.stokes_mode == PYRH_FULL_STOKES) {
      solve_stokes<R, MO, UP>(op, ds, nd, B0, B1, st);
    } else {
      st[0] = solve_scalar<R, MO, UP>(op, ds, nd, B0, B1);
    }
    R* out = static_cast<R*>(args.out) + 4 * loff;
#pragma unroll
    for (int s = 0; s < 4; ++s) out[(int64_t)s * nl + la] = st[s];
  }
}

// The same for blocks with lines that are not polarizable, out of line: the
// kernel's own register allocation then serves the common path alone (one
// call site, where little is live).
template <typename R, bool MO>
__device__ __noinline__ void synth_wavelength_unpol(const LteArgs& args, const Smem<R>& sm, int p,
                                                    int la0, int nl, int nd, int nline,
                                                    int64_t doff) {
  synth_wavelength<R, MO, true>(args, sm, p, la0, nl, nd, nline, doff);
}

// Phase 1 of the synthesis kernel in FP64: per depth, the path length and
// the projected field geometry (Bproject, project.c:38-79); per line and
// depth, the Doppler width, shift, damping, Zeeman splitting and LTE line
// opacity and emissivity (kurucz.c:638-680, 729-790).
template <typename R>
__device__ __forceinline__ void setup_f64(const LteArgs& args, const Smem<R>& sm, int64_t doff,
                                          int nd, int nline, double muz, double imu) {
  for (int k = threadIdx.x; k < nd; k += blockDim.x) {
    const int64_t d = doff + k;
    const double z_k = args.height[d];
    sm.geo[GF_DS * sm.maxd + k] = (k >= 1) ? R(fabs(z_k - args.height[d - 1]) * imu) : R(0);
    // Bproject (project.c:38-79)
    const double gam = args.gamma_B[d], chb = args.chi_B[d];
    double cg, c2c, s2c;
    if (muz == 1.0) {
      cg = cos(gam); c2c = cos(2.0 * chb); s2c = sin(2.0 * chb);
    } else {
      const double mux = sqrt(1.0 - muz * muz), csc = 1.0 / sqrt(1.0 - muz * muz);
      const double sg = sin(gam);
      const double bx = sg * cos(chb), by = sg * sin(chb), bz = cos(gam);
      const double b3 = mux * bx + muz * bz;
      const double b1 = csc * (bz - muz * b3);
      const double b2 = csc * (-mux * by);
      cg = b3;
      c2c = (b1 * b1 - b2 * b2) / (1.0 - b3 * b3);
      s2c = 2.0 * b1 * b2 / (1.0 - b3 * b3);
    }
    const double s2g = 1.0 - cg * cg;
    sm.geo[GF_GQ * sm.maxd + k] = R(s2g * c2c);
    sm.geo[GF_GU * sm.maxd + k] = R(s2g * s2c);
    sm.geo[GF_GV * sm.maxd + k] = R(cg);
    sm.geo[GF_SIN2G * sm.maxd + k] = R(s2g);
  }
  for (int i = threadIdx.x; i < nline * nd; i += blockDim.x) {
    const int l = i / nd, k = i % nd;
    const int64_t d = doff + k;
    const pyrh_line& L = args.lines[l];
    const double T = args.T[d], vt = args.vturb[d];
    const double vtherm = 2.0 * kKBOLTZMANN / (kAMU * L.weight);
    const double vb = sqrt(vtherm * T + vt * vt);
    const double sv = 1.0 / (kSQRTPI * vb);
    R* lp = sm.lp + (size_t)l * LF_N * sm.maxd;
    lp[LF_INVVB * sm.maxd + k] = R(kCLIGHT / (L.lambda0 * vb));
    lp[LF_VSHIFT * sm.maxd + k] = args.moving ? R(muz * args.vlos[d] / vb) : R(0);
    double adamp = -1.0;
    if (L.Grad != 0.0) {
      double GvdW;
      if (L.vdwaals == PYRH_VDW_UNSOLD) GvdW = L.cross * pow(T, 0.3);
      else if (L.vdwaals == PYRH_VDW_BARKLEM) GvdW = L.cross * pow(T, (1.0 - L.alpha) / 2.0);
      else GvdW = L.GvdWaals;
      adamp = (L.Grad + L.GStark * args.ne[d] + GvdW * (args.nHtot[d] - args.np[d])) *
              (L.lambda0 * kNM_TO_M) / (4.0 * kPI * vb);
    }
    lp[LF_ADAMP * sm.maxd + k] = R(adamp);
    lp[LF_VB * sm.maxd + k] = R((kLARMOR * L.lambda0) * args.B[d] / vb);
    // LTE line strength (kurucz.c:638-680)
    const double hc = kHPLANCK * kCLIGHT;
    const double hc_la = hc / (L.lambda0 * kNM_TO_M);
    const double Bijhc_4PI = hc / (4.0 * kPI) * L.Bij * L.isotope_frac * L.hyperfine_frac * L.gi;
    const double twohnu3_c2 = L.Aji / L.Bji;
    const double kT = 1.0 / (kKBOLTZMANN * T);
    const double nst = args.line_pops[((int64_t)l * 2 + 0) * args.total_depth + d];
    const double lnU = args.line_pops[((int64_t)l * 2 + 1) * args.total_depth + d];
    const double ni_gi = nst * exp(-L.Ei * kT - lnU);
    const double nj_gj = ni_gi * exp(-hc_la * kT);
    lp[LF_CHI * sm.maxd + k] = R(Bijhc_4PI * (ni_gi - nj_gj) * sv);
    lp[LF_ETA * sm.maxd + k] = R(Bijhc_4PI * twohnu3_c2 * nj_gj * sv);
  }
}

// Per-line constants of the FP32 set-up (formed in FP64, stored as float).
__device__ __forceinline__ void line_constants(const pyrh_line& L, float* c) {
  const double hc = kHPLANCK * kCLIGHT;
  c[LC_VTH] = float(2.0 * kKBOLTZMANN / (kAMU * L.weight));
  c[LC_CL0] = float(kCLIGHT / L.lambda0);
  c[LC_DAMP] = float((L.lambda0 * kNM_TO_M) / (4.0 * kPI));
  c[LC_LARM] = float(kLARMOR * L.lambda0);
  c[LC_XI] = float(L.Ei / kKBOLTZMANN);
  c[LC_XIJ] = float(hc / (L.lambda0 * kNM_TO_M * kKBOLTZMANN));
  const double bij = hc / (4.0 * kPI) * L.Bij * L.isotope_frac * L.hyperfine_frac * L.gi;
  c[LC_BIJ] = float(bij);
  c[LC_BIJE] = float(bij * (L.Aji / L.Bji));
  c[LC_GRAD] = float(L.Grad);
  c[LC_GSTARK] = float(L.GStark);
  if (L.vdwaals == PYRH_VDW_UNSOLD) {
    c[LC_CROSS] = float(L.cross); c[LC_VDWX] = 0.3f;
  } else if (L.vdwaals == PYRH_VDW_BARKLEM) {
    c[LC_CROSS] = float(L.cross); c[LC_VDWX] = float((1.0 - L.alpha) / 2.0);
  } else {
    c[LC_CROSS] = float(L.GvdWaals); c[LC_VDWX] = 0.0f;
  }
}

// Phase 1 in FP32 (the FP32 kernel): the same quantities from the per-line
// constants, without FP64 arithmetic except the path lengths (a difference
// of heights) and the geometry of oblique rays.
template <typename R>
__device__ __forceinline__ void setup_f32(const LteArgs& args, const Smem<R>& sm, int64_t doff,
                                          int nd, int nline, double muz, double imu) {
  const int maxd = sm.maxd;
  for (int k = threadIdx.x; k < nd; k += blockDim.x) {
    const int64_t d = doff + k;
    sm.geo[GF_DS * maxd + k] = (k >= 1) ? R(fabs(args.height[d] - args.height[d - 1]) * imu) : R(0);
    float cg, c2c, s2c;
    if (muz == 1.0) {
      cg = cosf((float)args.gamma_B[d]);
      sincosf(2.0f * (float)args.chi_B[d], &s2c, &c2c);
    } else {  // Bproject for an oblique ray, in FP64 (the denominators vanish along the ray)
      const double gam = args.gamma_B[d], chb = args.chi_B[d];
      const double mux = sqrt(1.0 - muz * muz), csc = 1.0 / sqrt(1.0 - muz * muz);
      const double sg = sin(gam);
      const double bx = sg * cos(chb), by = sg * sin(chb), bz = cos(gam);
      const double b3 = mux * bx + muz * bz;
      const double b1 = csc * (bz - muz * b3);
      const double b2 = csc * (-mux * by);
      cg = float(b3);
      c2c = float((b1 * b1 - b2 * b2) / (1.0 - b3 * b3));
      s2c = float(2.0 * b1 * b2 / (1.0 - b3 * b3));
    }
    const float s2g = 1.0f - cg * cg;
    sm.geo[GF_GQ * maxd + k] = R(s2g * c2c);
    sm.geo[GF_GU * maxd + k] = R(s2g * s2c);
    sm.geo[GF_GV * maxd + k] = R(cg);
    sm.geo[GF_SIN2G * maxd + k] = R(s2g);
  }
  const float rsqrtpi = float(1.0 / kSQRTPI);
  for (int i = threadIdx.x; i < nline * nd; i += blockDim.x) {
    const int l = i / nd, k = i % nd;
    const int64_t d = doff + k;
    const float* c = sm.lc + l * LC_N;
    const float T = (float)args.T[d], vt = (float)args.vturb[d];
    const float vb = sqrtf(fmaf(c[LC_VTH], T, vt * vt));
    const float rvb = 1.0f / vb;
    R* lp = sm.lp + (size_t)l * LF_N * maxd;
    lp[LF_INVVB * maxd + k] = R(c[LC_CL0] * rvb);
    lp[LF_VSHIFT * maxd + k] = args.moving ? R((float)(muz * args.vlos[d]) * rvb) : R(0);
    float adamp = -1.0f;
    if (c[LC_GRAD] != 0.0f) {
      const float GvdW = c[LC_CROSS] * powf(T, c[LC_VDWX]);
      adamp = (c[LC_GRAD] + c[LC_GSTARK] * (float)args.ne[d] +
               GvdW * (float)(args.nHtot[d] - args.np[d])) * c[LC_DAMP] * rvb;
    }
    lp[LF_ADAMP * maxd + k] = R(adamp);
    lp[LF_VB * maxd + k] = R(c[LC_LARM] * (float)args.B[d] * rvb);
    // LTE line strength (kurucz.c:638-680)
    const float rT = 1.0f / T;
    const float nst = (float)args.line_pops[((int64_t)l * 2 + 0) * args.total_depth + d];
    const float lnU = (float)args.line_pops[((int64_t)l * 2 + 1) * args.total_depth + d];
    const float ni_gi = nst * expf(-c[LC_XI] * rT - lnU);
    const float nj_gj = ni_gi * expf(-c[LC_XIJ] * rT);
    const float sv = rvb * rsqrtpi;
    lp[LF_CHI * maxd + k] = R(c[LC_BIJ] * (ni_gi - nj_gj) * sv);
    lp[LF_ETA * maxd + k] = R(c[LC_BIJE] * nj_gj * sv);
  }
}

// Resident blocks per SM the FP32 kernel is compiled for (register cap
// 65536 / (256 * N)); the FP64 kernel is compiled without a cap.
#ifndef PYRH_LTE_MIN_BLOCKS
#define PYRH_LTE_MIN_BLOCKS 4
#endif

template <typename R, bool MO>
__global__ void __launch_bounds__(256, (sizeof(R) == 4 ? PYRH_LTE_MIN_BLOCKS : 1))
lte_stokes_kernel(LteArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nline = args.nline < PYRH_MAX_LINES ? args.nline : PYRH_MAX_LINES;
  Smem<R> sm = carve<R>(smem_raw, nline, args.maxd);
  const int BL = blockDim.x;

  // line tables: once per block
  for (int i = threadIdx.x; i < nline * PYRH_MAX_COMPONENTS; i += BL) {
    const int l = i / PYRH_MAX_COMPONENTS, c = i % PYRH_MAX_COMPONENTS;
    const pyrh_line& L = args.lines[l];
    sm.cshift[i] = R(L.comp_shift[c]);
    sm.cweight[i] = R(L.comp_strength[c]);
    sm.cq[i] = L.comp_q[c];
  }
  for (int l = threadIdx.x; l < nline; l += BL) {
    sm.lam0[l] = args.lines[l].lambda0;
    const int nc = args.lines[l].ncomp;
    sm.meta[3 * l + 0] = args.lines[l].polarizable
                             ? (nc < 0 ? 0 : (nc > PYRH_MAX_COMPONENTS ? PYRH_MAX_COMPONENTS : nc))
                             : 0;
    sm.meta[3 * l + 1] = args.lines[l].polarizable;
    sm.meta[3 * l + 2] = args.lines[l].contributes;
    if (sizeof(R) == 4) line_constants(args.lines[l], sm.lc + l * LC_N);
  }

  const double muz = args.mu, imu = 1.0 / args.mu;
  const int64_t total = (int64_t)args.natm * args.tiles;
  for (int64_t w = blockIdx.x; w < total; w += gridDim.x) {
    const int p = (int)(w / args.tiles);
    const int tile = (int)(w % args.tiles);
    const int nl = args.nlam[p];
    const int la0 = tile * BL;
    if (la0 >= nl) continue;  // uniform across the block
    const int nd = args.ndep[p];
    if (nd < 3 || nd > args.maxd) continue;  // uniform across the block
    const int64_t doff = args.depth_off[p];
    __syncthreads();  // shared tables of the previous work item are consumed

    // ---- phase 1: depth- and line-dependent, wavelength-independent ----
    if (sizeof(R) == 4)
      setup_f32(args, sm, doff, nd, nline, muz, imu);
    else
      setup_f64(args, sm, doff, nd, nline, muz, imu);
    __syncthreads();

    // ---- phase 2: one wavelength per thread ----
    bool any_unpol = false;   // the same in every thread of the block
    for (int l = 0; l < nline; ++l) any_unpol |= sm.meta[3 * l + 2] && !sm.meta[3 * l + 1];
    if (any_unpol)
      synth_wavelength_unpol<R, MO>(args, sm, p, la0, nl, nd, nline, doff);
    else
      synth_wavelength<R, MO, false>(args, sm, p, la0, nl, nd, nline, doff);
  }
}

template <typename R>
static cudaError_t launch_t(const LteArgs& a, int block, int grid, cudaStream_t st) {
  const size_t sm = smem_bytes<R>(a.nline, a.maxd, block);
  if (a.magneto_optical) {
    auto k = lte_stokes_kernel<R, true>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k<<<grid, block, sm, st>>>(a);
  } else {
    auto k = lte_stokes_kernel<R, false>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k<<<grid, block, sm, st>>>(a);
  }
  return cudaGetLastError();
}

size_t lte_smem_bytes(int precision, int nline, int maxd, int block) {
  return precision == PYRH_FP32 ? smem_bytes<float>(nline, maxd, block)
                                : smem_bytes<double>(nline, maxd, block);
}

cudaError_t launch_lte_stokes(const LteArgs& a, int block, int grid, cudaStream_t st) {
  if (a.precision == PYRH_FP32) return launch_t<float>(a, block, grid, st);
  return launch_t<double>(a, block, grid, st);
}

}  // namespace pyrh
