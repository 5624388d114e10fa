// nlte.cu -- MALI lambda iteration for one active atom, batched over
// atmospheres.
//
// Per iteration (rh/iterate.c:48-143):
//   gamma_init    new J = 0, the tiles' rate sums = 0    (fillgamma.c:44-54)
//   formal        every (atmosphere, wavelength, ray): active-atom opacity
//                 (opacity.c:64-300), formal solution with the diagonal
//                 operator for both directions (bezier_1D.c:306-541) or
//                 Feautrier where no line is active (feautrier.c:56-202),
//                 cross-coupling (fillgamma.c:251-332) and the Gamma / J
//                 quadrature (fillgamma.c:82-246, formal.c:247-256)
//   jcopy         J = new J
//   stateq        per depth: Gamma = C + the tiles' rate sums, statEquil
//                 with Crout LU + one improvement (statequil.c:40-102,
//                 ludcmp.c:36-177), FP64
//   ng            per atmosphere: Ng acceleration and MaxChange
//                 (accelerate.c:68-146, maxchange.c:32-50), FP64;
//                 converged atmospheres drop out of later launches
// Line profiles (profile.c:67-371, Armstrong Voigt of voigt.c:126-243) are
// computed once in FP64 and kept in the workspace in the formal-solution
// precision.  The per-(wavelength, depth) opacity and rate contributions run
// in the formal-solution precision.  A warp owns one tile of 32 wavelengths
// of one atmosphere and runs the rays of its ray group through it; its rate
// and J contributions are summed over the tile's wavelengths with shuffles
// and added to sums that only this warp writes, in program order, and the
// (tile, group) sums are added in a fixed order when the rate matrix and J
// are assembled: every sum has a fixed order, so a solve is
// bit-reproducible.  Background, J and these partial sums are kept in the
// formal-solution precision.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pyrh_gb300.h"
#include "nlte.cuh"
#include "lu_device.cuh"
#include "rt_device.cuh"
#include "voigt_armstrong.cuh"

namespace pyrh {

// ------------------------------------------------------------ helpers ----

__device__ __forceinline__ double wlambda_line(const double* lam, const pyrh_nlte_transition& t,
                                               int la) {
  double Dw = kCLIGHT / t.lambda0;
  if (t.symmetric) Dw *= 2.0;
  const int nl = t.nlambda;
  double w;
  if (la == 0) w = 0.5 * (lam[1] - lam[0]);
  else if (la == nl - 1) w = 0.5 * (lam[la] - lam[la - 1]);
  else w = 0.5 * (lam[la + 1] - lam[la - 1]);
  return w * Dw;
}

__device__ __forceinline__ double wlambda_cont(const double* lam, const pyrh_nlte_transition& t,
                                               int la) {
  const int nl = t.nlambda;
  if (la == 0) return 0.5 * (lam[1] - lam[0]);
  if (la == nl - 1) return 0.5 * (lam[la] - lam[la - 1]);
  return 0.5 * (lam[la + 1] - lam[la - 1]);
}

// ---------------------------------------------------------- profiles -----
// phi block of a line: [k][2*nrays][nlambda], lambda fastest.

// One thread per (line, depth, wavelength) evaluates the profile of every
// ray and direction: the Doppler offset, the damping and the normalisation
// are formed once, the ray's velocity shift once per ray, and a static
// atmosphere (no shift) takes one evaluation for all of them.
template <typename R>
__global__ void nlte_profile_kernel(NlteArgs A) {
  const int p = blockIdx.y;
  const pyrh_nlte_batch& b = A.b;
  const int nd = b.ndep[p], nt = b.ntrans[p], nq = 2 * A.nrays;
  const pyrh_nlte_transition* tr = b.trans + b.trans_off[p];
  const int64_t doff = b.depth_off[p];
  const double* lam = b.lambda + b.lam_off[p];
  int64_t total = 0;
  for (int t = 0; t < nt; ++t)
    if (tr[t].type == 0) total += (int64_t)tr[t].nlambda * nd;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = e;
    int t = 0;
    for (; t < nt; ++t) {
      if (tr[t].type != 0) continue;
      const int64_t sz = (int64_t)tr[t].nlambda * nd;
      if (r < sz) break;
      r -= sz;
    }
    const pyrh_nlte_transition& L = tr[t];
    const int la = (int)(r % L.nlambda);
    const int k = (int)(r / L.nlambda);
    const double vb = b.vbroad[doff + k];
    const double v0 = (lam[L.nblue + la] - L.lambda0 - L.c_shift) * kCLIGHT / (vb * L.lambda0);
    const double a = L.voigt ? b.adamp[b.adamp_off[p] + (int64_t)L.line_index * nd + k] : 0.0;
    const double den = kSQRTPI * vb;
    // the first element of the line's block for this depth and wavelength;
    // direction q is nlambda further on per q
    const int64_t base = L.phi_off + (int64_t)k * nq * L.nlambda + la;
    if (base + (int64_t)(nq - 1) * L.nlambda >= A.phi_cap) {
      atomicOr(A.err, 1);
      continue;
    }
    R* out = static_cast<R*>(A.phi) + base;
    double H_static = 0.0;
    for (int q = 0; q < nq; ++q) {
      const int mu = q / 2, to_obs = q % 2;
      double v = v0;
      double H;
      if (A.moving) {
        const double d = A.muz[mu] * b.vel[doff + k] / vb;
        v += to_obs ? d : -d;
      }
      if (A.moving || q == 0) {
        // Armstrong's function in FP64; for FP32 profiles with the Gaussian
        // factor in FP32 and the Dawson sum cut at 1e-10 (H within 2e-7 of
        // itself).  Evaluated wholly in FP32 (its own error up to 1.5e-5)
        // the converged populations moved from 2.5e-4 to 5.9e-4 of the
        // reference's over the 1024-atmosphere batch and past 1e-3 at 160
        // depths.
        H = sizeof(R) == 4 ? voigt_armstrong_t<double, true>(a, v) : voigt_armstrong(a, v);
        H_static = H;
      } else {
        H = H_static;
      }
      out[(int64_t)q * L.nlambda] = R(H * L.c_fraction / den);
    }
  }
}

// wphi = 1 / sum_{la, mu, dir} phi * wlambda * wmu / 2   (profile.c:210-364)
template <typename R>
__global__ void nlte_wphi_kernel(NlteArgs A) {
  const int p = blockIdx.y;
  const pyrh_nlte_batch& b = A.b;
  const int nd = b.ndep[p], nt = b.ntrans[p], nq = 2 * A.nrays;
  const pyrh_nlte_transition* tr = b.trans + b.trans_off[p];
  const double* lam = b.lambda + b.lam_off[p];
  for (int e = threadIdx.x + blockIdx.x * blockDim.x; e < nt * nd; e += blockDim.x * gridDim.x) {
    const int t = e / nd, k = e % nd;
    const pyrh_nlte_transition& L = tr[t];
    if (L.type != 0) continue;
    if (L.phi_off + (int64_t)(k + 1) * nq * L.nlambda > A.phi_cap) {
      atomicOr(A.err, 1);
      continue;
    }
    const R* ph = static_cast<const R*>(A.phi) + L.phi_off + (int64_t)k * nq * L.nlambda;
    double s = 0.0;
    for (int la = 0; la < L.nlambda; ++la) {
      const double wl = wlambda_line(lam + L.nblue, L, la);
      for (int mu = 0; mu < A.nrays; ++mu) {
        const double wlamu = wl * 0.5 * A.wmu[mu];
        for (int to = 0; to <= 1; ++to) s += (double)ph[(2 * mu + to) * L.nlambda + la] * wlamu;
      }
    }
    A.wphi[b.adamp_off[p] + (int64_t)L.line_index * nd + k] = 1.0 / s;
  }
}

// Rate-matrix partial sums of a wavelength tile and ray group: the
// off-diagonal entries (i, j), i != j, of the tile's 32 wavelengths and the
// group's rays, one value per (tile, group, entry, depth) at
// (((tile * ngroup + group) * nslot + gamma_slot) * total_depth + depth).
__host__ __device__ inline int gamma_slot(int i, int j, int nlev) {
  return i * (nlev - 1) + j - (j > i ? 1 : 0);
}

// The new J = 0 and the tiles' rate partial sums = 0 for atmospheres still
// iterating (Gamma = C is added back when statEquil assembles the matrix).
template <typename R>
__global__ void nlte_gamma_init_kernel(NlteArgs A) {
  const pyrh_nlte_batch& b = A.b;
  const int p = blockIdx.y;
  if (blockIdx.x == 0 && p == 0 && threadIdx.x == 0) *A.any = 0;   // nlte_ng_kernel sets it
  if (!A.active[p]) return;
  const int nd = b.ndep[p], nslot = b.nlevel * (b.nlevel - 1);
  const int ntg = (b.nspect[p] + 31) / 32 * A.ngroup;   // (tile, ray group) pairs
  const int64_t doff = b.depth_off[p];
  for (int e = threadIdx.x + blockIdx.x * blockDim.x; e < ntg * nslot * nd;
       e += blockDim.x * gridDim.x) {
    const int ts = e / nd, k = e % nd;
    static_cast<R*>(A.gslab)[(int64_t)ts * b.total_depth + doff + k] = R(0);
  }
  if (A.rslab) {
    if (b.ntrans[p] > A.max_ntrans) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(A.err, 4);
    }
    const int nr = 2 * A.max_ntrans;
    for (int e = threadIdx.x + blockIdx.x * blockDim.x; e < ntg * nr * nd;
         e += blockDim.x * gridDim.x) {
      const int ts = e / nd, k = e % nd;
      static_cast<R*>(A.rslab)[(int64_t)ts * b.total_depth + doff + k] = R(0);
    }
  }
  const int64_t coff = b.cont_off[p], ncont = (int64_t)nd * b.nspect[p];
  for (int g = 0; g < A.ngroup; ++g)
    for (int64_t e = threadIdx.x + (int64_t)blockIdx.x * blockDim.x; e < ncont;
         e += (int64_t)blockDim.x * gridDim.x)
      static_cast<R*>(A.Jnew)[g * b.total_cont + coff + e] = R(0);
}

// Once per solve: the background and the starting J in the formal-solution
// precision, so that the depth loops convert nothing (in FP32 mode a
// conversion from or to double runs on the FP64 pipe, a small fraction of
// the FP32 rate on this GPU).
template <typename R>
__global__ void nlte_prepare_kernel(NlteArgs A) {
  const pyrh_nlte_batch& b = A.b;
  const int64_t tc = b.total_cont;
  R* bg = static_cast<R*>(A.bgr);
  R* Jr = static_cast<R*>(A.Jr);
  for (int64_t e = threadIdx.x + (int64_t)blockIdx.x * blockDim.x; e < tc;
       e += (int64_t)blockDim.x * gridDim.x) {
    bg[e] = R(b.chi_c[e]);
    bg[tc + e] = R(b.eta_c[e]);
    bg[2 * tc + e] = R(b.sca_c[e]);
    Jr[e] = R(b.J[e]);
  }
}

// ------------------------------------------------------------ formal -----

// Transitions active across a warp's tile of 32 wavelengths: the union of
// the lanes' active sets, each transition once, continua in transition order
// and then lines (the order of every lane's own active set), in shared
// memory.  Line quantities are kept without the factor h c / (4 pi) where
// products would leave the single-precision range (V W reaches 1e15 and W
// alone 1e33).
constexpr int kMaxUnion = 32;

template <typename R>
struct UnionEntry {
  int64_t phi_off;
  int t, type, i, j, key;        // transition index, type, levels, key i nlev + j
  int nblue, nlambda, line_index;
  // the entries (bits) whose lower level is i (not this one), whose upper
  // level is j, and whose upper level is i: what the cross-coupling sums of
  // addtoCoupling select
  unsigned up_i, up_j, dn_i;
  R vb, gl, tw;                  // lines: B_ij isotope_frac, B_ji / B_ij, A_ji / B_ji
};

// One lane's active set: its entries of the warp's union and its
// wavelength-only constants, in the formal-solution precision R.
template <typename R>
struct ActiveSet {
  const UnionEntry<R>* ue;       // the warp's union (shared memory)
  unsigned lm;                   // this lane's entries (bit u: entry u)
  int la;                        // wavelength index in the atmosphere's grid
  bool bb;                       // a line is active (containsBoundBound)
  bool pol;                      // a polarized line is active (containsPolarized)
  R hckl;                        // h c / (k_B lambda)
  R twc;                         // continua: 2 h c / lambda^3
  R vbc[kMaxUnion];              // continua: alpha(lambda) of entry u
  R wl[kMaxUnion];               // lines: wlambda (Hz); continua: 4 pi wlambda / (h lambda)
};

// Per-block staging of the atmosphere's quantities that every thread reads
// at every depth (the block's warps are wavelength tiles of one atmosphere).
template <typename R>
struct NlteShared {
  R* n;       // [nlev][nd] populations
  R* lnst;    // [nlev][nd] log of the LTE populations
  R* iT;      // [nd] 1 / T
  R* ds;      // [nrays][nd] path lengths of each ray
  R* wphi;    // [nline][nd] line profile normalisation
};

template <typename R>
struct NlteOpacity {
  const NlteArgs* A;
  const pyrh_nlte_transition* tr;
  const ActiveSet<R>* as;
  const NlteShared<R>* sh;
  int nd, ns, la, q;
  int64_t coff;
  bool act;   // the lane's wavelength takes part in this solution (else no loads)

  // Total opacity, source function, the background part of the source
  // function (eta_c + sca_c J) / chi, the background opacity chi_c and the
  // atom's emissivity at depth k (opacity.c:64-300 for the active atom).
  // Lanes that do not take part in the current solution (the other solver's
  // wavelengths of a mixed warp, which run along so that the warp's rate sums
  // stay converged and add nothing) get unit opacity without reading memory.
  __device__ __forceinline__ void operator()(int k, R& chi, R& S, R& S_bg, R& chi_bg,
                                             R& eta_atom, R Jold) const {
    if (!act) {
      chi = chi_bg = R(1);
      S = S_bg = eta_atom = R(0);
      return;
    }
    const pyrh_nlte_batch& b = A->b;
    R chi_a = 0, eta_a = 0;
    for (unsigned r = as->lm; r; r &= r - 1) {
      const int u = __ffs(r) - 1;
      const UnionEntry<R>& e = as->ue[u];
      const R ni = sh->n[e.i * nd + k], nj = sh->n[e.j * nd + k];
      if (e.type == 0) {
        const int64_t pi = e.phi_off + ((int64_t)k * 2 * A->nrays + q) * e.nlambda + (as->la - e.nblue);
        const R phv = pi < A->phi_cap ? static_cast<const R*>(A->phi)[pi] : R(0);
        const R V = R(kHPLANCK * kCLIGHT / (4.0 * kPI)) * (e.vb * phv);
        chi_a += V * (ni - e.gl * nj);
        eta_a += (e.tw * e.gl) * (V * nj);
      } else {
        const R g = dev_exp(sh->lnst[e.i * nd + k] - sh->lnst[e.j * nd + k] -
                            as->hckl * sh->iT[k]);
        const R V = as->vbc[u];
        chi_a += V * (ni - g * nj);
        eta_a += (as->twc * g) * (V * nj);
      }
    }
    const int64_t c = coff + (int64_t)k * ns + la, tc = b.total_cont;
    const R* bg = static_cast<const R*>(A->bgr);
    chi_bg = bg[c];
    const R ct = chi_a + chi_bg;
    const R eta_bg = bg[tc + c] + bg[2 * tc + c] * Jold;
    chi = ct;
    S = (eta_a + eta_bg) / ct;
    S_bg = eta_bg / ct;
    eta_atom = eta_a;
  }
};

// Mean intensity of one wavelength at depth k ([depth][lambda] storage).
template <typename R>
struct JRow {
  const R* base;
  int stride;
  __device__ __forceinline__ R operator[](int k) const { return base[(int64_t)k * stride]; }
};

// Scalar Bezier3 with the diagonal operator along one direction
// (bezier_1D.c:306-541).  Each depth's intensity I, operator Psi, 1 - Psi,
// effective intensity and opacities are handed to emit(k, ...) as soon as
// they are known, so the rate and J quadratures run inside the recurrence
// and nothing is stored per depth.  Returns the intensity at the last depth
// of the sweep (the emergent one for to_obs).
template <typename R, typename Op, typename Emit>
__device__ __forceinline__ R bezier_sweep(const Op& op, const R* ds, int nd, int to_obs,
                                          double B0, double B1, const JRow<R>& Jold, Emit&& emit) {
  // Ieff = I - Psi S_atom, the effective intensity of the MALI rates
  // (fillgamma.c:121-134), is built term by term in the same recurrence: the
  // local source enters through S_bg = S - S_atom only, so no difference of
  // two nearly equal intensities is ever formed.  In optically thick line
  // cores I and Psi S_atom agree to many digits, and forming their
  // difference from single-precision I and Psi would lose all of them.
  const int dk = to_obs ? -1 : 1, k_start = to_obs ? nd - 1 : 0, k_end = to_obs ? 0 : nd - 1;
  R ea;
  R chi_u, chi_c, chi_d, chi_dd = 0, S_u, S_c, S_d, S_dd = 0, Sb_u, Sb_c, Sb_d, Sb_dd = 0;
  R cb_u, cb_c, cb_d, cb_dd = 0;
  op(k_start, chi_u, S_u, Sb_u, cb_u, ea, Jold[k_start]);
  op(k_start + dk, chi_c, S_c, Sb_c, cb_c, ea, Jold[k_start + dk]);
  op(k_start + 2 * dk, chi_d, S_d, Sb_d, cb_d, ea, Jold[k_start + 2 * dk]);
  // interval path length between depth a and a+1 is ds[a+1]
  auto dsi = [&](int a, int b2) { return ds[a > b2 ? a : b2]; };
  const R dtau0 = R(0.5) * (chi_u + chi_c) * dsi(k_start, k_start + dk);
  R I_upw = to_obs ? R(B1 - (B0 - B1) / (double)dtau0) : R(0);
  emit(k_start, I_upw, R(0), R(1), I_upw, chi_u, cb_u);
  int k = k_start + dk;
  R dsup = dsi(k, k - dk), dsdn = dsi(k + dk, k);
  R dchi_up = (chi_c - chi_u) / dsup;
  R dchi_c = cent_deriv<R>(dsup, dsdn, chi_u, chi_c, chi_d);
  R c1 = fmax(chi_c - (dsup / R(3)) * dchi_c, R(0));
  R c2 = fmax(chi_u + (dsup / R(3)) * dchi_up, R(0));
  R dtau_uw = dsup * (chi_c + chi_u + c1 + c2) * R(0.25);
  R dS_up = (S_c - S_u) / dtau_uw;
  for (k = k_start + dk; k != k_end; k += dk) {
    dsdn = dsi(k + dk, k);
    R dchi_dn;
    if (abs(k - k_end) > 1) {
      op(k + 2 * dk, chi_dd, S_dd, Sb_dd, cb_dd, ea, Jold[k + 2 * dk]);
      dchi_dn = cent_deriv<R>(dsdn, dsi(k + 2 * dk, k + dk), chi_c, chi_d, chi_dd);
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
    const R c1_raw = S_c - dt03 * dS_c;
    c1 = fmax(c1_raw, R(0));
    c2 = fmax(S_u + dt03 * dS_up, R(0));
    // control point minus S_atom: S_bg - dt03 dS_c, or -S_atom where it clips
    const R c1_eff = c1_raw > R(0) ? Sb_c - dt03 * dS_c : Sb_c - S_c;
    const R upw = I_upw * eps + beta * S_u + theta * c2;
    const R Ieff = upw + alpha * Sb_c + gamma * c1_eff;
    I_upw = upw + alpha * S_c + gamma * c1;
    // 1 - Psi without cancellation: the Bezier3 weights of a constant
    // source function sum to one (eps + alpha + beta + gamma + theta = 1)
    emit(k, I_upw, alpha + gamma, eps + beta + theta, Ieff, chi_c, cb_c);
    S_u = S_c; S_c = S_d; S_d = S_dd;
    Sb_u = Sb_c; Sb_c = Sb_d; Sb_d = Sb_dd;
    chi_u = chi_c; chi_c = chi_d; chi_d = chi_dd;
    cb_u = cb_c; cb_c = cb_d; cb_d = cb_dd;
    dchi_c = dchi_dn;
    dtau_uw = dtau_dw;
    dS_up = dS_c;
  }
  k = k_end;
  const double dtau = 0.5 * ((double)chi_c + (double)chi_u) * (double)dsi(k, k - dk);
  double w[3];
  w3(dtau, w);
  const R dS_uw = -(S_c - S_u) / R(dtau);
  const R I_last = (R(1) - R(w[0])) * I_upw + R(w[0]) * S_c + R(w[1]) * dS_uw;
  const R Ieff_last =
      (R(1) - R(w[0])) * I_upw + R(w[0]) * Sb_c + R(w[1]) * ((S_u - Sb_c) / R(dtau));
  emit(k, I_last, R(w[0] - w[1] / dtau), R((1.0 - w[0]) + w[1] / dtau), Ieff_last, chi_c, cb_c);
  return I_last;
}
// Feautrier (feautrier.c:56-202) with P, Psi, 1 - Psi and the MALI
// effective intensity P - Psi S_atom at every depth.  The effective
// intensity is not formed as that difference (which loses most of its
// digits in thick line cores, where P and Psi S_atom are both close to S):
// with the downward elimination P_k = P_{k+1} / (1 + F_k) + zt_k and the
// upward one P_k = P_{k-1} / (1 + G_k) + Zb_k, row k of the system gives
//   P_k = Psi_k (S_k + A_k zt_{k-1} + C_k Zb_{k+1}),
// so P_k - Psi_k S_atom,k = Psi_k (S_bg,k + A_k zt_{k-1} + C_k Zb_{k+1}), a sum
// of positive terms.  P may share storage with S, Psi with F, 1 - Psi with zt
// and Ieff with Sbg: each is written only after the last read of the array
// it shares.
template <typename R>
__device__ R feautrier_full(const R* chi, const R* S, const R* Sbg, const R* ds, int nd,
                            double B0, double B1, R* P, R* Psi, R* omPsi, R* Ieff, R* F, R* zt) {
  // dtau[k] = 0.5 (chi[k] + chi[k+1]) ds[k+1] for k = 0..nd-2 (ds already / mu)
  auto dtau = [&](int kk) { return R(0.5) * (chi[kk] + chi[kk + 1]) * ds[kk + 1]; };
  const R hN = R(B1 - (B0 - B1) / (double)dtau(nd - 2));
  // rows: -A1 P_{k-1} + (1 + A1 + C1) P_k - C1 P_{k+1} = S_k; the surface row
  // has diagonal abc0 + C10, the bottom row abcN + A1N and source StN
  const R d0 = dtau(0);
  const R abc0 = R(1) + R(2) / d0, C10 = R(2) / (d0 * d0);
  F[0] = abc0 / C10;
  zt[0] = S[0] / (abc0 + C10);
  for (int k = 1; k < nd - 1; ++k) {
    const R dm = dtau(k - 1), dp = dtau(k), dmid = R(0.5) * (dp + dm);
    const R A1 = R(1) / (dmid * dm), C1 = R(1) / (dmid * dp);
    F[k] = (R(1) + A1 * F[k - 1] / (R(1) + F[k - 1])) / C1;
    zt[k] = (S[k] + A1 * zt[k - 1]) / (C1 * (R(1) + F[k]));
  }
  const R dN = dtau(nd - 2);
  const R abcN = R(1) + R(2) / dN, A1N = R(2) / (dN * dN), bN = R(2) * hN / dN;
  const R StN = S[nd - 1] + bN;
  const R FoN = F[nd - 2] / (R(1) + F[nd - 2]);
  R Pk = (StN + A1N * zt[nd - 2]) / (abcN + A1N * FoN);
  // upward elimination, one step behind the downward back-substitution;
  // 1 - Psi = (denominator - 1) Psi, formed from the positive terms of the
  // denominator without cancellation
  R G = abcN / A1N;
  R Zb = StN / (A1N * (R(1) + G));
  {
    const R rest = R(2) / dN + A1N * FoN;
    const R psi = R(1) / (R(1) + rest);
    Ieff[nd - 1] = psi * (Sbg[nd - 1] + bN + A1N * zt[nd - 2]);
    P[nd - 1] = Pk;
    Psi[nd - 1] = psi;
    omPsi[nd - 1] = rest * psi;
  }
  for (int k = nd - 2; k >= 1; --k) {
    Pk = Pk / (R(1) + F[k]) + zt[k];
    const R dm = dtau(k - 1), dp = dtau(k), dmid = R(0.5) * (dp + dm);
    const R A1 = R(1) / (dmid * dm), C1 = R(1) / (dmid * dp);
    const R CG = C1 * G / (R(1) + G);
    const R rest = A1 * F[k - 1] / (R(1) + F[k - 1]) + CG;
    const R psi = R(1) / (R(1) + rest);
    const R ieff = psi * (Sbg[k] + A1 * zt[k - 1] + C1 * Zb);
    G = (R(1) + CG) / A1;
    Zb = (S[k] + C1 * Zb) / (A1 * (R(1) + G));
    P[k] = Pk;
    Psi[k] = psi;
    omPsi[k] = rest * psi;
    Ieff[k] = ieff;
  }
  {
    Pk = Pk / (R(1) + F[0]) + zt[0];
    const R rest = R(2) / d0 + C10 * G / (R(1) + G);
    const R psi = R(1) / (R(1) + rest);
    Ieff[0] = psi * (Sbg[0] + C10 * Zb);
    P[0] = Pk;
    Psi[0] = psi;
    omPsi[0] = rest * psi;
  }
  return R(2) * Pk;
}

template <typename R>
__host__ __device__ inline size_t formal_smem_layout(int nlev, int nd, int nrays, int nline,
                                                     NlteShared<R>* sh, unsigned char* base) {
  size_t off = 0;
  auto take = [&](size_t count) {
    R* p = base ? reinterpret_cast<R*>(base + off) : nullptr;
    off += ((sizeof(R) * count + 15) / 16) * 16;
    return p;
  };
  R* n = take((size_t)nlev * nd);
  R* lnst = take((size_t)nlev * nd);
  R* iT = take((size_t)nd);
  R* ds = take((size_t)nrays * nd);
  R* wphi = take((size_t)(nline > 0 ? nline : 1) * nd);
  if (sh) *sh = NlteShared<R>{n, lnst, iT, ds, wphi};
  return off;
}

// Wavelength tiles (warps) per block of the formal kernel.
constexpr int kFormalWarps = 4;

// Where one warp's rate and J contributions go: the warp is the only writer
// of its tile's rate partial sums and of its 32 wavelengths' new J, and adds
// to them in program order, so every sum has a fixed order and the solve is
// bit-reproducible.
template <typename R>
struct TileSink {
  R* gslab;           // this tile's partial sums: slot * total_depth + doff + k
  R* rslab;           // its radiative-rate sums (2 t + {0: R_ij, 1: R_ji}), or nullptr
  R* Jn;              // new J of this lane's wavelength, depth stride ns
  int64_t total_depth, doff;
  int ns;
};

// Sums a and c over the lanes of the warp that hold the same key, in an
// order fixed by the lane numbers (a shuffle tree when the whole warp shares
// the key); returns true on the one lane of each group with key >= 0, which
// then holds the group's sums.  All lanes of the warp call it together.
template <typename R>
__device__ __forceinline__ bool keyed_warp_sum(int key, R& a, R& c) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned peers = __match_any_sync(full, key);
  if (peers == full) {
    if (key < 0) return false;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(full, a, o);
      c += __shfl_xor_sync(full, c, o);
    }
    return lane == 0;
  }
  const int cnt = key >= 0 ? __popc(peers) : 0;
  const int maxc = __reduce_max_sync(full, cnt);
  unsigned rem = key >= 0 ? peers : 0u;
  R sa = R(0), sc = R(0);
  for (int s = 0; s < maxc; ++s) {
    const int src = rem ? __ffs(rem) - 1 : lane;
    const R x = __shfl_sync(full, a, src), y = __shfl_sync(full, c, src);
    if (rem) {
      sa += x;
      sc += y;
      rem &= rem - 1;
    }
  }
  a = sa;
  c = sc;
  return key >= 0 && lane == __ffs(peers) - 1;
}

// Rate (fillgamma.c:82-332) and J (formal.c:247-256) contributions of one
// depth of one ray direction, summed over the warp's 32 wavelengths.  All
// lanes of the warp call it together; lanes with mine == false add nothing.
template <typename R>
__device__ __forceinline__ void add_rates(const NlteArgs& A, const ActiveSet<R>& as, int nunion,
                                          const NlteShared<R>& sh, const TileSink<R>& out,
                                          int nd, int nlev, int q, int k, bool mine, R wdir,
                                          R I_k, R Psi_k, R omp, R Ieff_k, R chi_k, R chi_bg) {
  const unsigned full = 0xffffffffu;
  if (mine) atomicAdd(out.Jn + (int64_t)k * out.ns, wdir * I_k);
  if (!__any_sync(full, mine)) return;
  const unsigned lm = mine ? as.lm : 0u;
  const R psi = mine ? Psi_k / chi_k : R(0);
  const R ichi = mine ? R(1) / chi_k : R(0);
  // per entry: V W (product formed without the h c / 4 pi that cancels in
  // it), U = TW G V, the stimulated-emission factor G, the transition's own
  // opacity X and its opacity with the weight W, CC
  R VW[kMaxUnion], U[kMaxUnion], G[kMaxUnion], X[kMaxUnion], CC[kMaxUnion];
  for (unsigned r = lm; r; r &= r - 1) {
    const int u = __ffs(r) - 1;
    const UnionEntry<R>& e = as.ue[u];
    const R ni = sh.n[e.i * nd + k], nj = sh.n[e.j * nd + k];
    if (e.type == 0) {
      const int64_t pi = e.phi_off + ((int64_t)k * 2 * A.nrays + q) * e.nlambda + (as.la - e.nblue);
      const R phv = pi < A.phi_cap ? static_cast<const R*>(A.phi)[pi] : R(0);
      const R vph = e.vb * phv;
      const R V = R(kHPLANCK * kCLIGHT / (4.0 * kPI)) * vph;
      G[u] = e.gl;
      VW[u] = vph * (as.wl[u] * sh.wphi[e.line_index * nd + k]);
      U[u] = (e.tw * G[u]) * V;
      X[u] = V * (ni - G[u] * nj);
    } else {
      G[u] = dev_exp(sh.lnst[e.i * nd + k] - sh.lnst[e.j * nd + k] - as.hckl * sh.iT[k]);
      VW[u] = as.vbc[u] * as.wl[u];
      U[u] = (as.twc * G[u]) * as.vbc[u];
      X[u] = as.vbc[u] * (ni - G[u] * nj);
    }
    CC[u] = VW[u] * (ni - G[u] * nj);
  }
  const int nu = nunion;
  for (int u = 0; u < nu; ++u) {
    const bool has = (lm >> u) & 1u;
    const UnionEntry<R>& e = as.ue[u];
    int key = -1;
    R gij = 0, gji = 0;
    if (has) {
      key = e.key;
      const R tw = e.type == 0 ? e.tw : as.twc;
      // cross-coupling sums over the lane's active set (addtoCoupling), with
      // the transition's own terms kept apart: chi_up_o and U_down_o leave
      // out this transition, X_o is the opacity of everything but it
      // (background and the other transitions); each sum runs over the
      // transitions in active-set order
      R chi_up_o = 0, chi_down_j = 0, U_down_o = 0, U_down_i = 0, X_o = chi_bg;
      const R chi_self = CC[u];
      for (unsigned r = lm & ~(1u << u); r; r &= r - 1) X_o += X[__ffs(r) - 1];
      for (unsigned r = e.up_i & lm; r; r &= r - 1) chi_up_o += CC[__ffs(r) - 1];
      for (unsigned r = e.up_j & lm; r; r &= r - 1) {
        const int qq = __ffs(r) - 1;
        chi_down_j += CC[qq];
        if (qq != u) U_down_o += U[qq];
      }
      const unsigned di = e.dn_i & lm;
      for (unsigned r = di; r; r &= r - 1) U_down_i += U[__ffs(r) - 1];
      const int cnt = __popc(di);
      const R wlamu = VW[u] * wdir;
      gji = Ieff_k * wlamu;
      // fillgamma.c:185-196: (2 h nu^3 / c^2 + Ieff) g V W - chi_up Psi U_down.
      // The transition's own part of the coupling product,
      // 2 h nu^3 / c^2 g V W X_m Psi / chi, cancels the spontaneous term to
      // within the escape fraction 1 - X_m Psi / chi in optically thick
      // cores; that fraction is formed as X_o / chi + (X_m / chi)(1 - Psi)
      // from positive terms, and only the products with the other
      // transitions stay in the coupling term.
      const R esc = X_o * ichi + (X[u] * ichi) * omp;
      gij = (Ieff_k + tw * esc) * G[u] * wlamu -
            (chi_self * U_down_o + chi_up_o * (U[u] + U_down_o)) * (psi * wdir);
      // one term per active transition whose upper level is i
      if (cnt) gji += R(cnt) * chi_down_j * (psi * U_down_i) * wdir;
    }
    if (keyed_warp_sum<R>(key, gij, gji)) {
      const int i = key / nlev, j = key % nlev;
      atomicAdd(out.gslab + (int64_t)gamma_slot(i, j, nlev) * out.total_depth + out.doff + k, gij);
      atomicAdd(out.gslab + (int64_t)gamma_slot(j, i, nlev) * out.total_depth + out.doff + k, gji);
    }
    if (out.rslab) {
      // addtoRates (fillgamma.c:446-452): R_ij += I V W, R_ji += g (2 h nu^3 /
      // c^2 + I) V W, with the intensity itself (not Ieff)
      int rkey = -1;
      R rij = 0, rji = 0;
      if (has && e.t < A.max_ntrans) {
        rkey = e.t;
        const R wlamu = VW[u] * wdir;
        rij = I_k * wlamu;
        rji = G[u] * ((e.type == 0 ? e.tw : as.twc) + I_k) * wlamu;
      }
      if (keyed_warp_sum<R>(rkey, rij, rji)) {
        R* r = out.rslab + (int64_t)(2 * rkey) * out.total_depth + out.doff + k;
        atomicAdd(r, rij);
        atomicAdd(r + out.total_depth, rji);
      }
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(32 * kFormalWarps)
nlte_formal_kernel(NlteArgs A, int emergent_only, double* I_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const pyrh_nlte_batch& b = A.b;
  const int p = blockIdx.y;
  if (!emergent_only && !A.active[p]) return;
  const int nd = b.ndep[p], ns = b.nspect[p], nlev = b.nlevel, nt = b.ntrans[p];
  // block = kFormalWarps tiles of one atmosphere and one ray group: the
  // group takes rays grp, grp + ngroup, ... (one group unless the batch is
  // too small to fill the GPU with tiles)
  const int grp = blockIdx.x % A.ngroup;
  const int tile0 = (blockIdx.x / A.ngroup) * kFormalWarps;
  if (tile0 * 32 >= ns) return;
  if (nd < 3 || nd > b.max_ndep || nd > PYRH_NLTE_MAX_DEPTH) {   // uniform per block
    if (threadIdx.x == 0) atomicOr(A.err, 2);
    return;
  }
  const int64_t doff = b.depth_off[p], coff = b.cont_off[p];
  const pyrh_nlte_transition* tr = b.trans + b.trans_off[p];
  const double* lamp = b.lambda + b.lam_off[p];
  NlteShared<R> sh;
  // the union tables of the block's warps follow the staged arrays
  const size_t union_off = formal_smem_layout<R>(nlev, b.max_ndep, A.nrays, b.max_nline, &sh,
                                                 smem_raw);
  const int nthr = blockDim.x;
  for (int e = threadIdx.x; e < nlev * nd; e += nthr) {
    const int i = e / nd, k = e % nd;
    sh.n[e] = R(b.n[(int64_t)i * b.total_depth + doff + k]);
    sh.lnst[e] = R(log(b.nstar[(int64_t)i * b.total_depth + doff + k]));
  }
  for (int k = threadIdx.x; k < nd; k += nthr) sh.iT[k] = R(1.0 / b.T[doff + k]);
  for (int e = threadIdx.x; e < A.nrays * nd; e += nthr) {
    const int m = e / nd, k = e % nd;
    sh.ds[e] = k ? R(fabs(b.height[doff + k] - b.height[doff + k - 1]) / A.muz[m]) : R(0);
  }
  int nline = 0;
  for (int t = 0; t < nt; ++t) nline += (tr[t].type == 0);
  for (int e = threadIdx.x; e < nline * nd; e += nthr)
    sh.wphi[e] = R(A.wphi[b.adamp_off[p] + e]);
  __syncthreads();

  const int lane = threadIdx.x & 31, tile = tile0 + (threadIdx.x >> 5);
  if (tile * 32 >= ns) return;   // uniform per warp; no block barrier follows
  const unsigned full = 0xffffffffu;
  // lanes past the end of the spectrum run the recurrences of the last
  // wavelength in step with the others and add nothing
  const int la_raw = tile * 32 + lane;
  const bool live = la_raw < ns;
  const int la = live ? la_raw : ns - 1;
  const double lam = lamp[la];
  // the warp's union of active sets: every transition that covers some
  // lane's wavelength (each lane taking at most PYRH_NLTE_MAX_ACTIVE, the
  // first in continua-then-lines order, as the active set of one wavelength
  // holds them), built in that order by one ballot per transition
  UnionEntry<R>* ue = reinterpret_cast<UnionEntry<R>*>(smem_raw + union_off) +
                      (threadIdx.x >> 5) * kMaxUnion;
  ActiveSet<R> as;
  as.ue = ue;
  as.lm = 0u;
  as.la = la;
  as.bb = false;
  as.pol = false;
  as.hckl = R((kHPLANCK * kCLIGHT / (kKBOLTZMANN * kNM_TO_M)) / lam);
  as.twc = R(2.0 * kHPLANCK * kCLIGHT / (kNM_TO_M * kNM_TO_M * kNM_TO_M) / (lam * lam * lam));
  int nunion = 0, nown = 0;
  for (int pass = 1; pass >= 0; --pass)       // continua (type 1) first, then lines
    for (int t = 0; t < nt; ++t) {
      const pyrh_nlte_transition& T = tr[t];
      if (T.type != pass) continue;
      const bool mine_t = la >= T.nblue && la < T.nblue + T.nlambda && nown < PYRH_NLTE_MAX_ACTIVE;
      const unsigned who = __ballot_sync(full, mine_t);
      if (!who) continue;
      if (nunion == kMaxUnion) {            // uniform: more transitions than a table holds
        if (lane == 0) atomicOr(A.err, 8);
        continue;
      }
      const int u = nunion++;
      if (lane == (u & 31)) {
        UnionEntry<R>& e = ue[u];
        e.t = t;
        e.type = T.type;
        e.i = T.i;
        e.j = T.j;
        e.key = T.i * nlev + T.j;
        e.nblue = T.nblue;
        e.nlambda = T.nlambda;
        e.line_index = T.line_index;
        e.phi_off = T.phi_off;
        e.vb = T.type == 0 ? R(T.Bij * T.isotope_frac) : R(0);
        e.gl = T.type == 0 ? R(T.Bji / T.Bij) : R(0);
        e.tw = T.type == 0 ? R(T.Aji / T.Bji) : R(0);
      }
      if (mine_t) {
        ++nown;
        as.lm |= 1u << u;
        const int lt = la - T.nblue;
        if (T.type == 0) {
          as.bb = true;
          if (T.polarized) as.pol = true;
          as.vbc[u] = R(0);
          as.wl[u] = R(wlambda_line(lamp + T.nblue, T, lt));
        } else {
          as.vbc[u] = R(b.alpha[T.alpha_off + lt]);
          as.wl[u] = R(4.0 * kPI / kHPLANCK * (wlambda_cont(lamp + T.nblue, T, lt) / lam));
        }
      }
    }
  __syncwarp();
  for (int u = lane; u < nunion; u += 32) {   // coupling partners of each entry
    unsigned ui = 0, uj = 0, di = 0;
    for (int qq = 0; qq < nunion; ++qq) {
      if (ue[qq].i == ue[u].i && qq != u) ui |= 1u << qq;
      if (ue[qq].j == ue[u].j) uj |= 1u << qq;
      if (ue[qq].j == ue[u].i) di |= 1u << qq;
    }
    ue[u].up_i = ui;
    ue[u].up_j = uj;
    ue[u].dn_i = di;
  }
  __syncwarp();
  const double B0 = planck(b.T[doff + nd - 2], lam), B1 = planck(b.T[doff + nd - 1], lam);
  const JRow<R> Jold{static_cast<const R*>(A.Jr) + coff + la, ns};
  // angle-dependent wavelengths (formal.c:92-101: a polarized active set or
  // background, or a line in a moving atmosphere) take the Bezier3 solution
  // in both directions, the others Feautrier once per ray
  const int bgf = b.bgline[b.lam_off[p] + la];
  const bool angle_dep = as.pol || (bgf & 2) || (A.moving && (as.bb || (bgf & 1)));
  const bool bez = live && angle_dep, feau = live && !angle_dep;
  const bool any_bez = __any_sync(full, bez), any_feau = __any_sync(full, feau);
  NlteOpacity<R> op;
  op.A = &A; op.tr = tr; op.as = &as; op.sh = &sh;
  op.nd = nd; op.ns = ns; op.la = la; op.coff = coff;
  TileSink<R> out;
  out.gslab = static_cast<R*>(A.gslab) +
              ((int64_t)tile * A.ngroup + grp) * nlev * (nlev - 1) * b.total_depth;
  out.rslab = A.rslab ? static_cast<R*>(A.rslab) +
                            ((int64_t)tile * A.ngroup + grp) * 2 * A.max_ntrans * b.total_depth
                      : nullptr;
  out.Jn = static_cast<R*>(A.Jnew) + grp * b.total_cont + coff + la;
  out.total_depth = b.total_depth;
  out.doff = doff;
  out.ns = ns;
  R emergent = R(0);
  for (int ray = grp; ray < A.nrays; ray += A.ngroup) {
    const R* dsl = sh.ds + ray * nd;
    if (any_bez) {
      op.act = bez;
      for (int to_obs = emergent_only ? 1 : 0; to_obs <= 1; ++to_obs) {
        op.q = 2 * ray + to_obs;
        const R wdir = R(0.5 * A.wmu[ray]);
        const int q = op.q;
        auto emit = [&](int k, R I_k, R Psi_k, R omp, R Ieff_k, R chi_k, R chi_bg) {
          if (!emergent_only)
            add_rates<R>(A, as, nunion, sh, out, nd, nlev, q, k, bez, wdir, I_k, Psi_k, omp, Ieff_k,
                         chi_k, chi_bg);
        };
        const R Ie = bezier_sweep<R>(op, dsl, nd, to_obs, B0, B1, Jold, emit);
        if (to_obs && bez) emergent = Ie;
      }
    }
    if (any_feau) {
      // angle-independent: one Feautrier solution per ray (to_obs index 0)
      op.q = 2 * ray;
      op.act = feau;
      // P overwrites S, Psi F, 1 - Psi zt and Ieff Sb (feautrier_full allows it)
      R chis[PYRH_NLTE_MAX_DEPTH], S[PYRH_NLTE_MAX_DEPTH], F[PYRH_NLTE_MAX_DEPTH],
          zt[PYRH_NLTE_MAX_DEPTH], Sb[PYRH_NLTE_MAX_DEPTH], cbg[PYRH_NLTE_MAX_DEPTH];
      for (int k = 0; k < nd; ++k) {
        R eta_a;
        op(k, chis[k], S[k], Sb[k], cbg[k], eta_a, Jold[k]);
      }
      const R Ie = feautrier_full<R>(chis, S, Sb, dsl, nd, B0, B1, S, F, zt, Sb, F, zt);
      if (feau) emergent = Ie;
      if (!emergent_only) {
        const R wdir = R(A.wmu[ray]);
        for (int k = 0; k < nd; ++k)
          add_rates<R>(A, as, nunion, sh, out, nd, nlev, op.q, k, feau, wdir, S[k], F[k], zt[k],
                       Sb[k], chis[k], cbg[k]);
      }
    }
  }
  if (emergent_only && live) I_out[b.lam_off[p] + la] = (double)emergent;
}

// R_ij and R_ji of the atmospheres that took part in this formal solution
// (the others keep those of their last one): the (tile, ray group) sums
// added in a fixed order.
template <typename R>
__global__ void nlte_rates_kernel(NlteArgs A) {
  const pyrh_nlte_batch& b = A.b;
  const int p = blockIdx.y;
  if (!A.active[p]) return;
  const int nd = b.ndep[p];
  const int nt = b.ntrans[p] < A.max_ntrans ? b.ntrans[p] : A.max_ntrans;
  const int ntg = (b.nspect[p] + 31) / 32 * A.ngroup;
  const int64_t doff = b.depth_off[p], td = b.total_depth;
  const int64_t tstride = (int64_t)2 * A.max_ntrans * td;
  const R* rs = static_cast<const R*>(A.rslab);
  for (int e = threadIdx.x + blockIdx.x * blockDim.x; e < 2 * nt * nd;
       e += blockDim.x * gridDim.x) {
    const int slot = e / nd, k = e % nd;
    const R* s = rs + (int64_t)slot * td + doff + k;
    double r = 0.0;
    for (int t = 0; t < ntg; ++t) r += (double)s[t * tstride];
    b.rates[(int64_t)slot * td + doff + k] = r;
  }
}

// J <- new J for atmospheres still iterating (each wavelength replaces its
// own mean intensity, formal.c:128-139), the ray groups' sums added in
// group order; the formal-precision copy of J follows.
template <typename R>
__global__ void nlte_jcopy_kernel(NlteArgs A) {
  const pyrh_nlte_batch& b = A.b;
  const int p = blockIdx.y;
  if (!A.active[p]) return;
  const int64_t coff = b.cont_off[p], ncont = (int64_t)b.ndep[p] * b.nspect[p];
  const R* Jn = static_cast<const R*>(A.Jnew);
  R* Jr = static_cast<R*>(A.Jr);
  for (int64_t e = threadIdx.x + (int64_t)blockIdx.x * blockDim.x; e < ncont;
       e += (int64_t)blockDim.x * gridDim.x) {
    double J = (double)Jn[coff + e];
    for (int g = 1; g < A.ngroup; ++g) J += (double)Jn[g * b.total_cont + coff + e];
    b.J[coff + e] = J;
    Jr[coff + e] = R(J);
  }
}

// ------------------------------------------------ statistical equilibrium --

template <typename R>
__global__ void nlte_stateq_kernel(NlteArgs A) {
  const pyrh_nlte_batch& b = A.b;
  const int p = blockIdx.y;
  if (!A.active[p]) return;
  const int nd = b.ndep[p], nl = b.nlevel;
  const int64_t doff = b.depth_off[p];
  for (int k = threadIdx.x + blockIdx.x * blockDim.x; k < nd; k += blockDim.x * gridDim.x) {
    double M[PYRH_NLTE_MAX_LEVELS * PYRH_NLTE_MAX_LEVELS], x[PYRH_NLTE_MAX_LEVELS];
    int ie = 0;
    if (A.isum == -1) {
      double nmax = 0.0;
      for (int i = 0; i < nl; ++i) {
        const double v = b.n[(int64_t)i * b.total_depth + doff + k];
        if (v > nmax) { nmax = v; ie = i; }
      }
    } else {
      ie = A.isum;
    }
    // Gamma = C plus the rate sums of the atmosphere's (tile, ray group)
    // pairs, added in that order
    const int ntile = (b.nspect[p] + 31) / 32 * A.ngroup, nslot = nl * (nl - 1);
    for (int i = 0; i < nl; ++i)
      for (int j = 0; j < nl; ++j) {
        double g = b.C[(int64_t)(i * nl + j) * b.total_depth + doff + k];
        if (i != j) {
          const R* sl = static_cast<const R*>(A.gslab) +
                        (int64_t)gamma_slot(i, j, nl) * b.total_depth + doff + k;
          for (int t = 0; t < ntile; ++t) g += (double)sl[(int64_t)t * nslot * b.total_depth];
        }
        M[i * nl + j] = g;
      }
    for (int i = 0; i < nl; ++i) {
      double d = 0.0;
      M[i * nl + i] = 0.0;
      x[i] = 0.0;
      for (int j = 0; j < nl; ++j) d += M[j * nl + i];
      M[i * nl + i] = -d;
    }
    x[ie] = b.ntotal[doff + k];
    for (int j = 0; j < nl; ++j) M[ie * nl + j] = 1.0;
    lu_solve<PYRH_NLTE_MAX_LEVELS>(nl, M, x);
    for (int i = 0; i < nl; ++i) b.n[(int64_t)i * b.total_depth + doff + k] = x[i];
  }
}

// --------------------------------------------------------- Ng + MaxChange --
// One block per atmosphere; history prev[(order+2)][nlevel*ndep] per atmosphere.

__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
  __syncthreads();
  if (threadIdx.x == 0) red[0] = s;
  __syncthreads();
  const double r = red[0];
  __syncthreads();
  return r;
}

__device__ double block_max(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s = fmax(s, red[i]);
    red[0] = s;
  }
  __syncthreads();
  const double r = red[0];
  __syncthreads();
  return r;
}

__global__ void nlte_ng_kernel(NlteArgs A, int init) {
  __shared__ double red[32];
  __shared__ double Ab[PYRH_NLTE_MAX_NG * PYRH_NLTE_MAX_NG + PYRH_NLTE_MAX_NG];
  const pyrh_nlte_batch& b = A.b;
  const int p = blockIdx.x;
  if (!init && !A.active[p]) return;
  const int nd = b.ndep[p], nl = b.nlevel, N = nl * nd, No = A.ng_order, np2 = No + 2;
  const int64_t doff = b.depth_off[p];
  double* prev = A.ngprev + (int64_t)np2 * nl * doff;   // [np2][N]
  auto sol = [&](int e) -> double& {
    return b.n[(int64_t)(e / nd) * b.total_depth + doff + (e % nd)];
  };
  if (init) {                                     // NgInit (accelerate.c:34-63)
    for (int e = threadIdx.x; e < N; e += blockDim.x) prev[e] = sol(e);
    if (threadIdx.x == 0) { A.count[p] = 1; A.iters[p] = 0; A.dpops[p] = 0.0; A.active[p] = 1; }
    return;
  }
  const int count0 = A.count[p];
  const int slot = count0 % np2;
  for (int e = threadIdx.x; e < N; e += blockDim.x) prev[(int64_t)slot * N + e] = sol(e);
  const int count = count0 + 1;
  const int Ndelay = A.ng_delay > No + 2 ? A.ng_delay : No + 2;
  bool accel = (No > 0) && (count >= Ndelay) && !((count - Ndelay) % A.ng_period);
  __syncthreads();
  if (accel) {
    // A[i][j], b[j] over the weighted differences (accelerate.c:87-118)
    for (int j = 0; j < No; ++j) {
      const int ip0 = (count - 1) % np2, ipp0 = (count - 2) % np2;
      const int ipj = (count - 2 - j) % np2, ippj = (count - 3 - j) % np2;
      double sb = 0.0;
      for (int e = threadIdx.x; e < N; e += blockDim.x) {
        const double w = 1.0 / fabs(sol(e));
        const double d0 = prev[(int64_t)ip0 * N + e] - prev[(int64_t)ipp0 * N + e];
        const double dj = prev[(int64_t)ipj * N + e] - prev[(int64_t)ippj * N + e];
        sb += w * d0 * (d0 - dj);
      }
      sb = block_sum(sb, red);
      if (threadIdx.x == 0) Ab[No * No + j] = sb;
      for (int i = 0; i < No; ++i) {
        const int ipi = (count - 2 - i) % np2, ippi = (count - 3 - i) % np2;
        double sa = 0.0;
        for (int e = threadIdx.x; e < N; e += blockDim.x) {
          const double w = 1.0 / fabs(sol(e));
          const double d0 = prev[(int64_t)ip0 * N + e] - prev[(int64_t)ipp0 * N + e];
          const double dj = prev[(int64_t)ipj * N + e] - prev[(int64_t)ippj * N + e];
          const double di = prev[(int64_t)ipi * N + e] - prev[(int64_t)ippi * N + e];
          sa += w * (dj - d0) * (di - d0);
        }
        sa = block_sum(sa, red);
        if (threadIdx.x == 0) Ab[i * No + j] = sa;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) lu_solve<PYRH_NLTE_MAX_LEVELS>(No, Ab, Ab + No * No);
    __syncthreads();
    const int i0 = (count - 1) % np2;
    for (int e = threadIdx.x; e < N; e += blockDim.x) {
      double s = sol(e);
      for (int q = 0; q < No; ++q) {
        const int ip = (count - 2 - q) % np2;
        s += Ab[No * No + q] * (prev[(int64_t)ip * N + e] - prev[(int64_t)i0 * N + e]);
      }
      sol(e) = s;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < N; e += blockDim.x) prev[(int64_t)i0 * N + e] = sol(e);
    __syncthreads();
  }
  // MaxChange (maxchange.c:32-50)
  const int io = (count - 2) % np2, in = (count - 1) % np2;
  double dm = 0.0;
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    const double nw = prev[(int64_t)in * N + e], ol = prev[(int64_t)io * N + e];
    if (nw != 0.0) dm = fmax(dm, fabs((nw - ol) / nw));
  }
  dm = block_max(dm, red);
  if (threadIdx.x == 0) {
    A.count[p] = count;
    A.iters[p] += 1;
    A.dpops[p] = dm;
    if (dm < A.iter_limit || A.iters[p] >= A.nmax_iter) A.active[p] = 0;
    else atomicOr(A.any, 1);
  }
}

// ----------------------------------------------------------- launching ---

int nlte_ray_groups(int natm, int max_nspect, int nrays) {
  const long long tiles = (long long)natm * ((max_nspect + 31) / 32);
  const long long target = 4096;     // warps: about 27 per SM of a 152-SM GPU
  long long g = (target + tiles - 1) / (tiles > 0 ? tiles : 1);
  if (g > nrays) g = nrays;
  return g < 1 ? 1 : (int)g;
}

size_t nlte_formal_smem(int nlevel, int maxd, int nrays, int max_nline, int precision) {
  return precision == PYRH_FP32
             ? formal_smem_layout<float>(nlevel, maxd, nrays, max_nline, nullptr, nullptr) +
                   kFormalWarps * kMaxUnion * sizeof(UnionEntry<float>)
             : formal_smem_layout<double>(nlevel, maxd, nrays, max_nline, nullptr, nullptr) +
                   kFormalWarps * kMaxUnion * sizeof(UnionEntry<double>);
}

template <typename R>
static cudaError_t launch_profiles_t(const NlteArgs& A, int natm, int64_t max_elems,
                                     cudaStream_t st) {
  int64_t gx = (max_elems + 255) / 256;
  const int64_t cap = natm >= 4096 ? 1 : 4096 / natm;
  if (gx > cap) gx = cap;
  if (gx < 1) gx = 1;
  dim3 g((unsigned)gx, natm);
  nlte_profile_kernel<R><<<g, 256, 0, st>>>(A);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  dim3 g2(8, natm);
  nlte_wphi_kernel<R><<<g2, 128, 0, st>>>(A);
  return cudaGetLastError();
}

cudaError_t nlte_launch_profiles(const NlteArgs& A, int natm, int64_t max_elems, int precision,
                                 cudaStream_t st) {
  return precision == PYRH_FP32 ? launch_profiles_t<float>(A, natm, max_elems, st)
                                : launch_profiles_t<double>(A, natm, max_elems, st);
}

template <typename R>
static cudaError_t launch_formal_t(const NlteArgs& A, int natm, int max_nspect, int maxd,
                                   int emergent_only, double* I_out, cudaStream_t st,
                                   bool set_attr = true) {
  const size_t smem = nlte_formal_smem(A.b.nlevel, maxd, A.nrays, A.b.max_nline,
                                       sizeof(R) == 4 ? PYRH_FP32 : PYRH_FP64);
  cudaError_t e = cudaSuccess;
  if (set_attr)
    e = cudaFuncSetAttribute(nlte_formal_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
  if (e != cudaSuccess) return e;
  const int ntile = (max_nspect + 31) / 32;
  dim3 g((ntile + kFormalWarps - 1) / kFormalWarps * A.ngroup, natm);
  nlte_formal_kernel<R><<<g, 32 * kFormalWarps, smem, st>>>(A, emergent_only, I_out);
  return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_iteration_t(const NlteArgs& A, int natm, int max_nspect, int maxd,
                                      cudaStream_t st, bool set_attr) {
  dim3 gi(8, natm);
  nlte_gamma_init_kernel<R><<<gi, 256, 0, st>>>(A);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = launch_formal_t<R>(A, natm, max_nspect, maxd, 0, nullptr, st, set_attr);
  if (e != cudaSuccess) return e;
  if (A.rslab) {
    nlte_rates_kernel<R><<<gi, 256, 0, st>>>(A);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  nlte_jcopy_kernel<R><<<gi, 256, 0, st>>>(A);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  dim3 gs((maxd + 127) / 128, natm);
  nlte_stateq_kernel<R><<<gs, 128, 0, st>>>(A);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  nlte_ng_kernel<<<natm, 256, 0, st>>>(A, 0);
  return cudaGetLastError();
}

int nlte_iteration_launches(const NlteArgs& A) { return A.rslab ? 6 : 5; }

cudaError_t nlte_launch_iteration(const NlteArgs& A, int natm, int max_nspect, int maxd,
                                  int precision, cudaStream_t st, bool set_attr) {
  return precision == PYRH_FP32
             ? launch_iteration_t<float>(A, natm, max_nspect, maxd, st, set_attr)
             : launch_iteration_t<double>(A, natm, max_nspect, maxd, st, set_attr);
}

cudaError_t nlte_launch_prepare(const NlteArgs& A, int precision, cudaStream_t st) {
  const int64_t tc = A.b.total_cont;
  int64_t blocks = (tc + 255) / 256;
  if (blocks > 8192) blocks = 8192;
  if (blocks < 1) blocks = 1;
  if (precision == PYRH_FP32) nlte_prepare_kernel<float><<<(unsigned)blocks, 256, 0, st>>>(A);
  else nlte_prepare_kernel<double><<<(unsigned)blocks, 256, 0, st>>>(A);
  return cudaGetLastError();
}

cudaError_t nlte_launch_ng_init(const NlteArgs& A, int natm, cudaStream_t st) {
  nlte_ng_kernel<<<natm, 256, 0, st>>>(A, 1);
  return cudaGetLastError();
}

cudaError_t nlte_launch_emergent(const NlteArgs& A, int natm, int max_nspect, int maxd,
                                 int precision, double* I_out, cudaStream_t st) {
  return precision == PYRH_FP32
             ? launch_formal_t<float>(A, natm, max_nspect, maxd, 1, I_out, st)
             : launch_formal_t<double>(A, natm, max_nspect, maxd, 1, I_out, st);
}

}  // namespace pyrh
