// lte_rf_kernel.cuh -- response functions and chi^2 gradient of the LTE
// Stokes synthesis on the GPU: the kernel template, instantiated per
// precision and mode by lte_rf_fp{32,64}_{rf,chi2,vjp}.cu (units that compile in
// parallel); lte_rf.cu sizes its shared memory and dispatches.
//
// One thread owns one (atmosphere, wavelength) pair, as in lte_stokes.cu.
// A block holds several sub-blocks, each with its own work item (one
// atmosphere, one tile of wavelengths) and shared tables.  Per sub-block the
// per-(line, depth) quantities and the projected field geometry are computed once, in the
// working precision, with their derivatives with respect to (T, v_los,
// v_mic, B, gamma, chi) of the same depth, into shared memory (forward-mode
// dual numbers, lte_rf.cuh).  Each thread then
//   1. runs the DELO-Bezier3 recurrence (bezier_1D.c:52-300) to the surface,
//      evaluating the optical quantities q_k = (chi, S_I..S_V, K'_Q..K'_V) of
//      its wavelength two depths ahead of their first use, and writes the
//      recurrence state to a thread-private tape (local memory; depth-major,
//      so the tape words of a warp's threads are interleaved and coalesce);
//   2. runs the hand-written adjoint of that recurrence back down
//      (delo_reverse_stream), which hands over dL/dq_k as soon as depth k is
//      final;
//   3. at each handed-over depth, carries dL/dq_k backwards through the
//      opacity of that depth (local_q_vjp: through the line sums to the
//      per-line primitives, whose derivatives with respect to the parameters
//      are the dual parts in shared memory; the Zeeman profile sums and their
//      derivatives were evaluated once by the forward sweep and taped) and writes
//      dL/dx_k: for response functions the four
//      Stokes seeds give RF[s][x][k] (written wavelength-fastest, coalesced);
//      for the chi^2 gradient the single seed 2 w (S - obs), and for a
//      vector-Jacobian product the caller's dL/dS, give one value per
//      (x, k), summed over the sub-block's wavelengths in shared memory and
//      then added to the atmosphere's gradient in HBM.
// Steps 1 and 2-3 are separated by a block-wide barrier, so that all warps
// of the SM run the same sweep at a time.
// With the set-up's temperature derivatives (RfArgs::dT), the temperature
// slot also collects the continuum, population and path-length terms (the
// reference's finite-difference response functions re-run the set-up for
// every perturbed temperature, rf_ray.c:257-283).
// The tape holds 21 values per depth plus the Zeeman profile sums of the
// first kZLines lines; four depths of adjoints are live at a time.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pyrh_gb300.h"
#include "lte_rf.cuh"
#include "lte_stokes.cuh"

namespace pyrh {

namespace {

template <typename R>
struct RfSmem {
  LineDepth<R>* ld;   // [nline][maxd]
  GeoD<R>* geo;       // [maxd]
  R* ds;              // [maxd]
  R* cshift;          // [nline][PYRH_MAX_COMPONENTS]
  R* cweight;
  int* cq;
  int* ncomp;         // [nline]
  int* contrib;       // [nline]
  int* polar;         // [nline]
  double* lam0;       // [nline]
  R* grad;            // [kNX][maxd] (chi^2 mode)
  R* len_up;          // [maxd] d ds_k/dT_{k-1} (k >= 1; ds includes 1/mu), or zeros
  R* len_dn;          // [maxd] d ds_k/dT_k
  R* chi2;            // [1]
  R* gfs;             // [nline] log gf gradient of the block (modes 1-2)
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

template <typename R>
__host__ __device__ size_t rf_smem_t(int nline, int maxd, RfSmem<R>* s, unsigned char* base) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char* p = base ? base + off : nullptr;
    off = align16(off + bytes);
    return p;
  };
  unsigned char* p;
  p = take(sizeof(LineDepth<R>) * nline * maxd); if (s) s->ld = reinterpret_cast<LineDepth<R>*>(p);
  p = take(sizeof(GeoD<R>) * maxd);              if (s) s->geo = reinterpret_cast<GeoD<R>*>(p);
  p = take(sizeof(R) * maxd);                    if (s) s->ds = reinterpret_cast<R*>(p);
  p = take(sizeof(R) * nline * PYRH_MAX_COMPONENTS);   if (s) s->cshift = reinterpret_cast<R*>(p);
  p = take(sizeof(R) * nline * PYRH_MAX_COMPONENTS);   if (s) s->cweight = reinterpret_cast<R*>(p);
  p = take(sizeof(int) * nline * PYRH_MAX_COMPONENTS); if (s) s->cq = reinterpret_cast<int*>(p);
  p = take(sizeof(int) * nline);                 if (s) s->ncomp = reinterpret_cast<int*>(p);
  p = take(sizeof(int) * nline);                 if (s) s->contrib = reinterpret_cast<int*>(p);
  p = take(sizeof(int) * nline);                 if (s) s->polar = reinterpret_cast<int*>(p);
  p = take(sizeof(double) * nline);              if (s) s->lam0 = reinterpret_cast<double*>(p);
  p = take(sizeof(R) * kNX * maxd);              if (s) s->grad = reinterpret_cast<R*>(p);
  p = take(sizeof(R) * maxd);                    if (s) s->len_up = reinterpret_cast<R*>(p);
  p = take(sizeof(R) * maxd);                    if (s) s->len_dn = reinterpret_cast<R*>(p);
  p = take(sizeof(R) * 4);                       if (s) s->chi2 = reinterpret_cast<R*>(p);
  p = take(sizeof(R) * (nline > 0 ? nline : 1)); if (s) s->gfs = reinterpret_cast<R*>(p);
  return off;
}

// What one thread needs to evaluate q and dq/dx at any depth.
template <typename R>
struct Local {
  const RfSmem<R>* sm;
  int nline, maxd, nl;
  unsigned inwin;
  R dlam[PYRH_MAX_LINES];
  const R* chi_c;   // continuum of this (atmosphere, wavelength): index k * nl
  const R* eta_c;
  const R* dchi_c;  // their temperature derivatives, or nullptr (held fixed)
  const R* deta_c;
};

// Sum of every thread's per-line log gf gradient over the warp (shuffles)
// and the block (one shared atomic per warp and line).
template <typename R>
__device__ void gf_block_sum(const R* gfacc, int nline, R* gfs) {
  for (int l = 0; l < nline; ++l) {
    R v = gfacc[l];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31u) == 0) atomicAdd(&gfs[l], v);
  }
}

// UP: see local_q; lanes of blocks without unpolarizable lines use UP = false.
template <typename R, int MODE, bool UP>
struct Emit {
  const Local<R>* loc;
  const double* T;   // temperatures of this atmosphere
  double lam;
  int nd, nl, la;
  bool act;          // this lane holds a wavelength (writes and seeds)
  R* rf;             // mode 0: rf_out + 24 * cont_off + la
  R* gf;             // per-thread log gf accumulators [NS][PYRH_MAX_LINES] or nullptr
  const Tape<R>* tp;
  const ScalarAdj<R>* fa;  // lanes solved without polarization (Feautrier or scalar
                           // Bezier3): the adjoint of their Stokes I seed (their
                           // DELO seeds are zero)
  // k: the depth handed over; qb: dL_s/dq_k; bpl: dL_s/dB_k of the Planck
  // boundary; sdn, sup: dL_s/d ds_k and dL_s/d ds_{k+1} (path lengths)
  __device__ void operator()(int k, const R* qb_in, const R* bpl_in, const R* sdn_in,
                             const R* sup_in) const {
    constexpr int NS = MODE == 0 ? 4 : 1;
    const RfSmem<R>& sm = *loc->sm;
    // lanes solved without polarization take their own adjoints; selected by
    // value so that every lane reaches the warp sums below together
    R qb[NS * 8], bpl[NS], sdn[NS], sup[NS];
#pragma unroll
    for (int e = 0; e < NS * 8; ++e) qb[e] = qb_in[e];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      bpl[s] = bpl_in[s];
      sdn[s] = sdn_in[s];
      sup[s] = sup_in[s];
    }
    if (fa) {
#pragma unroll
      for (int e = 0; e < NS * 8; ++e) qb[e] = R(0);
      qb[0] = fa->chib[k];
      qb[1] = fa->Sb[k];
      bpl[0] = (k == nd - 2) ? fa->B0b : (k == nd - 1) ? fa->B1b : R(0);
      sdn[0] = fa->dsb[k];
      sup[0] = (k + 1 < nd) ? fa->dsb[k + 1] : R(0);
    }
    R g[NS][kNX];
#pragma unroll
    for (int s = 0; s < NS; ++s)
#pragma unroll
      for (int x = 0; x < kNX; ++x) g[s][x] = R(0);
    local_q_vjp<R, NS, UP>(loc->nline, sm.ld + k, loc->maxd, sm.geo[k], loc->dlam, loc->inwin,
                       sm.ncomp, sm.cshift, sm.cweight, sm.cq, PYRH_MAX_COMPONENTS, tp->q[k], qb,
                       g, gf, tp->z[k], loc->dchi_c ? loc->dchi_c[(int64_t)k * nl] : R(0),
                       loc->deta_c ? loc->deta_c[(int64_t)k * nl] : R(0));
    if (loc->dchi_c && k + 1 < nd) {   // the set-up derivatives of the next emit
      prefetch_l1(&loc->dchi_c[(int64_t)(k + 1) * nl]);
      prefetch_l1(&loc->deta_c[(int64_t)(k + 1) * nl]);
    }
    const R dB = (k >= nd - 2) ? R(planck_dT(T[k], lam)) : R(0);
    const R ldn = sm.len_dn[k], lup = (k + 1 < nd) ? sm.len_up[k + 1] : R(0);
#pragma unroll
    for (int s = 0; s < NS; ++s) {
#pragma unroll
      for (int x = 0; x < kNX; ++x) {
        R v = g[s][x];
        if (x == 0) v += bpl[s] * dB + sdn[s] * ldn + sup[s] * lup;
        if (MODE == 0) {
          if (act) rf[((int64_t)(s * kNX + x) * nd + k) * nl] = v;
        } else {   // modes 1 and 2: sum over the warp's wavelengths first
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          if ((threadIdx.x & 31u) == 0) atomicAdd(&sm.grad[x * loc->maxd + k], v);
        }
      }
    }
  }
};

// The work of one lane (atmosphere p, wavelength la0 + t; t the thread's
// place in its sub-block) of the response-function kernel: forward sweep
// with tape, reverse sweep, and the per-depth contraction.  Every thread of
// the block calls it (item: its sub-block holds a work item), because the
// two sweeps are separated by a block-wide barrier.
template <typename R, int MODE, bool UP>
__device__ __forceinline__ void rf_lane(const RfArgs& ra, const RfSmem<R>& sm, int nline, int p,
                                        int la0, int nl, int nd, int64_t doff, int t, bool item) {
  const LteArgs& args = ra.lte;
  // Every lane of a warp that holds at least one wavelength runs the sweep
  // (lanes past the spectrum repeat its last wavelength with zero seeds and
  // write nothing), so the per-depth gradient sums can use full-warp
  // shuffles before one shared atomic per warp.
  const bool act = item && la0 + t < nl;
  const int la = act ? la0 + t : nl - 1;
  const bool run = item && la0 + (t & ~31) < nl;   // the same in every lane of a warp
  int64_t loff = 0;
  double lam = 0.0, B0 = 0.0, B1 = 0.0;
  Local<R> loc;
  Tape<R> tp;
  R st[4] = {R(0), R(0), R(0), R(0)};
  bool pol = false, feaut = false;
  FeautTape<R> ftape;
  ScalarTape<R> stape;
  ScalarAdj<R> fadj;
  if (run) {
    loff = args.lam_off[p];
    lam = args.lambda[loff + la];
    const double dlc = lam * kQ_WING * (args.vmicro_char / kCLIGHT);
    loc.sm = &sm;
    loc.nline = nline;
    loc.maxd = args.maxd;
    loc.nl = nl;
    loc.inwin = 0u;
    for (int l = 0; l < nline; ++l) {
      loc.dlam[l] = R(lam - sm.lam0[l]);
      if (fabs(sm.lam0[l] - lam) <= dlc && sm.contrib[l]) loc.inwin |= 1u << l;
    }
    loc.chi_c = static_cast<const R*>(args.chi_c) + args.cont_off[p] + la;
    loc.eta_c = static_cast<const R*>(args.eta_c) + args.cont_off[p] + la;
    loc.dchi_c = ra.dT.dchi_c ? static_cast<const R*>(ra.dT.dchi_c) + args.cont_off[p] + la
                              : nullptr;
    loc.deta_c = ra.dT.deta_c ? static_cast<const R*>(ra.dT.deta_c) + args.cont_off[p] + la
                              : nullptr;

    auto qop = [&](int k, R* q) {
      if (k >= 1) {   // the continuum of the depth the next call takes
        prefetch_l1(&loc.chi_c[(int64_t)(k - 1) * nl]);
        prefetch_l1(&loc.eta_c[(int64_t)(k - 1) * nl]);
      }
      local_q<R, true, UP>(nline, sm.ld + k, args.maxd, sm.geo[k], loc.dlam, loc.inwin, sm.ncomp,
                       sm.cshift, sm.cweight, sm.cq, PYRH_MAX_COMPONENTS,
                       loc.chi_c[(int64_t)k * nl], loc.eta_c[(int64_t)k * nl], q, tp.z[k]);
    };
    B0 = planck(args.T[doff + nd - 2], lam);
    B1 = planck(args.T[doff + nd - 1], lam);
    delo_forward<R>(tp, sm.ds, nd, B0, B1, st, qop);
    // the reference's solver for this wavelength (formal.c:94-101,
    // 284-310): Feautrier where the wavelength is not angle dependent (no
    // line in window, or only unpolarizable lines in a static atmosphere),
    // scalar Bezier3 when none of the lines in window is polarizable,
    // DELO-Bezier3 otherwise (NO_STOKES: scalar where not Feautrier)
    for (int l = 0; l < nline; ++l) pol |= ((loc.inwin >> l) & 1u) && sm.polar[l];
    feaut = loc.inwin == 0u || (!pol && !args.moving);
    pol = pol && args.stokes_mode == PYRH_FULL_STOKES;
    if (feaut) {
      st[0] = feautrier_fwd<R>(tp, sm.ds, nd, B0, B1, ftape);
    } else if (!pol) {
      st[0] = scalar_bezier_fwd<R>(tp, sm.ds, nd, B0, B1, stape);
    }
    if (!pol) st[1] = st[2] = st[3] = R(0);
    R* out = static_cast<R*>(args.out) + 4 * loff;
    if (act)
#pragma unroll
      for (int s = 0; s < 4; ++s) out[(int64_t)s * nl + la] = st[s];
  }
  // Reached by every thread of the block: the forward sweeps of its
  // sub-blocks end together and their reverse sweeps start together, so
  // the resident warps run one sweep's instructions at a time.
  __syncthreads();
  if (!run) return;
  {
    const bool feaut_or_scalar = !pol;
    // adjoint of the unpolarized solvers for the Stokes I seed Ib
    auto unpol_vjp = [&](R Ib) {
      if (feaut) feautrier_vjp<R>(tp, sm.ds, nd, B0, B1, ftape, Ib, fadj);
      else scalar_bezier_vjp<R>(tp, sm.ds, nd, B0, B1, stape, Ib, fadj);
    };
    constexpr int NSG = MODE == 0 ? 4 : 1;
    const bool want_gf = MODE == 0 ? ra.rf_gf != nullptr : ra.grad_gf != nullptr;
    R gfacc[NSG * PYRH_MAX_LINES];
    if (want_gf)
      for (int e = 0; e < NSG * PYRH_MAX_LINES; ++e) gfacc[e] = R(0);
    Emit<R, MODE, UP> em;
    em.loc = &loc;
    em.tp = &tp;
    em.gf = want_gf ? gfacc : nullptr;
    em.T = args.T + doff;
    em.lam = lam;
    em.nd = nd;
    em.nl = nl;
    em.la = la;
    em.act = act;
    em.fa = feaut_or_scalar ? &fadj : nullptr;
    if (MODE == 0) {
      em.rf = static_cast<R*>(ra.rf) + 24 * args.cont_off[p] + la;
      const R one = pol ? R(1) : R(0);
      const R seed[4][4] = {{one, 0, 0, 0}, {0, one, 0, 0}, {0, 0, one, 0}, {0, 0, 0, one}};
      if (!pol) unpol_vjp(R(1));
      delo_reverse_stream<R, 4>(tp, sm.ds, nd, B0, B1, seed, em);
      if (want_gf && act) {
        R* o = static_cast<R*>(ra.rf_gf) + (int64_t)4 * nline * loff + la;
        for (int l = 0; l < nline; ++l)
          for (int s = 0; s < 4; ++s)
            o[(int64_t)(l * 4 + s) * nl] = gfacc[s * PYRH_MAX_LINES + l];
      }
    } else if (MODE == 2) {
      em.rf = nullptr;
      const R* dL = static_cast<const R*>(ra.weights) + 4 * loff;
      R seed[1][4];
#pragma unroll
      for (int s = 0; s < 4; ++s) seed[0][s] = act ? dL[(int64_t)s * nl + la] : R(0);
      if (!pol) {
        unpol_vjp(seed[0][0]);
#pragma unroll
        for (int s = 0; s < 4; ++s) seed[0][s] = R(0);
      }
      delo_reverse_stream<R, 1>(tp, sm.ds, nd, B0, B1, seed, em);
      if (want_gf) gf_block_sum(gfacc, nline, sm.gfs);
    } else {
      em.rf = nullptr;
      const R* obs = static_cast<const R*>(ra.obs) + 4 * loff;
      const R* wt = static_cast<const R*>(ra.weights) + 4 * loff;
      R seed[1][4];
      R c2 = 0;
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        const R wv = act ? wt[(int64_t)s * nl + la] : R(0);
        const R r = st[s] - obs[(int64_t)s * nl + la];
        seed[0][s] = R(2) * wv * r;
        c2 += wv * r * r;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) c2 += __shfl_xor_sync(0xffffffffu, c2, o);
      if ((threadIdx.x & 31u) == 0) atomicAdd(sm.chi2, c2);
      if (!pol) {
        unpol_vjp(seed[0][0]);
#pragma unroll
        for (int s = 0; s < 4; ++s) seed[0][s] = R(0);
      }
      delo_reverse_stream<R, 1>(tp, sm.ds, nd, B0, B1, seed, em);
      if (want_gf) gf_block_sum(gfacc, nline, sm.gfs);
    }
  }
}

template <typename R, int MODE>
__device__ __noinline__ void rf_lane_unpol(const RfArgs& ra, const RfSmem<R>& sm, int nline, int p,
                                           int la0, int nl, int nd, int64_t doff, int t,
                                           bool item) {
  rf_lane<R, MODE, true>(ra, sm, nline, p, la0, nl, nd, doff, t, item);
}

// A block holds ra.sub sub-blocks of blockDim.x / ra.sub threads, each
// with its own work item (atmosphere, tile of wavelengths) and its own
// shared tables, so that one block fills the SM and the barrier between the
// forward and reverse sweeps aligns the sweeps of all resident warps.
// Single-seed modes in FP32 are capped at 128 registers (512 threads per
// SM): measured 31.5 ms against 35.8 ms uncapped for the gradient of 4096
// atmospheres x 224 wavelengths, and 32.4 ms at 384 threads.  The four-seed
// full response functions at 168 registers (384 threads; 120 bytes of
// spills): 59.2 ms against 62.2 ms at 245 registers (256 threads) and 61.6 ms
// at 128 registers (512 threads, 900 bytes of spills).
template <typename R, int MODE>
constexpr int rf_max_threads() {
  return ::pyrh::rf_max_threads(sizeof(R) == 4 ? PYRH_FP32 : PYRH_FP64, MODE);
}

template <typename R, int MODE>
__global__ void __launch_bounds__(rf_max_threads<R, MODE>(), 1)
lte_rf_kernel(RfArgs ra) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const LteArgs& args = ra.lte;
  const int nline = args.nline < PYRH_MAX_LINES ? args.nline : PYRH_MAX_LINES;
  const int G = ra.sub;
  const int BL = blockDim.x / G;
  const int g = threadIdx.x / BL, t = threadIdx.x - g * BL;
  RfSmem<R> sm;
  const size_t per = rf_smem_t<R>(nline, args.maxd, nullptr, nullptr);
  rf_smem_t<R>(nline, args.maxd, &sm, smem_raw + per * g);

  for (int i = t; i < nline * PYRH_MAX_COMPONENTS; i += BL) {
    const int l = i / PYRH_MAX_COMPONENTS, c = i % PYRH_MAX_COMPONENTS;
    const pyrh_line& L = args.lines[l];
    sm.cshift[i] = R(L.comp_shift[c]);
    sm.cweight[i] = R(L.comp_strength[c]);
    sm.cq[i] = L.comp_q[c];
  }
  for (int l = t; l < nline; l += BL) {
    const pyrh_line& L = args.lines[l];
    const int nc = L.ncomp < 0 ? 0 : (L.ncomp > PYRH_MAX_COMPONENTS ? PYRH_MAX_COMPONENTS : L.ncomp);
    sm.ncomp[l] = L.polarizable ? nc : kArmstrong;
    sm.polar[l] = L.polarizable;
    sm.contrib[l] = L.contributes;
    sm.lam0[l] = L.lambda0;
  }

  const double muz = args.mu, imu = 1.0 / args.mu;
  const int64_t total = (int64_t)args.natm * args.tiles;
  // every barrier below is reached by every thread: the loop's trip count
  // is the same across the block, and sub-blocks without a work item skip
  // only the work between barriers
  for (int64_t w0 = (int64_t)blockIdx.x * G; w0 < total; w0 += (int64_t)gridDim.x * G) {
    const int64_t w = w0 + g;
    int p = 0, nl = 0, la0 = 0, nd = 0;
    int64_t doff = 0;
    bool item = w < total;
    if (item) {
      p = (int)(w / args.tiles);
      nl = args.nlam[p];
      la0 = (int)(w % args.tiles) * BL;
      nd = args.ndep[p];
      doff = args.depth_off[p];
      item = la0 < nl && nd >= 3 && nd <= args.maxd;
    }
    __syncthreads();  // shared tables of the previous work item are consumed

    // ---- per-depth and per-(line, depth) values with derivatives ----
    if (item) {
      for (int k = t; k < nd; k += BL) {
        const int64_t d = doff + k;
        sm.ds[k] = (k >= 1) ? R(fabs(args.height[d] - args.height[d - 1]) * imu) : R(0);
        sm.geo[k] = geometry_d<R>(R(args.gamma_B[d]), R(args.chi_B[d]), R(muz));
        sm.len_up[k] = (k >= 1 && ra.dT.dlen_up) ? R(ra.dT.dlen_up[d] * imu) : R(0);
        sm.len_dn[k] = (k >= 1 && ra.dT.dlen_dn) ? R(ra.dT.dlen_dn[d] * imu) : R(0);
        if (MODE != 0)
          for (int x = 0; x < kNX; ++x) sm.grad[x * args.maxd + k] = R(0);
      }
      if (MODE == 1 && t == 0) sm.chi2[0] = R(0);
      if (MODE != 0)
        for (int l = t; l < nline; l += BL) sm.gfs[l] = R(0);
      for (int i = t; i < nline * nd; i += BL) {
        const int l = i / nd, k = i % nd;
        const int64_t d = doff + k;
        const pyrh_line& L = args.lines[l];
        const LineConstD c = {L.lambda0, L.Ei, L.gi, L.Aji, L.Bji, L.Bij, L.Grad, L.GStark,
                              L.GvdWaals, L.cross, L.alpha, L.isotope_frac, L.hyperfine_frac,
                              L.weight, L.vdwaals};
        const double* dp = ra.dT.dline_pops;
        sm.ld[l * args.maxd + k] = line_depth<R>(
            c, R(args.T[d]), R(args.vlos[d]), R(args.vturb[d]), R(args.B[d]), R(args.ne[d]),
            R(args.nHtot[d]), R(args.np[d]),
            R(args.line_pops[((int64_t)l * 2 + 0) * args.total_depth + d]),
            R(args.line_pops[((int64_t)l * 2 + 1) * args.total_depth + d]), R(muz),
            args.moving != 0, dp ? R(dp[((int64_t)l * 2 + 0) * args.total_depth + d]) : R(0),
            dp ? R(dp[((int64_t)l * 2 + 1) * args.total_depth + d]) : R(0),
            ra.dT.dnp ? R(ra.dT.dnp[d]) : R(0));
      }
    }
    __syncthreads();

    // lines that are not polarizable take an out-of-line copy of the lane's
    // work that has their branch, the others a copy without it; the line
    // list is the same for every atmosphere, so the choice is the same in
    // every thread of the grid (and both copies hold the sweep barrier)
    bool any_unpol = false;
    for (int l = 0; l < nline; ++l) any_unpol |= sm.contrib[l] && !sm.polar[l];
    if (any_unpol)
      rf_lane_unpol<R, MODE>(ra, sm, nline, p, la0, nl, nd, doff, t, item);
    else
      rf_lane<R, MODE, false>(ra, sm, nline, p, la0, nl, nd, doff, t, item);
    if (MODE != 0) {
      __syncthreads();
      if (item) {
        R* grad = static_cast<R*>(ra.grad);
        for (int i = t; i < kNX * nd; i += BL) {
          const int x = i / nd, k = i % nd;
          atomicAdd(&grad[(int64_t)x * args.total_depth + doff + k], sm.grad[x * args.maxd + k]);
        }
        if (MODE == 1 && t == 0) atomicAdd(static_cast<R*>(ra.chi2) + p, sm.chi2[0]);
        if (ra.grad_gf)
          for (int l = t; l < nline; l += BL)
            atomicAdd(static_cast<R*>(ra.grad_gf) + (int64_t)p * nline + l, sm.gfs[l]);
      }
    }
  }
}

// block: threads of one sub-block (the tile width); smem: the shared tables
// of one sub-block.  The launch has a.sub sub-blocks per block.
template <typename R, int MODE>
cudaError_t launch_mode(const RfArgs& a, int block, int grid, size_t smem, cudaStream_t st) {
  if (a.sub < 1 || block * a.sub > rf_max_threads<R, MODE>()) return cudaErrorInvalidValue;
  auto k = lte_rf_kernel<R, MODE>;
  const size_t total = smem * a.sub;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)total);
  if (e != cudaSuccess) return e;
  k<<<grid, block * a.sub, total, st>>>(a);
  return cudaGetLastError();
}

}  // namespace

template <typename R>
size_t rf_smem_precision(int nline, int maxd) {
  return rf_smem_t<R>(nline, maxd, nullptr, nullptr);
}

}  // namespace pyrh
