// ltepops.cu -- LTE ionisation-stage populations, the stage densities and
// partition functions of Kurucz lines, and the electron density, on the
// device (one thread per depth point; the points are independent).
//
// Reference routines restated here (file:line in the reference tree):
//   LTEpops_elem   rh/ltepops.c:116-166  (Saha equation stage by stage from
//                                         the log partition functions)
//   rlk_opacity    rh/kurucz.c:662-677   (n[stage] and ln U of a line)
//   Solve_ne       rh/solvene.c:55-141   (Newton iteration on n_e with the
//                                         H- term; from hydrogen's
//                                         ionisation when from scratch)
//   getfjk         rh/solvene.c:145-198  (stage fractions and their n_e
//                                         derivatives, LTE branch)
//   Linear, Hunt   rh/linear.c:22-51, rh/hunt.c (ln U at T, held at the
//                                         ends of the grid)
// Every expression keeps the reference's operation order and constants
// (rh/constant.h), so the results agree with it to rounding.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <vector>

#include "../../include/pyrh_gb300.h"

namespace pyrh {
void set_error(const char* fmt, ...);
void set_launches(int n);
}

namespace {

constexpr double kH = 6.6260755E-34;
constexpr double kK = 1.380658E-23;
constexpr double kMe = 9.1093897E-31;
constexpr double kPi = 3.14159265358979;
constexpr double kEV = 1.60217733E-19;
// (HPLANCK / (2 PI M_ELECTRON)) (HPLANCK / KBOLTZMANN)
constexpr double kC1 = (kH / (2.0 * kPi * kMe)) * (kH / kK);
constexpr double kMaxElectronError = 1.0E-2;   // solvene.c:37
constexpr int kMaxElectronIter = 10;           // solvene.c:38
constexpr int kMaxSel = 128;                   // elements or lines per launch

struct DevTables {
  int nelem, npf;
  const double *Tpf, *abund, *lnpf, *ionpot;
  const int32_t *nstage, *stage_off;
};

// Linear() at one temperature: the bracket and weight, shared by every row
// of the tables (all rows are on the same grid).
struct PfAt {
  int j;        // bracket (or the end row when clamped)
  int clamped;  // 1: held at the end value y[j]
  double fx;
};

__device__ __forceinline__ PfAt pf_at(const double* t, int n, double x) {
  PfAt a;
  if (x <= t[0]) { a.j = 0; a.clamped = 1; a.fx = 0.0; return a; }
  if (x >= t[n - 1]) { a.j = n - 1; a.clamped = 1; a.fx = 0.0; return a; }
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (hi + lo) >> 1;
    if (x >= t[mid]) lo = mid;
    else hi = mid;
  }
  a.j = lo;
  a.clamped = 0;
  a.fx = (t[lo + 1] - x) / (t[lo + 1] - t[lo]);
  return a;
}

__device__ __forceinline__ double pf_eval(const double* y, const PfAt& a) {
  if (a.clamped) return y[a.j];
  return a.fx * y[a.j] + (1 - a.fx) * y[a.j + 1];
}

// LTEpops_elem at one point: the element's stage populations into n[].
__device__ __forceinline__ void stage_pops(const DevTables& t, int e, const PfAt& at, double T,
                                           double ne, double nHtot,
                                           double n[PYRH_PF_MAX_STAGES]) {
  const int ns = t.nstage[e];
  const double* lnpf = t.lnpf + (int64_t)t.stage_off[e] * t.npf;
  const double* ion = t.ionpot + t.stage_off[e];
  const double CT_ne = 2.0 * pow(kC1 / T, -1.5) / ne;
  double sum = 1.0;
  n[0] = 1.0;
  double Uk = pf_eval(lnpf, at);
#pragma unroll
  for (int i = 1; i < PYRH_PF_MAX_STAGES; ++i) {
    if (i < ns) {
      const double Ukp1 = pf_eval(lnpf + (int64_t)i * t.npf, at);
      n[i] = n[i - 1] * CT_ne * exp(Ukp1 - Uk - ion[i - 1] / (kK * T));
      sum += n[i];
      Uk = Ukp1;
    } else {
      n[i] = 0.0;
    }
  }
  n[0] = t.abund[e] * nHtot / sum;
#pragma unroll
  for (int i = 1; i < PYRH_PF_MAX_STAGES; ++i)
    if (i < ns) n[i] *= n[0];
}

struct SelArgs {
  int n;
  int elem[kMaxSel], stage[kMaxSel];
  int64_t row[kMaxSel];   // first output row of each selection
};

__global__ void stage_pops_kernel(DevTables t, int64_t npoint, const double* T, const double* ne,
                                  const double* nHtot, SelArgs s, double* pops) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= npoint) return;
  const double Tk = T[k];
  const PfAt at = pf_at(t.Tpf, t.npf, Tk);
  for (int m = 0; m < s.n; ++m) {
    double n[PYRH_PF_MAX_STAGES];
    const int e = s.elem[m];
    stage_pops(t, e, at, Tk, ne[k], nHtot[k], n);
    const int ns = t.nstage[e];
#pragma unroll
    for (int i = 0; i < PYRH_PF_MAX_STAGES; ++i)
      if (i < ns) pops[(s.row[m] + i) * npoint + k] = n[i];
  }
}

__global__ void line_pops_kernel(DevTables t, int64_t npoint, const double* T, const double* ne,
                                 const double* nHtot, SelArgs s, double* line_pops) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= npoint) return;
  const double Tk = T[k];
  const PfAt at = pf_at(t.Tpf, t.npf, Tk);
  for (int m = 0; m < s.n; ++m) {
    double n[PYRH_PF_MAX_STAGES];
    const int e = s.elem[m], st = s.stage[m];
    stage_pops(t, e, at, Tk, ne[k], nHtot[k], n);
    double nst = n[0];
#pragma unroll
    for (int i = 1; i < PYRH_PF_MAX_STAGES; ++i)
      if (i == st) nst = n[i];
    const double lnU = pf_eval(t.lnpf + (int64_t)(t.stage_off[e] + st) * t.npf, at);
    line_pops[(s.row[m] + 0) * npoint + k] = nst;
    line_pops[(s.row[m] + 1) * npoint + k] = lnU;
  }
}

// The factor of getfjk's stage recursion that does not depend on n_e,
// exp(ln U_{j+1} - ln U_j - chi_j / kT), for every element and stage j >= 1
// at one point: row stage_off[e] + j of E.  Solve_ne's iterations reuse it.
constexpr int kMaxRows = PYRH_NELEM * PYRH_PF_MAX_STAGES;

__device__ __forceinline__ void stage_factors(const DevTables& t, const PfAt& at, double T,
                                              double* E) {
  for (int e = 0; e < t.nelem; ++e) {
    const int ns = t.nstage[e], off = t.stage_off[e];
    const double* lnpf = t.lnpf + (int64_t)off * t.npf;
    const double* ion = t.ionpot + off;
    double Uk = pf_eval(lnpf, at);
    for (int j = 1; j < ns; ++j) {
      const double Ukp1 = pf_eval(lnpf + (int64_t)j * t.npf, at);
      E[off + j] = exp(Ukp1 - Uk - ion[j - 1] / (kK * T));
      Uk = Ukp1;
    }
  }
}

// getfjk (LTE branch) for element e at n_e = ne: the stage fractions and
// their n_e derivatives, accumulated straight into Solve_ne's error and sum.
__device__ __forceinline__ void add_element(const DevTables& t, int e, const double* E,
                                            double ne, double CT_ne_ref, double& error,
                                            double& sum, double PhiHmin) {
  const int ns = t.nstage[e], off = t.stage_off[e];
  const double CT_ne = CT_ne_ref / ne;
  double f[PYRH_PF_MAX_STAGES], df[PYRH_PF_MAX_STAGES];
  double sum1 = 1.0, sum2 = 0.0;
  f[0] = 1.0;
  df[0] = 0.0;
#pragma unroll
  for (int j = 1; j < PYRH_PF_MAX_STAGES; ++j) {
    if (j < ns) {
      f[j] = f[j - 1] * CT_ne * E[off + j];
      df[j] = -j * f[j] / ne;
      sum1 += f[j];
      sum2 += df[j];
    }
  }
#pragma unroll
  for (int j = 0; j < PYRH_PF_MAX_STAGES; ++j) {
    if (j < ns) {
      f[j] /= sum1;
      df[j] = (df[j] - f[j] * sum2) / sum1;
    }
  }
  if (e == 0) {   // H- (solvene.c:103-108)
    error += ne * f[0] * PhiHmin;
    sum -= (f[0] + ne * df[0]) * PhiHmin;
  }
  const double ab = t.abund[e];
#pragma unroll
  for (int j = 1; j < PYRH_PF_MAX_STAGES; ++j) {
    if (j < ns) {
      const double akj = ab * j;
      error -= akj * f[j];
      sum += akj * df[j];
    }
  }
}

__global__ void solve_ne_kernel(DevTables t, int64_t npoint, const double* T,
                                const double* nHtot, double* ne, int fromscratch,
                                int32_t* niter_out) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= npoint) return;
  const double Tk = T[k], nH = nHtot[k];
  const PfAt at = pf_at(t.Tpf, t.npf, Tk);
  double ne_old;
  if (fromscratch) {
    // ionisation of hydrogen alone (H in LTE), with hydrogen's neutral
    // partition function (Solve_ne, solvene.c:80-86) or with U = 1 (get_ne,
    // rh/rhf1d/pyrh_background.c:485-492, the start of the hydrostatic
    // equilibrium's electron densities)
    const double Uk =
        fromscratch == 2 ? 0.0 : pf_eval(t.lnpf + (int64_t)t.stage_off[0] * t.npf, at);
    const double PhiH = 0.5 * pow(kC1 / Tk, 1.5) * exp(Uk + t.ionpot[t.stage_off[0]] / (kK * Tk));
    ne_old = (sqrt(1.0 + 4.0 * nH * PhiH) - 1.0) / (2.0 * PhiH);
  } else {
    ne_old = ne[k];
  }
  const double CT_ne_ref = 2.0 * pow(kC1 / Tk, -1.5);
  const double PhiHmin = 0.25 * pow(kC1 / Tk, 1.5) * exp(0.754 * kEV / (kK * Tk));
  double E[kMaxRows];
  stage_factors(t, at, Tk, E);
  double ne_new = ne_old, dne = 0.0;
  int niter = 0;
  while (niter < kMaxElectronIter) {
    double error = ne_old / nH;
    double sum = 0.0;
    for (int e = 0; e < t.nelem; ++e) add_element(t, e, E, ne_old, CT_ne_ref, error, sum, PhiHmin);
    ne_new = ne_old - nH * error / (1.0 - nH * sum);
    dne = fabs((ne_new - ne_old) / ne_old);
    ne_old = ne_new;
    if (dne <= kMaxElectronError) break;
    niter++;
  }
  ne[k] = ne_new;
  if (niter_out) niter_out[k] = dne > kMaxElectronError ? -1 : niter + 1;
}

// Solve_ne with the work of one point spread over a warp, for batches too
// small to fill the GPU with one point per thread (the hydrostatic
// equilibrium's layers): lane l takes elements l, l + 32, l + 64, l + 96 and
// keeps their stage factors in registers; each Newton step adds the lanes'
// error and derivative terms by a butterfly, so every lane holds the same
// totals and the same n_e.  The terms are those of the reference; their
// summation order differs, and the divisions by n_e and by each element's
// stage sum are multiplications by the reciprocal (FP64 divisions dominate
// the work on this part's FP64 pipe): the results agree with the
// reference's to rounding.
constexpr int kWarpElems = (PYRH_NELEM + 31) / 32;

__device__ __forceinline__ void add_element_r(const DevTables& t, int e,
                                              const double (&Er)[PYRH_PF_MAX_STAGES], double ne,
                                              double inv_ne, double CT_ne_ref, double& error,
                                              double& sum, double PhiHmin) {
  const int ns = t.nstage[e];
  const double CT_ne = CT_ne_ref * inv_ne;
  double f[PYRH_PF_MAX_STAGES], df[PYRH_PF_MAX_STAGES];
  double sum1 = 1.0, sum2 = 0.0;
  f[0] = 1.0;
  df[0] = 0.0;
#pragma unroll
  for (int j = 1; j < PYRH_PF_MAX_STAGES; ++j) {
    if (j < ns) {
      f[j] = f[j - 1] * CT_ne * Er[j];
      df[j] = -j * f[j] * inv_ne;
      sum1 += f[j];
      sum2 += df[j];
    }
  }
  const double inv_sum1 = 1.0 / sum1;
#pragma unroll
  for (int j = 0; j < PYRH_PF_MAX_STAGES; ++j) {
    if (j < ns) {
      f[j] *= inv_sum1;
      df[j] = (df[j] - f[j] * sum2) * inv_sum1;
    }
  }
  if (e == 0) {
    error += ne * f[0] * PhiHmin;
    sum -= (f[0] + ne * df[0]) * PhiHmin;
  }
  const double ab = t.abund[e];
#pragma unroll
  for (int j = 1; j < PYRH_PF_MAX_STAGES; ++j) {
    if (j < ns) {
      const double akj = ab * j;
      error -= akj * f[j];
      sum += akj * df[j];
    }
  }
}

__global__ void solve_ne_warp_kernel(DevTables t, int64_t npoint, const double* T,
                                     const double* nHtot, double* ne, int fromscratch,
                                     int32_t* niter_out) {
  const int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (k >= npoint) return;   // k is the same for the whole warp
  const double Tk = T[k], nH = nHtot[k];
  const PfAt at = pf_at(t.Tpf, t.npf, Tk);
  double ne_old;
  if (fromscratch) {
    const double Uk =
        fromscratch == 2 ? 0.0 : pf_eval(t.lnpf + (int64_t)t.stage_off[0] * t.npf, at);
    const double PhiH = 0.5 * pow(kC1 / Tk, 1.5) * exp(Uk + t.ionpot[t.stage_off[0]] / (kK * Tk));
    ne_old = (sqrt(1.0 + 4.0 * nH * PhiH) - 1.0) / (2.0 * PhiH);
  } else {
    ne_old = ne[k];
  }
  const double CT_ne_ref = 2.0 * pow(kC1 / Tk, -1.5);
  const double PhiHmin = 0.25 * pow(kC1 / Tk, 1.5) * exp(0.754 * kEV / (kK * Tk));
  double E[kWarpElems][PYRH_PF_MAX_STAGES];
#pragma unroll
  for (int q = 0; q < kWarpElems; ++q) {
    const int e = lane + 32 * q;
#pragma unroll
    for (int j = 0; j < PYRH_PF_MAX_STAGES; ++j) E[q][j] = 0.0;
    if (e >= t.nelem) continue;
    const int ns = t.nstage[e], off = t.stage_off[e];
    const double* lnpf = t.lnpf + (int64_t)off * t.npf;
    double Uk = pf_eval(lnpf, at);
#pragma unroll
    for (int j = 1; j < PYRH_PF_MAX_STAGES; ++j) {
      if (j < ns) {
        const double Ukp1 = pf_eval(lnpf + (int64_t)j * t.npf, at);
        E[q][j] = exp(Ukp1 - Uk - t.ionpot[off + j - 1] / (kK * Tk));
        Uk = Ukp1;
      }
    }
  }
  double ne_new = ne_old, dne = 0.0;
  int niter = 0;
  while (niter < kMaxElectronIter) {
    double err = 0.0, sm = 0.0;
    const double inv_ne = 1.0 / ne_old;
#pragma unroll
    for (int q = 0; q < kWarpElems; ++q) {
      const int e = lane + 32 * q;
      if (e < t.nelem) add_element_r(t, e, E[q], ne_old, inv_ne, CT_ne_ref, err, sm, PhiHmin);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      err += __shfl_xor_sync(0xffffffffu, err, o);
      sm += __shfl_xor_sync(0xffffffffu, sm, o);
    }
    const double error = ne_old / nH + err;
    ne_new = ne_old - nH * error / (1.0 - nH * sm);
    dne = fabs((ne_new - ne_old) / ne_old);
    ne_old = ne_new;
    if (dne <= kMaxElectronError) break;
    niter++;
  }
  if (lane == 0) {
    ne[k] = ne_new;
    if (niter_out) niter_out[k] = dne > kMaxElectronError ? -1 : niter + 1;
  }
}

pyrh_status fail(pyrh_status s, const char* msg) {
  pyrh::set_error("%s", msg);
  return s;
}

// Checks the tables and copies their per-element stage counts and offsets
// to the host (one small synchronous copy on the stream).
pyrh_status load_tables(const pyrh_elem_tables* tab, cudaStream_t st, DevTables& d,
                        std::vector<int32_t>& nstage, std::vector<int32_t>& off) {
  if (!tab || !tab->Tpf || !tab->abund || !tab->nstage || !tab->stage_off || !tab->lnpf ||
      !tab->ionpot)
    return fail(PYRH_ERR_ARG, "element tables: NULL pointer");
  if (tab->nelem != PYRH_NELEM) return fail(PYRH_ERR_ARG, "element tables: nelem != PYRH_NELEM");
  if (tab->npf < 2) return fail(PYRH_ERR_ARG, "element tables: fewer than two temperatures");
  nstage.assign(PYRH_NELEM, 0);
  off.assign(PYRH_NELEM, 0);
  cudaError_t e = cudaMemcpyAsync(nstage.data(), tab->nstage, sizeof(int32_t) * PYRH_NELEM,
                                  cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(off.data(), tab->stage_off, sizeof(int32_t) * PYRH_NELEM,
                        cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    pyrh::set_error("element tables: %s", cudaGetErrorString(e));
    return PYRH_ERR_CUDA;
  }
  int64_t rows = 0;
  for (int n = 0; n < PYRH_NELEM; ++n) {
    if (nstage[n] < 1 || nstage[n] > PYRH_PF_MAX_STAGES || off[n] != rows)
      return fail(PYRH_ERR_ARG, "element tables: bad stage count or offset");
    rows += nstage[n];
  }
  d.nelem = tab->nelem;
  d.npf = tab->npf;
  d.Tpf = tab->Tpf;
  d.abund = tab->abund;
  d.lnpf = tab->lnpf;
  d.ionpot = tab->ionpot;
  d.nstage = tab->nstage;
  d.stage_off = tab->stage_off;
  return PYRH_OK;
}

pyrh_status finish(cudaError_t e, int launches) {
  pyrh::set_launches(launches);
  if (e != cudaSuccess) {
    pyrh::set_error("launch: %s", cudaGetErrorString(e));
    return PYRH_ERR_CUDA;
  }
  return PYRH_OK;
}

constexpr int kThreads = 128;

unsigned grid_for(int64_t npoint) { return (unsigned)((npoint + kThreads - 1) / kThreads); }

}  // namespace

extern "C" pyrh_status pyrh_lte_stage_pops(const pyrh_elem_tables* tables, int64_t npoint,
                                           const double* T, const double* ne,
                                           const double* nHtot, int32_t nsel, const int32_t* sel,
                                           double* pops, void* stream) {
  pyrh::set_launches(0);
  if (npoint < 0 || nsel < 0 || (nsel > 0 && !sel)) return fail(PYRH_ERR_ARG, "stage pops: bad sizes");
  if (npoint == 0 || nsel == 0) return PYRH_OK;
  if (!T || !ne || !nHtot || !pops) return fail(PYRH_ERR_ARG, "stage pops: NULL array");
  cudaStream_t st = (cudaStream_t)stream;
  DevTables d;
  std::vector<int32_t> ns, off;
  pyrh_status s = load_tables(tables, st, d, ns, off);
  if (s != PYRH_OK) return s;
  int launches = 0;
  int64_t row = 0;
  cudaError_t e = cudaSuccess;
  for (int m0 = 0; m0 < nsel && e == cudaSuccess; m0 += kMaxSel) {
    SelArgs a;
    a.n = nsel - m0 < kMaxSel ? nsel - m0 : kMaxSel;
    for (int m = 0; m < a.n; ++m) {
      const int el = sel[m0 + m];
      if (el < 0 || el >= PYRH_NELEM) return fail(PYRH_ERR_ARG, "stage pops: element index");
      a.elem[m] = el;
      a.stage[m] = 0;
      a.row[m] = row;
      row += ns[el];
    }
    stage_pops_kernel<<<grid_for(npoint), kThreads, 0, st>>>(d, npoint, T, ne, nHtot, a, pops);
    e = cudaGetLastError();
    ++launches;
  }
  return finish(e, launches);
}

extern "C" pyrh_status pyrh_line_pops(const pyrh_elem_tables* tables, int64_t npoint,
                                      const double* T, const double* ne, const double* nHtot,
                                      int32_t nline, const int32_t* elem, const int32_t* stage,
                                      double* line_pops, void* stream) {
  pyrh::set_launches(0);
  if (npoint < 0 || nline < 0 || (nline > 0 && (!elem || !stage)))
    return fail(PYRH_ERR_ARG, "line pops: bad sizes");
  if (npoint == 0 || nline == 0) return PYRH_OK;
  if (!T || !ne || !nHtot || !line_pops) return fail(PYRH_ERR_ARG, "line pops: NULL array");
  cudaStream_t st = (cudaStream_t)stream;
  DevTables d;
  std::vector<int32_t> ns, off;
  pyrh_status s = load_tables(tables, st, d, ns, off);
  if (s != PYRH_OK) return s;
  int launches = 0;
  cudaError_t e = cudaSuccess;
  for (int m0 = 0; m0 < nline && e == cudaSuccess; m0 += kMaxSel) {
    SelArgs a;
    a.n = nline - m0 < kMaxSel ? nline - m0 : kMaxSel;
    for (int m = 0; m < a.n; ++m) {
      const int el = elem[m0 + m], stg = stage[m0 + m];
      if (el < 0 || el >= PYRH_NELEM) return fail(PYRH_ERR_ARG, "line pops: element index");
      if (stg < 0 || stg >= ns[el]) return fail(PYRH_ERR_ARG, "line pops: stage beyond the element's");
      a.elem[m] = el;
      a.stage[m] = stg;
      a.row[m] = 2LL * (m0 + m);
    }
    line_pops_kernel<<<grid_for(npoint), kThreads, 0, st>>>(d, npoint, T, ne, nHtot, a,
                                                             line_pops);
    e = cudaGetLastError();
    ++launches;
  }
  return finish(e, launches);
}

namespace pyrh {
// pyrh_solve_ne's iteration with a warp per point (see solve_ne_warp_kernel);
// launches one kernel on the stream.
pyrh_status solve_ne_warp(const pyrh_elem_tables* tables, int64_t npoint, const double* T,
                          const double* nHtot, double* ne, int32_t fromscratch, int32_t* niter,
                          cudaStream_t st) {
  if (npoint < 0 || npoint > ((int64_t)1 << 26)) return fail(PYRH_ERR_ARG, "solve ne: npoint");
  if (npoint == 0) return PYRH_OK;
  if (!T || !nHtot || !ne) return fail(PYRH_ERR_ARG, "solve ne: NULL array");
  if (fromscratch < 0 || fromscratch > 2) return fail(PYRH_ERR_ARG, "solve ne: fromscratch not 0, 1 or 2");
  DevTables d;
  std::vector<int32_t> ns, off;
  pyrh_status s = load_tables(tables, st, d, ns, off);
  if (s != PYRH_OK) return s;
  solve_ne_warp_kernel<<<(unsigned)((npoint * 32 + kThreads - 1) / kThreads), kThreads, 0, st>>>(
      d, npoint, T, nHtot, ne, fromscratch, niter);
  return finish(cudaGetLastError(), 1);
}
}  // namespace pyrh

extern "C" pyrh_status pyrh_solve_ne(const pyrh_elem_tables* tables, int64_t npoint,
                                     const double* T, const double* nHtot, double* ne,
                                     int32_t fromscratch, int32_t* niter, void* stream) {
  pyrh::set_launches(0);
  if (npoint < 0) return fail(PYRH_ERR_ARG, "solve ne: npoint < 0");
  if (npoint == 0) return PYRH_OK;
  if (!T || !nHtot || !ne) return fail(PYRH_ERR_ARG, "solve ne: NULL array");
  if (fromscratch < 0 || fromscratch > 2) return fail(PYRH_ERR_ARG, "solve ne: fromscratch not 0, 1 or 2");
  cudaStream_t st = (cudaStream_t)stream;
  DevTables d;
  std::vector<int32_t> ns, off;
  pyrh_status s = load_tables(tables, st, d, ns, off);
  if (s != PYRH_OK) return s;
  solve_ne_kernel<<<grid_for(npoint), kThreads, 0, st>>>(d, npoint, T, nHtot, ne,
                                                          fromscratch, niter);
  return finish(cudaGetLastError(), 1);
}
