// chem.cu -- chemical equilibrium of the molecules, on the device (one thread
// per depth point; the points are independent).
//
// Reference routines restated here (file:line in the reference tree):
//   ChemicalEquilibrium  rh/chemequil.c:107-390 (Newton iteration on the
//                        nuclei's number conservation and the molecules'
//                        Saha equations, H- in the hydrogen balance; no Ng
//                        acceleration, NG_CHEM_ORDER 0; stopping on the
//                        largest relative change, MaxChange rh/maxchange.c)
//   equilconstant        rh/chemequil.c:456-535 (the four fit types)
//   getfjk               rh/solvene.c:145-198 (neutral fraction of a nucleus
//                        without an atom model)
//   SolveLinearEq        rh/ludcmp.c:36-177 (lu_device.cuh)
// Every expression keeps the reference's operation order and constants
// (rh/constant.h).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "../../include/pyrh_gb300.h"
#include "lu_device.cuh"

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
constexpr double kTHETA0 = 5.03974756E+03;
constexpr double kCM_TO_M = 1.0E-02;
constexpr double kERG_TO_JOULE = 1.0E-07;
constexpr double kLG10 = 2.30258509299404568402;
constexpr double kCI = (kH / (2.0 * kPi * kMe)) * (kH / kK);
constexpr int kMaxIter = 10;          // N_MAX_CHEM_ITER, rh/background.h:18
constexpr double kIterLimit = 1.0E-3; // CHEM_ITER_LIMIT, rh/background.h:19
constexpr int kMaxEq = PYRH_CHEM_MAX_NUCLEI + PYRH_CHEM_MAX_MOLECULES;

struct ChemArgs {
  int nmol, nnuc;
  pyrh_molecule mol[PYRH_CHEM_MAX_MOLECULES];
  int nuc_elem[PYRH_CHEM_MAX_NUCLEI];              // element index of each nucleus
  const double* fn0[PYRH_CHEM_MAX_NUCLEI];         // model neutral fraction or NULL
  int nucl_index[PYRH_CHEM_MAX_MOLECULES][PYRH_MOL_MAX_ELEMENTS];
  // element tables (getfjk)
  int npf;
  const double *Tpf, *abund, *lnpf, *ionpot;
  const int32_t *nstage, *stage_off;
};

__device__ double pow10r(double x) { return exp(kLG10 * (x)); }

// equilconstant (rh/chemequil.c:456-535)
__device__ double equilconstant(const pyrh_molecule& m, double T) {
  double kT, t, eqc = 0.0, theta, cgs_to_SI = 1.0;
  int mk;
  if (T < m.tmin || T > m.tmax) return eqc;
  switch (m.fit) {
    case PYRH_FIT_KURUCZ_70:
      kT = kK * T;
      mk = m.nnuclei - 1 - m.charge;
      eqc = m.eqc_coef[0];
      for (int i = 1; i < m.neqc; i++) eqc = eqc * T + m.eqc_coef[i];
      eqc = exp(m.ediss / kT + eqc - 1.5 * mk * log(T));
      cgs_to_SI = pow(kCM_TO_M * kCM_TO_M * kCM_TO_M, (double)mk);
      break;
    case PYRH_FIT_KURUCZ_85:
      t = T * 1.0E-4;
      kT = kK * T;
      mk = m.nnuclei - 1 - m.charge;
      eqc = m.eqc_coef[0];
      for (int i = 1; i < m.neqc; i++) eqc = eqc * t + m.eqc_coef[i];
      eqc = exp(m.ediss / kT + eqc - 1.5 * mk * log(T));
      cgs_to_SI = pow(kCM_TO_M * kCM_TO_M * kCM_TO_M, (double)mk);
      break;
    case PYRH_FIT_IRWIN_81:       // Sauval & Tatum for the constant
    case PYRH_FIT_SAUVAL_TATUM_84:
      theta = kTHETA0 / T;
      t = log10(theta);
      kT = kK * T;
      eqc = m.eqc_coef[0];
      for (int i = 1; i < m.neqc; i++) eqc = eqc * t + m.eqc_coef[i];
      eqc = pow10r((m.ediss / kEV) * theta - eqc) * kT;
      cgs_to_SI = 1.0;
      break;
    case PYRH_FIT_TSUJI_73:
      theta = kTHETA0 / T;
      kT = kK * T;
      eqc = m.eqc_coef[0];
      for (int i = 1; i < m.neqc; i++) eqc = eqc * theta + m.eqc_coef[i];
      eqc = (kT * kT) * pow10r(-eqc);
      cgs_to_SI = pow((kCM_TO_M * kCM_TO_M * kCM_TO_M) / kERG_TO_JOULE, (double)(m.nnuclei - 1));
      break;
    default:
      return 0.0;
  }
  return eqc * cgs_to_SI;
}

// Linear() of ln U at T (rh/linear.c:22-51)
__device__ double pf_at(const ChemArgs& A, int row, double T) {
  const double* t = A.Tpf;
  const double* y = A.lnpf + (int64_t)row * A.npf;
  const int n = A.npf;
  if (T <= t[0]) return y[0];
  if (T >= t[n - 1]) return y[n - 1];
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (hi + lo) >> 1;
    if (T >= t[mid]) lo = mid;
    else hi = mid;
  }
  const double fx = (t[lo + 1] - T) / (t[lo + 1] - t[lo]);
  return fx * y[lo] + (1 - fx) * y[lo + 1];
}

// fjk[0] of getfjk (rh/solvene.c:177-197): the neutral fraction
__device__ double neutral_fraction(const ChemArgs& A, int e, double ne, double T) {
  const int ns = A.nstage[e], off = A.stage_off[e];
  const double CT_ne = 2.0 * pow(kCI / T, -1.5) / ne;
  double f = 1.0, sum1 = 1.0;
  double Uk = pf_at(A, off, T);
  for (int j = 1; j < ns; ++j) {
    const double Ukp1 = pf_at(A, off + j, T);
    f = f * CT_ne * exp(Ukp1 - Uk - A.ionpot[off + j - 1] / (kK * T));
    sum1 += f;
    Uk = Ukp1;
  }
  return 1.0 / sum1;
}

__global__ void chem_kernel(const __grid_constant__ ChemArgs A, int64_t npoint, const double* Tv,
                            const double* nev, const double* nHv, double* nmol_out,
                            double* nHmin_out, double* nnuc_out, int32_t* niter_out) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= npoint) return;
  const double T = Tv[k], ne = nev[k], nHtot = nHv[k];
  const int Nn = A.nnuc, Nm = A.nmol, Neq = Nn + Nm;
  double fn0[PYRH_CHEM_MAX_NUCLEI], a[kMaxEq], n[kMaxEq], prev[kMaxEq], f[kMaxEq];
  double df[kMaxEq * kMaxEq], Phi[PYRH_CHEM_MAX_MOLECULES];
  for (int i = 0; i < Nn; ++i) {
    const int e = A.nuc_elem[i];
    fn0[i] = A.fn0[i] ? A.fn0[i][k] : neutral_fraction(A, e, ne, T);
    a[i] = A.abund[e] * nHtot;
  }
  for (int i = Nn; i < Neq; ++i) a[i] = 0.0;
  const double PhiHmin = 0.25 * pow(kCI / T, 1.5) * exp(0.754 * kEV / (kK * T));
  const double fHmin = ne * fn0[0] * PhiHmin;
  for (int i = 0; i < Nm; ++i) Phi[i] = equilconstant(A.mol[i], T);
  for (int i = 0; i < Nn; ++i) n[i] = a[i];
  for (int i = 0; i < Nm; ++i) n[Nn + i] = 0.0;
  for (int i = 0; i < Neq; ++i) prev[i] = n[i];
  double dnmax = 0.0;
  int niter = 1;
  while (niter <= kMaxIter) {
    for (int i = 0; i < Neq; ++i) {
      f[i] = n[i] - a[i];
      for (int j = 0; j < Neq; ++j) df[i * Neq + j] = 0.0;
      df[i * Neq + i] = 1.0;
    }
    f[0] += fHmin * n[0];
    df[0] += fHmin;
    for (int i = 0; i < Nm; ++i) {
      const pyrh_molecule& m = A.mol[i];
      double saha = Phi[i];
      for (int j = 0; j < m.nelement; ++j) {
        const int nu = A.nucl_index[i][j];
        saha *= pow(fn0[nu] * n[nu], (double)m.pt_count[j]);
        f[nu] += m.pt_count[j] * n[Nn + i];
      }
      saha /= pow(ne, (double)m.charge);
      f[Nn + i] -= saha;
      for (int j = 0; j < m.nelement; ++j) {
        const int nu = A.nucl_index[i][j];
        df[nu * Neq + Nn + i] += m.pt_count[j];
        df[(Nn + i) * Neq + nu] = -saha * (m.pt_count[j] / n[nu]);
      }
    }
    pyrh::lu_solve<kMaxEq>(Neq, df, f);
    for (int i = 0; i < Neq; ++i) n[i] -= f[i];
    // MaxChange with NG_CHEM_ORDER 0: the last two iterates
    dnmax = 0.0;
    for (int i = 0; i < Neq; ++i) {
      if (n[i]) dnmax = fmax(dnmax, fabs((n[i] - prev[i]) / n[i]));
      prev[i] = n[i];
    }
    if (dnmax <= kIterLimit) break;
    niter++;
  }
  for (int i = 0; i < Nm; ++i) nmol_out[(int64_t)i * npoint + k] = n[Nn + i];
  nHmin_out[k] = ne * (n[0] * PhiHmin);
  if (nnuc_out)
    for (int i = 0; i < Nn; ++i) nnuc_out[(int64_t)i * npoint + k] = n[i];
  if (niter_out) niter_out[k] = dnmax > kIterLimit ? -1 : (niter > kMaxIter ? kMaxIter : niter);
}

// Chemical equilibrium with a warp per point, for batches too small to fill
// the GPU one point per thread (the layers of the hydrostatic equilibrium, a
// single atmosphere's set-up): lane i owns equation i, its row of the
// Jacobian in shared memory.  Rows are filled in the reference's order.  The
// factorisation is the right-looking form of the reference's Crout
// elimination with the same implicit pivoting: every entry receives the same
// updates, with the same multipliers, in the same order.  The forward
// substitution runs column by column in the reference's order, the back
// substitution column by column from the last (another summation order);
// the results agree with the reference to rounding.
constexpr int kChemWarps = 2;

__device__ __forceinline__ void warp_lu_substitute(int Neq, const double* M, const int* piv,
                                                   double* x, int lane) {
  // the row interchanges in order (ludcmp.c LUbacksubst), then L y = P b
  if (lane == 0)
    for (int i = 0; i < Neq; ++i) {
      const int ip = piv[i];
      const double t = x[ip];
      x[ip] = x[i];
      x[i] = t;
    }
  __syncwarp();
  double xl = lane < Neq ? x[lane] : 0.0;
  for (int i = 0; i < Neq; ++i) {
    const double xi = __shfl_sync(0xffffffffu, xl, i);
    if (lane > i && lane < Neq) xl -= M[lane * Neq + i] * xi;
  }
  for (int i = Neq - 1; i >= 0; --i) {
    if (lane == i) xl = xl / M[i * Neq + i];
    const double xi = __shfl_sync(0xffffffffu, xl, i);
    if (lane < i) xl -= M[lane * Neq + i] * xi;
  }
  __syncwarp();
  if (lane < Neq) x[lane] = xl;
  __syncwarp();
}

__global__ void __launch_bounds__(32 * kChemWarps)
    chem_warp_kernel(const __grid_constant__ ChemArgs A, int64_t npoint, const double* Tv,
                     const double* nev, const double* nHv, double* nmol_out, double* nHmin_out,
                     double* nnuc_out, int32_t* niter_out) {
  __shared__ double sM[kChemWarps][kMaxEq * kMaxEq];
  __shared__ double sMc[kChemWarps][kMaxEq * kMaxEq];
  __shared__ double sx[kChemWarps][kMaxEq], sr[kChemWarps][kMaxEq], sn[kChemWarps][kMaxEq];
  __shared__ int spiv[kChemWarps][kMaxEq];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t k = blockIdx.x * (int64_t)kChemWarps + w;
  if (k >= npoint) return;   // the same for the whole warp
  double* M = sM[w];
  double* Mc = sMc[w];
  double* x = sx[w];
  double* r = sr[w];
  double* nS = sn[w];
  int* piv = spiv[w];
  const unsigned full = 0xffffffffu;
  const double T = Tv[k], ne = nev[k], nHtot = nHv[k];
  const int Nn = A.nnuc, Nm = A.nmol, Neq = Nn + Nm;
  double fl0 = 0.0, al = 0.0;
  if (lane < Nn) {
    const int e = A.nuc_elem[lane];
    fl0 = A.fn0[lane] ? A.fn0[lane][k] : neutral_fraction(A, e, ne, T);
    al = A.abund[e] * nHtot;
  }
  double fn0[PYRH_CHEM_MAX_NUCLEI];
#pragma unroll
  for (int i = 0; i < PYRH_CHEM_MAX_NUCLEI; ++i) fn0[i] = __shfl_sync(full, fl0, i);
  const double PhiHmin = 0.25 * pow(kCI / T, 1.5) * exp(0.754 * kEV / (kK * T));
  const double fHmin = ne * fn0[0] * PhiHmin;
  const bool mol_row = lane >= Nn && lane < Neq;
  const double Phi = mol_row ? equilconstant(A.mol[lane - Nn], T) : 0.0;
  double nl = lane < Nn ? al : 0.0;
  double prev = nl;
  double dnmax = 0.0;
  int niter = 1;
  while (niter <= kMaxIter) {
    nS[lane] = nl;
    __syncwarp();
    double fl = 0.0;
    if (lane < Neq) {
      double* row = M + lane * Neq;
      for (int j = 0; j < Neq; ++j) row[j] = 0.0;
      row[lane] = 1.0;
      fl = nl - al;
      if (lane == 0) {
        fl += fHmin * nl;
        row[0] += fHmin;
      }
      if (lane < Nn) {
        for (int i = 0; i < Nm; ++i) {
          const pyrh_molecule& m = A.mol[i];
          for (int j = 0; j < m.nelement; ++j)
            if (A.nucl_index[i][j] == lane) {
              fl += m.pt_count[j] * nS[Nn + i];
              row[Nn + i] += m.pt_count[j];
            }
        }
      } else {
        const pyrh_molecule& m = A.mol[lane - Nn];
        double saha = Phi;
        for (int j = 0; j < m.nelement; ++j) {
          const int nu = A.nucl_index[lane - Nn][j];
          saha *= pow(fn0[nu] * nS[nu], (double)m.pt_count[j]);
        }
        saha /= pow(ne, (double)m.charge);
        fl -= saha;
        for (int j = 0; j < m.nelement; ++j) {
          const int nu = A.nucl_index[lane - Nn][j];
          row[nu] = -saha * (m.pt_count[j] / nS[nu]);
        }
      }
      x[lane] = fl;
    }
    __syncwarp();
    for (int i = lane; i < Neq * Neq; i += 32) Mc[i] = M[i];
    // implicit scaling of each row (ludcmp.c LUdecomp)
    double vv = 0.0;
    if (lane < Neq) {
      double big = 0.0;
      for (int j = 0; j < Neq; ++j) big = fmax(big, fabs(M[lane * Neq + j]));
      vv = big == 0.0 ? 0.0 : 1.0 / big;
    }
    __syncwarp();
    for (int j = 0; j < Neq; ++j) {
      // pivot: the largest scaled |A[i][j]| of rows i >= j, the last of equals
      double best = (lane >= j && lane < Neq) ? vv * fabs(M[lane * Neq + j]) : -1.0;
      int imax = lane;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(full, best, o);
        const int oi = __shfl_xor_sync(full, imax, o);
        if (ob > best || (ob == best && oi > imax)) {
          best = ob;
          imax = oi;
        }
      }
      if (imax != j) {
        if (lane < Neq) {
          const double t = M[imax * Neq + lane];
          M[imax * Neq + lane] = M[j * Neq + lane];
          M[j * Neq + lane] = t;
        }
        const double vj = __shfl_sync(full, vv, j);
        if (lane == imax) vv = vj;
      }
      if (lane == 0) piv[j] = imax;
      __syncwarp();
      if (lane == 0 && M[j * Neq + j] == 0.0) M[j * Neq + j] = 1.0e-20;
      __syncwarp();
      const double dum = 1.0 / M[j * Neq + j];
      if (lane > j && lane < Neq) {
        double* row = M + lane * Neq;
        const double l = row[j] * dum;
        row[j] = l;
        for (int c = j + 1; c < Neq; ++c) row[c] -= l * M[j * Neq + c];
      }
      __syncwarp();
    }
    // solve, then one improvement with the residual of the original system
    warp_lu_substitute(Neq, M, piv, x, lane);
    if (lane < Neq) {
      double res = fl;
      for (int j = 0; j < Neq; ++j) res -= Mc[lane * Neq + j] * x[j];
      r[lane] = res;
    }
    __syncwarp();
    warp_lu_substitute(Neq, M, piv, r, lane);
    if (lane < Neq) nl -= x[lane] + r[lane];
    // MaxChange with NG_CHEM_ORDER 0: the last two iterates
    double d = 0.0;
    if (lane < Neq && nl) d = fabs((nl - prev) / nl);
    prev = nl;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d = fmax(d, __shfl_xor_sync(full, d, o));
    dnmax = d;
    if (dnmax <= kIterLimit) break;
    niter++;
  }
  if (mol_row) nmol_out[(int64_t)(lane - Nn) * npoint + k] = nl;
  const double n0 = __shfl_sync(full, nl, 0);
  if (lane == 0) {
    nHmin_out[k] = ne * (n0 * PhiHmin);
    if (niter_out) niter_out[k] = dnmax > kIterLimit ? -1 : (niter > kMaxIter ? kMaxIter : niter);
  }
  if (nnuc_out && lane < Nn) nnuc_out[(int64_t)lane * npoint + k] = nl;
}

pyrh_status fail(pyrh_status s, const char* msg) {
  pyrh::set_error("%s", msg);
  return s;
}

}  // namespace

namespace {
pyrh_status chem_launch(const pyrh_elem_tables* tables, const pyrh_molecule* mol, int32_t nmol,
                        int64_t npoint, const double* T, const double* ne, const double* nHtot,
                        const double* const* fn0_model, double* nmol_out, double* nHmin,
                        double* nnuc, int32_t* niter, void* stream, bool warp) {
  pyrh::set_launches(0);
  if (!tables || !mol || nmol < 1 || nmol > PYRH_CHEM_MAX_MOLECULES || npoint < 0)
    return fail(PYRH_ERR_ARG, "chem: bad arguments");
  if (npoint == 0) return PYRH_OK;
  if (!T || !ne || !nHtot || !nmol_out || !nHmin) return fail(PYRH_ERR_ARG, "chem: NULL array");
  if (tables->nelem != PYRH_NELEM || tables->npf < 2 || !tables->Tpf || !tables->abund ||
      !tables->lnpf || !tables->ionpot || !tables->nstage || !tables->stage_off)
    return fail(PYRH_ERR_ARG, "chem: element tables");
  static_assert(sizeof(ChemArgs) < 32000, "kernel parameter block (32 KB on this architecture)");
  ChemArgs A;
  memset(&A, 0, sizeof A);
  A.nmol = nmol;
  if (strncmp(mol[0].id, "H2", 3) != 0)
    return fail(PYRH_ERR_ARG, "chem: the first molecule must be H2");
  // nuclei: the elements bound in some molecule, in element order
  bool bound[PYRH_NELEM] = {false};
  for (int i = 0; i < nmol; ++i) {
    if (mol[i].nelement < 1 || mol[i].nelement > PYRH_MOL_MAX_ELEMENTS || mol[i].neqc < 0 ||
        mol[i].neqc > PYRH_MOL_MAX_COEF)
      return fail(PYRH_ERR_ARG, "chem: malformed molecule");
    for (int j = 0; j < mol[i].nelement; ++j) {
      const int e = mol[i].pt_index[j];
      if (e < 0 || e >= PYRH_NELEM) return fail(PYRH_ERR_ARG, "chem: element index");
      bound[e] = true;
    }
    A.mol[i] = mol[i];
  }
  int map[PYRH_NELEM];
  for (int e = 0; e < PYRH_NELEM; ++e) {
    map[e] = -1;
    if (!bound[e]) continue;
    if (A.nnuc == PYRH_CHEM_MAX_NUCLEI) return fail(PYRH_ERR_UNSUPPORTED, "chem: too many nuclei");
    map[e] = A.nnuc;
    A.nuc_elem[A.nnuc] = e;
    A.fn0[A.nnuc] = fn0_model ? fn0_model[e] : nullptr;
    ++A.nnuc;
  }
  if (A.nuc_elem[0] != 0) return fail(PYRH_ERR_ARG, "chem: the first nucleus must be hydrogen");
  for (int i = 0; i < nmol; ++i)
    for (int j = 0; j < mol[i].nelement; ++j) A.nucl_index[i][j] = map[mol[i].pt_index[j]];
  A.npf = tables->npf;
  A.Tpf = tables->Tpf;
  A.abund = tables->abund;
  A.lnpf = tables->lnpf;
  A.ionpot = tables->ionpot;
  A.nstage = tables->nstage;
  A.stage_off = tables->stage_off;
  cudaStream_t st = (cudaStream_t)stream;
  if (warp) {
    chem_warp_kernel<<<(unsigned)((npoint + kChemWarps - 1) / kChemWarps), 32 * kChemWarps, 0,
                       st>>>(A, npoint, T, ne, nHtot, nmol_out, nHmin, nnuc, niter);
  } else {
    const int threads = 64;
    chem_kernel<<<(unsigned)((npoint + threads - 1) / threads), threads, 0, st>>>(
        A, npoint, T, ne, nHtot, nmol_out, nHmin, nnuc, niter);
  }
  const cudaError_t e = cudaGetLastError();
  pyrh::set_launches(1);
  if (e != cudaSuccess) {
    pyrh::set_error("chem: %s", cudaGetErrorString(e));
    return PYRH_ERR_CUDA;
  }
  return PYRH_OK;
}
}  // namespace

extern "C" pyrh_status pyrh_chem_equil(const pyrh_elem_tables* tables, const pyrh_molecule* mol,
                                       int32_t nmol, int64_t npoint, const double* T,
                                       const double* ne, const double* nHtot,
                                       const double* const* fn0_model, double* nmol_out,
                                       double* nHmin, double* nnuc, int32_t* niter,
                                       void* stream) {
  return chem_launch(tables, mol, nmol, npoint, T, ne, nHtot, fn0_model, nmol_out, nHmin, nnuc,
                     niter, stream, false);
}

namespace pyrh {
// pyrh_chem_equil with a warp per point (chem_warp_kernel).
pyrh_status chem_equil_warp(const pyrh_elem_tables* tables, const pyrh_molecule* mol,
                            int32_t nmol, int64_t npoint, const double* T, const double* ne,
                            const double* nHtot, const double* const* fn0_model, double* nmol_out,
                            double* nHmin, double* nnuc, int32_t* niter, void* stream) {
  if (npoint > ((int64_t)1 << 31) - kChemWarps) {
    pyrh::set_error("chem: npoint too large for a warp per point");
    return PYRH_ERR_ARG;
  }
  return chem_launch(tables, mol, nmol, npoint, T, ne, nHtot, fn0_model, nmol_out, nHmin, nnuc,
                     niter, stream, true);
}
}  // namespace pyrh
