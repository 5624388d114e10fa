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

pyrh_status fail(pyrh_status s, const char* msg) {
  pyrh::set_error("%s", msg);
  return s;
}

}  // namespace

extern "C" pyrh_status pyrh_chem_equil(const pyrh_elem_tables* tables, const pyrh_molecule* mol,
                                       int32_t nmol, int64_t npoint, const double* T,
                                       const double* ne, const double* nHtot,
                                       const double* const* fn0_model, double* nmol_out,
                                       double* nHmin, double* nnuc, int32_t* niter,
                                       void* stream) {
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
  const int threads = 64;
  chem_kernel<<<(unsigned)((npoint + threads - 1) / threads), threads, 0, st>>>(
      A, npoint, T, ne, nHtot, nmol_out, nHmin, nnuc, niter);
  const cudaError_t e = cudaGetLastError();
  pyrh::set_launches(1);
  if (e != cudaSuccess) {
    pyrh::set_error("chem: %s", cudaGetErrorString(e));
    return PYRH_ERR_CUDA;
  }
  return PYRH_OK;
}
