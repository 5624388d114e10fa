// hse.cu -- hydrostatic equilibrium of a batch of atmospheres on the device
// (pyrh's hse()).
//
// Reference routines restated here (file:line in the reference tree):
//   hse              rh/rhf1d/pyrh_hse.c:67-399 (layer by layer from the top:
//                    the gas pressure from the layer above, then passes of
//                    electron density, LTE populations, chemical equilibrium
//                    and 500 nm opacity until the hydrogen density settles)
//   get_ne           rh/rhf1d/pyrh_background.c:459-540 (Solve_ne's iteration,
//                    fromscratch mode 2; a warp per atmosphere for batches
//                    too small to fill the GPU one atmosphere per thread)
//   LTEpops          rh/ltepops.c:33-109 (Saha-Boltzmann; the Debye lowering
//                    is switched off there, ltepops.c:53)
//   ChemicalEquilibrium's neutral fractions and population scaling
//                    rh/chemequil.c:219-238, 330-339 (pyrh_chem_equil does
//                    the Newton iteration)
//   pyrh_Background  rh/rhf1d/pyrh_background.c:144-457 (pyrh_background with
//                    a model without the metals' continua, scattering added)
//   convertScales    rh/rhf1d/multiatmos.c:100-177 (pyrh_convert_scales), with
//                    Linear (rh/linear.c:22-51) and Locate (rh/hunt.c:92-117)
//                    for the height where tau_ref = 1
//
// Work layout: a layer k of every atmosphere is one vector of natm points
// (the batch is [ndep][natm]); each pass is six launches over those points
// on the caller's stream, and one 4-byte read of the count of atmospheres
// still iterating ends the layer.  An atmosphere that has settled keeps the
// values of its last pass: the pass computes into scratch and the update
// kernel commits only for the atmospheres still iterating.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "../../include/pyrh_gb300.h"

namespace pyrh {
void set_error(const char* fmt, ...);
void set_launches(int n);
pyrh_status solve_ne_warp(const pyrh_elem_tables* tables, int64_t npoint, const double* T,
                          const double* nHtot, double* ne, int32_t fromscratch, int32_t* niter,
                          cudaStream_t st);
pyrh_status chem_equil_warp(const pyrh_elem_tables* tables, const pyrh_molecule* mol,
                            int32_t nmol, int64_t npoint, const double* T, const double* ne,
                            const double* nHtot, const double* const* fn0_model, double* nmol_out,
                            double* nHmin, double* nnuc, int32_t* niter, void* stream);
}

namespace {

constexpr double kH = 6.6260755E-34;
constexpr double kK = 1.380658E-23;
constexpr double kMe = 9.1093897E-31;
constexpr double kPi = 3.14159265358979;
constexpr double kAMU = 1.6605402E-27;
constexpr double kKM_TO_M = 1.0E+03;
constexpr double kG_TO_KG = 1.0E-03;
constexpr double kCM_TO_M = 1.0E-02;
constexpr double kLG10 = 2.30258509299404568402;   // ln 10 (rh.h POW10)
constexpr double kC1 = (kH / (2.0 * kPi * kMe)) * (kH / kK);
constexpr int kThreads = 128;

__device__ __forceinline__ double pow10r(double x) { return exp(kLG10 * (x)); }

struct AtomsDev {
  int natom;
  int elem[PYRH_MAX_PASSIVE_ATOMS];
  int lev_off[PYRH_MAX_PASSIVE_ATOMS + 1];
  const double *E, *g;
  const int32_t* stage;
  const double* abund;   // element tables
};

// Top of layer k: the pressure step from the layer above (pyrh_hse.c:
// 245-255) and the first hydrogen density (:257-260); the top layer starts
// from pg_top with no electrons (:185-187).
__global__ void hse_start_kernel(pyrh_hse_config c, pyrh_hse_batch b, int k, int32_t* active,
                                 int32_t* iter) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= b.natm) return;
  const int64_t n = b.natm;
  const double T = b.T[k * n + a];
  active[a] = 1;
  iter[a] = 0;
  if (k == 0) {
    const double pg0 = b.pg_top[a];
    b.pg[a] = pg0;
    b.ne[a] = 0.0;
    b.nHtot[a] = (pg0 / kK / T - 0.0) / c.total_abund;
    return;
  }
  const int64_t i = k * n + a, u = (k - 1) * n + a;
  double dP;
  if (c.scale == 0) {
    const double tk = pow10r(b.scale[i]), tu = pow10r(b.scale[u]);
    dP = c.gravity * b.rho[u] / b.opacity[u] * (tk - tu);
  } else {
    dP = c.gravity * b.rho[u] * (b.scale[u] * kKM_TO_M - b.scale[i] * kKM_TO_M);
  }
  const double pg = b.pg[u] + dP;
  b.pg[i] = pg;
  b.nHtot[i] = (pg / kK / T - b.ne[u]) / c.total_abund;
}

// LTE populations of every model atom at the pass's electron density
// (rows [level][natm] of pops) and the neutral fraction of each (fn0
// [atom][natm]); one thread per (atom, point), the points of an atom
// consecutive.
__global__ void hse_pops_kernel(AtomsDev A, int natm, const double* __restrict__ Tl,
                                const double* __restrict__ nHl, const double* __restrict__ ne_c,
                                double* __restrict__ pops, double* __restrict__ fn0) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)natm * A.natom) return;
  const int a = (int)(t % natm), m = (int)(t / natm);
  const double T = Tl[a], nH = nHl[a], ne = ne_c[a];
  const double cNe_T = 0.5 * ne * pow(kC1 / T, 1.5);
  {
    const int o = A.lev_off[m], nl = A.lev_off[m + 1] - o;
    const double ntotal = A.abund[A.elem[m]] * nH;
    const double E0 = A.E[o], g0 = A.g[o];
    const int z0 = A.stage[o];
    double sum = 1.0;
    for (int i = 1; i < nl; ++i) {
      const double dE_kT = (A.E[o + i] - E0) / (kK * T);
      double v = A.g[o + i] / g0 * exp(-dE_kT);
      for (int z = 1; z <= A.stage[o + i] - z0; ++z) v /= cNe_T;
      pops[(int64_t)(o + i) * natm + a] = v;
      sum += v;
    }
    const double n0 = ntotal / sum;
    pops[(int64_t)o * natm + a] = n0;
    double neutral = n0;
    bool more = A.stage[o] <= 0;
    if (!more) neutral = 0.0;
    for (int i = 1; i < nl; ++i) {
      const int64_t r = (int64_t)(o + i) * natm + a;
      const double v = pops[r] * n0;
      pops[r] = v;
      if (more && A.stage[o + i] > 0) more = false;
      if (more) neutral += v;
    }
    fn0[(int64_t)m * natm + a] = neutral / ntotal;
  }
}

// chemequil.c:330-339: a nucleus' model atom keeps the fraction of its
// nuclei left atomic.
__global__ void hse_scale_kernel(AtomsDev A, int natm, int nnuc, const int* __restrict__ nuc_atom,
                                 const double* __restrict__ nHl, const double* __restrict__ nnuc_d,
                                 double* __restrict__ pops) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= natm) return;
  const double nH = nHl[a];
  for (int i = 0; i < nnuc; ++i) {
    const int m = nuc_atom[i];
    if (m < 0) continue;
    const double fraction = nnuc_d[(int64_t)i * natm + a] / (A.abund[A.elem[m]] * nH);
    for (int r = A.lev_off[m]; r < A.lev_off[m + 1]; ++r) pops[(int64_t)r * natm + a] *= fraction;
  }
}

// End of a pass (pyrh_hse.c:191-217 for the top layer, :262-338 below it):
// the atmospheres still iterating take the pass's electron density, density
// and opacity, the new gas pressure and hydrogen density, and stop once the
// hydrogen density changed by at most eta_limit.
__global__ void hse_update_kernel(pyrh_hse_config c, pyrh_hse_batch b, int k,
                                  const double* __restrict__ ne_c, const double* __restrict__ chi,
                                  int32_t* active, int32_t* iter, int32_t* still) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= b.natm || !active[a]) return;
  const int64_t n = b.natm, i = k * n + a;
  const double T = b.T[i];
  const double nH_old = b.nHtot[i];
  const double rho = (kAMU * c.wght_per_H) * nH_old;
  const double ne = ne_c[a], op = chi[a];
  b.rho[i] = rho;
  b.ne[i] = ne;
  if (b.opacity) b.opacity[i] = op;
  double pg = b.pg[i];
  if (k > 0) {
    const int64_t u = (k - 1) * n + a;
    if (c.scale == 0) {
      const double tk = pow10r(b.scale[i]), tu = pow10r(b.scale[u]);
      const double dlogtau = log10(tk) - log10(tu);
      const double beta1 = b.rho[u] / b.opacity[u] * tu;
      const double beta2 = rho / op * tk;
      pg = b.pg[u] + kLG10 * c.gravity * (beta2 + beta1) / 2 * dlogtau;
    } else {
      const double dP = c.gravity * (b.scale[u] * kKM_TO_M - b.scale[i] * kKM_TO_M) *
                        sqrt(rho * b.rho[u]);
      pg = b.pg[u] + dP;
    }
    b.pg[i] = pg;
  }
  const double nH = (pg / kK / T - ne) / c.total_abund;
  b.nHtot[i] = nH;
  const int it = ++iter[a];
  const double eta = fabs((nH - nH_old) / nH);
  if (eta <= c.eta_limit) {
    active[a] = 0;
    if (b.niter) b.niter[i] = it;
  } else if (it >= c.nmax_iter) {
    active[a] = 0;
    if (b.niter) b.niter[i] = -1;
  } else {
    atomicAdd(still, 1);
  }
}

__global__ void hse_bg_layout_kernel(int natm, int32_t* ndep, int32_t* nspect, int64_t* depth_off,
                                     int64_t* lam_off, int64_t* cont_off, double* lambda) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= natm) return;
  ndep[a] = 1;
  nspect[a] = 1;
  depth_off[a] = a;
  lam_off[a] = 0;
  cont_off[a] = a;
  if (a == 0) lambda[0] = 500.0;   // pyrh_hse.c:229-232
}

pyrh_status fail(pyrh_status s, const char* msg) {
  pyrh::set_error("%s", msg);
  return s;
}

// Device scratch of one call, carved from one allocation.
struct Scratch {
  char* base = nullptr;
  size_t off = 0, size = 0;
  template <typename T>
  T* take(size_t n) {
    off = (off + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base + off);
    off += n * sizeof(T);
    return p;
  }
};

int find_molecule(const pyrh_molecule* mol, int nmol, const char* id) {
  for (int i = 0; i < nmol; ++i)
    if (strncmp(mol[i].id, id, sizeof mol[i].id) == 0) return i;
  return -1;
}

pyrh_status check_atoms(const pyrh_passive_atoms* atoms) {
  if (atoms->natom < 1 || atoms->natom > PYRH_MAX_PASSIVE_ATOMS || !atoms->E || !atoms->g ||
      !atoms->stage || atoms->lev_off[0] != 0)
    return fail(PYRH_ERR_ARG, "passive atoms: count, arrays or first offset");
  for (int m = 0; m < atoms->natom; ++m) {
    if (atoms->lev_off[m + 1] <= atoms->lev_off[m] || atoms->elem[m] < 0 ||
        atoms->elem[m] >= PYRH_NELEM)
      return fail(PYRH_ERR_ARG, "passive atoms: levels or element");
    for (int q = 0; q < m; ++q)
      if (atoms->elem[q] == atoms->elem[m])
        return fail(PYRH_ERR_ARG, "passive atoms: two atoms of one element");
  }
  return PYRH_OK;
}

// The nuclei (elements bound in some molecule, in element order, as
// pyrh_chem_equil numbers them) and the model atom of each (-1: none);
// -1 when there are more than PYRH_CHEM_MAX_NUCLEI.
int nuclei_atoms(const pyrh_molecule* mol, int nmol, const pyrh_passive_atoms* atoms,
                 int* nuc_atom) {
  bool bound[PYRH_NELEM] = {false};
  for (int i = 0; i < nmol; ++i)
    for (int j = 0; j < mol[i].nelement && j < PYRH_MOL_MAX_ELEMENTS; ++j)
      if (mol[i].pt_index[j] >= 0 && mol[i].pt_index[j] < PYRH_NELEM) bound[mol[i].pt_index[j]] = true;
  int nnuc = 0;
  for (int e = 0; e < PYRH_NELEM; ++e) {
    if (!bound[e]) continue;
    if (nnuc == PYRH_CHEM_MAX_NUCLEI) return -1;
    nuc_atom[nnuc] = -1;
    for (int m = 0; m < atoms->natom; ++m)
      if (atoms->elem[m] == e) nuc_atom[nnuc] = m;
    ++nnuc;
  }
  return nnuc;
}

AtomsDev atoms_dev(const pyrh_passive_atoms* atoms, const double* abund) {
  AtomsDev A;
  A.natom = atoms->natom;
  for (int m = 0; m < A.natom; ++m) A.elem[m] = atoms->elem[m];
  for (int m = 0; m <= A.natom; ++m) A.lev_off[m] = atoms->lev_off[m];
  A.E = atoms->E;
  A.g = atoms->g;
  A.stage = atoms->stage;
  A.abund = abund;
  return A;
}

// Up to this many points a call takes the warp-per-point forms of Solve_ne
// and of the chemistry (the one-point-per-thread forms leave most of the GPU
// idle and are bound by one thread's latency; above it they are faster:
// 1024 atmospheres of hse 122 against 487 ms, 16384 875 against 598 ms).
constexpr int64_t kSmallBatch = 8192;
bool small_batch(int64_t npoint) { return npoint <= kSmallBatch; }

// LTE populations, chemical equilibrium and the scaled populations at
// npoint points (three launches); fn0 [natom]
// [npoint] and nnuc_d [nnuc][npoint] are scratch, nuc_atom the device copy
// of nuclei_atoms' map.
pyrh_status equilibria_core(const pyrh_elem_tables* tables, const pyrh_molecule* mol, int nmol,
                            const AtomsDev& A, int nnuc, const int* nuc_atom, int64_t npoint,
                            const double* T, const double* ne, const double* nH, double* pops,
                            double* fn0, double* nmol_out, double* nHmin, double* nnuc_d,
                            cudaStream_t st, int& launches) {
  const unsigned grid = (unsigned)((npoint + kThreads - 1) / kThreads);
  const unsigned grid_atoms = (unsigned)((npoint * A.natom + kThreads - 1) / kThreads);
  const double* fn0_ptr[PYRH_NELEM];
  for (int e = 0; e < PYRH_NELEM; ++e) fn0_ptr[e] = nullptr;
  for (int m = 0; m < A.natom; ++m) fn0_ptr[A.elem[m]] = fn0 + (size_t)m * npoint;
  hse_pops_kernel<<<grid_atoms, kThreads, 0, st>>>(A, npoint, T, nH, ne, pops, fn0);
  ++launches;
  const pyrh_status s =
      small_batch(npoint)
          ? pyrh::chem_equil_warp(tables, mol, nmol, npoint, T, ne, nH, fn0_ptr, nmol_out, nHmin,
                                  nnuc_d, nullptr, st)
          : pyrh_chem_equil(tables, mol, nmol, npoint, T, ne, nH, fn0_ptr, nmol_out, nHmin,
                            nnuc_d, nullptr, st);
  if (s != PYRH_OK) return s;
  launches += pyrh_last_launch_count();
  hse_scale_kernel<<<grid, kThreads, 0, st>>>(A, npoint, nnuc, nuc_atom, nH, nnuc_d, pops);
  ++launches;
  return PYRH_OK;
}

// convertScales for one atmosphere per thread, walking down its layers.
__global__ void convert_scales_kernel(pyrh_scales_batch b) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= b.natm) return;
  const int64_t n = b.natm;
  const int nd = b.ndep;
  auto at = [&](const double* x, int k) { return x[k * n + a]; };
  double* tau = b.tau_ref;
  double* cm = b.cmass;
  double* h = b.height;
  const double rho_c = kAMU * b.wght_per_H;
  // the given scale in SI (pyrh_compute1dray.c:229-245)
  for (int k = 0; k < nd; ++k) {
    const double v = at(b.scale_in, k);
    if (b.scale == 0) tau[k * n + a] = pow10r(v);
    else if (b.scale == 1) cm[k * n + a] = pow10r(v) * (kG_TO_KG / (kCM_TO_M * kCM_TO_M));
    else h[k * n + a] = v * kKM_TO_M;
  }
  double rho_u = rho_c * at(b.nHtot, 0), chi_u = at(b.chi_ref, 0);
  if (b.scale == 1) {
    h[a] = 0.0;
    tau[a] = chi_u / rho_u * cm[a];
  } else if (b.scale == 0) {
    h[a] = 0.0;
    cm[a] = (tau[a] / chi_u) * rho_u;
  } else {
    cm[a] = (at(b.nHtot, 0) * b.total_abund + at(b.ne, 0)) * (kK * at(b.T, 0) / b.gravity);
    tau[a] = 0.5 * chi_u * (h[a] - h[n + a]);
    if (tau[a] > 1.0) tau[a] = 0.0;
  }
  for (int k = 1; k < nd; ++k) {
    const int64_t i = k * n + a, u = (k - 1) * n + a;
    const double rho = rho_c * b.nHtot[i], chi = b.chi_ref[i];
    if (b.scale == 1) {
      h[i] = h[u] - 2.0 * (cm[i] - cm[u]) / (rho_u + rho);
      tau[i] = tau[u] + 0.5 * (chi_u + chi) * (h[u] - h[i]);
    } else if (b.scale == 0) {
      h[i] = h[u] - 2.0 * (tau[i] - tau[u]) / (chi_u + chi);
      cm[i] = cm[u] + 0.5 * (rho_u + rho) * (h[u] - h[i]);
    } else {
      cm[i] = cm[u] + 0.5 * (rho_u + rho) * (h[u] - h[i]);
      tau[i] = tau[u] + 0.5 * (chi_u + chi) * (h[u] - h[i]);
    }
    rho_u = rho;
    chi_u = chi;
  }
  if (b.scale == 0 || b.scale == 1) {
    // Linear(Ndep, tau_ref, height, 1, &unity, &h_zero, FALSE)
    const bool ascend = tau[n + a] > tau[a];
    const double xmin = ascend ? tau[a] : tau[(nd - 1) * n + a];
    const double xmax = ascend ? tau[(nd - 1) * n + a] : tau[a];
    const double x = 1.0;
    double h0;
    if (x <= xmin) {
      h0 = ascend ? h[a] : h[(nd - 1) * n + a];
    } else if (x >= xmax) {
      h0 = ascend ? h[(nd - 1) * n + a] : h[a];
    } else {
      // Locate: bisection for the interval holding x
      const bool asc = tau[(nd - 1) * n + a] > tau[a];
      int lo = 0, hi = nd;
      while (hi - lo > 1) {
        const int mid = (hi + lo) >> 1;
        const double t = tau[mid * n + a];
        if (asc ? (x >= t) : (x <= t)) lo = mid;
        else hi = mid;
      }
      const double t0 = tau[lo * n + a], t1 = tau[(lo + 1) * n + a];
      const double fx = (t1 - x) / (t1 - t0);
      h0 = fx * h[lo * n + a] + (1 - fx) * h[(lo + 1) * n + a];
    }
    for (int k = 0; k < nd; ++k) h[k * n + a] = h[k * n + a] - h0;
  }
}

}  // namespace

extern "C" pyrh_status pyrh_equilibria(const pyrh_elem_tables* tables, const pyrh_molecule* mol,
                                       int32_t nmol, const pyrh_passive_atoms* atoms,
                                       int64_t npoint, const double* T, const double* ne,
                                       const double* nHtot, double* pops, double* nmol_out,
                                       double* nHmin, void* stream) {
  pyrh::set_launches(0);
  if (!tables || !mol || !atoms) return fail(PYRH_ERR_ARG, "equilibria: NULL argument");
  if (npoint < 0 || npoint > ((int64_t)1 << 31) - kThreads)
    return fail(PYRH_ERR_ARG, "equilibria: npoint outside [0, 2^31)");
  if (npoint == 0) return PYRH_OK;
  if (!T || !ne || !nHtot || !pops || !nmol_out || !nHmin)
    return fail(PYRH_ERR_ARG, "equilibria: NULL array");
  if (nmol < 1 || nmol > PYRH_CHEM_MAX_MOLECULES) return fail(PYRH_ERR_ARG, "equilibria: molecules");
  const pyrh_status sa = check_atoms(atoms);
  if (sa != PYRH_OK) return sa;
  int nuc_atom_h[PYRH_CHEM_MAX_NUCLEI];
  const int nnuc = nuclei_atoms(mol, nmol, atoms, nuc_atom_h);
  if (nnuc < 0) return fail(PYRH_ERR_UNSUPPORTED, "equilibria: too many nuclei");
  cudaStream_t st = (cudaStream_t)stream;
  Scratch S;
  S.size = 4 * 256 + sizeof(double) * (size_t)npoint * (atoms->natom + nnuc) +
           sizeof(int) * PYRH_CHEM_MAX_NUCLEI;
  if (cudaMalloc(&S.base, S.size) != cudaSuccess)
    return fail(PYRH_ERR_CUDA, "equilibria: scratch allocation");
  double* fn0 = S.take<double>((size_t)atoms->natom * npoint);
  double* nnuc_d = S.take<double>((size_t)(nnuc > 0 ? nnuc : 1) * npoint);
  int* nuc_atom = S.take<int>(PYRH_CHEM_MAX_NUCLEI);
  cudaMemcpyAsync(nuc_atom, nuc_atom_h, sizeof(int) * nnuc, cudaMemcpyHostToDevice, st);
  int launches = 0;
  pyrh_status s = equilibria_core(tables, mol, nmol, atoms_dev(atoms, tables->abund), nnuc, nuc_atom,
                                  npoint, T, ne, nHtot, pops, fn0, nmol_out, nHmin, nnuc_d, st,
                                  launches);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (s == PYRH_OK && e != cudaSuccess) {
    pyrh::set_error("equilibria: %s", cudaGetErrorString(e));
    s = PYRH_ERR_CUDA;
  }
  cudaFree(S.base);
  pyrh::set_launches(launches);
  return s;
}

extern "C" pyrh_status pyrh_convert_scales(const pyrh_scales_batch* b, void* stream) {
  pyrh::set_launches(0);
  if (!b || b->natm < 1 || b->ndep < 2 || !b->scale_in || !b->T || !b->ne || !b->nHtot ||
      !b->chi_ref || !b->tau_ref || !b->cmass || !b->height)
    return fail(PYRH_ERR_ARG, "convert scales: NULL array, no atmosphere or fewer than 2 depths");
  if (b->scale < 0 || b->scale > 2) return fail(PYRH_ERR_ARG, "convert scales: scale not 0, 1 or 2");
  if (b->scale == 2 && !(b->gravity > 0.0)) return fail(PYRH_ERR_ARG, "convert scales: gravity");
  const unsigned grid = (unsigned)((b->natm + kThreads - 1) / kThreads);
  convert_scales_kernel<<<grid, kThreads, 0, (cudaStream_t)stream>>>(*b);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    pyrh::set_error("convert scales: %s", cudaGetErrorString(e));
    return PYRH_ERR_CUDA;
  }
  pyrh::set_launches(1);
  return PYRH_OK;
}

extern "C" pyrh_status pyrh_hse(const pyrh_elem_tables* tables, const pyrh_molecule* mol,
                                int32_t nmol, const pyrh_bg_model* bg, const pyrh_passive_atoms* atoms,
                                const pyrh_hse_config* cfg, const pyrh_hse_batch* b,
                                void* stream) {
  pyrh::set_launches(0);
  if (!tables || !mol || !bg || !atoms || !cfg || !b) return fail(PYRH_ERR_ARG, "hse: NULL argument");
  if (b->natm < 1 || b->natm > 65535 || b->ndep < 1)
    return fail(PYRH_ERR_ARG, "hse: natm outside [1, 65535] or no depth points");
  if (!b->scale || !b->T || !b->pg_top || !b->ne || !b->nHtot || !b->rho || !b->pg)
    return fail(PYRH_ERR_ARG, "hse: NULL batch array");
  if (cfg->scale != 0 && cfg->scale != 2)
    return fail(PYRH_ERR_UNSUPPORTED,
                "hse: scale must be 0 (log tau500) or 2 (height); the reference's column-mass "
                "branch leaves its pressure step unset");
  if (cfg->nmax_iter < 1 || !(cfg->total_abund > 0.0) || !(cfg->wght_per_H > 0.0))
    return fail(PYRH_ERR_ARG, "hse: config");
  const pyrh_status sa = check_atoms(atoms);
  if (sa != PYRH_OK) return sa;
  const int npop = atoms->lev_off[atoms->natom];
  if (bg->npop != npop) return fail(PYRH_ERR_ARG, "hse: background rows differ from the atoms' levels");
  if (nmol < 1 || nmol > PYRH_CHEM_MAX_MOLECULES) return fail(PYRH_ERR_ARG, "hse: molecules");
  const int iH2 = find_molecule(mol, nmol, "H2"), iOH = find_molecule(mol, nmol, "OH"),
            iCH = find_molecule(mol, nmol, "CH");
  if ((bg->has_h2 && iH2 < 0) || (bg->has_oh && iOH < 0) || (bg->has_ch && iCH < 0))
    return fail(PYRH_ERR_ARG, "hse: the background names a molecule the list lacks");
  int nuc_atom_h[PYRH_CHEM_MAX_NUCLEI];
  const int nnuc = nuclei_atoms(mol, nmol, atoms, nuc_atom_h);
  if (nnuc < 0) return fail(PYRH_ERR_UNSUPPORTED, "hse: too many nuclei");

  cudaStream_t st = (cudaStream_t)stream;
  const int natm = b->natm;
  Scratch S;
  S.size = 64 * 256 + sizeof(double) * (size_t)natm * (8 + npop + atoms->natom + nmol + nnuc) +
           sizeof(int64_t) * 3 * (size_t)natm + sizeof(int32_t) * 4 * (size_t)natm + 256;
  if (cudaMalloc(&S.base, S.size) != cudaSuccess) return fail(PYRH_ERR_CUDA, "hse: scratch allocation");
  double* ne_c = S.take<double>(natm);
  double* pops = S.take<double>((size_t)npop * natm);
  double* fn0 = S.take<double>((size_t)atoms->natom * natm);
  double* nmol_d = S.take<double>((size_t)nmol * natm);
  double* nHmin = S.take<double>(natm);
  double* nnuc_d = S.take<double>((size_t)nnuc * natm);
  double* chi = S.take<double>(natm);
  double* eta = S.take<double>(natm);
  double* sca = S.take<double>(natm);
  double* lambda = S.take<double>(1);
  int32_t* ndep = S.take<int32_t>(natm);
  int32_t* nspect = S.take<int32_t>(natm);
  int64_t* depth_off = S.take<int64_t>(natm);
  int64_t* lam_off = S.take<int64_t>(natm);
  int64_t* cont_off = S.take<int64_t>(natm);
  int32_t* active = S.take<int32_t>(natm);
  int32_t* iter = S.take<int32_t>(natm);
  int32_t* still = S.take<int32_t>(1);
  int* nuc_atom = S.take<int>(PYRH_CHEM_MAX_NUCLEI);
  double* op_tmp = nullptr;
  pyrh_hse_batch B = *b;
  if (!B.opacity) {   // the update and start kernels read the layer above's opacity
    if (cudaMalloc(&op_tmp, sizeof(double) * (size_t)natm * b->ndep) != cudaSuccess) {
      cudaFree(S.base);
      return fail(PYRH_ERR_CUDA, "hse: scratch allocation");
    }
    B.opacity = op_tmp;
  }
  int32_t* still_h = nullptr;
  if (cudaMallocHost(&still_h, sizeof(int32_t)) != cudaSuccess) {
    if (op_tmp) cudaFree(op_tmp);
    cudaFree(S.base);
    return fail(PYRH_ERR_CUDA, "hse: pinned host allocation");
  }

  const AtomsDev A = atoms_dev(atoms, tables->abund);

  pyrh_bg_batch bb;
  memset(&bb, 0, sizeof bb);
  bb.natm = natm;
  bb.max_nspect = 1;
  bb.max_ndep = 1;
  bb.precision = PYRH_FP64;
  bb.total_depth = natm;
  bb.ndep = ndep;
  bb.nspect = nspect;
  bb.depth_off = depth_off;
  bb.lam_off = lam_off;
  bb.cont_off = cont_off;
  bb.lambda = lambda;
  bb.ne = ne_c;
  bb.nHmin = nHmin;
  bb.nH2 = iH2 >= 0 ? nmol_d + (size_t)iH2 * natm : nullptr;
  bb.nOH = iOH >= 0 ? nmol_d + (size_t)iOH * natm : nullptr;
  bb.nCH = iCH >= 0 ? nmol_d + (size_t)iCH * natm : nullptr;
  bb.pops = pops;
  bb.chi_c = chi;
  bb.eta_c = eta;
  bb.sca_c = sca;

  pyrh_status s = PYRH_OK;
  int launches = 0;
  const unsigned grid = (unsigned)((natm + kThreads - 1) / kThreads);
  cudaMemcpyAsync(nuc_atom, nuc_atom_h, sizeof(int) * nnuc, cudaMemcpyHostToDevice, st);
  hse_bg_layout_kernel<<<grid, kThreads, 0, st>>>(natm, ndep, nspect, depth_off, lam_off,
                                                  cont_off, lambda);
  ++launches;
  for (int k = 0; k < b->ndep && s == PYRH_OK; ++k) {
    const double* Tl = b->T + (size_t)k * natm;
    double* nHl = B.nHtot + (size_t)k * natm;
    hse_start_kernel<<<grid, kThreads, 0, st>>>(*cfg, B, k, active, iter);
    ++launches;
    bb.T = Tl;
    for (int pass = 0; pass < cfg->nmax_iter; ++pass) {
      s = small_batch(natm) ? pyrh::solve_ne_warp(tables, natm, Tl, nHl, ne_c, 2, nullptr, st)
                            : pyrh_solve_ne(tables, natm, Tl, nHl, ne_c, 2, nullptr, st);
      if (s != PYRH_OK) break;
      launches += pyrh_last_launch_count();
      s = equilibria_core(tables, mol, nmol, A, nnuc, nuc_atom, natm, Tl, ne_c, nHl, pops, fn0,
                          nmol_d, nHmin, nnuc_d, st, launches);
      if (s != PYRH_OK) break;
      s = pyrh_background(bg, &bb, stream);
      if (s != PYRH_OK) break;
      launches += pyrh_last_launch_count();
      cudaMemsetAsync(still, 0, sizeof(int32_t), st);
      hse_update_kernel<<<grid, kThreads, 0, st>>>(*cfg, B, k, ne_c, chi, active, iter, still);
      ++launches;
      cudaMemcpyAsync(still_h, still, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
      const cudaError_t e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) {
        pyrh::set_error("hse: %s", cudaGetErrorString(e));
        s = PYRH_ERR_CUDA;
        break;
      }
      if (*still_h == 0) break;
    }
  }
  const cudaError_t e = cudaGetLastError();
  if (s == PYRH_OK && e != cudaSuccess) {
    pyrh::set_error("hse: %s", cudaGetErrorString(e));
    s = PYRH_ERR_CUDA;
  }
  cudaStreamSynchronize(st);
  if (op_tmp) cudaFree(op_tmp);
  cudaFree(S.base);
  cudaFreeHost(still_h);
  pyrh::set_launches(launches);
  return s;
}
