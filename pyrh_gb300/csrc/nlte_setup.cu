// nlte_setup.cu -- per-depth set-up of an NLTE batch for one model atom, on
// the device: LTE populations, the collision rate matrix and the Doppler
// widths, for every depth point of every atmosphere in one launch (one
// thread per depth point; the points are independent).
//
// Reference routines restated here (file:line in the reference tree):
//   LTEpops         rh/ltepops.c:33-109 (Saha-Boltzmann from the atom's own
//                   levels; Debye shielding is switched off there)
//   CollisionRate   rh/collision.c:450-700 (OMEGA, CE, CI, CP, CH, CH0, CH+
//                   records interpolated in T on their TEMP grid)
//   splineCoef / splineEval  rh/spline.c (natural cubic spline, clamped
//                   outside the table), Linear rh/linear.c (two points)
//   vbroad          rh/readatom.c:178-186
// The spline moments of each record depend on its table only and are
// computed once on the host; the device evaluates them at each T.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "../../include/pyrh_gb300.h"

namespace pyrh {
void set_error(const char* fmt, ...);
void set_launches(int n);
}

namespace {

constexpr double kH = 6.6260755E-34;
constexpr double kK = 1.380658E-23;
constexpr double kAMU = 1.6605402E-27;
constexpr double kMe = 9.1093897E-31;
constexpr double kERyd = 2.1798741E-18;
constexpr double kRBohr = 5.29177349E-11;
constexpr double kPi = 3.14159265358979;

// Compact device table of one atom: levels, then the collision records,
// then the records' temperatures, values and spline moments.
struct SetupLevel {
  double E, g;
  int stage, pad;
};
struct SetupRecord {
  int type, i, j, ntemp;
  int64_t temp, value, moment;    // offsets into the value pool
};
struct SetupTable {
  int nlevel, nrec;
  double weight;                  // atomic weight (amu)
  const SetupLevel* level;
  const SetupRecord* rec;
  const double* pool;
};

// splineCoef of rh/spline.c for one table (moments M, natural ends)
void spline_moments(int N, const double* x, const double* y, double* M) {
  std::vector<double> u(N);
  double* q = M;
  double hj = x[1] - x[0];
  double D = (y[1] - y[0]) / hj;
  q[0] = u[0] = 0.0;
  for (int j = 1; j < N - 1; j++) {
    const double hj1 = x[j + 1] - x[j];
    const double mu = hj / (hj + hj1);
    const double D1 = (y[j + 1] - y[j]) / hj1;
    const double p = mu * q[j - 1] + 2;
    q[j] = (mu - 1) / p;
    u[j] = ((D1 - D) * 6 / (hj + hj1) - mu * u[j - 1]) / p;
    hj = hj1;
    D = D1;
  }
  M[N - 1] = 0.0;
  for (int j = N - 2; j >= 0; j--) M[j] = q[j] * M[j + 1] + u[j];
}

// splineEval (N > 2) or Linear (N == 2) of rh/spline.c, rh/linear.c at T;
// the temperature tables are ascending.
__device__ double interp_T(int N, const double* x, const double* y, const double* M, double T) {
  if (T <= x[0]) return y[0];
  if (T >= x[N - 1]) return y[N - 1];
  int lo = 0, hi = N;
  while (hi - lo > 1) {
    const int mid = (hi + lo) >> 1;
    if (T >= x[mid]) lo = mid;
    else hi = mid;
  }
  const int j = lo;
  if (N > 2) {
    const double hj = x[j + 1] - x[j];
    const double fx = (T - x[j]) / hj;
    const double fx1 = 1 - fx;
    return fx1 * y[j] + fx * y[j + 1] +
           (fx1 * ((fx1) * (fx1)-1) * M[j] + fx * ((fx) * (fx)-1) * M[j + 1]) * ((hj) * (hj)) /
               6.0;
  }
  const double fx = (x[j + 1] - T) / (x[j + 1] - x[j]);
  return fx * y[j] + (1 - fx) * y[j + 1];
}

__global__ void nlte_setup_kernel(SetupTable tab, pyrh_nlte_setup_batch b, int32_t* err) {
  const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= b.total_depth) return;
  const int nl = tab.nlevel;
  const double T = b.T[d], ne = b.ne[d];
  // ---- LTEpops (ltepops.c:80-103)
  double nst[PYRH_ATOM_MAX_LEVELS];
  const double c1 = (kH / (2.0 * kPi * kMe)) * (kH / kK);
  const double cNe_T = 0.5 * ne * pow(c1 / T, 1.5);
  double sum = 1.0;
  for (int i = 1; i < nl; i++) {
    const double dE = tab.level[i].E - tab.level[0].E;
    const double gi0 = tab.level[i].g / tab.level[0].g;
    const int dZ = tab.level[i].stage - tab.level[0].stage;
    const double dE_kT = dE / (kK * T);
    nst[i] = gi0 * exp(-dE_kT);
    for (int m = 1; m <= dZ; m++) nst[i] /= cNe_T;
    sum += nst[i];
  }
  nst[0] = b.ntotal[d] / sum;
  for (int i = 1; i < nl; i++) nst[i] *= nst[0];
  for (int i = 0; i < nl; i++) b.nstar[(int64_t)i * b.total_depth + d] = nst[i];
  // ---- CollisionRate (collision.c:470-700)
  double* C = b.C;
  const int64_t td = b.total_depth;
  for (int ij = 0; ij < nl * nl; ij++) C[(int64_t)ij * td + d] = 0.0;
  const double C0 = ((kERyd / sqrt(kMe)) * kPi * ((kRBohr) * (kRBohr))) * sqrt(8.0 / (kPi * kK));
  for (int r = 0; r < tab.nrec; r++) {
    const SetupRecord& R = tab.rec[r];
    const int i = R.i, j = R.j;
    const int64_t ij = (int64_t)(i * nl + j) * td + d, ji = (int64_t)(j * nl + i) * td + d;
    const double Cv = interp_T(R.ntemp, tab.pool + R.temp, tab.pool + R.value,
                               tab.pool + R.moment, T);
    switch (R.type) {
      case PYRH_COLL_OMEGA: {
        const double Cdown = C0 * ne * Cv / (tab.level[j].g * sqrt(T));
        C[ij] += Cdown;
        C[ji] += Cdown * nst[j] / nst[i];
        break;
      }
      case PYRH_COLL_CE: {
        const double gij = tab.level[i].g / tab.level[j].g;
        const double Cdown = Cv * ne * gij * sqrt(T);
        C[ij] += Cdown;
        C[ji] += Cdown * nst[j] / nst[i];
        break;
      }
      case PYRH_COLL_CI: {
        const double dE = tab.level[j].E - tab.level[i].E;
        const double Cup = Cv * ne * exp(-dE / (kK * T)) * sqrt(T);
        C[ji] += Cup;
        C[ij] += Cup * nst[i] / nst[j];
        break;
      }
      case PYRH_COLL_CP: {
        if (!b.np) { atomicOr(err, 1); break; }
        const double Cdown = b.np[d] * Cv;
        C[ij] += Cdown;
        C[ji] += Cdown * nst[j] / nst[i];
        break;
      }
      case PYRH_COLL_CH: {
        if (!b.nh0) { atomicOr(err, 1); break; }
        const double Cup = b.nh0[d] * Cv;
        C[ji] += Cup;
        C[ij] += Cup * nst[i] / nst[j];
        break;
      }
      case PYRH_COLL_CH0:
        if (!b.nh0) { atomicOr(err, 1); break; }
        C[ij] += b.nh0[d] * Cv;
        break;
      case PYRH_COLL_CHP:
        if (!b.np) { atomicOr(err, 1); break; }
        C[ji] += b.np[d] * Cv;
        break;
      default:
        atomicOr(err, 2);
    }
  }
  // ---- Doppler width (readatom.c:178-186)
  if (b.vbroad) {
    const double vtherm = 2.0 * kK / (kAMU * tab.weight);
    b.vbroad[d] = sqrt(vtherm * T + ((b.vturb[d]) * (b.vturb[d])));
  }
}

struct HostTable {
  std::vector<SetupLevel> level;
  std::vector<SetupRecord> rec;
  std::vector<double> pool;
};

pyrh_status build_table(const pyrh_atom* a, HostTable& t) {
  t.level.resize(a->nlevel);
  for (int i = 0; i < a->nlevel; ++i)
    t.level[i] = SetupLevel{a->level[i].E, a->level[i].g, a->level[i].stage, 0};
  for (int r = 0; r < a->ncoll; ++r) {
    const pyrh_atom_coll& c = a->coll[r];
    if (c.type == PYRH_COLL_CR) {
      pyrh::set_error("nlte_setup: collision type CR is not supported");
      return PYRH_ERR_UNSUPPORTED;
    }
    if (c.ntemp < 2 || c.i < 0 || c.j >= a->nlevel || c.i == c.j) {
      pyrh::set_error("nlte_setup: collision record %d (%d points, levels %d-%d)", r, c.ntemp,
                      c.i, c.j);
      return PYRH_ERR_ARG;
    }
    const double* x = a->coll_values + c.temp_off;
    const double* y = a->coll_values + c.value_off;
    for (int n = 1; n < c.ntemp; ++n)
      if (!(x[n] > x[n - 1])) {
        pyrh::set_error("nlte_setup: TEMP grid of record %d is not ascending", r);
        return PYRH_ERR_ARG;
      }
    SetupRecord R;
    R.type = c.type;
    R.i = c.i;
    R.j = c.j;
    R.ntemp = c.ntemp;
    R.temp = (int64_t)t.pool.size();
    t.pool.insert(t.pool.end(), x, x + c.ntemp);
    R.value = (int64_t)t.pool.size();
    t.pool.insert(t.pool.end(), y, y + c.ntemp);
    R.moment = (int64_t)t.pool.size();
    t.pool.resize(t.pool.size() + c.ntemp, 0.0);
    if (c.ntemp > 2) spline_moments(c.ntemp, x, y, t.pool.data() + R.moment);
    t.rec.push_back(R);
  }
  return PYRH_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" {

size_t pyrh_nlte_setup_workspace_bytes(const pyrh_atom* atom) {
  if (!atom) return 0;
  size_t vals = 0;
  for (int r = 0; r < atom->ncoll; ++r) vals += 3 * (size_t)atom->coll[r].ntemp;
  return align256(sizeof(SetupLevel) * PYRH_ATOM_MAX_LEVELS) +
         align256(sizeof(SetupRecord) * (atom->ncoll > 0 ? atom->ncoll : 1)) +
         align256(sizeof(double) * (vals > 0 ? vals : 1)) + 256;
}

pyrh_status pyrh_nlte_setup(const pyrh_atom* atom, double weight_amu,
                            const pyrh_nlte_setup_batch* b, void* ws, size_t ws_bytes,
                            void* stream) {
  pyrh::set_launches(0);
  if (!atom || !b || !b->T || !b->ne || !b->ntotal || !b->nstar || !b->C ||
      (b->vbroad && !b->vturb) || b->total_depth < 1) {
    pyrh::set_error("nlte_setup: a required pointer is NULL or the batch is empty");
    return PYRH_ERR_ARG;
  }
  if (atom->nlevel < 2 || atom->nlevel > PYRH_ATOM_MAX_LEVELS || !(weight_amu > 0.0)) {
    pyrh::set_error("nlte_setup: %d levels / atomic weight %g", atom->nlevel, weight_amu);
    return PYRH_ERR_ARG;
  }
  HostTable t;
  pyrh_status s = build_table(atom, t);
  if (s != PYRH_OK) return s;
  const size_t need = pyrh_nlte_setup_workspace_bytes(atom);
  if (!ws || ws_bytes < need) {
    pyrh::set_error("nlte_setup: workspace of %zu bytes is smaller than %zu", ws_bytes, need);
    return PYRH_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(ws);
  const size_t o_lev = 0;
  const size_t o_rec = align256(sizeof(SetupLevel) * PYRH_ATOM_MAX_LEVELS);
  const size_t o_pool = o_rec + align256(sizeof(SetupRecord) * (t.rec.empty() ? 1 : t.rec.size()));
  const size_t o_err = o_pool + align256(sizeof(double) * (t.pool.empty() ? 1 : t.pool.size()));
  // pageable sources: each copy has completed when cudaMemcpyAsync returns
  cudaError_t e = cudaMemcpyAsync(w + o_lev, t.level.data(), sizeof(SetupLevel) * t.level.size(),
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !t.rec.empty())
    e = cudaMemcpyAsync(w + o_rec, t.rec.data(), sizeof(SetupRecord) * t.rec.size(),
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !t.pool.empty())
    e = cudaMemcpyAsync(w + o_pool, t.pool.data(), sizeof(double) * t.pool.size(),
                        cudaMemcpyHostToDevice, st);
  int32_t* err = reinterpret_cast<int32_t*>(w + o_err);
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int32_t), st);
  SetupTable tab;
  tab.nlevel = atom->nlevel;
  tab.nrec = (int)t.rec.size();
  tab.weight = weight_amu;
  tab.level = reinterpret_cast<const SetupLevel*>(w + o_lev);
  tab.rec = reinterpret_cast<const SetupRecord*>(w + o_rec);
  tab.pool = reinterpret_cast<const double*>(w + o_pool);
  if (e == cudaSuccess) {
    const int threads = 128;
    const int64_t blocks = (b->total_depth + threads - 1) / threads;
    nlte_setup_kernel<<<(unsigned)blocks, threads, 0, st>>>(tab, *b, err);
    e = cudaGetLastError();
  }
  int32_t herr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  pyrh::set_launches(1);
  if (e != cudaSuccess) {
    pyrh::set_error("nlte_setup: %s", cudaGetErrorString(e));
    return PYRH_ERR_CUDA;
  }
  if (herr) {
    pyrh::set_error(herr & 1 ? "nlte_setup: proton or hydrogen densities needed (CP, CH, CH0, CH+)"
                             : "nlte_setup: unknown collision type");
    return PYRH_ERR_ARG;
  }
  return PYRH_OK;
}

}  // extern "C"
