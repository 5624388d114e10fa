// capi.cu -- extern "C" entry points of libpyrh_gb300.so (include/pyrh_gb300.h).
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "../../include/pyrh_gb300.h"
#include "lte_stokes.cuh"

namespace {

thread_local char g_err[512] = "";
int g_last_launches = 0;

pyrh_status fail(pyrh_status s, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return s;
}

#define CUDA_TRY(x)                                                                   \
  do {                                                                                \
    cudaError_t e_ = (x);                                                             \
    if (e_ != cudaSuccess)                                                            \
      return fail(PYRH_ERR_CUDA, "%s failed: %s", #x, cudaGetErrorString(e_));        \
  } while (0)

int round_up(int x, int m) { return (x + m - 1) / m * m; }

pyrh_status check_lines_host(const pyrh_line* lines, int nline, int stokes_mode) {
  for (int l = 0; l < nline; ++l) {
    const pyrh_line& L = lines[l];
    if (L.ncomp < 0 || L.ncomp > PYRH_MAX_COMPONENTS)
      return fail(PYRH_ERR_ARG, "line %d: ncomp %d outside [0, %d]", l, L.ncomp,
                  PYRH_MAX_COMPONENTS);
    if (!(L.lambda0 > 0.0) || !(L.weight > 0.0) || !(L.Bji > 0.0))
      return fail(PYRH_ERR_ARG, "line %d: non-positive lambda0, weight or Bji", l);
    for (int c = 0; c < L.ncomp; ++c)
      if (L.comp_q[c] < -1 || L.comp_q[c] > 1)
        return fail(PYRH_ERR_ARG, "line %d component %d: q = %d", l, c, L.comp_q[c]);
    if (l > 0 && lines[l].lambda0 < lines[l - 1].lambda0)
      return fail(PYRH_ERR_ARG, "lines must be sorted by lambda0 (background.c:293)");
  }
  (void)stokes_mode;
  return PYRH_OK;
}

pyrh_status check_cfg(const pyrh_lte_config* cfg) {
  if (!cfg) return fail(PYRH_ERR_ARG, "cfg is NULL");
  if (cfg->precision != PYRH_FP64 && cfg->precision != PYRH_FP32)
    return fail(PYRH_ERR_ARG, "precision %d", cfg->precision);
  if (cfg->stokes_mode != PYRH_FULL_STOKES && cfg->stokes_mode != PYRH_NO_STOKES)
    return fail(PYRH_ERR_ARG, "stokes_mode %d", cfg->stokes_mode);
  if (!(cfg->mu > 0.0 && cfg->mu <= 1.0)) return fail(PYRH_ERR_ARG, "mu %g outside (0, 1]", cfg->mu);
  if (!(cfg->vmicro_char >= 0.0)) return fail(PYRH_ERR_ARG, "vmicro_char %g", cfg->vmicro_char);
  if (cfg->block_lambda < 0 || cfg->block_lambda > 256 || (cfg->block_lambda % 32))
    return fail(PYRH_ERR_ARG, "block_lambda %d must be 0 or a multiple of 32 <= 256",
                cfg->block_lambda);
  return PYRH_OK;
}

pyrh_status check_batch_shape(const pyrh_lte_batch* b, int nline) {
  if (!b) return fail(PYRH_ERR_ARG, "batch is NULL");
  if (b->natm < 1) return fail(PYRH_ERR_ARG, "natm %d", b->natm);
  if (b->max_ndep < 3 || b->max_ndep > PYRH_MAX_DEPTH)
    return fail(PYRH_ERR_ARG, "max_ndep %d outside [3, %d]", b->max_ndep, PYRH_MAX_DEPTH);
  if (b->max_nlam < 1) return fail(PYRH_ERR_ARG, "max_nlam %d", b->max_nlam);
  if (b->total_depth < b->max_ndep) return fail(PYRH_ERR_ARG, "total_depth %lld", (long long)b->total_depth);
  if (nline < 0 || nline > PYRH_MAX_LINES)
    return fail(PYRH_ERR_ARG, "nline %d outside [0, %d]", nline, PYRH_MAX_LINES);
  const void* ptrs[] = {b->ndep, b->depth_off, b->nlam, b->lam_off, b->cont_off, b->lambda,
                        b->height, b->T, b->ne, b->nHtot, b->np, b->vturb, b->vlos, b->B,
                        b->gamma_B, b->chi_B, b->chi_c, b->eta_c};
  for (const void* p : ptrs)
    if (!p) return fail(PYRH_ERR_ARG, "a batch array pointer is NULL");
  if (nline > 0 && !b->line_pops) return fail(PYRH_ERR_ARG, "line_pops is NULL");
  return PYRH_OK;
}

// Dynamic shared memory a block of these kernels may use on the current
// device: the opt-in maximum per block less 1 KB for static shared memory
// (200 KB where the device cannot be queried).
size_t smem_limit() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
      v <= 2048) {
    cudaGetLastError();
    return 200 * 1024;
  }
  return (size_t)v - 1024;
}

pyrh::LteArgs make_args(const pyrh_lte_batch* b, const pyrh_line* d_lines, int nline,
                        const pyrh_lte_config* cfg, void* out, int block) {
  pyrh::LteArgs a;
  a.natm = b->natm;
  a.tiles = (b->max_nlam + block - 1) / block;
  a.maxd = b->max_ndep;
  a.nline = nline;
  a.precision = cfg->precision;
  a.stokes_mode = cfg->stokes_mode;
  a.magneto_optical = cfg->magneto_optical ? 1 : 0;
  a.moving = cfg->moving ? 1 : 0;
  a.mu = cfg->mu;
  a.vmicro_char = cfg->vmicro_char;
  a.total_depth = b->total_depth;
  a.ndep = b->ndep; a.nlam = b->nlam;
  a.depth_off = b->depth_off; a.lam_off = b->lam_off; a.cont_off = b->cont_off;
  a.lambda = b->lambda; a.height = b->height; a.T = b->T; a.ne = b->ne;
  a.nHtot = b->nHtot; a.np = b->np; a.vturb = b->vturb; a.vlos = b->vlos; a.B = b->B;
  a.gamma_B = b->gamma_B; a.chi_B = b->chi_B; a.line_pops = b->line_pops;
  a.chi_c = b->chi_c; a.eta_c = b->eta_c;
  a.lines = d_lines;
  a.out = out;
  return a;
}

int default_block(int max_nlam, int requested) {
  if (requested > 0) return requested;
  int b = round_up(max_nlam, 32);
  if (b > 256) {
    // split into equal tiles of at most 256 wavelengths
    int tiles = (max_nlam + 255) / 256;
    b = round_up((max_nlam + tiles - 1) / tiles, 32);
  }
  return b < 32 ? 32 : b;
}

pyrh_status launch(const pyrh_lte_batch* b, const pyrh_line* d_lines, int nline,
                   const pyrh_lte_config* cfg, void* out, cudaStream_t st) {
  const int block = default_block(b->max_nlam, cfg->block_lambda);
  pyrh::LteArgs a = make_args(b, d_lines, nline, cfg, out, block);
  const size_t smem = pyrh::lte_smem_bytes(cfg->precision, nline, a.maxd, block);
  if (smem > smem_limit())
    return fail(PYRH_ERR_UNSUPPORTED, "shared memory %zu B for %d lines x %d depths", smem,
                nline, a.maxd);
  // One block per (atmosphere, wavelength tile) by default: a block that
  // finishes early frees its SM slot for the next one, where a persistent
  // grid would make its warps wait at the next work item's barrier
  // (measured 18.9 ms against 22.2 ms for 16384 atmospheres x 224 lambda).
  // persistent_blocks > 0 caps the grid; blocks then loop over work items.
  const long long work = (long long)a.natm * a.tiles;
  long long grid = cfg->persistent_blocks > 0 ? cfg->persistent_blocks : work;
  if (grid > work) grid = work;
  if (grid > 0x7fffffffLL) grid = 0x7fffffffLL;
  cudaError_t e = pyrh::launch_lte_stokes(a, block, (int)grid, st);
  if (e != cudaSuccess) return fail(PYRH_ERR_CUDA, "lte_stokes launch: %s", cudaGetErrorString(e));
  g_last_launches = 1;
  return PYRH_OK;
}

pyrh_status check_rf(const pyrh_lte_batch* b, const pyrh_lte_config* cfg, int nline,
                     const pyrh_line* lines) {
  pyrh_status s = check_cfg(cfg);
  if (s != PYRH_OK) return s;
  s = check_batch_shape(b, nline);
  if (s != PYRH_OK) return s;
  if (nline > 0 && !lines) return fail(PYRH_ERR_ARG, "lines is NULL");
  if (cfg->magneto_optical)
    return fail(PYRH_ERR_UNSUPPORTED,
                "response functions without magneto-optical terms only");
  if (b->max_ndep > PYRH_RF_MAX_DEPTH)
    return fail(PYRH_ERR_UNSUPPORTED, "max_ndep %d above PYRH_RF_MAX_DEPTH %d", b->max_ndep,
                PYRH_RF_MAX_DEPTH);
  if (cfg->block_lambda > pyrh::rf_max_threads(cfg->precision))
    return fail(PYRH_ERR_ARG, "block_lambda %d above %d for response functions",
                cfg->block_lambda, pyrh::rf_max_threads(cfg->precision));
  return PYRH_OK;
}

pyrh_status launch_rf(const pyrh_lte_batch* b, const pyrh_line* d_lines, int nline,
                      const pyrh_lte_config* cfg, int mode, const void* obs, const void* weights,
                      void* stokes_out, void* rf, void* chi2, void* grad, void* rf_gf,
                      void* grad_gf, cudaStream_t st) {
  const int block = cfg->block_lambda > 0 ? cfg->block_lambda : 128;
  pyrh::RfArgs ra;
  ra.lte = make_args(b, d_lines, nline, cfg, stokes_out, block);
  ra.mode = mode;
  ra.obs = obs;
  ra.weights = weights;
  ra.rf = rf;
  ra.chi2 = chi2;
  ra.grad = grad;
  ra.rf_gf = rf_gf;
  ra.grad_gf = grad_gf;
  if (b->setup_dT) ra.dT = *b->setup_dT;
  else memset(&ra.dT, 0, sizeof(ra.dT));
  const size_t smem = pyrh::rf_smem_bytes(cfg->precision, nline, ra.lte.maxd);
  if (smem > smem_limit())
    return fail(PYRH_ERR_UNSUPPORTED, "shared memory %zu B for %d lines x %d depths", smem,
                nline, ra.lte.maxd);
  // Sub-blocks (one work item each) per block: in FP32 one block holds the
  // registers of a whole SM, so that the barrier between the forward and
  // reverse sweeps aligns every resident warp; fewer where their shared
  // tables do not fit together.
  int sub = pyrh::rf_max_threads(cfg->precision, mode) / block;
  if (sub < 1) return fail(PYRH_ERR_ARG, "block_lambda %d too wide for this mode", block);
  while (sub > 1 && smem * sub > smem_limit()) --sub;
  ra.sub = sub;
  const long long work = (long long)ra.lte.natm * ra.lte.tiles;
  const long long blocks = (work + sub - 1) / sub;
  long long grid = cfg->persistent_blocks > 0 ? cfg->persistent_blocks : blocks;
  if (grid > blocks) grid = blocks;
  if (grid > 0x7fffffffLL) grid = 0x7fffffffLL;
  cudaError_t e = pyrh::launch_lte_rf(ra, block, (int)grid, st);
  if (e != cudaSuccess) return fail(PYRH_ERR_CUDA, "lte_rf launch: %s", cudaGetErrorString(e));
  return PYRH_OK;
}

// Workspace of the host-buffer entry point: device buffers cached between
// calls, and four streams (host-to-device copies, two for kernels,
// device-to-host copies) with per-chunk events for the pipelined upload.
struct HostWs {
  std::mutex mu;
  cudaStream_t stream = nullptr;      // host-to-device copies
  cudaStream_t kstream[2] = {};       // kernels of even and odd chunks
  cudaStream_t ostream = nullptr;     // device-to-host copies
  std::vector<cudaEvent_t> ev_in, ev_k;
  std::vector<void*> bufs;
  std::vector<size_t> caps;
  cudaError_t init(int nchunk) {
    cudaError_t e = cudaSuccess;
    for (cudaStream_t* s : {&stream, &kstream[0], &kstream[1], &ostream})
      if (!*s && (e = cudaStreamCreateWithFlags(s, cudaStreamNonBlocking)) != cudaSuccess) return e;
    while ((int)ev_in.size() < nchunk) {
      cudaEvent_t a, b;
      if ((e = cudaEventCreateWithFlags(&a, cudaEventDisableTiming)) != cudaSuccess) return e;
      if ((e = cudaEventCreateWithFlags(&b, cudaEventDisableTiming)) != cudaSuccess) return e;
      ev_in.push_back(a);
      ev_k.push_back(b);
    }
    return e;
  }
  void* get(int slot, size_t bytes, cudaError_t* err) {
    if ((int)bufs.size() <= slot) { bufs.resize(slot + 1, nullptr); caps.resize(slot + 1, 0); }
    if (caps[slot] < bytes) {
      if (bufs[slot]) cudaFree(bufs[slot]);
      bufs[slot] = nullptr;
      caps[slot] = 0;
      *err = cudaMalloc(&bufs[slot], bytes);
      if (*err != cudaSuccess) return nullptr;
      caps[slot] = bytes;
    }
    return bufs[slot];
  }
};
HostWs g_ws;

}  // namespace

namespace pyrh {
void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
void set_launches(int n) { g_last_launches = n; }
}  // namespace pyrh

extern "C" {

const char* pyrh_version(void) { return "pyrh_gb300 0.1 (sm_103a)"; }
const char* pyrh_last_error(void) { return g_err; }
int32_t pyrh_last_launch_count(void) { return g_last_launches; }

pyrh_status pyrh_lte_stokes(const pyrh_lte_batch* batch, const pyrh_line* lines, int32_t nline,
                            const pyrh_lte_config* cfg, void* stokes_out, void* stream) {
  g_last_launches = 0;
  pyrh_status s = check_cfg(cfg);
  if (s != PYRH_OK) return s;
  s = check_batch_shape(batch, nline);
  if (s != PYRH_OK) return s;
  if (!stokes_out) return fail(PYRH_ERR_ARG, "stokes_out is NULL");
  if (nline > 0 && !lines) return fail(PYRH_ERR_ARG, "lines is NULL");
  // The line table lives in device memory and is not read back here (that
  // would synchronise the stream); pyrh_check_lines validates a host copy,
  // and the kernel clamps component counts to PYRH_MAX_COMPONENTS.
  return launch(batch, lines, nline, cfg, stokes_out, (cudaStream_t)stream);
}

pyrh_status pyrh_lte_rf(const pyrh_lte_batch* batch, const pyrh_line* lines, int32_t nline,
                        const pyrh_lte_config* cfg, void* stokes_out, void* rf_out,
                        void* rf_loggf_out, void* stream) {
  g_last_launches = 0;
  pyrh_status s = check_rf(batch, cfg, nline, lines);
  if (s != PYRH_OK) return s;
  if (!stokes_out || !rf_out) return fail(PYRH_ERR_ARG, "stokes_out or rf_out is NULL");
  s = launch_rf(batch, lines, nline, cfg, 0, nullptr, nullptr, stokes_out, rf_out, nullptr,
                nullptr, rf_loggf_out, nullptr, (cudaStream_t)stream);
  if (s == PYRH_OK) g_last_launches = 1;
  return s;
}

pyrh_status pyrh_lte_chi2_grad(const pyrh_lte_batch* batch, const pyrh_line* lines,
                               int32_t nline, const pyrh_lte_config* cfg, const void* obs,
                               const void* weights, void* stokes_out, void* chi2_out,
                               void* grad_out, void* grad_loggf_out, void* stream) {
  g_last_launches = 0;
  pyrh_status s = check_rf(batch, cfg, nline, lines);
  if (s != PYRH_OK) return s;
  if (!obs || !weights || !stokes_out || !chi2_out || !grad_out)
    return fail(PYRH_ERR_ARG, "obs, weights, stokes_out, chi2_out or grad_out is NULL");
  const size_t real = cfg->precision == PYRH_FP32 ? sizeof(float) : sizeof(double);
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(cudaMemsetAsync(chi2_out, 0, real * batch->natm, st));
  CUDA_TRY(cudaMemsetAsync(grad_out, 0, real * PYRH_RF_NPARAM * batch->total_depth, st));
  if (grad_loggf_out) CUDA_TRY(cudaMemsetAsync(grad_loggf_out, 0, real * batch->natm * nline, st));
  s = launch_rf(batch, lines, nline, cfg, 1, obs, weights, stokes_out, nullptr, chi2_out, grad_out,
                nullptr, grad_loggf_out, st);
  if (s == PYRH_OK) g_last_launches = 1;
  return s;
}

pyrh_status pyrh_lte_stokes_vjp(const pyrh_lte_batch* batch, const pyrh_line* lines,
                                int32_t nline, const pyrh_lte_config* cfg,
                                const void* dL_dstokes, void* stokes_out, void* grad_out,
                                void* grad_loggf_out, void* stream) {
  g_last_launches = 0;
  pyrh_status s = check_rf(batch, cfg, nline, lines);
  if (s != PYRH_OK) return s;
  if (!dL_dstokes || !stokes_out || !grad_out)
    return fail(PYRH_ERR_ARG, "dL_dstokes, stokes_out or grad_out is NULL");
  const size_t real = cfg->precision == PYRH_FP32 ? sizeof(float) : sizeof(double);
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(cudaMemsetAsync(grad_out, 0, real * PYRH_RF_NPARAM * batch->total_depth, st));
  if (grad_loggf_out) CUDA_TRY(cudaMemsetAsync(grad_loggf_out, 0, real * batch->natm * nline, st));
  s = launch_rf(batch, lines, nline, cfg, 2, nullptr, dL_dstokes, stokes_out, nullptr, nullptr,
                grad_out, nullptr, grad_loggf_out, st);
  if (s == PYRH_OK) g_last_launches = 1;
  return s;
}

struct pyrh_lte_plan_s {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int block = 0;
  double ms = 0.0;
};

pyrh_status pyrh_lte_plan_create(const pyrh_lte_batch* batch, const pyrh_line* lines,
                                 int32_t nline, const pyrh_lte_config* cfg, void* stokes_out,
                                 void* stream, pyrh_lte_plan* plan_out) {
  g_last_launches = 0;
  if (!plan_out) return fail(PYRH_ERR_ARG, "plan_out is NULL");
  *plan_out = nullptr;
  pyrh_status s = check_cfg(cfg);
  if (s != PYRH_OK) return s;
  s = check_batch_shape(batch, nline);
  if (s != PYRH_OK) return s;
  if (!stokes_out) return fail(PYRH_ERR_ARG, "stokes_out is NULL");
  if (nline > 0 && !lines) return fail(PYRH_ERR_ARG, "lines is NULL");
  cudaStream_t own = nullptr;
  cudaStream_t st = (cudaStream_t)stream;
  if (!st) {
    CUDA_TRY(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
    st = own;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  pyrh_lte_config c = *cfg;
  auto cleanup = [&]() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (own) cudaStreamDestroy(own);
  };
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cleanup();
    return fail(PYRH_ERR_CUDA, "event creation failed");
  }
  // ---- tune the wavelength tile on the caller's buffers ----
  const int widest = round_up(batch->max_nlam, 32);
  int best = 0;
  double best_ms = 0.0;
  for (int blk = 32; blk <= 256 && blk <= (widest < 32 ? 32 : widest); blk += 32) {
    c.block_lambda = blk;
    s = launch(batch, lines, nline, &c, stokes_out, st);   // first launch sets up the kernel
    if (s != PYRH_OK) { cleanup(); return s; }
    cudaEventRecord(e0, st);
    for (int r = 0; r < 3; ++r) {
      s = launch(batch, lines, nline, &c, stokes_out, st);
      if (s != PYRH_OK) { cleanup(); return s; }
    }
    cudaEventRecord(e1, st);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e != cudaSuccess) {
      cleanup();
      return fail(PYRH_ERR_CUDA, "tuning: %s", cudaGetErrorString(e));
    }
    if (!best || ms / 3.0 < best_ms) { best = blk; best_ms = ms / 3.0; }
  }
  // ---- record the tuned launch as a graph ----
  c.block_lambda = best;
  pyrh_lte_plan plan = new pyrh_lte_plan_s;
  plan->block = best;
  plan->ms = best_ms;
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    s = launch(batch, lines, nline, &c, stokes_out, st);
    cudaError_t e2 = cudaStreamEndCapture(st, &plan->graph);
    if (s == PYRH_OK && e2 != cudaSuccess) e = e2;
  }
  if (e == cudaSuccess && s == PYRH_OK) e = cudaGraphInstantiate(&plan->exec, plan->graph, 0);
  cleanup();
  if (e != cudaSuccess || s != PYRH_OK) {
    pyrh_lte_plan_destroy(plan);
    if (s != PYRH_OK) return s;
    return fail(PYRH_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  }
  g_last_launches = 1;
  *plan_out = plan;
  return PYRH_OK;
}

pyrh_status pyrh_lte_plan_launch(pyrh_lte_plan plan, void* stream) {
  g_last_launches = 0;
  if (!plan || !plan->exec) return fail(PYRH_ERR_ARG, "plan is NULL");
  CUDA_TRY(cudaGraphLaunch(plan->exec, (cudaStream_t)stream));
  g_last_launches = 1;
  return PYRH_OK;
}

int32_t pyrh_lte_plan_block(pyrh_lte_plan plan) { return plan ? plan->block : 0; }
double pyrh_lte_plan_ms(pyrh_lte_plan plan) { return plan ? plan->ms : 0.0; }

void pyrh_lte_plan_destroy(pyrh_lte_plan plan) {
  if (!plan) return;
  if (plan->exec) cudaGraphExecDestroy(plan->exec);
  if (plan->graph) cudaGraphDestroy(plan->graph);
  delete plan;
}

pyrh_status pyrh_check_lines(const pyrh_line* host_lines, int32_t nline, int32_t stokes_mode) {
  if (nline < 0 || nline > PYRH_MAX_LINES)
    return fail(PYRH_ERR_ARG, "nline %d outside [0, %d]", nline, PYRH_MAX_LINES);
  if (nline > 0 && !host_lines) return fail(PYRH_ERR_ARG, "host_lines is NULL");
  return check_lines_host(host_lines, nline, stokes_mode);
}

pyrh_status pyrh_lte_stokes_host(const pyrh_lte_batch* hb, const pyrh_line* host_lines,
                                 int32_t nline, const pyrh_lte_config* cfg,
                                 void* host_stokes_out) {
  g_last_launches = 0;
  pyrh_status s = check_cfg(cfg);
  if (s != PYRH_OK) return s;
  s = check_batch_shape(hb, nline);
  if (s != PYRH_OK) return s;
  if (!host_stokes_out) return fail(PYRH_ERR_ARG, "host_stokes_out is NULL");
  if (nline > 0) {
    if (!host_lines) return fail(PYRH_ERR_ARG, "host_lines is NULL");
    s = check_lines_host(host_lines, nline, cfg->stokes_mode);
    if (s != PYRH_OK) return s;
  }
  const int natm = hb->natm;
  long long nlam_tot = 0, cont_tot = 0;
  // atmospheres whose continuum and spectrum follow each other in memory
  // can be uploaded and synthesised in chunks that overlap
  bool ordered = true;
  for (int p = 0; p < natm; ++p) {
    const long long e = hb->lam_off[p] + hb->nlam[p];
    if (e > nlam_tot) nlam_tot = e;
    const long long c = hb->cont_off[p] + (long long)hb->ndep[p] * hb->nlam[p];
    if (c > cont_tot) cont_tot = c;
    if (hb->ndep[p] < 3 || hb->ndep[p] > hb->max_ndep || hb->nlam[p] < 1 ||
        hb->nlam[p] > hb->max_nlam || hb->depth_off[p] + hb->ndep[p] > hb->total_depth)
      return fail(PYRH_ERR_ARG, "atmosphere %d: inconsistent ndep/nlam/offsets", p);
    if (p > 0 && (hb->cont_off[p] < hb->cont_off[p - 1] + (long long)hb->ndep[p - 1] * hb->nlam[p - 1] ||
                  hb->lam_off[p] < hb->lam_off[p - 1] + hb->nlam[p - 1] ||
                  hb->depth_off[p] < hb->depth_off[p - 1] + hb->ndep[p - 1]))
      ordered = false;
  }
  const size_t real = cfg->precision == PYRH_FP32 ? sizeof(float) : sizeof(double);
  // about 128 MB of continuum per chunk, at most 16 chunks, after a lead
  // chunk of an eighth of that size whose short upload is all that the
  // first launch waits for
  const long long cont_bytes = 2LL * (long long)real * cont_tot;
  int neq = ordered ? (int)(cont_bytes / (128LL << 20)) : 1;
  if (neq > 16) neq = 16;
  if (neq < 1) neq = 1;
  std::vector<int> pb(1, 0);   // chunk c holds atmospheres [pb[c], pb[c+1])
  int lead = 0;
  if (neq > 1) {
    lead = (int)((long long)natm / (8LL * neq));
    if (lead > 0) pb.push_back(lead);
  }
  for (int c = 1; c <= neq; ++c) {
    const int e = lead + (int)((long long)(natm - lead) * c / neq);
    if (e > pb.back()) pb.push_back(e);
  }
  const int nchunk = (int)pb.size() - 1;
  std::lock_guard<std::mutex> lock(g_ws.mu);
  CUDA_TRY(g_ws.init(nchunk));
  cudaError_t err = cudaSuccess;
  pyrh_lte_batch db = *hb;
  db.setup_dT = nullptr;   // the forward synthesis does not read it
  int slot = 0;
  auto up = [&](const void* src, size_t bytes) -> void* {
    void* d = g_ws.get(slot++, bytes, &err);
    if (!d) return nullptr;
    err = cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, g_ws.stream);
    return err == cudaSuccess ? d : nullptr;
  };
#define UP(field, bytes)                                                       \
  do {                                                                         \
    db.field = (decltype(db.field))up(hb->field, bytes);                       \
    if (!db.field) return fail(PYRH_ERR_CUDA, "upload %s: %s", #field,         \
                               cudaGetErrorString(err));                       \
  } while (0)
  UP(ndep, sizeof(int32_t) * natm);
  UP(depth_off, sizeof(int64_t) * natm);
  UP(nlam, sizeof(int32_t) * natm);
  UP(lam_off, sizeof(int64_t) * natm);
  UP(cont_off, sizeof(int64_t) * natm);
#undef UP
  pyrh_line* d_lines = nullptr;
  if (nline > 0) {
    d_lines = (pyrh_line*)up(host_lines, sizeof(pyrh_line) * nline);
    if (!d_lines) return fail(PYRH_ERR_CUDA, "upload lines: %s", cudaGetErrorString(err));
  }
  // Device arrays for the per-depth, per-wavelength and continuum data; each
  // chunk uploads its own ranges of them.
  const long long ndt = hb->total_depth;
  const double* const* hdepth[10] = {&hb->height, &hb->T, &hb->ne, &hb->nHtot, &hb->np,
                                     &hb->vturb, &hb->vlos, &hb->B, &hb->gamma_B, &hb->chi_B};
  const double** ddepth[10] = {&db.height, &db.T, &db.ne, &db.nHtot, &db.np,
                               &db.vturb, &db.vlos, &db.B, &db.gamma_B, &db.chi_B};
  for (int f = 0; f < 10; ++f) {
    *ddepth[f] = (const double*)g_ws.get(slot++, sizeof(double) * ndt, &err);
    if (!*ddepth[f]) return fail(PYRH_ERR_CUDA, "depth buffers: %s", cudaGetErrorString(err));
  }
  if (nline > 0) {
    db.line_pops = (const double*)g_ws.get(slot++, sizeof(double) * ndt * 2 * nline, &err);
    if (!db.line_pops) return fail(PYRH_ERR_CUDA, "line_pops buffer: %s", cudaGetErrorString(err));
  }
  db.lambda = (const double*)g_ws.get(slot++, sizeof(double) * nlam_tot, &err);
  if (!db.lambda) return fail(PYRH_ERR_CUDA, "lambda buffer: %s", cudaGetErrorString(err));
  unsigned char* d_chi = (unsigned char*)g_ws.get(slot++, real * cont_tot, &err);
  unsigned char* d_eta = d_chi ? (unsigned char*)g_ws.get(slot++, real * cont_tot, &err) : nullptr;
  if (!d_eta) return fail(PYRH_ERR_CUDA, "continuum buffers: %s", cudaGetErrorString(err));
  db.chi_c = d_chi;
  db.eta_c = d_eta;
  const size_t out_bytes = real * 4 * nlam_tot;
  unsigned char* d_out = (unsigned char*)g_ws.get(slot++, out_bytes, &err);
  if (!d_out) return fail(PYRH_ERR_CUDA, "output buffer: %s", cudaGetErrorString(err));
  auto h2d = [&](const void* dst, const void* src, size_t bytes) {
    return cudaMemcpyAsync(const_cast<void*>(dst), src, bytes, cudaMemcpyHostToDevice,
                           g_ws.stream);
  };
  // Chunk c: upload its depths, wavelengths and continuum (copy stream),
  // synthesise its atmospheres once the upload is done (kernel stream
  // c % 2), copy its spectra back (output stream).  Chunk c+1's upload runs
  // under chunk c's kernel, and with two kernel streams chunk c+1's blocks
  // fill the SMs that chunk c's last, partial wave leaves idle.
  const unsigned char* h_chi = (const unsigned char*)hb->chi_c;
  const unsigned char* h_eta = (const unsigned char*)hb->eta_c;
  for (int c = 0; c < nchunk; ++c) {
    const int p0 = pb[c], p1 = pb[c + 1];
    const bool whole = nchunk == 1;   // also the layout without ordered offsets
    const long long c0 = whole ? 0 : hb->cont_off[p0];
    const long long c1 = whole ? cont_tot
                               : hb->cont_off[p1 - 1] + (long long)hb->ndep[p1 - 1] * hb->nlam[p1 - 1];
    const long long d0 = whole ? 0 : hb->depth_off[p0];
    const long long d1 = whole ? ndt : hb->depth_off[p1 - 1] + hb->ndep[p1 - 1];
    const long long l0 = whole ? 0 : hb->lam_off[p0];
    const long long l1 = whole ? nlam_tot : hb->lam_off[p1 - 1] + hb->nlam[p1 - 1];
    for (int f = 0; f < 10; ++f)
      CUDA_TRY(h2d(*ddepth[f] + d0, *hdepth[f] + d0, sizeof(double) * (d1 - d0)));
    for (long long r = 0; r < 2LL * nline; ++r)
      CUDA_TRY(h2d(db.line_pops + r * ndt + d0, hb->line_pops + r * ndt + d0,
                   sizeof(double) * (d1 - d0)));
    CUDA_TRY(h2d(db.lambda + l0, hb->lambda + l0, sizeof(double) * (l1 - l0)));
    CUDA_TRY(h2d(d_chi + real * c0, h_chi + real * c0, real * (c1 - c0)));
    CUDA_TRY(h2d(d_eta + real * c0, h_eta + real * c0, real * (c1 - c0)));
    CUDA_TRY(cudaEventRecord(g_ws.ev_in[c], g_ws.stream));
    cudaStream_t ks = g_ws.kstream[c & 1];
    CUDA_TRY(cudaStreamWaitEvent(ks, g_ws.ev_in[c], 0));
    pyrh_lte_batch cb = db;   // atmospheres [p0, p1): offsets stay absolute
    cb.natm = p1 - p0;
    cb.ndep = db.ndep + p0;
    cb.depth_off = db.depth_off + p0;
    cb.nlam = db.nlam + p0;
    cb.lam_off = db.lam_off + p0;
    cb.cont_off = db.cont_off + p0;
    s = launch(&cb, d_lines, nline, cfg, d_out, ks);
    if (s != PYRH_OK) return s;
    CUDA_TRY(cudaEventRecord(g_ws.ev_k[c], ks));
    CUDA_TRY(cudaStreamWaitEvent(g_ws.ostream, g_ws.ev_k[c], 0));
    // Stokes of atmosphere p occupy [4 lam_off[p], 4 lam_off[p] + 4 nlam[p])
    CUDA_TRY(cudaMemcpyAsync((unsigned char*)host_stokes_out + real * 4 * l0,
                             d_out + real * 4 * l0, real * 4 * (l1 - l0),
                             cudaMemcpyDeviceToHost, g_ws.ostream));
  }
  CUDA_TRY(cudaStreamSynchronize(g_ws.ostream));
  CUDA_TRY(cudaStreamSynchronize(g_ws.kstream[0]));
  CUDA_TRY(cudaStreamSynchronize(g_ws.kstream[1]));
  CUDA_TRY(cudaStreamSynchronize(g_ws.stream));
  g_last_launches = nchunk;
  return PYRH_OK;
}

}  // extern "C"
