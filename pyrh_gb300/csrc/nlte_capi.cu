// nlte_capi.cu -- extern "C" entry points of the NLTE solver.
#include <cuda_runtime.h>
#include <stdio.h>

#include <vector>

#include "../../include/pyrh_gb300.h"
#include "nlte.cuh"

namespace pyrh {
void set_error(const char* fmt, ...);
void set_launches(int n);
}  // namespace pyrh

namespace {

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct Layout {
  size_t wphi, Jnew, gslab, rslab, bgr, Jr, ngprev, count, active, iters, err, any, dpops, phi,
      fixed;
};

int groups_of(const pyrh_nlte_batch* b, const pyrh_nlte_config* cfg) {
  return pyrh::nlte_ray_groups(b->natm, b->max_nspect, cfg->nrays);
}

// Workspace layout for `ngroup` ray groups of the formal kernel.
Layout layout(const pyrh_nlte_batch* b, const pyrh_nlte_config* cfg, int ngroup) {
  Layout L;
  size_t off = 0;
  const int nlev = b->nlevel, natm = b->natm;
  L.wphi = off; off = align256(off + sizeof(double) * (size_t)(b->max_nline > 0 ? b->max_nline : 1) * b->total_depth);
  // in the formal-solution precision: the new J of each ray group, the
  // rate sums per (wavelength tile of 32, ray group, off-diagonal entry,
  // depth), the background and J
  const size_t r = cfg->precision == PYRH_FP32 ? sizeof(float) : sizeof(double);
  L.Jnew = off; off = align256(off + r * (size_t)ngroup * b->total_cont);
  const size_t ntile = (size_t)(b->max_nspect + 31) / 32;
  L.gslab = off; off = align256(off + r * ntile * ngroup * nlev * (nlev - 1) * b->total_depth);
  // the radiative rates' sums, only when the batch keeps the rates
  const size_t nr = b->rates && b->max_ntrans > 0 ? 2 * (size_t)b->max_ntrans : 0;
  L.rslab = off; off = align256(off + r * ntile * ngroup * nr * b->total_depth);
  L.bgr = off; off = align256(off + r * 3 * (size_t)b->total_cont);
  L.Jr = off; off = align256(off + r * (size_t)b->total_cont);
  L.ngprev = off; off = align256(off + sizeof(double) * (size_t)(cfg->ng_order + 2) * nlev * b->total_depth);
  L.count = off; off = align256(off + sizeof(int32_t) * natm);
  L.active = off; off = align256(off + sizeof(int32_t) * natm);
  L.iters = off; off = align256(off + sizeof(int32_t) * natm);
  L.err = off; off = align256(off + sizeof(int32_t));
  L.any = off; off = align256(off + sizeof(int32_t));
  L.dpops = off; off = align256(off + sizeof(double) * natm);
  L.phi = off;
  L.fixed = off;
  return L;
}

pyrh_status check(const pyrh_nlte_batch* b, const pyrh_nlte_config* cfg) {
  if (!b || !cfg) { pyrh::set_error("batch or cfg is NULL"); return PYRH_ERR_ARG; }
  if (b->natm < 1 || b->nlevel < 2 || b->nlevel > PYRH_NLTE_MAX_LEVELS) {
    pyrh::set_error("natm %d / nlevel %d outside limits", b->natm, b->nlevel);
    return PYRH_ERR_ARG;
  }
  if (b->max_ndep < 3 || b->max_ndep > PYRH_NLTE_MAX_DEPTH) {
    pyrh::set_error("max_ndep %d outside [3, %d]", b->max_ndep, PYRH_NLTE_MAX_DEPTH);
    return PYRH_ERR_ARG;
  }
  if (cfg->nrays < 1 || cfg->nrays > PYRH_NLTE_MAX_RAYS) {
    pyrh::set_error("nrays %d outside [1, %d]", cfg->nrays, PYRH_NLTE_MAX_RAYS);
    return PYRH_ERR_ARG;
  }
  if (cfg->ng_order < 0 || cfg->ng_order > PYRH_NLTE_MAX_NG || (cfg->ng_order > 0 && cfg->ng_period < 1)) {
    pyrh::set_error("ng_order %d / ng_period %d", cfg->ng_order, cfg->ng_period);
    return PYRH_ERR_ARG;
  }
  if (cfg->precision != PYRH_FP32 && cfg->precision != PYRH_FP64) {
    pyrh::set_error("precision %d", cfg->precision);
    return PYRH_ERR_ARG;
  }
  if (cfg->isum < -1 || cfg->isum >= b->nlevel || cfg->nmax_iter < 1) {
    pyrh::set_error("isum %d / nmax_iter %d", cfg->isum, cfg->nmax_iter);
    return PYRH_ERR_ARG;
  }
  const void* ptrs[] = {b->ndep, b->nspect, b->ntrans, b->depth_off, b->lam_off, b->cont_off,
                        b->trans_off, b->adamp_off, b->lambda, b->height, b->T, b->vel,
                        b->vbroad, b->ntotal, b->nstar, b->C, b->chi_c, b->eta_c, b->sca_c,
                        b->bgline, b->trans, b->n, b->J};
  for (const void* p : ptrs)
    if (!p) { pyrh::set_error("a batch array pointer is NULL"); return PYRH_ERR_ARG; }
  if (b->rates && b->max_ntrans < 1) {
    pyrh::set_error("rates requested with max_ntrans %d", b->max_ntrans);
    return PYRH_ERR_ARG;
  }
  return PYRH_OK;
}

pyrh::NlteArgs make_args(const pyrh_nlte_batch* b, const pyrh_nlte_config* cfg, void* ws,
                         size_t ws_bytes, const Layout& L, int ngroup) {
  pyrh::NlteArgs A;
  A.b = *b;
  A.nrays = cfg->nrays;
  A.ngroup = ngroup;
  for (int m = 0; m < PYRH_NLTE_MAX_RAYS; ++m) {
    A.muz[m] = m < cfg->nrays ? cfg->muz[m] : 1.0;
    A.wmu[m] = m < cfg->nrays ? cfg->wmu[m] : 0.0;
  }
  A.moving = cfg->moving;
  A.isum = cfg->isum;
  A.ng_order = cfg->ng_order;
  A.ng_delay = cfg->ng_delay;
  A.ng_period = cfg->ng_period > 0 ? cfg->ng_period : 1;
  A.nmax_iter = cfg->nmax_iter;
  A.iter_limit = cfg->iter_limit;
  char* w = static_cast<char*>(ws);
  A.wphi = reinterpret_cast<double*>(w + L.wphi);
  A.Jnew = w + L.Jnew;
  A.gslab = w + L.gslab;
  A.rslab = b->rates ? w + L.rslab : nullptr;
  A.max_ntrans = b->rates ? b->max_ntrans : 0;
  A.bgr = w + L.bgr;
  A.Jr = w + L.Jr;
  A.ngprev = reinterpret_cast<double*>(w + L.ngprev);
  A.count = reinterpret_cast<int32_t*>(w + L.count);
  A.active = reinterpret_cast<int32_t*>(w + L.active);
  A.iters = reinterpret_cast<int32_t*>(w + L.iters);
  A.err = reinterpret_cast<int32_t*>(w + L.err);
  A.any = reinterpret_cast<int32_t*>(w + L.any);
  A.dpops = reinterpret_cast<double*>(w + L.dpops);
  A.phi = w + L.phi;
  const size_t r = cfg->precision == PYRH_FP32 ? sizeof(float) : sizeof(double);
  A.phi_cap = (int64_t)((ws_bytes - L.phi) / r);
  return A;
}

// Iterations launched back to back before the host looks at the device's
// "an atmosphere is still iterating" flag.  Each atmosphere's convergence
// test runs on the device (nlte_ng_kernel) and converged atmospheres skip
// the later launches, so at most kChunk - 1 launches of empty iterations
// follow the last atmosphere's convergence.
constexpr int kChunk = 4;

cudaError_t iterate(const pyrh::NlteArgs& A, const pyrh_nlte_batch* b,
                    const pyrh_nlte_config* cfg, cudaStream_t st, int* launches) {
  cudaError_t e = cudaSuccess;
  for (int it = 0; e == cudaSuccess && it < cfg->nmax_iter;) {
    const int n = cfg->nmax_iter - it < kChunk ? cfg->nmax_iter - it : kChunk;
    for (int c = 0; c < n && e == cudaSuccess; ++c) {
      e = pyrh::nlte_launch_iteration(A, b->natm, b->max_nspect, b->max_ndep, cfg->precision,
                                      st);
      *launches += pyrh::nlte_iteration_launches(A);
    }
    it += n;
    int32_t any = 0;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&any, A.any, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (!any) break;
  }
  return e;
}


// The same loop with one chunk of kChunk iterations recorded as a CUDA graph
// and replayed per chunk on the caller's stream (one graph launch instead
// of kChunk iterations of kernel launches).  The recording uses a private stream, since
// the caller's may be the legacy default stream, which cannot be captured;
// nothing runs while recording.  The first chunk runs uncaptured, which
// also sets the formal kernel's shared-memory attribute before the
// recording; if the capture or the instantiation fails, the remaining
// chunks run uncaptured.
cudaError_t iterate_graph(const pyrh::NlteArgs& A, const pyrh_nlte_batch* b,
                          const pyrh_nlte_config* cfg, cudaStream_t st, int* launches) {
  cudaError_t e = cudaSuccess;
  int it = 0;
  int32_t any = 1;
  {   // first chunk, uncaptured
    const int n = cfg->nmax_iter < kChunk ? cfg->nmax_iter : kChunk;
    for (int c = 0; c < n && e == cudaSuccess; ++c) {
      e = pyrh::nlte_launch_iteration(A, b->natm, b->max_nspect, b->max_ndep, cfg->precision,
                                      st);
      *launches += pyrh::nlte_iteration_launches(A);
    }
    it += n;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&any, A.any, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess || !any || it >= cfg->nmax_iter) return e;
  }
  cudaStream_t cs = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool captured = false;
  if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess &&
      cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    cudaError_t ce = cudaSuccess;
    for (int c = 0; c < kChunk && ce == cudaSuccess; ++c)
      ce = pyrh::nlte_launch_iteration(A, b->natm, b->max_nspect, b->max_ndep, cfg->precision,
                                       cs, false);
    const cudaError_t ee = cudaStreamEndCapture(cs, &graph);
    captured = ce == cudaSuccess && ee == cudaSuccess && graph &&
               cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
  }
  cudaGetLastError();   // a failed capture leaves no sticky error; clear the last one
  // iterations beyond nmax_iter do nothing: nlte_ng_kernel retires an
  // atmosphere once it reaches nmax_iter, so whole chunks are safe
  for (; e == cudaSuccess && it < cfg->nmax_iter && any; it += kChunk) {
    if (captured) {
      e = cudaGraphLaunch(exec, st);
    } else {
      for (int c = 0; c < kChunk && e == cudaSuccess; ++c)
        e = pyrh::nlte_launch_iteration(A, b->natm, b->max_nspect, b->max_ndep, cfg->precision,
                                        st);
    }
    *launches += pyrh::nlte_iteration_launches(A) * kChunk;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&any, A.any, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cs) cudaStreamDestroy(cs);
  return e;
}

}  // namespace

extern "C" {

size_t pyrh_nlte_workspace_bytes(const pyrh_nlte_batch* b, const pyrh_nlte_config* cfg,
                                 int64_t phi_elems) {
  if (!b || !cfg) return 0;
  const Layout L = layout(b, cfg, groups_of(b, cfg));
  const size_t r = cfg->precision == PYRH_FP32 ? sizeof(float) : sizeof(double);
  return L.fixed + r * (size_t)(phi_elems > 0 ? phi_elems : 1);
}

pyrh_status pyrh_nlte_solve(const pyrh_nlte_batch* b, const pyrh_nlte_config* cfg, void* ws,
                            size_t ws_bytes, int32_t* iterations, double* dpops, void* stream) {
  pyrh::set_launches(0);
  pyrh_status s = check(b, cfg);
  if (s != PYRH_OK) return s;
  const int ngroup = groups_of(b, cfg);
  const Layout L = layout(b, cfg, ngroup);
  if (!ws || ws_bytes <= L.fixed) {
    pyrh::set_error("workspace of %zu bytes is smaller than %zu", ws_bytes, L.fixed);
    return PYRH_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  pyrh::NlteArgs A = make_args(b, cfg, ws, ws_bytes, L, ngroup);
  const size_t smem = pyrh::nlte_formal_smem(b->nlevel, b->max_ndep, cfg->nrays, b->max_nline, cfg->precision);
  if (smem > 220 * 1024) {
    pyrh::set_error("shared memory %zu B for %d levels x %d depths", smem, b->nlevel, b->max_ndep);
    return PYRH_ERR_UNSUPPORTED;
  }
  cudaError_t e = cudaMemsetAsync(A.err, 0, sizeof(int32_t), st);
  int launches = 1;
  if (e == cudaSuccess) e = pyrh::nlte_launch_ng_init(A, b->natm, st), ++launches;
  if (e == cudaSuccess) e = pyrh::nlte_launch_prepare(A, cfg->precision, st), ++launches;
  const int64_t max_elems = (int64_t)b->max_nspect * 2 * cfg->nrays * b->max_ndep;
  if (e == cudaSuccess)
    e = pyrh::nlte_launch_profiles(A, b->natm, max_elems, cfg->precision, st), launches += 2;
  if (e == cudaSuccess) e = iterate_graph(A, b, cfg, st, &launches);
  int32_t err = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, A.err, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && iterations)
    e = cudaMemcpyAsync(iterations, A.iters, sizeof(int32_t) * b->natm, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && dpops)
    e = cudaMemcpyAsync(dpops, A.dpops, sizeof(double) * b->natm, cudaMemcpyDeviceToDevice, st);
  std::vector<double> dp(b->natm);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dp.data(), A.dpops, sizeof(double) * b->natm, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  pyrh::set_launches(launches);
  if (e != cudaSuccess) {
    pyrh::set_error("NLTE solve: %s", cudaGetErrorString(e));
    return PYRH_ERR_CUDA;
  }
  if (err) {
    pyrh::set_error(err & 8   ? "more than 32 transitions active across one tile of 32 wavelengths"
                    : err & 4 ? "an atmosphere's ntrans exceeds max_ntrans (rates)"
                    : err & 2 ? "an atmosphere's ndep exceeds max_ndep or the depth limit"
                              : "line profiles do not fit the workspace (phi_off beyond capacity)");
    return PYRH_ERR_ARG;
  }
  for (int p = 0; p < b->natm; ++p)
    if (!(dp[p] < cfg->iter_limit)) {
      pyrh::set_error("atmosphere %d not converged after %d iterations (dpops %g)", p,
                      cfg->nmax_iter, dp[p]);
      return PYRH_ERR_NONCONVERGED;
    }
  return PYRH_OK;
}

pyrh_status pyrh_nlte_emergent(const pyrh_nlte_batch* b, const pyrh_nlte_config* cfg,
                               double mu_out, void* ws, size_t ws_bytes, double* I_out,
                               void* stream) {
  pyrh::set_launches(0);
  pyrh_status s = check(b, cfg);
  if (s != PYRH_OK) return s;
  if (!(mu_out > 0.0 && mu_out <= 1.0) || !I_out) {
    pyrh::set_error("mu_out %g or I_out", mu_out);
    return PYRH_ERR_ARG;
  }
  pyrh_nlte_config one = *cfg;
  one.nrays = 1;
  one.muz[0] = mu_out;
  one.wmu[0] = 1.0;
  const Layout L = layout(b, &one, 1);
  if (!ws || ws_bytes <= L.fixed) {
    pyrh::set_error("workspace of %zu bytes is smaller than %zu", ws_bytes, L.fixed);
    return PYRH_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  pyrh::NlteArgs A = make_args(b, &one, ws, ws_bytes, L, 1);
  cudaError_t e = cudaMemsetAsync(A.err, 0, sizeof(int32_t), st);
  const int64_t max_elems = (int64_t)b->max_nspect * 2 * b->max_ndep;
  if (e == cudaSuccess) e = pyrh::nlte_launch_prepare(A, one.precision, st);
  if (e == cudaSuccess) e = pyrh::nlte_launch_profiles(A, b->natm, max_elems, one.precision, st);
  if (e == cudaSuccess)
    e = pyrh::nlte_launch_emergent(A, b->natm, b->max_nspect, b->max_ndep, one.precision, I_out, st);
  int32_t err = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, A.err, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  pyrh::set_launches(4);
  if (e != cudaSuccess) {
    pyrh::set_error("NLTE emergent: %s", cudaGetErrorString(e));
    return PYRH_ERR_CUDA;
  }
  if (err) {
    pyrh::set_error(err & 8 ? "more than 32 transitions active across one tile of 32 wavelengths"
                            : "line profiles do not fit the workspace");
    return PYRH_ERR_ARG;
  }
  return PYRH_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------
// Allocation-free variant of pyrh_nlte_solve.
//
// Some callers cannot call cudaMalloc: code that runs while another
// component owns all device memory through its own pool, programs embedded
// in hosts that forbid device allocation after start-up, and latency-bound
// loops that cannot afford the implicit device synchronisation an
// allocation may cause.  For them the solver's scratch (line profiles,
// profile normalisation, second mean-intensity buffer, rate matrices, Ng
// history, per-atmosphere state) lives in one fixed, file-scope device
// array.  Every GPU that loads this library holds that array until the
// process exits.
// ------------------------------------------------------------------------

static __device__ __align__(256) unsigned char g_nlte_static_scratch[PYRH_NLTE_STATIC_SCRATCH_BYTES];

namespace {

constexpr int kMaxStaticAtm = 256;

// Device address of the static scratch in the current context, looked up
// with cudaGetSymbolAddress on every call (with the caller's device
// current) and never cached: after cudaDeviceReset, or with another context
// current on the same device, the module and its array may sit at another
// address.  The host-side name of the array is not a device address and is
// never passed to a kernel.
cudaError_t static_scratch(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_nlte_static_scratch);
  if (e != cudaSuccess) return e;
  *out = p;
  return cudaSuccess;
}

}  // namespace

extern "C" pyrh_status pyrh_nlte_solve_static(const pyrh_nlte_batch* b,
                                              const pyrh_nlte_config* cfg, int64_t phi_elems,
                                              int32_t* iterations, double* dpops, void* stream) {
  pyrh::set_launches(0);
  pyrh_status s = check(b, cfg);
  if (s != PYRH_OK) return s;
  if (b->natm > kMaxStaticAtm) {
    pyrh::set_error("pyrh_nlte_solve_static: %d atmospheres exceed the limit of %d", b->natm,
                    kMaxStaticAtm);
    return PYRH_ERR_ARG;
  }
  // the workspace solve's ray groups if their partial sums fit, else one
  const size_t r = cfg->precision == PYRH_FP32 ? sizeof(float) : sizeof(double);
  const size_t phi_bytes = r * (size_t)(phi_elems > 0 ? phi_elems : 1);
  int ngroup = groups_of(b, cfg);
  Layout L = layout(b, cfg, ngroup);
  if (L.fixed + phi_bytes > (size_t)PYRH_NLTE_STATIC_SCRATCH_BYTES && ngroup > 1) {
    ngroup = 1;
    L = layout(b, cfg, 1);
  }
  const size_t need = L.fixed + phi_bytes;
  if (need > (size_t)PYRH_NLTE_STATIC_SCRATCH_BYTES) {
    pyrh::set_error("pyrh_nlte_solve_static: batch needs %zu bytes of scratch, the static "
                    "scratch holds %zu (PYRH_NLTE_STATIC_SCRATCH_BYTES)",
                    need, (size_t)PYRH_NLTE_STATIC_SCRATCH_BYTES);
    return PYRH_ERR_ARG;
  }
  const size_t smem = pyrh::nlte_formal_smem(b->nlevel, b->max_ndep, cfg->nrays, b->max_nline, cfg->precision);
  if (smem > 220 * 1024) {
    pyrh::set_error("shared memory %zu B for %d levels x %d depths", smem, b->nlevel, b->max_ndep);
    return PYRH_ERR_UNSUPPORTED;
  }
  void* ws = nullptr;
  cudaError_t e = static_scratch(&ws);
  if (e != cudaSuccess) {
    pyrh::set_error("pyrh_nlte_solve_static: static scratch lookup: %s", cudaGetErrorString(e));
    return PYRH_ERR_CUDA;
  }
  cudaStream_t st = (cudaStream_t)stream;
  pyrh::NlteArgs A = make_args(b, cfg, ws, need, L, ngroup);
  // The array keeps the previous call's contents; the error word is the
  // only part a kernel reads before this call writes it, so it alone is
  // cleared (the kernels write profiles, rate matrices, Ng history and
  // per-atmosphere state before reading them, as in pyrh_nlte_solve, whose
  // workspace also arrives uninitialised).
  e = cudaMemsetAsync(A.err, 0, sizeof(int32_t), st);
  int launches = 1;
  if (e == cudaSuccess) e = pyrh::nlte_launch_ng_init(A, b->natm, st), ++launches;
  if (e == cudaSuccess) e = pyrh::nlte_launch_prepare(A, cfg->precision, st), ++launches;
  const int64_t max_elems = (int64_t)b->max_nspect * 2 * cfg->nrays * b->max_ndep;
  if (e == cudaSuccess)
    e = pyrh::nlte_launch_profiles(A, b->natm, max_elems, cfg->precision, st), launches += 2;
  if (e == cudaSuccess) e = iterate(A, b, cfg, st, &launches);
  int32_t err = 0;
  double dp[kMaxStaticAtm];
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, A.err, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && iterations)
    e = cudaMemcpyAsync(iterations, A.iters, sizeof(int32_t) * b->natm, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && dpops)
    e = cudaMemcpyAsync(dpops, A.dpops, sizeof(double) * b->natm, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dp, A.dpops, sizeof(double) * b->natm, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  pyrh::set_launches(launches);
  if (e != cudaSuccess) {
    pyrh::set_error("pyrh_nlte_solve_static: %s", cudaGetErrorString(e));
    return PYRH_ERR_CUDA;
  }
  if (err) {
    pyrh::set_error(err & 8   ? "more than 32 transitions active across one tile of 32 wavelengths"
                    : err & 4 ? "an atmosphere's ntrans exceeds max_ntrans (rates)"
                    : err & 2 ? "an atmosphere's ndep exceeds max_ndep or the depth limit"
                              : "line profiles do not fit the static scratch (phi_off beyond phi_elems)");
    return PYRH_ERR_ARG;
  }
  for (int p = 0; p < b->natm; ++p)
    if (!(dp[p] < cfg->iter_limit)) {
      pyrh::set_error("atmosphere %d not converged after %d iterations (dpops %g)", p,
                      cfg->nmax_iter, dp[p]);
      return PYRH_ERR_NONCONVERGED;
    }
  return PYRH_OK;
}
