// lte_stokes.cuh -- launch interface of the fused LTE Stokes kernel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pyrh_gb300.h"

namespace pyrh {

struct LteArgs {
  int natm, tiles, maxd, nline;
  int precision, stokes_mode, magneto_optical, moving;
  double mu, vmicro_char;
  int64_t total_depth;
  const int32_t *ndep, *nlam;
  const int64_t *depth_off, *lam_off, *cont_off;
  const double *lambda, *height, *T, *ne, *nHtot, *np, *vturb, *vlos, *B, *gamma_B, *chi_B;
  const double *line_pops;
  const void *chi_c, *eta_c;
  const pyrh_line *lines;
  void *out;
};

// Response-function / gradient launch (lte_rf.cu).  mode 0 writes rf;
// mode 1 accumulates chi2 and grad (zeroed by the caller) with obs and
// weights; mode 2 accumulates grad with dL/dS passed in `weights`.  The
// log gf outputs are written or accumulated (zeroed by the caller) when set.
struct RfArgs {
  LteArgs lte;
  int mode;
  const void *obs, *weights;
  void *rf, *chi2, *grad;
  void *rf_gf;    // mode 0, optional: dS/dlog10(gf) [nline][4][lambda] per atmosphere
  void *grad_gf;  // modes 1-2, optional: dL/dlog10(gf) [natm][nline]
  pyrh_lte_setup_dT dT;   // set-up temperature derivatives (NULL members: held fixed)
  int sub;                // sub-blocks (work items) per block of the kernel
};

size_t rf_smem_bytes(int precision, int nline, int maxd);
// Threads per block of the response-function kernel (its launch bound):
// in FP32 one block takes an SM's registers at 128 per thread (168 for the
// four-seed full response functions, mode 0); mode < 0 gives the largest
// over the modes.
constexpr int rf_max_threads(int precision, int mode = -1) {
  return precision != PYRH_FP32 ? 128 : (mode == 0 ? 384 : 512);
}
cudaError_t launch_lte_rf(const RfArgs &a, int block, int grid, cudaStream_t st);

size_t lte_smem_bytes(int precision, int nline, int maxd, int block);
cudaError_t launch_lte_stokes(const LteArgs &a, int block, int grid, cudaStream_t st);

}  // namespace pyrh
