// nlte.cuh -- launch interface of the NLTE MALI kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pyrh_gb300.h"

namespace pyrh {

struct NlteArgs {
  pyrh_nlte_batch b;              // pointers of the batch (device)
  int nrays;
  double muz[PYRH_NLTE_MAX_RAYS], wmu[PYRH_NLTE_MAX_RAYS];
  int moving, isum, ng_order, ng_delay, ng_period, nmax_iter;
  int ngroup;                     // ray groups of the formal kernel (nlte_ray_groups)
  double iter_limit;
  // workspace
  void *phi;
  int64_t phi_cap;                // elements of phi
  double *wphi, *ngprev, *dpops;
  // in the formal-solution precision: per (tile, ray group) rate sums, the
  // ray groups' new J, the background [chi_c, eta_c, sca_c] and J
  void *gslab, *Jnew, *bgr, *Jr;
  // per (tile, ray group) sums of the radiative rates R_ij, R_ji
  // ([2 max_ntrans][total_depth] each), or nullptr when b.rates is NULL
  void *rslab;
  int max_ntrans;
  int32_t *count, *active, *iters, *err;
  int32_t *any;                   // set by nlte_ng_kernel while an atmosphere iterates
};

// Ray groups for a batch: enough (tile, group) warps to fill the GPU, at
// most one group per ray; depends on the batch's shape only.
int nlte_ray_groups(int natm, int max_nspect, int nrays);

size_t nlte_formal_smem(int nlevel, int maxd, int nrays, int max_nline, int precision);
cudaError_t nlte_launch_profiles(const NlteArgs &A, int natm, int64_t max_elems, int precision,
                                 cudaStream_t st);
cudaError_t nlte_launch_ng_init(const NlteArgs &A, int natm, cudaStream_t st);
// background and starting J in the formal-solution precision (once per solve)
cudaError_t nlte_launch_prepare(const NlteArgs &A, int precision, cudaStream_t st);
// Kernel launches of one MALI iteration: 5, and one more that keeps the
// radiative rates when the batch asks for them.
int nlte_iteration_launches(const NlteArgs &A);
// One MALI iteration.  set_attr = false leaves the formal
// kernel's shared-memory attribute as an earlier call set it (for stream
// capture, where the launches are recorded rather than issued).
cudaError_t nlte_launch_iteration(const NlteArgs &A, int natm, int max_nspect, int maxd,
                                  int precision, cudaStream_t st, bool set_attr = true);
cudaError_t nlte_launch_emergent(const NlteArgs &A, int natm, int max_nspect, int maxd,
                                 int precision, double *I_out, cudaStream_t st);

}  // namespace pyrh
