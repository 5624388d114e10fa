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
  double iter_limit;
  // workspace
  void *phi;
  int64_t phi_cap;                // elements of phi
  double *wphi, *Jnew, *gslab, *ngprev, *dpops;   // gslab: per-tile rate sums
  int32_t *count, *active, *iters, *err;
  int32_t *any;                   // set by nlte_ng_kernel while an atmosphere iterates
};

size_t nlte_formal_smem(int nlevel, int maxd, int nrays, int max_nline, int precision);
cudaError_t nlte_launch_profiles(const NlteArgs &A, int natm, int64_t max_elems, int precision,
                                 cudaStream_t st);
cudaError_t nlte_launch_ng_init(const NlteArgs &A, int natm, cudaStream_t st);
cudaError_t nlte_launch_iteration(const NlteArgs &A, int natm, int max_nspect, int maxd,
                                  int precision, cudaStream_t st);
cudaError_t nlte_launch_emergent(const NlteArgs &A, int natm, int max_nspect, int maxd,
                                 int precision, double *I_out, cudaStream_t st);

}  // namespace pyrh
