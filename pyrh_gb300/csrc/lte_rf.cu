// lte_rf.cu -- shared-memory sizing and launch of the response-function
// kernels (lte_rf_kernel.cuh), whose instantiations live in
// lte_rf_fp{32,64}_{rf,chi2,vjp}.cu.
#include <cuda_runtime.h>

#include "../../include/pyrh_gb300.h"
#include "lte_stokes.cuh"

namespace pyrh {

cudaError_t launch_lte_rf_fp32_m0(const RfArgs& a, int block, int grid, size_t smem,
                                  cudaStream_t st);
cudaError_t launch_lte_rf_fp32_m1(const RfArgs& a, int block, int grid, size_t smem,
                                  cudaStream_t st);
cudaError_t launch_lte_rf_fp32_m2(const RfArgs& a, int block, int grid, size_t smem,
                                  cudaStream_t st);
cudaError_t launch_lte_rf_fp64_m0(const RfArgs& a, int block, int grid, size_t smem,
                                  cudaStream_t st);
cudaError_t launch_lte_rf_fp64_m1(const RfArgs& a, int block, int grid, size_t smem,
                                  cudaStream_t st);
cudaError_t launch_lte_rf_fp64_m2(const RfArgs& a, int block, int grid, size_t smem,
                                  cudaStream_t st);
size_t rf_smem_bytes_fp32(int nline, int maxd);
size_t rf_smem_bytes_fp64(int nline, int maxd);

size_t rf_smem_bytes(int precision, int nline, int maxd) {
  return precision == PYRH_FP32 ? rf_smem_bytes_fp32(nline, maxd)
                                : rf_smem_bytes_fp64(nline, maxd);
}

cudaError_t launch_lte_rf(const RfArgs& a, int block, int grid, cudaStream_t st) {
  const size_t smem = rf_smem_bytes(a.lte.precision, a.lte.nline, a.lte.maxd);
  const bool f32 = a.lte.precision == PYRH_FP32;
  switch (a.mode) {
    case 0: return f32 ? launch_lte_rf_fp32_m0(a, block, grid, smem, st)
                       : launch_lte_rf_fp64_m0(a, block, grid, smem, st);
    case 1: return f32 ? launch_lte_rf_fp32_m1(a, block, grid, smem, st)
                       : launch_lte_rf_fp64_m1(a, block, grid, smem, st);
    default: return f32 ? launch_lte_rf_fp32_m2(a, block, grid, smem, st)
                        : launch_lte_rf_fp64_m2(a, block, grid, smem, st);
  }
}

}  // namespace pyrh
