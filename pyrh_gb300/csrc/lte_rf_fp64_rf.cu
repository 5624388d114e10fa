// lte_rf_fp64_rf.cu -- the double-precision response-function kernel for the
// full response functions (mode 0) (lte_rf_kernel.cuh), in a unit of its own so that the kernel
// instantiations compile in parallel.
#include "lte_rf_kernel.cuh"

namespace pyrh {

cudaError_t launch_lte_rf_fp64_m0(const RfArgs& a, int block, int grid, size_t smem,
                                  cudaStream_t st) {
  return launch_mode<double, 0>(a, block, grid, smem, st);
}

size_t rf_smem_bytes_fp64(int nline, int maxd) { return rf_smem_precision<double>(nline, maxd); }

}  // namespace pyrh
