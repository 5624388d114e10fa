// lte_rf_fp64_chi2.cu -- the double-precision response-function kernel for the
// chi^2 gradient (mode 1) (lte_rf_kernel.cuh), in a unit of its own so that the kernel
// instantiations compile in parallel.
#include "lte_rf_kernel.cuh"

namespace pyrh {

cudaError_t launch_lte_rf_fp64_m1(const RfArgs& a, int block, int grid, size_t smem,
                                  cudaStream_t st) {
  return launch_mode<double, 1>(a, block, grid, smem, st);
}

}  // namespace pyrh
