// lte_rf_fp64_vjp.cu -- the double-precision response-function kernel for the
// vector-Jacobian product (mode 2) (lte_rf_kernel.cuh), in a unit of its own so that the kernel
// instantiations compile in parallel.
#include "lte_rf_kernel.cuh"

namespace pyrh {

cudaError_t launch_lte_rf_fp64_m2(const RfArgs& a, int block, int grid, size_t smem,
                                  cudaStream_t st) {
  return launch_mode<double, 2>(a, block, grid, smem, st);
}

}  // namespace pyrh
