// Instantiations of the one-warp-per-cell sweep in double-float (FP64 accuracy on the FP32 pipes): 2-D and 3-D Q1..Q5.
#include "sweep_wide.cuh"

namespace ouranos {

template <>
cudaError_t launch_sweep_wide<df64>(int dim, int p1, const SweepArgs<df64>& a, int grid, int block, cudaStream_t s) {
  return launch_sweep_wide_any<df64>(dim, p1, a, grid, block, s);
}

}  // namespace ouranos
