// Instantiations of the one-warp-per-cell sweep in native FP64: 2-D and 3-D Q1..Q5.
#include "sweep_wide.cuh"

namespace ouranos {

template <>
cudaError_t launch_sweep_wide<double>(int dim, int p1, const SweepArgs<double>& a, int grid, int block, cudaStream_t s) {
  return launch_sweep_wide_any<double>(dim, p1, a, grid, block, s);
}

}  // namespace ouranos
