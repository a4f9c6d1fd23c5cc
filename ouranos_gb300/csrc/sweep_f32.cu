// Instantiations of the sweep kernel in float: 2-D Q1..Q4, 3-D Q1..Q2
// (one warp per cell for the 1 x 1 x 1 tiling and the higher orders:
// sweep_wide_f32.cu).
#include "sweep.cuh"

namespace ouranos {

template <>
cudaError_t launch_sweep<float>(int dim, int p1, int fm, const SweepArgs<float>& a, int grid, int block,
                                cudaStream_t s) {
  if (a.lpc == 32) return launch_sweep_wide<float>(dim, p1, a, grid, block, s);
  if (dim == 2) {
    switch (p1) {
      case 2: return launch_sweep_impl<float, 2, 2>(fm, a, grid, block, s);
      case 3: return launch_sweep_impl<float, 2, 3>(fm, a, grid, block, s);
      case 4: return launch_sweep_impl<float, 2, 4>(fm, a, grid, block, s);
      case 5: return launch_sweep_impl<float, 2, 5>(fm, a, grid, block, s);
    }
  } else if (dim == 3) {
    switch (p1) {
      case 2: return launch_sweep_impl<float, 3, 2>(fm, a, grid, block, s);
      case 3: return launch_sweep_impl<float, 3, 3>(fm, a, grid, block, s);
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace ouranos
