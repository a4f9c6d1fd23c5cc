// Instantiations of the batched sweep kernel in float: 2-D Q1..Q4, 3-D Q1..Q2.
#include "sweep.cuh"

namespace ouranos {

template <>
cudaError_t launch_sweep_batch<float>(int dim, int p1, int fm, int lpc, const SweepArgs<float>* args, const int2* tmap,
                                   int n_total, int* ticket, const int* status, const unsigned* epoch,
                                   int grid, int block, cudaStream_t s) {
#define ARGS fm, lpc, args, tmap, n_total, ticket, status, epoch, grid, block, s
  if (dim == 2) {
    switch (p1) {
      case 2: return launch_sweep_batch_impl<float, 2, 2>(ARGS);
      case 3: return launch_sweep_batch_impl<float, 2, 3>(ARGS);
      case 4: return launch_sweep_batch_impl<float, 2, 4>(ARGS);
      case 5: return launch_sweep_batch_impl<float, 2, 5>(ARGS);
    }
  } else if (dim == 3) {
    switch (p1) {
      case 2: return launch_sweep_batch_impl<float, 3, 2>(ARGS);
      case 3: return launch_sweep_batch_impl<float, 3, 3>(ARGS);
    }
  }
#undef ARGS
  return cudaErrorInvalidValue;
}

}  // namespace ouranos
