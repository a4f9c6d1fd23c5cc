// Kernels of the learned preconditioner's convolutional network.
//
// Activations are channels-last BF16 tensors [voxel][C] on an nx*ny*nz grid
// (voxel = x + nx*(y + ny*z)); weights are FP32 masters [tap][cin][cout] with
// BF16 copies in the layouts the tensor-core kernels read.  Convolutions are
// 3x3x3, stride 1, zero padding, written as implicit GEMMs:
//   out[v][co] = sum_{tap, ci} in[v + off(tap)][ci] * W[tap][ci][co]
// M = voxels, N = cout, K = 27 * cin, on tcgen05.mma (BF16 inputs, FP32
// accumulation in tensor memory, input bricks staged by TMA; cnn_tc.cu).  The
// gradient with respect to the input is the same implicit GEMM over the
// output gradient with the taps mirrored; the weight gradient is a GEMM with
// the voxels as K (rows (tap, cin), columns cout), also on tcgen05.mma.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>

namespace ouranos {
namespace cnn {

struct Grid {
  int nx, ny, nz;
  __host__ __device__ long voxels() const { return (long)nx * ny * nz; }
};

__device__ __forceinline__ int tap_dx(int t) { return t % 3 - 1; }
__device__ __forceinline__ int tap_dy(int t) { return (t / 3) % 3 - 1; }
__device__ __forceinline__ int tap_dz(int t) { return t / 9 - 1; }

// 3x3x3 convolution, out[v][co] = sum_{tap, ci} in[v + off(tap)][ci] W[tap][co][ci],
// as a tcgen05 implicit GEMM (cnn_tc.cu); cin, cout in {16, 32}; wt BF16
// [27][cout][cin].  Outputs (each may be NULL): pre, the BF16 convolution;
// gated, BF16 of pre times the layer's gate a[3c] + a[3c+1] m.x + a[3c+2] m.y
// (mat per voxel, gate per channel); pre_f32 and gated_f32 the same in FP32.
// A bounded wait that runs out sets bit 0 of *status.
cudaError_t conv3_tc(int cin, int cout, const Grid& g, const __nv_bfloat16* in, const __nv_bfloat16* wt,
                     const float2* mat, const float* gate, __nv_bfloat16* pre, __nv_bfloat16* gated, float* pre_f32,
                     float* gated_f32, int* status, long long limit_ns, cudaStream_t s, std::string* err);

// Weight gradient dW[tap][ci][co] += sum_v in[v + off(tap)][ci] * g[v][co]
// as a tcgen05 GEMM over voxel chunks (cnn_tc.cu): rows (tap, ci), columns
// co, BF16 products accumulated in FP32 in tensor memory, one FP32 atomic add
// per weight per CTA; in and g 16-byte aligned.  A bounded wait that runs out
// sets bit 0 of *status.
cudaError_t conv3_wgrad_tc(int cin, int cout, const Grid& g, const __nv_bfloat16* in, const __nv_bfloat16* grad,
                           float* dw, int* status, long long limit_ns, cudaStream_t s);

// ---------------------------------------------------------------- continuity projection
// Nodal fields on a grid of Q1 cells: value k (0..7) of a cell sits at its
// corner (k&1, (k>>1)&1, k>>2).  The projection S onto continuous fields
// averages the values that share a mesh vertex and copies the average back
// to each of them (S is symmetric and S S = S).
__host__ __device__ inline long n_vertices(const Grid& g) {
  return (long)(g.nx + 1) * (g.ny + 1) * (g.nz + 1);
}

// vert[v] = scale * mean of nodal[cell*ld + corner] over the pairs at vertex v
static __global__ void vertex_average_kernel(Grid g, const float* nodal, int ld, float scale, float* vert) {
  const long nv = n_vertices(g);
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < nv; v += (long)gridDim.x * blockDim.x) {
    const int vx = (int)(v % (g.nx + 1)), vy = (int)((v / (g.nx + 1)) % (g.ny + 1));
    const int vz = (int)(v / ((long)(g.nx + 1) * (g.ny + 1)));
    float s = 0.f;
    int n = 0;
    for (int k = 0; k < 8; ++k) {
      const int cx = vx - (k & 1), cy = vy - ((k >> 1) & 1), cz = vz - (k >> 2);
      if (cx < 0 || cy < 0 || cz < 0 || cx >= g.nx || cy >= g.ny || cz >= g.nz) continue;
      s += nodal[(cx + (long)g.nx * (cy + (long)g.ny * cz)) * ld + k];
      ++n;
    }
    vert[v] = n ? scale * s / (float)n : 0.f;
  }
}

__device__ __forceinline__ long corner_vertex(const Grid& g, long cell, int k) {
  const int x = (int)(cell % g.nx), y = (int)((cell / g.nx) % g.ny), z = (int)(cell / ((long)g.nx * g.ny));
  return (x + (k & 1)) + (long)(g.nx + 1) * ((y + ((k >> 1) & 1)) + (long)(g.ny + 1) * (z + (k >> 2)));
}

// nodal[cell*8 + k] = vert[vertex of (cell, k)], one cell per thread
static __global__ void vertex_scatter_kernel(Grid g, const float* vert, float* nodal) {
  const long n = g.voxels();
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
    const long v0 = corner_vertex(g, c, 0);
    const long sy = g.nx + 1, sz = (long)(g.nx + 1) * (g.ny + 1);
    float4* o = reinterpret_cast<float4*>(nodal + c * 8);
    o[0] = make_float4(vert[v0], vert[v0 + 1], vert[v0 + sy], vert[v0 + sy + 1]);
    o[1] = make_float4(vert[v0 + sz], vert[v0 + sz + 1], vert[v0 + sz + sy], vert[v0 + sz + sy + 1]);
  }
}

}  // namespace cnn
}  // namespace ouranos
