// Kernels of the learned preconditioner's convolutional network.
//
// Activations are channels-last BF16 tensors [voxel][C] on an nx*ny*nz grid
// (voxel = x + nx*(y + ny*z)); weights are FP32 masters [tap][cin][cout] with
// BF16 copies in the layouts the tensor-core kernels read.  Convolutions are
// 3x3x3, stride 1, zero padding, written as implicit GEMMs:
//   out[v][co] = sum_{tap, ci} in[v + off(tap)][ci] * W[tap][ci][co]
// M = voxels, N = cout, K = 27 * cin, on mma.sync.m16n8k16 (BF16 inputs, FP32
// accumulation); every warp owns 16 voxels and all output channels.  The
// gradient with respect to the input is the same implicit GEMM over the
// output gradient with the taps mirrored; the weight gradient reduces over
// voxels in FP32.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace ouranos {
namespace cnn {

struct Grid {
  int nx, ny, nz;
  __host__ __device__ long voxels() const { return (long)nx * ny * nz; }
};

__device__ __forceinline__ int tap_dx(int t) { return t % 3 - 1; }
__device__ __forceinline__ int tap_dy(int t) { return (t / 3) % 3 - 1; }
__device__ __forceinline__ int tap_dz(int t) { return t / 9 - 1; }

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<unsigned*>(&v);
}

// D += A(16x16 bf16, row) * B(16x8 bf16, col), FP32 accumulators
__device__ __forceinline__ void mma_bf16_16816(float* d, const unsigned* a, const unsigned* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Implicit-GEMM 3x3x3 convolution.  CIN, COUT multiples of 16 (COUT of 8).
// wt: BF16 weights [27][COUT][CIN] (k contiguous per output channel).
// out_bf16 (and/or out_f32) receive bias + optional ReLU.
template <int CIN, int COUT, bool RELU>
__global__ void __launch_bounds__(128) conv3_fwd(Grid g, const __nv_bfloat16* __restrict__ in,
                                                 const __nv_bfloat16* __restrict__ wt,
                                                 const float* __restrict__ bias,
                                                 __nv_bfloat16* __restrict__ out_bf16,
                                                 float* __restrict__ out_f32) {
  constexpr int NT = COUT / 8;  // n tiles of 8 channels
  const long V = g.voxels();
  const int lane = threadIdx.x & 31;
  const int grp = lane >> 2, tig = lane & 3;
  const long warp_global = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  const long v0 = warp_global * 16;
  if (v0 >= V) return;
  // the two voxel rows this thread feeds into A: grp and grp + 8
  long vr[2];
  int xr[2], yr[2], zr[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    vr[h] = v0 + grp + 8 * h;
    const long v = vr[h] < V ? vr[h] : V - 1;
    xr[h] = (int)(v % g.nx);
    yr[h] = (int)((v / g.nx) % g.ny);
    zr[h] = (int)(v / ((long)g.nx * g.ny));
  }
  float acc[NT][4];
#pragma unroll
  for (int n = 0; n < NT; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
  for (int tap = 0; tap < 27; ++tap) {
    const int dx = tap_dx(tap), dy = tap_dy(tap), dz = tap_dz(tap);
    const __nv_bfloat16* src[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int x = xr[h] + dx, y = yr[h] + dy, z = zr[h] + dz;
      const bool ok = vr[h] < V && x >= 0 && x < g.nx && y >= 0 && y < g.ny && z >= 0 && z < g.nz;
      src[h] = ok ? in + ((long)x + (long)g.nx * (y + (long)g.ny * z)) * CIN : nullptr;
    }
    const __nv_bfloat16* wtap = wt + (long)tap * COUT * CIN;
#pragma unroll
    for (int k0 = 0; k0 < CIN; k0 += 16) {
      unsigned a[4];
      const int c0 = k0 + tig * 2;
      a[0] = src[0] ? *reinterpret_cast<const unsigned*>(src[0] + c0) : 0u;
      a[1] = src[1] ? *reinterpret_cast<const unsigned*>(src[1] + c0) : 0u;
      a[2] = src[0] ? *reinterpret_cast<const unsigned*>(src[0] + c0 + 8) : 0u;
      a[3] = src[1] ? *reinterpret_cast<const unsigned*>(src[1] + c0 + 8) : 0u;
#pragma unroll
      for (int n = 0; n < NT; ++n) {
        const __nv_bfloat16* wrow = wtap + (long)(n * 8 + grp) * CIN + c0;
        unsigned b[2];
        b[0] = __ldg(reinterpret_cast<const unsigned*>(wrow));
        b[1] = __ldg(reinterpret_cast<const unsigned*>(wrow + 8));
        mma_bf16_16816(acc[n], a, b);
      }
    }
  }
  // epilogue: C[row][col] rows grp, grp+8; cols tig*2, tig*2+1 of each n tile
#pragma unroll
  for (int n = 0; n < NT; ++n) {
    const int co = n * 8 + tig * 2;
    const float b0 = bias ? bias[co] : 0.f, b1 = bias ? bias[co + 1] : 0.f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (vr[h] >= V) continue;
      float o0 = acc[n][2 * h + 0] + b0, o1 = acc[n][2 * h + 1] + b1;
      if (RELU) {
        o0 = fmaxf(o0, 0.f);
        o1 = fmaxf(o1, 0.f);
      }
      if (out_bf16)
        *reinterpret_cast<unsigned*>(out_bf16 + vr[h] * COUT + co) = pack_bf16(o0, o1);
      if (out_f32) {
        out_f32[vr[h] * COUT + co] = o0;
        out_f32[vr[h] * COUT + co + 1] = o1;
      }
    }
  }
}

// Weight gradient: dW[tap][ci][co] += sum_v in[v + off(tap)][ci] * g[v][co],
// dbias[co] += sum_v g[v][co].  One block per (tap, voxel chunk); thread
// (ci, co) pairs; FP32 accumulation, one atomicAdd per weight per block.
template <int CIN, int COUT>
__global__ void conv3_wgrad(Grid g, const __nv_bfloat16* __restrict__ in,
                            const __nv_bfloat16* __restrict__ grad, float* __restrict__ dw,
                            float* __restrict__ dbias, int chunk) {
  constexpr int PAIRS = CIN * COUT;
  __shared__ float s_in[64][CIN];
  __shared__ float s_g[64][COUT];
  const long V = g.voxels();
  const int tap = blockIdx.y;
  const int dx = tap_dx(tap), dy = tap_dy(tap), dz = tap_dz(tap);
  const long vbeg = (long)blockIdx.x * chunk;
  const long vend = vbeg + chunk < V ? vbeg + chunk : V;
  float acc[(PAIRS + 255) / 256];
  float bacc = 0.f;
#pragma unroll
  for (int k = 0; k < (PAIRS + 255) / 256; ++k) acc[k] = 0.f;
  for (long vb = vbeg; vb < vend; vb += 64) {
    const int nv = (int)(vend - vb < 64 ? vend - vb : 64);
    for (int e = threadIdx.x; e < 64 * CIN; e += blockDim.x) {
      const int r = e / CIN, c = e % CIN;
      float val = 0.f;
      if (r < nv) {
        const long v = vb + r;
        const int x = (int)(v % g.nx) + dx, y = (int)((v / g.nx) % g.ny) + dy,
                  z = (int)(v / ((long)g.nx * g.ny)) + dz;
        if (x >= 0 && x < g.nx && y >= 0 && y < g.ny && z >= 0 && z < g.nz)
          val = __bfloat162float(in[((long)x + (long)g.nx * (y + (long)g.ny * z)) * CIN + c]);
      }
      s_in[r][c] = val;
    }
    for (int e = threadIdx.x; e < 64 * COUT; e += blockDim.x) {
      const int r = e / COUT, c = e % COUT;
      s_g[r][c] = r < nv ? __bfloat162float(grad[(vb + r) * COUT + c]) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < (PAIRS + 255) / 256; ++k) {
      const int pr = threadIdx.x + 256 * k;
      if (pr < PAIRS) {
        const int ci = pr / COUT, co = pr % COUT;
        float s = 0.f;
        for (int r = 0; r < nv; ++r) s += s_in[r][ci] * s_g[r][co];
        acc[k] += s;
      }
    }
    if (tap == 13 && threadIdx.x < COUT)
      for (int r = 0; r < nv; ++r) bacc += s_g[r][threadIdx.x];
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < (PAIRS + 255) / 256; ++k) {
    const int pr = threadIdx.x + 256 * k;
    if (pr < PAIRS) {
      const int ci = pr / COUT, co = pr % COUT;
      atomicAdd(dw + ((long)tap * CIN + ci) * COUT + co, acc[k]);
    }
  }
  if (tap == 13 && threadIdx.x < COUT && dbias) atomicAdd(dbias + threadIdx.x, bacc);
}

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

// nodal[cell*8 + k] = vert[vertex of (cell, k)]
static __global__ void vertex_scatter_kernel(Grid g, const float* vert, float* nodal) {
  const long n = g.voxels() * 8;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
    nodal[e] = vert[corner_vertex(g, e >> 3, (int)(e & 7))];
}

}  // namespace cnn
}  // namespace ouranos
