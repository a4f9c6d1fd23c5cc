// The network's 3x3x3 convolutions as tcgen05 implicit GEMMs.
//
//   out[v][co] = sum_{tap, ci} in[v + off(tap)][ci] * W[tap][co][ci]
//
// M = 128 voxels per tile: an 8 (x) x 16 (y) patch of one z-plane, one
// tensor-memory lane per voxel; N = the output channels (16 or 32); K = 27
// taps x the input channels, one MMA of K = 16 per tap and 16 input channels.
// The input brick of a tile (10 x 18 x 3 voxels with the one-voxel halo) is
// brought into shared memory by TMA, one 4-D box per 8-channel chunk of the
// channels-last activations ([z][y][x][8 channels], zero outside the grid),
// which is exactly the K-major core-matrix layout the MMA reads: eight
// consecutive x voxels of one chunk are one core matrix (8 rows x 16 bytes),
// the 16 y rows of the patch are 160 bytes apart (the stride-dimension
// offset), the next chunk of channels one plane further (the leading-dimension
// offset), and a tap is a start-address shift inside the brick.  The weights
// of all 27 taps stay in shared memory in the same layout.  One thread issues
// the MMAs and commits them to an mbarrier; the next tile's brick is loaded
// while this tile's accumulators are written out; every wait is bounded.
// The epilogue applies the layer's gate (per voxel and channel, affine in
// the pooled material features) and writes the pre-gate and gated outputs
// the forward and backward passes read.
#include <cuda.h>

#include <algorithm>
#include <cstdio>
#include <string>

#include "cnn_kernels.cuh"
#include "tc5.cuh"

namespace ouranos {
namespace cnn {
namespace {

constexpr int kThreads = 128;
constexpr int kTx = 8, kTy = 16;                     // tile: 8 x 16 voxels of one plane
constexpr int kBx = kTx + 2, kBy = kTy + 2, kBz = 3;  // the brick with its halo
constexpr uint32_t kPlaneBytes = kBx * kBy * kBz * 16;  // one 8-channel chunk of the brick: 8640
constexpr uint32_t kPlaneStride = 8704;                 // chunk planes 128-byte aligned
constexpr uint32_t kSboA = kBx * 16;                    // y rows of the patch

struct TmapSet {
  CUtensorMap m[4];  // one per 8-channel chunk of the input (at most 32 channels)
};

// NBUF brick buffers: with two, the next-but-one tile's brick is loaded
// while this tile's MMAs and epilogue run
template <int CIN, int COUT, int NBUF>
__global__ void __launch_bounds__(kThreads) conv3_tc_kernel(const __grid_constant__ TmapSet maps, Grid g,
                                                            const __nv_bfloat16* __restrict__ wt,
                                                            const float2* __restrict__ mat,
                                                            const float* __restrict__ gate, __nv_bfloat16* pre,
                                                            __nv_bfloat16* gated, float* pre_f32, float* gated_f32,
                                                            int* status, long long limit_ns) {
  constexpr int NCH = CIN / 8;
  constexpr uint32_t kWtap = COUT * CIN * 2;
  constexpr uint32_t kSboB = NCH * 128;
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t kBrick = NCH * kPlaneStride;
  uint8_t* W = smem + NBUF * kBrick;
  // mbarriers: MMAs done [0], error path [1], brick b loaded [2 + b]
  uint64_t* bar = reinterpret_cast<uint64_t*>(W + 27 * kWtap);
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 4);
  float* sgate = reinterpret_cast<float*>(slot + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // W[tap][n][k] -> tap * kWtap + (n / 8) * kSboB + (k / 8) * 128 + (n % 8) * 16 + (k % 8) * 2
  for (int i = tid; i < 27 * COUT * NCH; i += kThreads) {
    const int tap = i / (COUT * NCH), rem = i % (COUT * NCH), n = rem / NCH, kc = rem % NCH;
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(wt + ((long)tap * COUT + n) * CIN + 8 * kc));
    *reinterpret_cast<uint4*>(W + tap * kWtap + (n >> 3) * kSboB + kc * 128 + (n & 7) * 16) = v;
  }
  if (gate)
    for (int i = tid; i < 3 * COUT; i += kThreads) sgate[i] = gate[i];
  if (tid == 0) {
    for (int i = 0; i < 2 + NBUF; ++i) tc5::mbar_init(bar + i, 1);
    tc5::mbar_init_fence();
  }
  if (warp == 0) {
    tc5::tmem_alloc(slot, 32);
    tc5::tmem_relinquish();
  }
  tc5::fence_smem_to_async();
  tc5::fence_before_sync();
  __syncthreads();
  tc5::fence_after_sync();
  const uint32_t tmem = *slot;
  constexpr uint32_t idesc = tc5::idesc_bf16_f32(128, COUT);
  const int tx = (g.nx + kTx - 1) / kTx, ty = (g.ny + kTy - 1) / kTy;
  const long ntiles = (long)tx * ty * g.nz;
  auto origin = [&](long t, int& x0, int& y0, int& z0) {
    x0 = (int)(t % tx) * kTx;
    y0 = (int)((t / tx) % ty) * kTy;
    z0 = (int)(t / ((long)tx * ty));
  };
  auto load = [&](long t, int b) {  // one thread: the brick of tile t into buffer b
    int x0, y0, z0;
    origin(t, x0, y0, z0);
    uint8_t* dst = smem + b * kBrick;
    tc5::mbar_arrive_expect_tx(bar + 2 + b, NCH * kPlaneBytes);
#pragma unroll
    for (int c = 0; c < NCH; ++c)
      tc5::tma_load_4d(dst + c * kPlaneStride, &maps.m[c], 0, x0 - 1, y0 - 1, z0 - 1, bar + 2 + b);
  };
  uint32_t ph_load = 0, ph_mma = 0;  // ph_load bit b: the parity awaited next on brick b
  uint32_t pending = 0;              // bit b: a load into brick b is in flight
  bool ok = true;
  const long stride = gridDim.x;
  if (tid == 0)
    for (int b = 0; b < NBUF; ++b)
      if ((long)blockIdx.x + b * stride < ntiles) load(blockIdx.x + b * stride, b);
  for (int b = 0; b < NBUF; ++b)
    if ((long)blockIdx.x + b * stride < ntiles) pending |= 1u << b;
  int it = 0;
  for (long tile = blockIdx.x; tile < ntiles; tile += stride, ++it) {
    const int b = NBUF == 1 ? 0 : (it & 1);
    uint8_t* brick = smem + b * kBrick;
    bool w = true;
    if (tid == 0) w = tc5::mbar_wait(bar + 2 + b, (ph_load >> b) & 1u, limit_ns);
    ph_load ^= 1u << b;
    pending &= ~(1u << b);
    ok = __syncthreads_and(w);
    if (!ok) break;
    if (tid == 0) {
      tc5::fence_after_sync();
      // one descriptor per operand; a tap or a K step only moves the start
      // address (the low field, in 16-byte units), so the 27 x CIN/16 MMAs
      // issue back to back from constant offsets
      const uint64_t a0 = tc5::smem_desc(tc5::smem_addr(brick), kPlaneStride, kSboA);
      const uint64_t b0 = tc5::smem_desc(tc5::smem_addr(W), 128, kSboB);
#pragma unroll
      for (int tap = 0; tap < 27; ++tap) {
        const uint32_t shift = (uint32_t)(((tap / 9) * kBy + (tap / 3) % 3) * kBx + tap % 3);  // 16-byte units
#pragma unroll
        for (int ks = 0; ks < CIN / 16; ++ks)
          tc5::mma_bf16(tmem, a0 + shift + (uint64_t)(ks * 2 * (kPlaneStride >> 4)),
                        b0 + (uint64_t)((tap * kWtap + ks * 256) >> 4), idesc, tap > 0 || ks > 0);
      }
      tc5::mma_commit(bar);
    }
    if (tid == 0) w = tc5::mbar_wait(bar, ph_mma, limit_ns);
    ph_mma ^= 1u;
    ok = __syncthreads_and(w);
    if (!ok) break;
    // this brick is free: the tile NBUF steps ahead loads into it while this
    // epilogue (and, with two buffers, the next tile's MMAs) run
    if (tile + NBUF * stride < ntiles) {
      if (tid == 0) load(tile + NBUF * stride, b);
      pending |= 1u << b;
    }
    tc5::fence_after_sync();
    int x0, y0, z0;
    origin(tile, x0, y0, z0);
    const int r = 32 * warp + lane, x = x0 + (r & 7), y = y0 + (r >> 3);
    float acc[COUT];
#pragma unroll
    for (int c0 = 0; c0 < COUT; c0 += 16) {
      float t16[16];
      tc5::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, t16);
#pragma unroll
      for (int k = 0; k < 16; ++k) acc[c0 + k] = t16[k];
    }
    if (x < g.nx && y < g.ny) {
      const long v = x + (long)g.nx * (y + (long)g.ny * z0);
      const float2 m = gate ? mat[v] : make_float2(0.f, 0.f);
#pragma unroll
      for (int c0 = 0; c0 < COUT; c0 += 8) {
        uint32_t pk[4], gk[4];
#pragma unroll
        for (int k = 0; k < 8; k += 2) {
          const __nv_bfloat162 o = __floats2bfloat162_rn(acc[c0 + k], acc[c0 + k + 1]);
          pk[k / 2] = *reinterpret_cast<const uint32_t*>(&o);
          if (gated) {  // the gate applies to the BF16 pre-gate value, as the backward pass sees it
            const float g0 = sgate[3 * (c0 + k)] + sgate[3 * (c0 + k) + 1] * m.x + sgate[3 * (c0 + k) + 2] * m.y;
            const float g1 =
                sgate[3 * (c0 + k + 1)] + sgate[3 * (c0 + k + 1) + 1] * m.x + sgate[3 * (c0 + k + 1) + 2] * m.y;
            const __nv_bfloat162 q = __floats2bfloat162_rn(__low2float(o) * g0, __high2float(o) * g1);
            gk[k / 2] = *reinterpret_cast<const uint32_t*>(&q);
          }
        }
        if (pre) *reinterpret_cast<uint4*>(pre + v * COUT + c0) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        if (gated) *reinterpret_cast<uint4*>(gated + v * COUT + c0) = make_uint4(gk[0], gk[1], gk[2], gk[3]);
        if (pre_f32 || gated_f32) {
#pragma unroll
          for (int k = 0; k < 8; k += 4) {
            if (pre_f32)
              *reinterpret_cast<float4*>(pre_f32 + v * COUT + c0 + k) =
                  make_float4(acc[c0 + k], acc[c0 + k + 1], acc[c0 + k + 2], acc[c0 + k + 3]);
            if (gated_f32) {
              float gv[4];
#pragma unroll
              for (int j = 0; j < 4; ++j) {
                const int c = c0 + k + j;
                gv[j] = acc[c] * (sgate[3 * c] + sgate[3 * c + 1] * m.x + sgate[3 * c + 2] * m.y);
              }
              *reinterpret_cast<float4*>(gated_f32 + v * COUT + c0 + k) = make_float4(gv[0], gv[1], gv[2], gv[3]);
            }
          }
        }
      }
    }
    tc5::fence_before_sync();
    __syncthreads();
  }
  if (!ok) {  // a wait ran out: bounded waits for the MMAs and the loads still in flight
    if (tid == 0) {
      if (status) atomicOr(status, 1);
      tc5::mma_commit(bar + 1);
      tc5::mbar_wait(bar + 1, 0u, limit_ns);
      for (int b = 0; b < NBUF; ++b)
        if ((pending >> b) & 1u) tc5::mbar_wait(bar + 2 + b, (ph_load >> b) & 1u, limit_ns);
    }
    __syncthreads();
  }
  if (warp == 0) {
    tc5::fence_after_sync();
    tc5::tmem_dealloc(tmem, 32);
  }
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder(std::string* err) {
  static EncodeTiled fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p) {
      if (err) *err = "cuTensorMapEncodeTiled is not available from the driver";
      return nullptr;
    }
    fn = reinterpret_cast<EncodeTiled>(p);
  }
  return fn;
}

template <int CIN, int COUT, int NBUF>
cudaError_t launch(const TmapSet& maps, const Grid& g, const __nv_bfloat16* wt, const float2* mat, const float* gate,
                   __nv_bfloat16* pre, __nv_bfloat16* gated, float* pre_f32, float* gated_f32, int* status,
                   long long limit_ns, cudaStream_t s) {
  constexpr size_t smem = NBUF * (CIN / 8) * kPlaneStride + 27 * COUT * CIN * 2 + 4 * 8 + 16 + 3 * COUT * 4;
  // the function's attributes and its resident-CTA count, once per device
  // (a forward pass launches ten convolutions; host work per launch shows)
  static int slots[64] = {};  // resident CTAs per device, 0 = not configured yet
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!slots[dev]) {
    e = cudaFuncSetAttribute(conv3_tc_kernel<CIN, COUT, NBUF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(conv3_tc_kernel<CIN, COUT, NBUF>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    slots[dev] = sms * tc5::resident_ctas(conv3_tc_kernel<CIN, COUT, NBUF>, kThreads, smem, 32, dev);
  }
  const long ntiles = (long)((g.nx + kTx - 1) / kTx) * ((g.ny + kTy - 1) / kTy) * g.nz;
  const int grid = (int)std::max(1L, std::min(ntiles, (long)slots[dev]));
  conv3_tc_kernel<CIN, COUT, NBUF><<<grid, kThreads, smem, s>>>(maps, g, wt, mat, gate, pre, gated, pre_f32, gated_f32,
                                                          status, limit_ns);
  return cudaGetLastError();
}

}  // namespace

cudaError_t conv3_tc(int cin, int cout, const Grid& g, const __nv_bfloat16* in, const __nv_bfloat16* wt,
                     const float2* mat, const float* gate, __nv_bfloat16* pre, __nv_bfloat16* gated, float* pre_f32,
                     float* gated_f32, int* status, long long limit_ns, cudaStream_t s, std::string* err) {
  EncodeTiled enc = encoder(err);
  if (!enc) return cudaErrorNotSupported;
  if ((cin != 16 && cin != 32) || (cout != 16 && cout != 32) || (reinterpret_cast<uintptr_t>(in) & 15)) {
    if (err) *err = "convolution: 16 or 32 channels in and out, 16-byte aligned input";
    return cudaErrorInvalidValue;
  }
  TmapSet maps;
  const cuuint64_t dims[4] = {8, (cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
  const cuuint64_t strides[3] = {(cuuint64_t)cin * 2, (cuuint64_t)g.nx * cin * 2, (cuuint64_t)g.nx * g.ny * cin * 2};
  const cuuint32_t box[4] = {8, kBx, kBy, kBz};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  for (int c = 0; c < cin / 8; ++c) {
    const CUresult r = enc(&maps.m[c], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)(in + 8 * c), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      if (err) {
        char buf[96];
        std::snprintf(buf, sizeof buf, "convolution: tensor map encoding failed (%d)", (int)r);
        *err = buf;
      }
      return cudaErrorInvalidValue;
    }
  }
  // two brick buffers where shared memory leaves room for several CTAs per SM
  if (cin == 16 && cout == 16)
    return launch<16, 16, 2>(maps, g, wt, mat, gate, pre, gated, pre_f32, gated_f32, status, limit_ns, s);
  if (cin == 16 && cout == 32)
    return launch<16, 32, 2>(maps, g, wt, mat, gate, pre, gated, pre_f32, gated_f32, status, limit_ns, s);
  if (cin == 32 && cout == 32)
    return launch<32, 32, 1>(maps, g, wt, mat, gate, pre, gated, pre_f32, gated_f32, status, limit_ns, s);
  return launch<32, 16, 2>(maps, g, wt, mat, gate, pre, gated, pre_f32, gated_f32, status, limit_ns, s);
}

}  // namespace cnn
}  // namespace ouranos
