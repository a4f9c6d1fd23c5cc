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

// ------------------------------------------------------------ weight gradient
// dW[tap][ci][co] += sum_v in[v + off(tap)][ci] g[v][co] as a tcgen05 GEMM:
// M = the 27 CIN rows (tap, ci) in 128-row tiles, N = COUT, K = voxels in
// chunks of 32 (two MMAs of K = 16 per tile).  Both operands are K-major, so
// a chunk is staged as the transpose of the channels-last tensors: a warp
// reads 512 contiguous bytes (16 voxels x 8 channels for one tap of A, the
// tap's voxel shift applied, zero outside the grid and past the last voxel),
// neighbouring lanes swap halves so that each holds four channels of a voxel
// pair, and each writes those as four 4-byte (voxel, voxel + 1) pairs into
// the rows of its core matrix, bank-conflict free.  Two staging buffers, each
// reused once the MMAs that read it have completed; the next chunk's gathers
// are in flight while this chunk's MMAs are issued.  Each CTA sums its
// chunks in tensor memory (all M tiles at once) and adds its partial into dW
// with 16-byte vector atomics.  The CUDA-core form this replaces (one block
// per tap and 2048 voxels, thread per (ci, co)) took 2.02 ms for 32 -> 32
// channels on a 64^3 grid on GB300; this takes 0.133 ms.
constexpr int kWgThreads = 512;
constexpr int kWgChunk = 32;  // voxels per K chunk

template <int CIN, int COUT>
struct WgShape {
  static constexpr int ROWS = 27 * CIN;
  static constexpr int MT = (ROWS + 127) / 128;            // 128-row tiles of A
  static constexpr uint32_t SBO = kWgChunk / 8 * 128;      // four core matrices of K per row group
  static constexpr uint32_t ATILE = 128 / 8 * SBO;         // 8 KB
  static constexpr uint32_t ABUF = MT * ATILE;
  static constexpr uint32_t BBUF = COUT / 8 * SBO;
  static constexpr uint32_t COLS = MT * COUT <= 32 ? 32 : MT * COUT <= 64 ? 64 : MT * COUT <= 128 ? 128 : 256;
  static constexpr size_t SMEM = 2 * (size_t)(ABUF + BBUF) + 64;  // + 4 mbarriers and the column slot
  static_assert((size_t)ROWS * COUT * 4 <= 2 * (size_t)(ABUF + BBUF), "the partial dW fits the staging buffers");
};

// One voxel pair's share of a core matrix.  This thread holds channels
// [8 c8, 8 c8 + 8) of voxel j of the chunk (u); lane ^ q holds the same
// channels of voxel j ^ 1.  The two swap two words, then the even voxel's
// thread writes the BF16 pairs (voxel j low, j + 1 high) of channels 0-3 into
// rows 0-3 of the core matrix at base, the odd one those of channels 4-7 into
// rows 4-7.  Rows are visited from kk ^ rot (the pairs permuted to match by
// two conditional swaps, so that indices stay static) so that the stores of
// a warp cover the 32 banks once.
__device__ __forceinline__ void stage_half(uint8_t* base, const uint4& u, int q, bool odd, int rot) {
  const uint32_t r0 = __shfl_xor_sync(0xffffffffu, odd ? u.x : u.z, q);
  const uint32_t r1 = __shfl_xor_sync(0xffffffffu, odd ? u.y : u.w, q);
  const uint32_t a0 = odd ? r0 : u.x, a1 = odd ? r1 : u.y;  // the even voxel's four channels
  const uint32_t b0 = odd ? u.z : r0, b1 = odd ? u.w : r1;  // the odd voxel's
  uint32_t p[4] = {__byte_perm(a0, b0, 0x5410), __byte_perm(a0, b0, 0x7632), __byte_perm(a1, b1, 0x5410),
                   __byte_perm(a1, b1, 0x7632)};
#pragma unroll
  for (int bit = 1; bit < 4; bit <<= 1)
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (!(j & bit)) {
        const bool sw = (rot & bit) != 0;
        const uint32_t lo = p[j], hi = p[j | bit];
        p[j] = sw ? hi : lo;
        p[j | bit] = sw ? lo : hi;
      }
  uint8_t* rows = base + (odd ? 64 : 0);
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) *reinterpret_cast<uint32_t*>(rows + (kk ^ rot) * 16) = p[kk];
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(kWgThreads, 1) conv3_wgrad_tc_kernel(Grid g, const __nv_bfloat16* __restrict__ in,
                                                                      const __nv_bfloat16* __restrict__ grad,
                                                                      float* __restrict__ dw, int* status,
                                                                      long long limit_ns) {
  using S = WgShape<CIN, COUT>;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* A = smem;
  uint8_t* B = smem + 2 * S::ABUF;
  // mbarriers: staging buffers 0 and 1, all MMAs 2, the error path 3
  uint64_t* bar = reinterpret_cast<uint64_t*>(B + 2 * S::BBUF);
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // zero both buffers once: the rows past 27 CIN are never written
  for (uint32_t o = tid * 16u; o < 2 * (S::ABUF + S::BBUF); o += kWgThreads * 16u)
    *reinterpret_cast<uint4*>(smem + o) = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) {
    for (int i = 0; i < 4; ++i) tc5::mbar_init(bar + i, 1);
    tc5::mbar_init_fence();
  }
  if (warp == 0) {
    tc5::tmem_alloc(slot, S::COLS);
    tc5::tmem_relinquish();
  }
  tc5::fence_before_sync();
  __syncthreads();
  tc5::fence_after_sync();
  const uint32_t tmem = *slot;
  const long V = g.voxels();
  const long nchunks = (V + kWgChunk - 1) / kWgChunk;
  constexpr uint32_t idesc = tc5::idesc_bf16_f32(128, COUT);
  // Staging: A task (tap, voxel j of the chunk, 8-channel group c8), B task
  // (j, c8), c8 fastest, so that the 32 lanes of a warp read 512 contiguous
  // bytes of one tap.  A thread's j and c8 are the same in every round (the
  // thread count is a multiple of 32 QA): its voxel's position is found once
  // per chunk, and all of its gathers are issued before its first store.
  constexpr int QA = CIN / 8, QB = COUT / 8;
  constexpr int TA = 27 * kWgChunk * QA, TB = kWgChunk * QB;
  constexpr int NT = (TA + kWgThreads - 1) / kWgThreads;
  constexpr int TAPS = kWgThreads / (kWgChunk * QA);  // taps per round
  static_assert(kWgThreads % (kWgChunk * QA) == 0 && TA % 32 == 0 && TB % 32 == 0 && TB <= kWgThreads,
                "whole warps per task range, a thread keeps its voxel");
  const int ca = tid % QA, ja = (tid / QA) % kWgChunk, tap0 = tid / (kWgChunk * QA);
  const int cb = tid % QB, jb = (tid / QB) % kWgChunk;
  // first rows: the lanes that share a bank column differ in c8 and in j / 8
  const int rota = (ca + QA * (ja >> 3)) & 3, rotb = (cb + QB * (jb >> 3)) & 3;
  // the 16 bytes of channels [8 c8, 8 c8 + 8) at (x, y, z), 0 outside the grid or when !live
  auto at = [&](const __nv_bfloat16* t, int C, bool live, int x, int y, int z, int c8) {
    uint4 u = make_uint4(0u, 0u, 0u, 0u);
    if (live && x >= 0 && x < g.nx && y >= 0 && y < g.ny && z >= 0 && z < g.nz)
      u = __ldg(reinterpret_cast<const uint4*>(t + ((long)x + (long)g.nx * (y + (long)g.ny * z)) * C) + c8);
    return u;
  };
  // the byte offset of voxel j's pair in a row group
  const uint32_t cola = (uint32_t)(ja >> 3) * 128u + (uint32_t)(ja & 6) * 2u;
  const uint32_t colb = (uint32_t)(jb >> 3) * 128u + (uint32_t)(jb & 6) * 2u;
  // the gathers of chunk ch: ra[i] for tap tap0 + TAPS i, rgv from the
  // output gradient (past the last voxel: not live, staged as 0)
  uint4 ra[NT], rgv;
  auto gather = [&](long ch) {
    const long va = ch * kWgChunk + ja, vb = ch * kWgChunk + jb;
    const int xa = (int)(va % g.nx), ya = (int)((va / g.nx) % g.ny), za = (int)(va / ((long)g.nx * g.ny));
#pragma unroll
    for (int i = 0; i < NT; ++i) {
      const int tap = tap0 + TAPS * i;
      ra[i] = at(in, CIN, tap < 27 && va < V, xa + tap_dx(tap), ya + tap_dy(tap), za + tap_dz(tap), ca);
    }
    rgv = make_uint4(0u, 0u, 0u, 0u);
    if (tid < TB && vb < V) rgv = __ldg(reinterpret_cast<const uint4*>(grad + vb * COUT) + cb);
  };
  uint32_t ph_buf = 0u;
  long k = 0;  // chunks this CTA has staged
  bool ok = true;
  if (blockIdx.x < nchunks) gather(blockIdx.x);
  for (long ch = blockIdx.x; ch < nchunks; ch += gridDim.x, ++k) {
    const int b = (int)(k & 1);
    if (k >= 2) {  // the MMAs that read this buffer two chunks ago
      bool w = true;
      if (tid == 0) w = tc5::mbar_wait(bar + b, (ph_buf >> b) & 1u, limit_ns);
      ph_buf ^= 1u << b;
      ok = __syncthreads_and(w);
      if (!ok) break;
    }
    uint8_t* Ab = A + b * S::ABUF;
    uint8_t* Bb = B + b * S::BBUF;
#pragma unroll
    for (int i = 0; i < NT; ++i) {
      const int tap = tap0 + TAPS * i;
      const int grp = (tap * CIN + 8 * ca) >> 3;  // row group (tap, 8 ca .. 8 ca + 7)
      if (tap < 27)  // whole warps
        stage_half(Ab + (grp >> 4) * S::ATILE + (grp & 15) * S::SBO + cola, ra[i], QA, ja & 1, rota);
    }
    if (tid < TB) stage_half(Bb + cb * S::SBO + colb, rgv, QB, jb & 1, rotb);
    // the next chunk's gathers are in flight during the barrier and the MMAs
    if (ch + gridDim.x < nchunks) gather(ch + gridDim.x);
    tc5::fence_smem_to_async();
    tc5::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc5::fence_after_sync();
#pragma unroll
      for (int mt = 0; mt < S::MT; ++mt)
#pragma unroll
        for (int ks = 0; ks < kWgChunk / 16; ++ks) {
          const uint64_t ad = tc5::smem_desc(tc5::smem_addr(Ab + mt * S::ATILE + ks * 256), 128, S::SBO);
          const uint64_t bd = tc5::smem_desc(tc5::smem_addr(Bb + ks * 256), 128, S::SBO);
          tc5::mma_bf16(tmem + (uint32_t)(mt * COUT), ad, bd, idesc, k > 0 || ks > 0);
        }
      tc5::mma_commit(bar + b);
    }
  }
  if (ok && k > 0) {  // every MMA of this CTA done: the partial sums into dW
    bool w = true;
    if (tid == 0) {
      tc5::mma_commit(bar + 2);
      w = tc5::mbar_wait(bar + 2, 0u, limit_ns);
    }
    ok = __syncthreads_and(w);
    if (ok) {
      tc5::fence_after_sync();
      // the CTA's partial dW [ROWS][COUT] goes through the staging buffers
      // (free: every MMA has completed), its 16-byte column groups XOR-swizzled
      // by the row so that the writes of a warp spread over the banks, then
      // into dW with 16-byte vector atomics on consecutive addresses
      constexpr int C4 = COUT / 4;
      float4* part = reinterpret_cast<float4*>(smem);
      const int sub = warp & 3;
      for (int mt = warp >> 2; mt < S::MT; mt += kWgThreads / 128) {
        const int row = mt * 128 + 32 * sub + lane;
        const uint32_t base = tmem + ((uint32_t)(32 * sub) << 16) + (uint32_t)(mt * COUT);
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
          float v[16];
          tc5::tmem_ld16(base + (uint32_t)c0, v);
          if (row < S::ROWS) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
              part[row * C4 + ((c0 / 4 + q) ^ (row & (C4 - 1)))] =
                  make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
          }
        }
      }
      __syncthreads();
      for (int i = tid; i < S::ROWS * C4; i += kWgThreads) {
        const int row = i / C4, c4 = i % C4;
        const float4 v = part[row * C4 + (c4 ^ (row & (C4 - 1)))];
        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dw + 4L * i), "f"(v.x), "f"(v.y),
                     "f"(v.z), "f"(v.w)
                     : "memory");
      }
    }
  }
  if (!ok) {  // a wait ran out: one more bounded wait for every MMA issued, then free the columns
    if (tid == 0) {
      if (status) atomicOr(status, 1);
      tc5::mma_commit(bar + 3);
      tc5::mbar_wait(bar + 3, 0u, limit_ns);
    }
  }
  tc5::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc5::fence_after_sync();
    tc5::tmem_dealloc(tmem, S::COLS);
  }
}

template <int CIN, int COUT>
cudaError_t wgrad_launch(const Grid& g, const __nv_bfloat16* in, const __nv_bfloat16* grad, float* dw, int* status,
                         long long limit_ns, cudaStream_t s) {
  using S = WgShape<CIN, COUT>;
  static int sms[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!sms[dev]) {
    e = cudaFuncSetAttribute(conv3_wgrad_tc_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)S::SMEM);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  // at most one CTA per SM (the shared memory allows no second), each summing
  // at least 8 chunks before its 27 CIN COUT atomic adds
  const long nchunks = (g.voxels() + kWgChunk - 1) / kWgChunk;
  if (nchunks == 0) return cudaSuccess;
  const int grid = (int)std::max(1L, std::min((nchunks + 7) / 8, (long)sms[dev]));
  conv3_wgrad_tc_kernel<CIN, COUT><<<grid, kWgThreads, S::SMEM, s>>>(g, in, grad, dw, status, limit_ns);
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

cudaError_t conv3_wgrad_tc(int cin, int cout, const Grid& g, const __nv_bfloat16* in, const __nv_bfloat16* grad,
                           float* dw, int* status, long long limit_ns, cudaStream_t s) {
  if ((reinterpret_cast<uintptr_t>(in) & 15) || (reinterpret_cast<uintptr_t>(grad) & 15) ||
      (reinterpret_cast<uintptr_t>(dw) & 15))
    return cudaErrorInvalidValue;
  if (cin == 16 && cout == 16) return wgrad_launch<16, 16>(g, in, grad, dw, status, limit_ns, s);
  if (cin == 16 && cout == 32) return wgrad_launch<16, 32>(g, in, grad, dw, status, limit_ns, s);
  if (cin == 32 && cout == 32) return wgrad_launch<32, 32>(g, in, grad, dw, status, limit_ns, s);
  if (cin == 32 && cout == 16) return wgrad_launch<32, 16>(g, in, grad, dw, status, limit_ns, s);
  return cudaErrorInvalidValue;
}

}  // namespace cnn
}  // namespace ouranos
