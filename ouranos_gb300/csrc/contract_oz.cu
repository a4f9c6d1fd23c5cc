// Direction-axis contractions of the double-float sweep on the tensor cores
// (tcgen05.mma, BF16 operands, FP32 accumulators in tensor memory) at FP64
// accuracy, by exact digit products (the splitting scheme of Ozaki, Ogita,
// Oishi and Rump, 2012, with BF16 digits):
//
//   expansion  q[d][e]   = sum_m M2D[d][m] T[m][e] (+ iso[e])
//              (reference: the M2D source assembly, src/RadiativeTransfer.cc:907-913)
//   reduction  phi[m][e] = sum_d D2M[m][d] psi[d][e]
//              (reference: the D2M accumulation, src/RadiativeTransfer.cc:990-996)
//
// Digits.  A row of the vector operand (one dof's values over the K axis, or
// over a chunk of it) is scaled by a power of two 2^-E so that every value is
// below 1 in magnitude, and each value x = hi + lo (a double-float pair) is
// cut into seven digits on the fixed grids 2^-8, 2^-16, ..., 2^-56:
// digit k is a multiple of 2^-8(k+1) of at most 256 units, so it is exactly a
// BF16 number, and x - sum_k digit_k is below 2^-56.  The digits come from
// round-to-nearest extractions t = (x + 1.5 * 2^(15-8k)) - 1.5 * 2^(15-8k)
// in FP32 (exact, with an exact remainder x - t).  The matrix (M2D or D2M)
// is cut the same way on the host, per direction (expansion) or per moment
// and chunk (reduction).
//
// Products.  A digit product a_i b_j is a multiple of 2^-8(i+j+2) below 2^16
// units, so a sum of them over K values stays an integer number of units.
// Level L = i + j collects the pairs of that level; levels 0..3 each get
// their own FP32 accumulator, and while a level's sum stays below 2^24 units
// (K <= 64 for level 3's four pairs) the tensor core adds it exactly.
// Levels 4..6 share a fifth accumulator: its value is below 2^-24 of the
// scale, so its FP32 rounding stays near 2^-48 of the scale, the precision
// of the double-float inputs; levels 7 and up are dropped (below 2^-62 of
// the scale).  28 MMAs per K step.  The epilogue sums the five accumulators in compensated
// FP32 arithmetic (a double-float result), scales back by 2^(E + F) and
// stores: the same ~48-bit accuracy as the double-float contractions on the
// CUDA cores, with the multiply-adds on the tensor pipe.
//
// Operand tiles in shared memory are K-major without swizzling (tc5.cuh).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "df64.cuh"
#include "internal.h"
#include "tc5.cuh"

namespace ouranos {
namespace {

constexpr int kRows = 128;   // dofs per tile: the MMA's M, one tensor-memory lane each
constexpr int kDig = 7;      // BF16 digits per value
constexpr int kLmax = 6;     // highest digit level kept
constexpr int kSlots = 5;    // accumulators: levels 0, 1, 2, 3, and 4..6 together
constexpr int kPart = 48;    // expansion: directions per accumulator set (5 x 48 tensor-memory columns)
constexpr int kChunk = 48;   // reduction: directions per exponent chunk
constexpr int kWorkers = 512;  // staging / epilogue threads (16 warps); warp 16 issues the MMAs
constexpr int kThreads = kWorkers + 32;

__device__ __forceinline__ float pow2f(int k) { return __uint_as_float((uint32_t)(k + 127) << 23); }
// E with max |value| < 2^E, from the largest |hi| of a row (0 -> -126: every
// digit is 0).  Capped at 126 so that 2^-E and 2^E are normal FP32 numbers:
// rows beyond 2^126 (8.5e37, past what the double-float sweep carries) would
// leave the digit bounds.
__device__ __forceinline__ int row_exponent(float maxabs) {
  return min((int)((__float_as_uint(maxabs) >> 23) & 0xffu) - 126, 126);
}

// round-to-nearest extraction of x on the grid of sigma / 1.5 * 2^-23
__device__ __forceinline__ float extract(float& x, float sigma) {
  const float t = __fsub_rn(__fadd_rn(x, sigma), sigma);
  x = __fsub_rn(x, t);
  return t;
}
// The seven digits of hi + lo, |hi + lo| < 1.  |lo| <= 2^-25 is zero on the
// grids of levels 0 and 1; after level 3 the two remainders are below 2^-33
// and their FP32 sum rounds below 2^-57, so levels 4..6 extract from it.
__device__ __forceinline__ void digits7(float hi, float lo, float (&d)[kDig]) {
  d[0] = extract(hi, 0x1.8p15f);
  d[1] = extract(hi, 0x1.8p7f);
  d[2] = extract(hi, 0x1.8p-1f) + extract(lo, 0x1.8p-1f);
  d[3] = extract(hi, 0x1.8p-9f) + extract(lo, 0x1.8p-9f);
  float r = hi + lo;
  d[4] = extract(r, 0x1.8p-17f);
  d[5] = extract(r, 0x1.8p-25f);
  d[6] = extract(r, 0x1.8p-33f);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);  // exact: digits are BF16 numbers
  return *reinterpret_cast<const uint32_t*>(&v);
}

// compensated sum of FP32 terms (df64.cuh's accumulator, one term at a time)
__device__ __forceinline__ void acc_addf(df64_acc& acc, float a) {
  const float s = acc.s + a;
  const float bb = s - acc.s;
  acc.c += (acc.s - (s - bb)) + (a - bb);
  acc.s = s;
}
// the five accumulators of one output as a double-float number
__device__ __forceinline__ df64 slot_sum(const float (&v)[kSlots]) {
  df64_acc a = {v[kSlots - 1], 0.f};  // smallest first
#pragma unroll
  for (int s = kSlots - 2; s >= 0; --s) acc_addf(a, v[s]);
  return acc_result(a);
}

// The 28 digit products, highest level first (the shared accumulator adds
// its smallest terms first); one MMA per pair and K step.
template <typename F>
__device__ __forceinline__ void for_each_pair(F&& f) {
#pragma unroll
  for (int L = kLmax; L >= 0; --L)
#pragma unroll
    for (int i = 0; i < kDig; ++i) {
      const int j = L - i;
      if (j < 0 || j >= kDig) continue;
      const int slot = L < kSlots - 1 ? L : kSlots - 1;
      const bool first = (L < kSlots - 1 || L == kLmax) && i == (L >= kDig ? L - kDig + 1 : 0);
      f(i, j, slot, first);
    }
}

// Pipeline waits.  Every wait is bounded by the handle's wait limit; the
// first that runs out raises the CTA's abort flag (and bit 4 of the status
// word), and every other wait gives up as soon as it sees the flag, so all
// threads reach the end of the kernel.  Waits run on one lane of a warp.
__device__ __forceinline__ bool pipe_wait(uint64_t* bar, uint32_t parity, long long limit_ns, volatile int* abort,
                                          int* status) {
  if (tc5::mbar_try_wait(bar, parity)) return true;
  const long long t0 = tc5::globaltimer();
  for (;;) {
    if (tc5::mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if (tc5::globaltimer() - t0 > limit_ns) {
      *abort = 1;
      if (status) atomicOr(status, 4);
      return false;
    }
  }
}
// the whole warp waits (lane 0 polls)
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity, long long limit_ns, volatile int* abort,
                                          int* status) {
  int ok = 1;
  if ((threadIdx.x & 31) == 0) ok = pipe_wait(bar, parity, limit_ns, abort, status);
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

// After every role has left its loop: if the pipeline was aborted, the MMAs
// already issued get one more bounded wait before the columns are freed.
__device__ __forceinline__ void finish(volatile int* abort, uint64_t* bar_err, long long limit_ns, int mma_warp,
                                       uint32_t tmem, uint32_t cols) {
  __syncthreads();
  const int warp = threadIdx.x >> 5;
  if (*abort && warp == mma_warp && (threadIdx.x & 31) == 0) {
    tc5::mma_commit(bar_err);
    tc5::mbar_wait(bar_err, 0u, limit_ns);
  }
  __syncthreads();
  if (warp == mma_warp) {
    tc5::fence_after_sync();
    tc5::tmem_dealloc(tmem, cols);
  }
}

// ------------------------------------------------------------- expansion
// Tile = 128 dofs; A = the dofs' moments (K = 16 slots), one row exponent per
// dof; B = M2D (N = directions, npad rows), digits per direction.  The
// directions run in parts of 48: 28 MMAs into 5 x 48 accumulator columns.
// Roles: warp 16 issues the MMAs; warps 0-15 stage A (two buffers, one per
// tile in flight) and drain the accumulators (two sets of 256 columns, so
// the MMAs of the next part run while the current one is drained).
//   afull[ab]    A staged (512 arrivals)      aempty[ab]   A read (commit)
//   accfull[pb]  part's MMAs done (commit)    accempty[pb] part drained (512 arrivals)
//   staged[t&1]  every worker has staged tile t (512 arrivals; the row exponents are visible)
__global__ void __launch_bounds__(kThreads, 1) expand_oz_kernel(const df64* __restrict__ T,
                                                               const df64* __restrict__ iso,
                                                               const uint8_t* __restrict__ bimg,
                                                               const int* __restrict__ bexp,
                                                               df64* __restrict__ q, int n_dir, int n_mom, int npad,
                                                               long n_dofs, long len, int* status,
                                                               long long limit_ns) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t kSbo = 256;                    // two core matrices of K per row group
  constexpr uint32_t kAdig = kRows / 8 * kSbo;      // 128 rows x 16 moments, BF16
  constexpr uint32_t kAbuf = kDig * kAdig;
  const uint32_t bdig = (uint32_t)npad / 8 * kSbo;  // npad rows x 16 moments, BF16
  uint8_t* A = smem;
  uint8_t* B = A + 2 * kAbuf;
  float* Fs = reinterpret_cast<float*>(B + kDig * bdig);  // [npad] 2^F per direction
  int* Es = reinterpret_cast<int*>(Fs + npad);             // [2][128] row exponents per tile parity
  uint64_t* bar = reinterpret_cast<uint64_t*>(Es + 2 * kRows);
  uint64_t* afull = bar;        // [2]
  uint64_t* aempty = bar + 2;   // [2]
  uint64_t* accfull = bar + 4;  // [2]
  uint64_t* accempty = bar + 6; // [2]
  uint64_t* staged = bar + 8;   // [2]
  uint64_t* bar_err = bar + 10;
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 11);
  volatile int* abort = reinterpret_cast<volatile int*>(slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int kMmaWarp = kWorkers / 32;
  for (uint32_t o = tid * 16u; o < kDig * bdig; o += kThreads * 16u)
    *reinterpret_cast<uint4*>(B + o) = __ldg(reinterpret_cast<const uint4*>(bimg + o));
  for (int k = tid; k < npad; k += kThreads) Fs[k] = pow2f(bexp[k]);
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      tc5::mbar_init(afull + i, kWorkers);
      tc5::mbar_init(aempty + i, 1);
      tc5::mbar_init(accfull + i, 1);
      tc5::mbar_init(accempty + i, kWorkers);
      tc5::mbar_init(staged + i, kWorkers);
    }
    tc5::mbar_init(bar_err, 1);
    *abort = 0;
    tc5::mbar_init_fence();
  }
  if (warp == kMmaWarp) {
    tc5::tmem_alloc(slot, 512);
    tc5::tmem_relinquish();
  }
  tc5::fence_before_sync();
  __syncthreads();
  tc5::fence_after_sync();
  const uint32_t tmem = *slot;
  const long ntiles = (len + kRows - 1) / kRows;
  const int nparts = (npad + kPart - 1) / kPart;

  if (warp == kMmaWarp) {
    if (lane == 0) {
      long gp = 0;  // parts issued
      int tl = 0;   // tiles of this CTA
      for (long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++tl) {
        const int ab = tl & 1;
        if (!pipe_wait(afull + ab, (uint32_t)(tl >> 1) & 1u, limit_ns, abort, status)) break;
        bool ok = true;
        for (int p = 0; p < nparts; ++p, ++gp) {
          const int pb = (int)(gp & 1);
          if (gp >= 2 && !pipe_wait(accempty + pb, (uint32_t)((gp >> 1) - 1) & 1u, limit_ns, abort, status)) {
            ok = false;
            break;
          }
          tc5::fence_after_sync();
          const int c0 = p * kPart;
          const int np = min(kPart, npad - c0);  // a multiple of 16
          const uint32_t idesc = tc5::idesc_bf16_f32(kRows, np);
          const uint32_t dbase = tmem + (uint32_t)(pb * 256);
          for_each_pair([&](int i, int j, int s, bool first) {
            const uint64_t ad = tc5::smem_desc(tc5::smem_addr(A + ab * kAbuf + i * kAdig), 128, kSbo);
            const uint64_t bd = tc5::smem_desc(tc5::smem_addr(B + j * bdig + (c0 / 8) * kSbo), 128, kSbo);
            tc5::mma_bf16(dbase + (uint32_t)(s * kPart), ad, bd, idesc, !first);
          });
          tc5::mma_commit(accfull + pb);
        }
        if (!ok) break;
        tc5::mma_commit(aempty + ab);
      }
    }
    __syncwarp();
  } else {
    long gp = 0;
    int tl = 0;
    bool ok = true;
    for (long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++tl) {
      const int ab = tl & 1;
      const long e0 = tile * kRows;
      if (tl >= 2 && !warp_wait(aempty + ab, (uint32_t)((tl >> 1) - 1) & 1u, limit_ns, abort, status)) break;
      {  // stage A: thread (row r, quarter u) cuts moments [4u, 4u + 4) of dof e0 + r
        const int r = tid >> 2, u = tid & 3;
        const long e = e0 + r;
        float hi[4], lo[4];
        float mx = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int m = 4 * u + k;
          float2 v = make_float2(0.f, 0.f);
          if (e < len && m < n_mom) v = __ldg(reinterpret_cast<const float2*>(T + (long)m * n_dofs + e));
          hi[k] = v.x;
          lo[k] = v.y;
          mx = fmaxf(mx, fabsf(v.x));
        }
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
        const int E = row_exponent(mx);
        if (u == 0) Es[ab * kRows + r] = E;
        const float sc = pow2f(-E);
        float d[4][kDig];
#pragma unroll
        for (int k = 0; k < 4; ++k) digits7(hi[k] * sc, lo[k] * sc, d[k]);
        const uint32_t off = tc5::kmajor_offset(r, 4 * u, kSbo);
#pragma unroll
        for (int g = 0; g < kDig; ++g)
          *reinterpret_cast<uint2*>(A + ab * kAbuf + g * kAdig + off) =
              make_uint2(pack_bf16(d[0][g], d[1][g]), pack_bf16(d[2][g], d[3][g]));
      }
      tc5::fence_smem_to_async();
      tc5::mbar_arrive(afull + ab);
      tc5::mbar_arrive(staged + (tl & 1));
      if (!warp_wait(staged + (tl & 1), (uint32_t)(tl >> 1) & 1u, limit_ns, abort, status)) break;
      // epilogue: warp w reads the lanes of sub-partition w & 3 and columns
      // [12 (w >> 2), +12) of each part; q is read once, by the sweep, so it
      // is stored with streaming (evict-first) stores
      const int sub = warp & 3, cg = warp >> 2;
      const int rr = 32 * sub + lane;
      const long e = e0 + rr;
      const float sE = pow2f(Es[ab * kRows + rr]);
      float2 is = make_float2(0.f, 0.f);
      if (iso && e < len) is = __ldg(reinterpret_cast<const float2*>(iso + e));
      for (int p = 0; p < nparts; ++p, ++gp) {
        const int pb = (int)(gp & 1);
        if (!warp_wait(accfull + pb, (uint32_t)(gp >> 1) & 1u, limit_ns, abort, status)) {
          ok = false;
          break;
        }
        tc5::fence_after_sync();
        const int c0 = p * kPart;
        const int np = min(kPart, npad - c0);
        const uint32_t lane_base = tmem + ((uint32_t)(32 * sub) << 16) + (uint32_t)(pb * 256);
#pragma unroll
        for (int blk = 0; blk < 3; ++blk) {
          const int cb = 12 * cg + 4 * blk;
          if (cb >= np) break;  // warp-uniform
          float v[kSlots][4];
#pragma unroll
          for (int s = 0; s < kSlots; ++s) tc5::tmem_ld4(lane_base + (uint32_t)(s * kPart + cb), v[s]);
          if (e < len) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const int d = c0 + cb + k;
              if (d < n_dir) {
                const float u5[kSlots] = {v[0][k], v[1][k], v[2][k], v[3][k], v[4][k]};
                const df64 x = slot_sum(u5);
                const float sc = sE * Fs[d];
                df64 y(x.hi * sc, x.lo * sc);
                if (iso) {
                  df64_acc a = acc_from(y);
                  acc_add(a, df64(is.x, is.y));
                  y = acc_result(a);
                }
                __stcs(reinterpret_cast<float2*>(q + (long)d * n_dofs + e), make_float2(y.hi, y.lo));
              }
            }
          }
        }
        tc5::fence_before_sync();
        tc5::mbar_arrive(accempty + pb);
      }
    }
  }
  finish(abort, bar_err, limit_ns, kMmaWarp, tmem, 512);
}

// ------------------------------------------------------------- reduction
// Tile = 128 dofs; K = directions in NCH chunks of 48, each chunk with its
// own row exponents; N = the D2M digits stacked (7 x 16 moment slots), so
// one MMA multiplies digit i of psi by every digit j <= 6 - i of D2M and
// writes pair (i, j) into column block i + j: seven accumulator blocks per
// chunk, one per level, 7 MMAs per K step.  Levels 0..4 stay below 2^24
// units (at most five pairs x 48 values x 2^16) and are exact; levels 5 and
// 6 round below 2^-56 of the scale.  Roles: warp 16 issues the MMAs; worker thread (row r = tid >> 2,
// quarter u = tid & 3) loads the 12 values of directions [48 c + 12 u, +12)
// of its dof (the next chunk's values are in flight while this one is cut),
// stages them (two buffers), and after the tile's last chunk the workers
// drain the accumulators.
//   full[b]   chunk staged (512 arrivals)   empty[b]  chunk read (commit)
//   tfull     tile's MMAs done (commit)      tempty    tile drained (512 arrivals)
//   staged[t&1]  every worker has staged tile t (its row exponents are visible)
template <int NCH>
__global__ void __launch_bounds__(kThreads, 1) reduce_oz_kernel(const df64* __restrict__ psi,
                                                               const uint8_t* __restrict__ bimg,
                                                               const int* __restrict__ bexp,
                                                               double* __restrict__ phi, int n_dir, int n_mom,
                                                               long n_dofs, long len, int* status,
                                                               long long limit_ns, const double* __restrict__ xc) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t kSbo = kChunk / 8 * 128;     // six core matrices of K per row group
  constexpr uint32_t kAdig = kRows / 8 * kSbo;    // 128 rows x 48 directions, BF16
  constexpr uint32_t kAbuf = kDig * kAdig;
  constexpr uint32_t kBdig = 2 * kSbo;            // 16 moment rows x 48 directions, BF16
  constexpr int kCols = kDig * 16;                // accumulator columns per chunk: one block per level
  constexpr uint32_t kTmemCols = NCH * kCols <= 128 ? 128 : NCH * kCols <= 256 ? 256 : 512;
  static_assert(NCH * kCols <= 512, "tensor memory holds four chunks");
  uint8_t* A = smem;
  uint8_t* B = A + 2 * kAbuf;
  float* Fs = reinterpret_cast<float*>(B + NCH * kDig * kBdig);  // [NCH][16] 2^F per moment
  int* Es = reinterpret_cast<int*>(Fs + NCH * 16);                // [2][NCH][128] row exponents
  uint64_t* bar = reinterpret_cast<uint64_t*>(Es + 2 * NCH * kRows);
  uint64_t* full = bar;         // [2]
  uint64_t* empty = bar + 2;    // [2]
  uint64_t* tfull = bar + 4;
  uint64_t* tempty = bar + 5;
  uint64_t* staged = bar + 6;   // [2]
  uint64_t* bar_err = bar + 8;
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 9);
  volatile int* abort = reinterpret_cast<volatile int*>(slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int kMmaWarp = kWorkers / 32;
  for (uint32_t o = tid * 16u; o < NCH * kDig * kBdig; o += kThreads * 16u)
    *reinterpret_cast<uint4*>(B + o) = __ldg(reinterpret_cast<const uint4*>(bimg + o));
  for (int k = tid; k < NCH * 16; k += kThreads) Fs[k] = pow2f(bexp[k]);
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      tc5::mbar_init(full + i, kWorkers);
      tc5::mbar_init(empty + i, 1);
      tc5::mbar_init(staged + i, kWorkers);
    }
    tc5::mbar_init(tfull, 1);
    tc5::mbar_init(tempty, kWorkers);
    tc5::mbar_init(bar_err, 1);
    *abort = 0;
    tc5::mbar_init_fence();
  }
  if (warp == kMmaWarp) {
    tc5::tmem_alloc(slot, kTmemCols);
    tc5::tmem_relinquish();
  }
  tc5::fence_before_sync();
  __syncthreads();
  tc5::fence_after_sync();
  const uint32_t tmem = *slot;
  const long ntiles = (len + kRows - 1) / kRows;

  if (warp == kMmaWarp) {
    if (lane == 0) {
      long g = 0;  // chunks issued
      int tl = 0;
      bool ok = true;
      for (long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++tl) {
        for (int c = 0; c < NCH; ++c, ++g) {
          const int b = (int)(g & 1);
          if (!pipe_wait(full + b, (uint32_t)(g >> 1) & 1u, limit_ns, abort, status)) {
            ok = false;
            break;
          }
          if (c == 0 && tl > 0 && !pipe_wait(tempty, (uint32_t)(tl - 1) & 1u, limit_ns, abort, status)) {
            ok = false;
            break;
          }
          tc5::fence_after_sync();
          const uint32_t dc = tmem + (uint32_t)(c * kCols);
          uint8_t* Ab = A + b * kAbuf;
          // digit i of psi against digits 0 .. 6 - i of D2M, stacked along N
          // (the chunk's seven digit images are consecutive row groups): the
          // product with digit j lands in column block i + j, its level
#pragma unroll
          for (int ks = 0; ks < kChunk / 16; ++ks)
#pragma unroll
            for (int i = 0; i < kDig; ++i) {
              const uint64_t ad = tc5::smem_desc(tc5::smem_addr(Ab + i * kAdig + ks * 256), 128, kSbo);
              const uint64_t bd = tc5::smem_desc(tc5::smem_addr(B + c * kDig * kBdig + ks * 256), 128, kSbo);
              tc5::mma_bf16(dc + (uint32_t)(16 * i), ad, bd, tc5::idesc_bf16_f32(kRows, 16 * (kDig - i)),
                            ks > 0 || i > 0);
            }
          tc5::mma_commit(empty + b);
          if (c == NCH - 1) tc5::mma_commit(tfull);
        }
      }
    }
    __syncwarp();
  } else {
    const int r = tid >> 2, u = tid & 3;
    auto load = [&](long tile, int c, float (&h)[12], float (&l)[12]) {
      const long e = tile * kRows + r;
#pragma unroll
      for (int k = 0; k < 12; ++k) {
        const int d = kChunk * c + 12 * u + k;
        float2 v = make_float2(0.f, 0.f);
        if (e < len && d < n_dir) v = __ldg(reinterpret_cast<const float2*>(psi + (long)d * n_dofs + e));
        h[k] = v.x;
        l[k] = v.y;
      }
    };
    float hn[12], ln[12];
    if ((long)blockIdx.x < ntiles) load(blockIdx.x, 0, hn, ln);
    long g = 0;
    int tl = 0;
    bool ok = true;
    for (long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++tl) {
      int* Et = Es + (tl & 1) * NCH * kRows;
      for (int c = 0; c < NCH; ++c, ++g) {
        float hc[12], lc[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) {
          hc[k] = hn[k];
          lc[k] = ln[k];
        }
        if (c + 1 < NCH) load(tile, c + 1, hn, ln);
        else if (tile + gridDim.x < ntiles) load(tile + gridDim.x, 0, hn, ln);
        float mx = 0.f;
#pragma unroll
        for (int k = 0; k < 12; ++k) mx = fmaxf(mx, fabsf(hc[k]));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
        const int E = row_exponent(mx);
        const float sc = pow2f(-E);
        const int b = (int)(g & 1);
        if (g >= 2 && !warp_wait(empty + b, (uint32_t)((g >> 1) - 1) & 1u, limit_ns, abort, status)) {
          ok = false;
          break;
        }
        if (u == 0) Et[c * kRows + r] = E;
        uint8_t* Ab = A + b * kAbuf;
#pragma unroll
        for (int t = 0; t < 3; ++t) {  // four directions at a time: one 8-byte piece per digit
          float d[4][kDig];
#pragma unroll
          for (int k = 0; k < 4; ++k) digits7(hc[4 * t + k] * sc, lc[4 * t + k] * sc, d[k]);
          const uint32_t off = tc5::kmajor_offset(r, 12 * u + 4 * t, kSbo);
#pragma unroll
          for (int qd = 0; qd < kDig; ++qd)
            *reinterpret_cast<uint2*>(Ab + qd * kAdig + off) =
                make_uint2(pack_bf16(d[0][qd], d[1][qd]), pack_bf16(d[2][qd], d[3][qd]));
        }
        tc5::fence_smem_to_async();
        tc5::mbar_arrive(full + b);
      }
      if (!ok) break;
      tc5::mbar_arrive(staged + (tl & 1));
      if (!warp_wait(staged + (tl & 1), (uint32_t)(tl >> 1) & 1u, limit_ns, abort, status)) break;
      if (!warp_wait(tfull, (uint32_t)tl & 1u, limit_ns, abort, status)) break;
      tc5::fence_after_sync();
      // epilogue: warp w reads the lanes of sub-partition w & 3 and moments
      // [4 (w >> 2), +4); per chunk the five accumulators are summed, scaled
      // by 2^(E + F) and added to the moment's double-float sum
      {
        const int sub = warp & 3, m0 = 4 * (warp >> 2);
        const int rr = 32 * sub + lane;
        const long e = tile * kRows + rr;
        const uint32_t lane_base = tmem + ((uint32_t)(32 * sub) << 16);
        if (m0 < n_mom) {  // warp-uniform
          df64_acc acc[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) acc[k] = acc_zero();
#pragma unroll
          for (int c = 0; c < NCH; ++c) {
            float v[kDig][4];
#pragma unroll
            for (int L = 0; L < kDig; ++L) tc5::tmem_ld4(lane_base + (uint32_t)(c * kCols + L * 16 + m0), v[L]);
            const float sE = pow2f(Et[c * kRows + rr]);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              df64_acc a7 = {v[kDig - 1][k], 0.f};  // smallest level first
#pragma unroll
              for (int L = kDig - 2; L >= 0; --L) acc_addf(a7, v[L][k]);
              const df64 x = acc_result(a7);
              const float s2 = sE * Fs[c * 16 + m0 + k];
              acc_add(acc[k], df64(x.hi * s2, x.lo * s2));
            }
          }
          if (e < len) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
              if (m0 + k < n_mom) {
                const long i = (long)(m0 + k) * n_dofs + e;
                const double p = df64_to(acc_result(acc[k]));
                phi[i] = xc ? xc[i] - p : p;  // with xc: the Apply's y = x - phi, fused
              }
          }
        }
      }
      tc5::fence_before_sync();
      tc5::mbar_arrive(tempty);
    }
  }
  finish(abort, bar_err, limit_ns, kMmaWarp, tmem, kTmemCols);
}

template <int NCH>
size_t reduce_oz_smem() {
  return 2 * (size_t)kDig * (kRows / 8) * (kChunk / 8 * 128) + (size_t)NCH * kDig * 2 * (kChunk / 8 * 128) +
         sizeof(float) * NCH * 16 + sizeof(int) * 2 * NCH * kRows + 128;
}

template <int NCH>
cudaError_t reduce_oz_launch(const df64* psi, const OzTables& t, double* phi, long n_dofs, long len, int* status,
                             long long limit_ns, cudaStream_t s, const double* xc) {
  const size_t smem = reduce_oz_smem<NCH>();
  cudaError_t e = cudaFuncSetAttribute(reduce_oz_kernel<NCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long ntiles = (len + kRows - 1) / kRows;
  const int grid = (int)std::max(1L, std::min(ntiles, (long)sms));
  reduce_oz_kernel<NCH><<<grid, kThreads, smem, s>>>(psi, t.d2m_img, t.d2m_exp, phi, t.n_dir, t.n_mom, n_dofs, len,
                                                     status, limit_ns, xc);
  return cudaGetLastError();
}

size_t expand_oz_smem(int npad) {
  return 2 * (size_t)kDig * (kRows / 8) * 256 + (size_t)kDig * (npad / 8) * 256 + sizeof(float) * npad +
         sizeof(int) * 2 * kRows + 128;
}

// ------------------------------------------------------------------ host
uint16_t bf16_exact_bits(double x) {  // x is a BF16 number (a digit): truncation is exact
  const float f = (float)x;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (uint16_t)(u >> 16);
}
// exponent F with max |v| < 2^F (0 for an all-zero set), within [-126, 126]
// so that 2^F is a normal FP32 number (the tables hold harmonics times weights)
int set_exponent(double maxabs) {
  if (!(maxabs > 0.0)) return 0;
  int e = 0;
  std::frexp(maxabs, &e);
  return std::max(-126, std::min(126, e));
}
// the seven digits of x * 2^-F (|x| < 2^F) on the grids 2^-8 ... 2^-56
void host_digits(double x, int F, double (&d)[kDig]) {
  double r = std::ldexp(x, -F);
  for (int k = 0; k < kDig; ++k) {
    const double t = std::ldexp(std::nearbyint(std::ldexp(r, 8 * (k + 1))), -8 * (k + 1));
    d[k] = t;
    r -= t;
  }
}

}  // namespace

// up to 16 moments (the K of the expansion, the N of the reduction) and four
// chunks of 48 directions (7 x 16 accumulator columns per chunk in the 512
// of an SM's tensor memory)
bool oz_contractions_fit(int n_dir, int n_mom) {
  return n_dir >= 1 && n_mom >= 1 && n_mom <= 16 && n_dir <= 4 * kChunk;
}

void oz_build_tables(const std::vector<double>& m2d, const std::vector<double>& d2m, int n_dir, int n_mom,
                     OzHost& h) {
  h.n_dir = n_dir;
  h.n_mom = n_mom;
  h.npad = (n_dir + 15) / 16 * 16;
  h.nch = (n_dir + kChunk - 1) / kChunk;
  // expansion B: digit g of M2D[d][m] * 2^-F_d at (row d, K = m)
  {
    const uint32_t sbo = 256, dig = (uint32_t)h.npad / 8 * sbo;
    h.m2d_img.assign((size_t)kDig * dig, 0);
    h.m2d_exp.assign(h.npad, 0);
    for (int d = 0; d < n_dir; ++d) {
      double mx = 0.0;
      for (int m = 0; m < n_mom; ++m) mx = std::max(mx, std::fabs(m2d[(size_t)d * n_mom + m]));
      const int F = set_exponent(mx);
      h.m2d_exp[d] = F;
      for (int m = 0; m < n_mom; ++m) {
        double dg[kDig];
        host_digits(m2d[(size_t)d * n_mom + m], F, dg);
        for (int g = 0; g < kDig; ++g) {
          const uint16_t b = bf16_exact_bits(dg[g]);
          std::memcpy(&h.m2d_img[(size_t)g * dig + tc5::kmajor_offset(d, m, sbo)], &b, 2);
        }
      }
    }
  }
  // reduction B: per chunk c and digit g, D2M[m][d] * 2^-F_{c,m} at (row m, K = d - 48 c)
  {
    const uint32_t sbo = kChunk / 8 * 128, dig = 2 * sbo;
    h.d2m_img.assign((size_t)h.nch * kDig * dig, 0);
    h.d2m_exp.assign((size_t)h.nch * 16, 0);
    for (int c = 0; c < h.nch; ++c)
      for (int m = 0; m < n_mom; ++m) {
        double mx = 0.0;
        for (int d = c * kChunk; d < std::min(n_dir, (c + 1) * kChunk); ++d)
          mx = std::max(mx, std::fabs(d2m[(size_t)m * n_dir + d]));
        const int F = set_exponent(mx);
        h.d2m_exp[(size_t)c * 16 + m] = F;
        for (int d = c * kChunk; d < std::min(n_dir, (c + 1) * kChunk); ++d) {
          double dg[kDig];
          host_digits(d2m[(size_t)m * n_dir + d], F, dg);
          for (int g = 0; g < kDig; ++g) {
            const uint16_t b = bf16_exact_bits(dg[g]);
            std::memcpy(&h.d2m_img[((size_t)c * kDig + g) * dig + tc5::kmajor_offset(m, d - c * kChunk, sbo)], &b,
                        2);
          }
        }
      }
  }
}

cudaError_t launch_expand_oz(const df64* T, const df64* iso, const OzTables& t, df64* q, long n_dofs, int* status,
                             long long limit_ns, cudaStream_t s, long len) {
  if (len < 0) len = n_dofs;
  if (len == 0) return cudaSuccess;
  const size_t smem = expand_oz_smem(t.npad);
  cudaError_t e = cudaFuncSetAttribute(expand_oz_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(expand_oz_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                           (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // one CTA per SM: it holds all 512 tensor-memory columns
  const long ntiles = (len + kRows - 1) / kRows;
  const int grid = (int)std::max(1L, std::min(ntiles, (long)sms));
  expand_oz_kernel<<<grid, kThreads, smem, s>>>(T, iso, t.m2d_img, t.m2d_exp, q, t.n_dir, t.n_mom, t.npad, n_dofs,
                                                len, status, limit_ns);
  return cudaGetLastError();
}

cudaError_t launch_reduce_oz(const df64* psi, const OzTables& t, double* phi, long n_dofs, int* status,
                             long long limit_ns, cudaStream_t s, long len, const double* xc) {
  if (len < 0) len = n_dofs;
  if (len == 0) return cudaSuccess;
  switch (t.nch) {
    case 1: return reduce_oz_launch<1>(psi, t, phi, n_dofs, len, status, limit_ns, s, xc);
    case 2: return reduce_oz_launch<2>(psi, t, phi, n_dofs, len, status, limit_ns, s, xc);
    case 3: return reduce_oz_launch<3>(psi, t, phi, n_dofs, len, status, limit_ns, s, xc);
    case 4: return reduce_oz_launch<4>(psi, t, phi, n_dofs, len, status, limit_ns, s, xc);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace ouranos
