// Direction-axis contractions of the FP32 sweep on the tensor cores
// (tcgen05.mma, BF16 operands, FP32 accumulators in tensor memory):
//
//   expansion  q[d][e]   = sum_m M2D[d][m] T[m][e] (+ iso[e])
//              (reference: the M2D source assembly, src/RadiativeTransfer.cc:907-913)
//   reduction  phi[m][e] = sum_d D2M[m][d] psi[d][e]
//              (reference: the D2M accumulation, src/RadiativeTransfer.cc:990-996)
//
// Both are GEMMs with the dofs e as the M dimension, 128 per tile (one
// tensor-memory lane per dof):
//   expansion: D[e][d] = A[e][m] B[d][m],  A = T^T (K = moments, padded to 16),
//              B = M2D (N = directions, padded to a multiple of 16);
//   reduction: D[e][m] = A[e][d] B[m][d],  A = psi^T (K = directions, padded
//              to a multiple of 32), B = D2M (N = 16 moment slots).
// FP32 accuracy from BF16 operands: every FP32 value is split into three
// BF16 parts x = x0 + x1 + x2 (8 significant bits each, so the parts hold the
// value's 24 bits), and the products x_i y_j with i + j <= 2 are summed in the
// FP32 accumulator, smallest first; the dropped products are below 2^-24 of
// the result, and the accumulation rounds like an FP32 dot product.  The
// matrix parts (M2D, D2M) are split once on the host; the vector parts are
// split by the threads that stage the tile in shared memory.  Each CTA owns
// one tile at a time: threads stage A, one thread issues the MMAs and commits
// them to an mbarrier, all threads wait (bounded by the handle's wait limit)
// and the epilogue moves the accumulators from tensor memory to HBM with
// coalesced stores (32 consecutive dofs per warp store).
#include <algorithm>
#include <cstring>
#include <vector>

#include "internal.h"
#include "tc5.cuh"

namespace ouranos {
namespace {

constexpr int kRows = 128;   // dofs per tile: the MMA's M, one tensor-memory lane each
constexpr int kPairs = 6;    // part products (i, j) with i + j <= 2
constexpr int kExpandThreads = 512;
constexpr int kReduceThreads = 256;

// part pairs, the smallest products first
__device__ __forceinline__ int pair_a(int p) { return p == 0 ? 2 : p == 2 ? 1 : p == 3 ? 1 : 0; }
__device__ __forceinline__ int pair_b(int p) { return p == 1 ? 2 : p == 2 ? 1 : p == 4 ? 1 : 0; }

// A wait that ran out leaves bit 4 in the status word; the MMAs it waited
// for get one more bounded wait before the tensor memory is freed.
__device__ __forceinline__ void finish_tile_loop(bool ok, uint64_t* bar, uint32_t phase, long long limit_ns,
                                                 int* status) {
  if (!ok) {
    if (threadIdx.x == 0) {
      if (status) atomicOr(status, 4);
      tc5::mbar_wait(bar, phase ^ 1u, limit_ns);
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kExpandThreads) expand_tc_kernel(const float* __restrict__ T,
                                                                   const float* __restrict__ iso,
                                                                   const uint8_t* __restrict__ bimg,
                                                                   float* __restrict__ q, int n_dir, int n_mom,
                                                                   int npad, long n_dofs, long len, int* status,
                                                                   long long limit_ns) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t kApart = kRows * 16 * 2;      // 128 rows x 16 moments, BF16
  constexpr uint32_t kSbo = 256;                   // two core matrices of K per row group
  const uint32_t bpart = (uint32_t)npad * 32;      // npad rows x 16 moments, BF16
  uint8_t* A = smem;
  uint8_t* B = smem + 3 * kApart;
  uint64_t* bar = reinterpret_cast<uint64_t*>(B + 3 * bpart);
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (uint32_t o = tid * 16u; o < 3 * bpart; o += kExpandThreads * 16u)
    *reinterpret_cast<uint4*>(B + o) = __ldg(reinterpret_cast<const uint4*>(bimg + o));
  if (tid == 0) {
    tc5::mbar_init(bar, 1);
    tc5::mbar_init_fence();
  }
  if (warp == 0) {
    tc5::tmem_alloc(slot, 256);
    tc5::tmem_relinquish();
  }
  tc5::fence_before_sync();
  __syncthreads();
  tc5::fence_after_sync();
  const uint32_t tmem = *slot;
  const uint32_t idesc = tc5::idesc_bf16_f32(kRows, npad);
  const long ntiles = (len + kRows - 1) / kRows;
  uint32_t phase = 0;
  bool ok = true;
  for (long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long e0 = tile * kRows;
    if (tid < 2 * kRows) {  // stage A: row r = dof e0 + r; thread half h splits moments [8h, 8h + 8)
      const int r = tid & (kRows - 1), h = tid >> 7;
      const long e = e0 + r;
      float x[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int m = 8 * h + k;
        x[k] = (e < len && m < n_mom) ? __ldg(T + (long)m * n_dofs + e) : 0.f;
      }
      tc5::split8_store(x, A, A + kApart, A + 2 * kApart, tc5::kmajor_offset(r, 8 * h, kSbo));
    }
    tc5::fence_smem_to_async();
    tc5::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc5::fence_after_sync();
#pragma unroll
      for (int p = 0; p < kPairs; ++p) {
        const uint64_t ad = tc5::smem_desc(tc5::smem_addr(A + pair_a(p) * kApart), 128, kSbo);
        const uint64_t bd = tc5::smem_desc(tc5::smem_addr(B + pair_b(p) * bpart), 128, kSbo);
        tc5::mma_bf16(tmem, ad, bd, idesc, p > 0);
      }
      tc5::mma_commit(bar);
    }
    ok = tc5::mbar_wait(bar, phase, limit_ns);
    ok = __syncthreads_and(ok);
    phase ^= 1u;
    if (!ok) break;
    tc5::fence_after_sync();
    // epilogue: warp w reads the lanes of sub-partition w & 3 and every
    // fourth 8-column piece from piece w >> 2 on; q is read once, by the
    // sweep, so it is stored with streaming (evict-first) stores
    const int sub = warp & 3, quarter = warp >> 2;
    const long e = e0 + 32 * sub + lane;
    const float is = (iso && e < len) ? __ldg(iso + e) : 0.f;
    for (int c = 8 * quarter; c < npad; c += 32) {
      float v[8];
      tc5::tmem_ld8(tmem + ((uint32_t)(32 * sub) << 16) + (uint32_t)c, v);
      if (e < len) {
#pragma unroll
        for (int k = 0; k < 8; ++k)
          if (c + k < n_dir) __stcs(q + (long)(c + k) * n_dofs + e, v[k] + is);
      }
    }
    tc5::fence_before_sync();
    __syncthreads();
  }
  finish_tile_loop(ok, bar, phase, limit_ns, status);
  if (warp == 0) {
    tc5::fence_after_sync();
    tc5::tmem_dealloc(tmem, 256);
  }
}

// The reduction streams psi through shared memory in chunks of 32
// directions: thread (row r = tid & 127, half h = tid >> 7) loads the 16
// values of directions [32 c + 16 h, 32 c + 16 h + 16) of its dof, and the
// next chunk's values are already in flight while this one is split, staged
// (two staging buffers, each reused once the MMAs that read it have
// completed) and multiplied.  The tile's accumulator (16 tensor-memory
// columns) is complete after its last chunk.  K = 32 NCH directions.
template <int NCH>
__global__ void __launch_bounds__(kReduceThreads, 2) reduce_tc_kernel(const float* __restrict__ psi,
                                                                   const uint8_t* __restrict__ bimg,
                                                                   float* __restrict__ phi, int n_dir,
                                                                   int n_mom, long n_dofs, long len, int* status,
                                                                   long long limit_ns) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr int KPAD = 32 * NCH;
  constexpr uint32_t kSboA = 512;                  // four core matrices of K per row group
  constexpr uint32_t kApart = kRows / 8 * kSboA;   // 128 rows x 32 directions, BF16
  constexpr uint32_t kAbuf = 3 * kApart;           // the three parts of one chunk
  constexpr uint32_t kSboB = KPAD * 16;
  constexpr uint32_t kBpart = 2 * kSboB;           // 16 moment rows x KPAD directions, BF16
  uint8_t* A = smem;
  uint8_t* B = smem + 2 * kAbuf;
  // mbarriers: staging buffers 0 and 1, the tile's accumulator 2, the error path 3
  uint64_t* bar = reinterpret_cast<uint64_t*>(B + 3 * kBpart);
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (uint32_t o = tid * 16u; o < 3 * kBpart; o += kReduceThreads * 16u)
    *reinterpret_cast<uint4*>(B + o) = __ldg(reinterpret_cast<const uint4*>(bimg + o));
  if (tid == 0) {
    for (int i = 0; i < 4; ++i) tc5::mbar_init(bar + i, 1);
    tc5::mbar_init_fence();
  }
  if (warp == 0) {
    tc5::tmem_alloc(slot, 32);
    tc5::tmem_relinquish();
  }
  tc5::fence_before_sync();
  __syncthreads();
  tc5::fence_after_sync();
  const uint32_t tmem = *slot;
  constexpr uint32_t idesc = tc5::idesc_bf16_f32(kRows, 16);
  const long ntiles = (len + kRows - 1) / kRows;
  const int r = tid & (kRows - 1), h = tid >> 7;
  auto load = [&](long tile, int kc, float (&x)[16]) {
    const long e = tile * kRows + r;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const int d = 32 * kc + 16 * h + k;
      x[k] = (e < len && d < n_dir) ? __ldg(psi + (long)d * n_dofs + e) : 0.f;
    }
  };
  float xn[16];
  if ((long)blockIdx.x < ntiles) load(blockIdx.x, 0, xn);
  uint32_t ph_buf = 0u, ph_tile = 0u;  // bit b: the parity awaited next on staging buffer b
  long g = 0;  // chunks this CTA has staged
  bool ok = true;
  for (long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    for (int kc = 0; kc < NCH; ++kc, ++g) {
      float x[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) x[k] = xn[k];
      if (kc + 1 < NCH) load(tile, kc + 1, xn);
      else if (tile + gridDim.x < ntiles) load(tile + gridDim.x, 0, xn);
      const int b = (int)(g & 1);
      uint8_t* Ab = A + b * kAbuf;
      if (g >= 2) {  // the MMAs that read this buffer two chunks ago
        bool w = true;
        if (tid == 0) w = tc5::mbar_wait(bar + b, (ph_buf >> b) & 1u, limit_ns);
        ph_buf ^= 1u << b;
        ok = __syncthreads_and(w);
        if (!ok) break;
      }
      float lo[8], hi[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        lo[k] = x[k];
        hi[k] = x[8 + k];
      }
      tc5::split8_store(lo, Ab, Ab + kApart, Ab + 2 * kApart, tc5::kmajor_offset(r, 16 * h, kSboA));
      tc5::split8_store(hi, Ab, Ab + kApart, Ab + 2 * kApart, tc5::kmajor_offset(r, 16 * h + 8, kSboA));
      tc5::fence_smem_to_async();
      tc5::fence_before_sync();
      __syncthreads();
      if (tid == 0) {
        tc5::fence_after_sync();
#pragma unroll
        for (int p = 0; p < kPairs; ++p)
#pragma unroll
          for (int ks = 0; ks < 2; ++ks) {
            const uint64_t ad = tc5::smem_desc(tc5::smem_addr(Ab + pair_a(p) * kApart + ks * 256), 128, kSboA);
            const uint64_t bd =
                tc5::smem_desc(tc5::smem_addr(B + pair_b(p) * kBpart + (2 * kc + ks) * 256), 128, kSboB);
            tc5::mma_bf16(tmem, ad, bd, idesc, kc > 0 || ks > 0 || p > 0);
          }
        tc5::mma_commit(bar + b);
        if (kc == NCH - 1) tc5::mma_commit(bar + 2);
      }
    }
    if (!ok) break;
    bool w = true;
    if (tid == 0) w = tc5::mbar_wait(bar + 2, ph_tile, limit_ns);
    ph_tile ^= 1u;
    ok = __syncthreads_and(w);
    if (!ok) break;
    tc5::fence_after_sync();
    if (warp < 4) {
      const long e = tile * kRows + 32 * warp + lane;
      float v[16];
      tc5::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16), v);
      if (e < len) {
#pragma unroll
        for (int m = 0; m < 16; ++m)
          if (m < n_mom) phi[(long)m * n_dofs + e] = v[m];
      }
    }
    tc5::fence_before_sync();
    __syncthreads();
  }
  if (!ok) {  // a wait ran out: one more bounded wait for every MMA issued, then free the columns
    if (tid == 0) {
      if (status) atomicOr(status, 4);
      tc5::mma_commit(bar + 3);
      tc5::mbar_wait(bar + 3, 0u, limit_ns);
    }
    __syncthreads();
  }
  if (warp == 0) {
    tc5::fence_after_sync();
    tc5::tmem_dealloc(tmem, 32);
  }
}

template <int NCH>
cudaError_t reduce_tc_launch(const float* psi, const uint8_t* img, float* phi, int n_dir, int n_mom, long n_dofs,
                             long len, int* status, long long limit_ns, cudaStream_t s) {
  constexpr size_t smem = 2 * 3 * (size_t)(kRows / 8) * 512 + 3 * (size_t)2 * (32 * NCH * 16) + 64;  // + 4 mbarriers, slot
  const cudaError_t e =
      cudaFuncSetAttribute(reduce_tc_kernel<NCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // the whole carveout as shared memory, so that two CTAs fit on an SM (the
  // default split left room for one)
  const cudaError_t e2 = cudaFuncSetAttribute(reduce_tc_kernel<NCH>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                              (int)cudaSharedmemCarveoutMaxShared);
  if (e2 != cudaSuccess) return e2;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int per_sm = tc5::resident_ctas(reduce_tc_kernel<NCH>, kReduceThreads, smem, 32, dev);
  const long ntiles = (len + kRows - 1) / kRows;
  const int grid = (int)std::max(1L, std::min(ntiles, (long)sms * per_sm));
  reduce_tc_kernel<NCH><<<grid, kReduceThreads, smem, s>>>(psi, img, phi, n_dir, n_mom, n_dofs, len, status,
                                                           limit_ns);
  return cudaGetLastError();
}

// host BF16 rounding (round to nearest even; the tables hold finite values)
uint16_t bf16_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
float bf16_value(uint16_t b) {
  const uint32_t u = (uint32_t)b << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// three K-major BF16 part images of W[rows][k] (FP32 values), padded to
// rows_pad x k_pad with zeros
std::vector<uint8_t> part_images(const std::vector<float>& W, int rows, int k, int rows_pad, int k_pad) {
  const uint32_t sbo = (uint32_t)k_pad * 16;
  const size_t part = (size_t)rows_pad / 8 * sbo;
  std::vector<uint8_t> img(3 * part, 0);
  for (int r = 0; r < rows; ++r)
    for (int c = 0; c < k; ++c) {
      const float x = W[(size_t)r * k + c];
      const uint16_t p0 = bf16_bits(x);
      const float r1 = x - bf16_value(p0);
      const uint16_t p1 = bf16_bits(r1);
      const uint16_t p2 = bf16_bits(r1 - bf16_value(p1));
      const uint32_t off = tc5::kmajor_offset(r, c, sbo);
      std::memcpy(&img[off], &p0, 2);
      std::memcpy(&img[part + off], &p1, 2);
      std::memcpy(&img[2 * part + off], &p2, 2);
    }
  return img;
}

}  // namespace

bool tc_contractions_fit(int n_dir, int n_mom) { return n_dir >= 1 && n_dir <= 256 && n_mom >= 1 && n_mom <= 16; }

// FP32 M2D [n_dir][n_mom] and D2M [n_mom][n_dir] -> the B operand images
void tc_build_images(const std::vector<double>& m2d, const std::vector<double>& d2m, int n_dir, int n_mom,
                     std::vector<uint8_t>& m2d_img, std::vector<uint8_t>& d2m_img, int& npad, int& kpad) {
  npad = (n_dir + 15) / 16 * 16;
  kpad = (n_dir + 31) / 32 * 32;
  std::vector<float> a((size_t)n_dir * n_mom), b((size_t)n_mom * n_dir);
  for (size_t i = 0; i < a.size(); ++i) a[i] = (float)m2d[i];
  for (size_t i = 0; i < b.size(); ++i) b[i] = (float)d2m[i];
  m2d_img = part_images(a, n_dir, n_mom, npad, 16);
  d2m_img = part_images(b, n_mom, n_dir, 16, kpad);
}

cudaError_t launch_expand_tc(const float* T, const float* iso, const TcTables& t, float* q, long n_dofs, int* status,
                             long long limit_ns, cudaStream_t s, long len) {
  if (len < 0) len = n_dofs;
  if (len == 0) return cudaSuccess;
  // 100 KB of shared memory per CTA (the tiles need under 40 KB) keeps at
  // most two CTAs on an SM: two hold all 512 tensor-memory columns, a third
  // would wait in tcgen05.alloc until one of them had finished
  const size_t smem = std::max<size_t>(3 * (size_t)kRows * 32 + 3 * (size_t)t.npad * 32 + 64, 100 * 1024);
  const cudaError_t e = cudaFuncSetAttribute(expand_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const cudaError_t e2 = cudaFuncSetAttribute(expand_tc_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                              (int)cudaSharedmemCarveoutMaxShared);
  if (e2 != cudaSuccess) return e2;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long ntiles = (len + kRows - 1) / kRows;
  const int grid = (int)std::max(1L, std::min(ntiles, 2L * sms));
  expand_tc_kernel<<<grid, kExpandThreads, smem, s>>>(T, iso, t.m2d_img, q, t.n_dir, t.n_mom, t.npad, n_dofs, len,
                                                      status, limit_ns);
  return cudaGetLastError();
}

cudaError_t launch_reduce_tc(const float* psi, const TcTables& t, float* phi, long n_dofs, int* status,
                             long long limit_ns, cudaStream_t s, long len) {
  if (len < 0) len = n_dofs;
  if (len == 0) return cudaSuccess;
  switch (t.kpad / 32) {
    case 1: return reduce_tc_launch<1>(psi, t.d2m_img, phi, t.n_dir, t.n_mom, n_dofs, len, status, limit_ns, s);
    case 2: return reduce_tc_launch<2>(psi, t.d2m_img, phi, t.n_dir, t.n_mom, n_dofs, len, status, limit_ns, s);
    case 3: return reduce_tc_launch<3>(psi, t.d2m_img, phi, t.n_dir, t.n_mom, n_dofs, len, status, limit_ns, s);
    case 4: return reduce_tc_launch<4>(psi, t.d2m_img, phi, t.n_dir, t.n_mom, n_dofs, len, status, limit_ns, s);
    case 5: return reduce_tc_launch<5>(psi, t.d2m_img, phi, t.n_dir, t.n_mom, n_dofs, len, status, limit_ns, s);
    case 6: return reduce_tc_launch<6>(psi, t.d2m_img, phi, t.n_dir, t.n_mom, n_dofs, len, status, limit_ns, s);
    case 7: return reduce_tc_launch<7>(psi, t.d2m_img, phi, t.n_dir, t.n_mom, n_dofs, len, status, limit_ns, s);
    case 8: return reduce_tc_launch<8>(psi, t.d2m_img, phi, t.n_dir, t.n_mom, n_dofs, len, status, limit_ns, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace ouranos
