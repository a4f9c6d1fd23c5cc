// Fifth-generation tensor-core (tcgen05) building blocks for sm_103a, as
// inline PTX: tensor-memory allocation, shared-memory matrix descriptors, the
// instruction descriptor of kind::f16 (BF16 operands, FP32 accumulators),
// the MMA issue, its commit to an mbarrier, bounded mbarrier waits and the
// tensor-memory loads of the epilogue.
//
// Operand tiles in shared memory use the K-major layout without swizzling:
// the tile is cut into core matrices of 8 rows x 16 bytes (8 BF16 values of
// K), each stored as 128 contiguous bytes (row r of the core matrix at byte
// 16 r).  The core matrix holding rows [8 g, 8 g + 8) and K values
// [8 c, 8 c + 8) sits at byte g * SBO + c * LBO; one MMA of K = 16 reads the
// two core matrices c, c + 1 of every row group.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

namespace ouranos {
namespace tc5 {

// CTAs of a kernel that fit on one SM at the same time, from its registers,
// its threads and its dynamic shared memory (228 KB per SM, 1 KB reserved per
// CTA), capped by the tensor-memory columns each CTA allocates (512 per SM)
template <typename K>
inline int resident_ctas(K kernel, int threads, size_t smem, int tmem_cols, int device) {
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(kernel)) != cudaSuccess) return 1;
  int smem_sm = 0, regs_sm = 0, threads_sm = 0;
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device);
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, device);
  cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, device);
  const int warps = (threads + 31) / 32;
  const int regs_warp = ((fa.numRegs > 0 ? fa.numRegs : 32) * 32 + 255) / 256 * 256;
  int n = 32;
  if (smem_sm > 0) n = std::min(n, (int)(smem_sm / (smem + fa.sharedSizeBytes + 1024)));
  if (regs_sm > 0) n = std::min(n, regs_sm / (regs_warp * warps));
  if (threads_sm > 0) n = std::min(n, threads_sm / threads);
  if (tmem_cols > 0) n = std::min(n, 512 / tmem_cols);
  return std::max(n, 1);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ long long globaltimer() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// byte offset of (row, k) in a K-major, unswizzled BF16 tile whose row
// groups are sbo bytes apart (core matrices along K 128 bytes apart)
__host__ __device__ __forceinline__ uint32_t kmajor_offset(int row, int k, uint32_t sbo) {
  return (uint32_t)(row >> 3) * sbo + (uint32_t)(k >> 3) * 128u + (uint32_t)(row & 7) * 16u + (uint32_t)(k & 7) * 2u;
}

// Shared-memory matrix descriptor: start address, leading-dimension byte
// offset (between core matrices adjacent in K), stride-dimension byte offset
// (between row groups), the fixed descriptor version 1 (bits 46-48 = 0b001),
// base offset 0, no swizzle (bits 61-63 = 0).  Addresses and offsets are
// stored in 16-byte units.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: D FP32 (bits 4-5 = 1),
// A and B BF16 (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ------------------------------------------------------------------ TMEM
// allocate ncols (a power of 2, >= 32) columns; one whole warp executes it,
// the base address lands in *slot
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy writes to shared memory become visible to the tensor core
__device__ __forceinline__ void fence_smem_to_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// wait for the phase of the given parity to complete, at most limit_ns
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = globaltimer();
  while (!mbar_try_wait(bar, parity))
    if (globaltimer() - t0 > limit_ns) return false;
  return true;
}

// one arrival of this thread (release: its earlier shared-memory writes are
// seen by the threads that wait for the phase)
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// the arrival of this thread, announcing `bytes` of bulk copies that
// complete on the barrier (the phase ends when both have happened)
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// ------------------------------------------------------------------- TMA
// one box of a 4-D tensor map (tmap: the generic address of a
// __grid_constant__ CUtensorMap) into shared memory at dst, completing on
// bar; coordinates may lie outside the tensor (those elements read as zero)
__device__ __forceinline__ void tma_load_4d(void* dst, const void* tmap, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
      "%5}], [%6];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(tmap)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
      : "memory");
}

// ------------------------------------------------------------------ MMA
// D[tmem] (+)= A[smem] * B[smem]^T, one thread issues
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}
// the mbarrier receives one arrival once every MMA this thread issued before
// has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_addr(bar))
               : "memory");
}

// ------------------------------------------------------- TMEM -> registers
// warp w reads lanes [32 (w % 4), 32 (w % 4) + 32): thread i gets lane
// 32 (w % 4) + i, columns [col, col + 4) / [col, col + 8) / [col, col + 16)
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float (&v)[4]) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 4; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

// ------------------------------------------------- FP32 -> three BF16 parts
// x = p0 + p1 + p2 (+ a remainder below 2^-24 |x|): each part is x's
// remainder rounded to BF16; the subtractions are exact in FP32
__device__ __forceinline__ void split3(float x, __nv_bfloat16& p0, __nv_bfloat16& p1, __nv_bfloat16& p2) {
  p0 = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(p0);
  p1 = __float2bfloat16_rn(r1);
  p2 = __float2bfloat16_rn(r1 - __bfloat162float(p1));
}
__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}
// 8 consecutive K values of one row -> the row's 16-byte piece of each part
__device__ __forceinline__ void split8_store(const float (&x)[8], uint8_t* part0, uint8_t* part1, uint8_t* part2,
                                             uint32_t off) {
  __nv_bfloat16 a[8], b[8], c[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) split3(x[k], a[k], b[k], c[k]);
  *reinterpret_cast<uint4*>(part0 + off) = make_uint4(pack2(a[0], a[1]), pack2(a[2], a[3]), pack2(a[4], a[5]), pack2(a[6], a[7]));
  *reinterpret_cast<uint4*>(part1 + off) = make_uint4(pack2(b[0], b[1]), pack2(b[2], b[3]), pack2(b[4], b[5]), pack2(b[6], b[7]));
  *reinterpret_cast<uint4*>(part2 + off) = make_uint4(pack2(c[0], c[1]), pack2(c[2], c[3]), pack2(c[4], c[5]), pack2(c[6], c[7]));
}

}  // namespace tc5
}  // namespace ouranos
