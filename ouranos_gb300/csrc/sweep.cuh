// Transport sweep kernel for sm_103a.
//
// Replaces the reference's task loop
//   initialize_scheduler(); while (n_tasks_to_execute) sweep(*get_next_task(), ...)
// (src/RadiativeTransfer.cc:605-692, 780-809, 878-1012), whose scheduler walks a
// (cell, direction) task DAG with FIFO ready counters and MPI face messages.
//
// Canonical orientation.  A direction with Omega_a < 0 is swept in the mirrored
// coordinate x'_a = N_a - 1 - x_a, and each cell's local dofs are visited in the
// mirrored order, so every direction looks like one of the all-positive octant:
// the inflow face of axis a is local index c_a = 0 and the outflow face
// c_a = p.  Face dof positions are then compile-time constants and the cell
// matrix depends only on (sigma_t, |Omega|) (its inverse is precomputed).
//
// Work decomposition.  The sweep axis S is y in 2-D and z in 3-D; the
// transverse plane (x, or x-y) is cut into tiles of wx (x wy) cells.  One warp
// runs one task = (group of kd directions of one octant, one tile): lane
// (lx, ly, k) handles cell (x'_0 + lx, y'_0 + ly) of direction k and, at step
// s, the plane s' = s - lx - ly of the sweep axis (a skewed wavefront inside
// the warp).  Upwind face values arrive
//   - along S: from the lane's own previous step (registers),
//   - along x/y inside the tile: from lane-1 / lane-wx by warp shuffle,
//   - across tiles: from an HBM edge buffer written by the upwind tile's warp
//     -- the GPU form of the reference's MPI_Isend/Iprobe of outflow faces
//     (src/RadiativeTransfer.cc:633-750).  Every edge value travels in a
//     64-bit word together with a 32-bit tag (sweep epoch, plane); an FP64
//     value is split into two tagged halves.  The consumer polls the words it
//     needs until the tags match: single-copy atomicity of aligned 64-bit
//     accesses makes each word self-validating, so no fence or counter is
//     needed on the producer side.
// Tasks are handed out through one atomic ticket in dependency order (tile
// level first), so a warp only ever waits on tasks that live warps already
// hold: any grid size is deadlock-free.  Every wait is bounded (iteration cap
// and %globaltimer); a wait that runs out sets `status`, and all warps leave.
//
// Per lane and step: b = q_d[cell] (the source expanded to this direction by
// the expansion kernel, or sum_m M2D(d,m) T_m[cell] + isotropic source for one
// or two moments) + |Omega_a| F_a psi_up,a over the inflow faces; x = A'^-1 b;
// the outflow faces are the c_a = p entries of x; x is stored as psi_d[cell].
// The source values of the next kPrefetch planes stream into a per-warp
// shared-memory ring with cp.async, so their memory latency overlaps the
// solves of the planes before them.  The moments phi = D2M psi are formed
// afterwards by the reduction kernel over the direction axis (no atomics: the
// sweep is deterministic).
#pragma once

#include "internal.h"

namespace ouranos {

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ long long global_ns() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Tagged edge words: value bits in the low half, tag in the high half.
template <typename real>
struct Tagged;
template <>
struct Tagged<float> {
  static constexpr int W = 1;  // 64-bit words per value
  static __device__ __forceinline__ void put(unsigned long long* w, float v, unsigned tag) {
    st_relaxed_u64(w, ((unsigned long long)tag << 32) | __float_as_uint(v));
  }
  static __device__ __forceinline__ bool decode(const unsigned long long* raw, unsigned tag, float& v) {
    const unsigned long long a = raw[0];
    v = __uint_as_float((unsigned)a);
    return (unsigned)(a >> 32) == tag;
  }
  static __device__ __forceinline__ bool get(const unsigned long long* w, unsigned tag, float& v) {
    const unsigned long long a = ld_relaxed_u64(w);
    return decode(&a, tag, v);
  }
};
template <>
struct Tagged<double> {
  static constexpr int W = 2;
  static __device__ __forceinline__ void put(unsigned long long* w, double v, unsigned tag) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    st_relaxed_u64(w, ((unsigned long long)tag << 32) | (b & 0xffffffffull));
    st_relaxed_u64(w + 1, ((unsigned long long)tag << 32) | (b >> 32));
  }
  static __device__ __forceinline__ bool decode(const unsigned long long* raw, unsigned tag, double& v) {
    const unsigned long long lo = raw[0], hi = raw[1];
    v = __longlong_as_double((long long)((hi << 32) | (lo & 0xffffffffull)));
    return (unsigned)(lo >> 32) == tag && (unsigned)(hi >> 32) == tag;
  }
  static __device__ __forceinline__ bool get(const unsigned long long* w, unsigned tag, double& v) {
    const unsigned long long raw[2] = {ld_relaxed_u64(w), ld_relaxed_u64(w + 1)};
    return decode(raw, tag, v);
  }
};

template <>
struct Tagged<df64> {  // a double-float travels as its two tagged halves
  static constexpr int W = 2;
  static __device__ __forceinline__ void put(unsigned long long* w, df64 v, unsigned tag) {
    st_relaxed_u64(w, ((unsigned long long)tag << 32) | __float_as_uint(v.hi));
    st_relaxed_u64(w + 1, ((unsigned long long)tag << 32) | __float_as_uint(v.lo));
  }
  static __device__ __forceinline__ bool decode(const unsigned long long* raw, unsigned tag, df64& v) {
    const unsigned long long a = raw[0], b = raw[1];
    v = df64(__uint_as_float((unsigned)a), __uint_as_float((unsigned)b));
    return (unsigned)(a >> 32) == tag && (unsigned)(b >> 32) == tag;
  }
  static __device__ __forceinline__ bool get(const unsigned long long* w, unsigned tag, df64& v) {
    const unsigned long long raw[2] = {ld_relaxed_u64(w), ld_relaxed_u64(w + 1)};
    return decode(raw, tag, v);
  }
};

// Arithmetic of the cell solve.  float / double: plain fused multiply-adds.
// df64 (FP64 accuracy on the FP32 pipes): the products and sums of each dot
// product go through the compensated accumulator of df64.cuh, renormalised once.
template <typename real>
struct Arith {
  using acc = real;
  static __device__ __forceinline__ acc zero() { return real(0); }
  static __device__ __forceinline__ acc from(real v) { return v; }
  // explicit roundings (no contraction left to the compiler), so every form
  // of the sweep rounds a dot product the same way: s = fma(a, b, s)
  static __device__ __forceinline__ void fma(acc& s, real a, real b) {
    if constexpr (sizeof(real) == 4) s = __fmaf_rn(a, b, s);
    else s = __fma_rn(a, b, s);
  }
  // the first term of a dot product: the value fma(zero(), a, b) gives
  static __device__ __forceinline__ acc prod(real a, real b) {
    if constexpr (sizeof(real) == 4) return __fmul_rn(a, b);
    else return __dmul_rn(a, b);
  }
  // an intermediate that only feeds further multiply-adds
  static __device__ __forceinline__ real raw(acc s) { return s; }
  static __device__ __forceinline__ real get(acc s) { return s; }
  static __device__ __forceinline__ real ldg(const real* p) { return __ldg(p); }
  static __device__ __forceinline__ real shfl_up(real v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
  static __device__ __forceinline__ real shfl_xor(real v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
};
template <>
struct Arith<df64> {
  using acc = df64_acc;
  static __device__ __forceinline__ acc zero() { return acc_zero(); }
  static __device__ __forceinline__ acc from(df64 v) { return acc_from(v); }
  static __device__ __forceinline__ void fma(acc& s, df64 a, df64 b) { acc_fma(s, a, b); }
  static __device__ __forceinline__ acc prod(df64 a, df64 b) { return acc_prod(a, b); }
  // an intermediate that only feeds further compensated multiply-adds, which
  // take any hi + lo pair with a small low part: left unrenormalised
  static __device__ __forceinline__ df64 raw(acc s) { return df64(s.s, s.c); }
  static __device__ __forceinline__ df64 get(acc s) { return acc_result(s); }
  static __device__ __forceinline__ df64 ldg(const df64* p) {
    const float2 t = __ldg(reinterpret_cast<const float2*>(p));
    return df64(t.x, t.y);
  }
  static __device__ __forceinline__ df64 shfl_up(df64 v, int d) {
    return df64(__shfl_up_sync(0xffffffffu, v.hi, d), __shfl_up_sync(0xffffffffu, v.lo, d));
  }
  static __device__ __forceinline__ df64 shfl_xor(df64 v, int m) {
    return df64(__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m));
  }
};

// Read FD tagged values; poll until every tag matches.  Returns false when the
// wait ran out (and then records status 1) or when another warp has already
// recorded an error.
template <typename real, int FD>
static __device__ __forceinline__ bool fetch_edge(const unsigned long long* w, unsigned tag,
                                                  real* out, int* status, long long limit_ns) {
  constexpr int W = Tagged<real>::W;
  bool ok = true;
#pragma unroll
  for (int t = 0; t < FD; ++t) ok &= Tagged<real>::get(w + t * W, tag, out[t]);
  if (ok) return true;
  const long long t0 = global_ns();
  unsigned sleep_ns = 16;
  for (unsigned it = 0; it < (1u << 26); ++it) {
    if (it >= 8) {  // the first re-polls go straight back (a value in flight lands within them)
      __nanosleep(sleep_ns);
      if (sleep_ns < 256) sleep_ns <<= 1;
    }
    ok = true;
#pragma unroll
    for (int t = 0; t < FD; ++t) ok &= Tagged<real>::get(w + t * W, tag, out[t]);
    if (ok) return true;
    if (*(volatile int*)status) return false;
    if (global_ns() - t0 > limit_ns) break;
  }
  atomicCAS(status, 0, 1);
  return false;
}

// cp.async of one 4- or 8-byte element into shared memory
template <typename real>
__device__ __forceinline__ void cp_async_elem(real* smem_dst, const real* gsrc) {
  const unsigned dst = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(dst), "l"(gsrc), "n"(sizeof(real))
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// 16-byte cp.async (to shared memory through L2) and a cell's N contiguous
// values copied in 16-byte pieces (N * sizeof(real) a multiple of 16, both
// addresses 16-byte aligned)
__device__ __forceinline__ void cp_async_16(void* smem_dst, const void* gsrc) {
  const unsigned dst = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(gsrc) : "memory");
}
template <typename real, int N>
__device__ __forceinline__ void cp_async_cell(real* smem_dst, const real* gsrc) {
#pragma unroll
  for (int k = 0; k < (int)(N * sizeof(real) / 16); ++k)
    cp_async_16(reinterpret_cast<char*>(smem_dst) + 16 * k, reinterpret_cast<const char*>(gsrc) + 16 * k);
}

// 32-bit words of a value (little endian), for 16-byte vector stores
template <typename real>
struct Bits;
template <>
struct Bits<float> {
  static constexpr int W = 1;
  static __device__ __forceinline__ unsigned word(float v, int) { return __float_as_uint(v); }
};
template <>
struct Bits<double> {
  static constexpr int W = 2;
  static __device__ __forceinline__ unsigned word(double v, int w) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return w ? (unsigned)(b >> 32) : (unsigned)b;
  }
};
template <>
struct Bits<df64> {
  static constexpr int W = 2;
  static __device__ __forceinline__ unsigned word(df64 v, int w) {
    return w ? __float_as_uint(v.lo) : __float_as_uint(v.hi);
  }
};
// value from its 32-bit words (little endian)
template <typename real>
__device__ __forceinline__ real from_words(unsigned w0, unsigned w1);
template <>
__device__ __forceinline__ float from_words<float>(unsigned w0, unsigned) { return __uint_as_float(w0); }
template <>
__device__ __forceinline__ double from_words<double>(unsigned w0, unsigned w1) {
  return __longlong_as_double((long long)(((unsigned long long)w1 << 32) | w0));
}
template <>
__device__ __forceinline__ df64 from_words<df64>(unsigned w0, unsigned w1) {
  return df64(__uint_as_float(w0), __uint_as_float(w1));
}
// 16 bytes through the read-only path, kept in L1 with evict-last priority:
// the cell tables are re-read every step, while the sources streamed into
// the ring by cp.async also pass through L1 and are read once
__device__ __forceinline__ uint4 ldg_keep(const uint4* p) {
  uint4 u;
  // (not volatile: a read of read-only data, which the compiler may schedule like __ldg)
  asm("ld.global.nc.L1::evict_last.v4.u32 {%0, %1, %2, %3}, [%4];"
      : "=r"(u.x), "=r"(u.y), "=r"(u.z), "=r"(u.w)
      : "l"(p));
  return u;
}
// A table row of NV values stored padded to whole 16-byte pieces (p 16-byte
// aligned): read through the read-only path in 16-byte loads
template <typename real, int NV>
__device__ __forceinline__ void load_row(const real* p, real (&o)[NV]) {
  constexpr int PER = 16 / (int)sizeof(real);  // values per piece: 4 floats, 2 doubles or pairs
  constexpr int W = Bits<real>::W;
#pragma unroll
  for (int k = 0; k < (NV + PER - 1) / PER; ++k) {
    const uint4 u = ldg_keep(reinterpret_cast<const uint4*>(p) + k);
    const unsigned w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int t = 0; t < PER; ++t)
      if (k * PER + t < NV) o[k * PER + t] = from_words<real>(w[t * W], W == 2 ? w[t * W + 1] : 0u);
  }
}
__host__ __device__ constexpr int pad4(int n) { return (n + 3) & ~3; }

// o[0..N) = src[0..N) with 16-byte shared-memory loads (src 16-byte aligned)
template <typename real, int N>
__device__ __forceinline__ void load_cell(const real* src, real (&o)[N]) {
  constexpr int W = Bits<real>::W;
#pragma unroll
  for (int k = 0; k < (int)(N * sizeof(real) / 16); ++k) {
    const uint4 u = *reinterpret_cast<const uint4*>(reinterpret_cast<const char*>(src) + 16 * k);
    if (W == 1) {
      o[4 * k + 0] = from_words<real>(u.x, 0);
      o[4 * k + 1] = from_words<real>(u.y, 0);
      o[4 * k + 2] = from_words<real>(u.z, 0);
      o[4 * k + 3] = from_words<real>(u.w, 0);
    } else {
      o[2 * k + 0] = from_words<real>(u.x, u.y);
      o[2 * k + 1] = from_words<real>(u.z, u.w);
    }
  }
}

// Streaming (evict-first) stores of the angular flux: written once per sweep
// and read back once by the reduction, it should not push the cell tables and
// the sources out of the caches.
__device__ __forceinline__ void store_stream(float* p, float v) { __stcs(p, v); }
__device__ __forceinline__ void store_stream(double* p, double v) { __stcs(p, v); }
__device__ __forceinline__ void store_stream(df64* p, df64 v) {
  __stcs(reinterpret_cast<float2*>(p), make_float2(v.hi, v.lo));
}

// dst[0..N) = o[0..N) with 16-byte streaming stores (dst 16-byte aligned)
template <typename real, int N>
__device__ __forceinline__ void store_cell(real* dst, const real (&o)[N]) {
  constexpr int W = Bits<real>::W;
#pragma unroll
  for (int k = 0; k < (int)(N * sizeof(real) / 16); ++k) {
    unsigned u[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) u[t] = Bits<real>::word(o[(4 * k + t) / W], (4 * k + t) % W);
    __stcs(reinterpret_cast<uint4*>(reinterpret_cast<char*>(dst) + 16 * k), make_uint4(u[0], u[1], u[2], u[3]));
  }
}
// o[j] <- o[j ^ m] for every j (conditional swaps along each index bit)
template <typename real, int N>
__device__ __forceinline__ void xor_permute(real (&o)[N], int m) {
#pragma unroll
  for (int bit = 1; bit < N; bit <<= 1) {
    const bool sw = (m & bit) != 0;
#pragma unroll
    for (int j = 0; j < N; ++j)
      if (!(j & bit)) {
        const real t0 = o[j], t1 = o[j | bit];
        o[j] = sw ? t1 : t0;
        o[j | bit] = sw ? t0 : t1;
      }
  }
}

// planes prefetched ahead of the one being solved; the ring has one more slot
// so the slot being refilled was consumed a step earlier
// (measured on GB300: 3 planes for FP32 values, 2 for 8-byte values, whose
// smaller ring lets more blocks share an SM)
template <typename real>
struct Prefetch {
  static constexpr int PF = sizeof(real) == 8 ? 2 : 3;
  static constexpr int RING = PF + 1;
};

template <int DIM, int P1>
struct Cell {
  static constexpr int N = DIM == 2 ? P1 * P1 : P1 * P1 * P1;
  static constexpr int FD = DIM == 2 ? P1 : P1 * P1;
  static constexpr int PN = N / P1;  // dofs per sweep-axis layer
  // canonical local component of dof i on axis a
  static __device__ __forceinline__ constexpr int comp(int i, int a) {
    return a == 0 ? i % P1 : (a == 1 ? (i / P1) % P1 : i / (P1 * P1));
  }
  // dof on the inflow (c_a = 0) face of the x axis, transverse index t
  static __device__ __forceinline__ constexpr int x_in(int t) { return P1 * t; }
  static __device__ __forceinline__ constexpr int x_out(int t) { return P1 * t + P1 - 1; }
  // y axis (3-D only), transverse t = c_x + P1 c_z
  static __device__ __forceinline__ constexpr int y_in(int t) { return (t % P1) + P1 * P1 * (t / P1); }
  static __device__ __forceinline__ constexpr int y_out(int t) { return y_in(t) + P1 * (P1 - 1); }
  // sweep axis (y in 2-D, z in 3-D)
  static __device__ __forceinline__ constexpr int s_in(int t) { return t; }
  static __device__ __forceinline__ constexpr int s_out(int t) { return t + N - PN; }
};

template <typename real, int FM, int N>
struct Stream {
  // values streamed per plane and lane: the expanded source (FM = 0) or FM
  // moments plus the isotropic source
  static constexpr int NV = FM == 0 ? N : (FM + 1) * N;
  // Q1 cells (N = 4 in 2-D, 8 in 3-D) move in 16-byte pieces; their ring slots
  // are read back with 16-byte shared loads, so each lane's stride is padded to
  // an odd number of 16-byte units: the 8 lanes of one access phase then fall
  // on 8 different 4-bank groups
  static constexpr bool VEC = (N == 4 || N == 8) && (N * sizeof(real)) % 16 == 0;
  static constexpr int PAD = VEC && ((NV * sizeof(real) / 16) % 2 == 0) ? (int)(16 / sizeof(real)) : 0;
  static constexpr int NVP = NV + PAD;  // per-slot stride of the ring, in values
  // FP32 cells solved by two lanes share one ring slot per cell (each lane
  // copies half of the cell's values): half the ring, so more blocks fit
  // beside the L1 the tables need (2-D Q2 S16 FP32 sweep: 0.865 -> 0.771 ms).
  // The 8-byte sweeps keep a slot per lane: shared slots measured slower
  // there (1.159 -> 1.258 ms at the same two blocks per SM).
  template <int H>
  static constexpr bool shared_slots = H == 2 && sizeof(real) == 4;
  template <int H>
  static constexpr size_t warp_bytes =
      (size_t)Prefetch<real>::RING * (shared_slots<H> ? 16 : 32) * (NVP * sizeof(real) + sizeof(int));
};

// Row r of a cell solve split over H lanes: lane `half` of the pair holds rows
// k H + half in xr[k]; both lanes return row r (a converged shuffle).
template <typename real, int H, int NR>
__device__ __forceinline__ real cell_row(const real (&xr)[NR], int r, int half) {
  if (H == 1) return xr[r];
  const real mine = xr[r / 2];
  const real other = Arith<real>::shfl_xor(mine, 1);
  return (r & 1) == half ? mine : other;
}

// One task: a tile of wx x wy columns for kd directions, swept over the whole
// sweep axis.  Shared by the single-problem and the batched kernels.  The
// arguments come by value: inlined into the single-problem kernel they stay
// parameter reads the compiler can keep out of the inner loop (a reference
// to the parameter block made them loads it had to repeat after every store).
// H lanes solve one cell (H = 2 for cells of 9 or more dofs may be chosen by
// the tiling): both assemble the right-hand side, each computes half of the
// rows of A'^-1 b, and the outflow values they pass on are exchanged; a warp
// then covers 32 / H cells, so twice as many warps share the wavefront and
// each does half the cell-solve arithmetic per step.
template <typename real, int DIM, int P1, int FM, int H>
__device__ __forceinline__ void sweep_task(const SweepArgs<real> a, const int task,
                                           unsigned char* smem_raw) {
  using C = Cell<DIM, P1>;
  constexpr int N = C::N;
  constexpr int FD = C::FD;
  constexpr int NV = Stream<real, FM, N>::NV;
  constexpr int NVP = Stream<real, FM, N>::NVP;
  constexpr int W = Tagged<real>::W;
  constexpr unsigned FULL = 0xffffffffu;
  using A = Arith<real>;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  real* ring = reinterpret_cast<real*>(smem_raw + warp * Stream<real, FM, N>::template warp_bytes<H>);
  constexpr int kPrefetch = Prefetch<real>::PF;
  constexpr int kRing = Prefetch<real>::RING;
  constexpr bool kShare = Stream<real, FM, N>::template shared_slots<H>;
  constexpr int SL = kShare ? 16 : 32;  // ring slots per plane
  constexpr int HS = kShare ? 2 : 1;    // lanes that fill one slot
  int* cring = reinterpret_cast<int*>(ring + kRing * SL * NVP);
  static_assert(H == 1 || H == 2, "one or two lanes per cell");
  static_assert(H == 1 || !Stream<real, FM, N>::VEC, "16-byte cells are solved by one lane");
  constexpr int NR = (N + H - 1) / H;  // rows of the cell solve per lane
  const int cell_lane = lane / H;
  const int half = H == 2 ? (lane & 1) : 0;
  const unsigned pair_mask = H == 2 ? (3u << (lane & 30)) : (1u << lane);
  const int wc = a.wx * a.wy;
  const int kslot = cell_lane / wc;
  const int cl = cell_lane - kslot * wc;
  const int lx = cl % a.wx;
  const int ly = cl / a.wx;
  const int tiles = a.tiles_x * a.tiles_y;
  const int NS = a.n_sweep;
  const int NX = a.nx;
  const int NY = DIM == 3 ? a.ny : 1;
  const int nsteps = NS + (a.wx - 1) + (a.wy - 1);
  constexpr int AS = DIM - 1;  // physical axis of the sweep direction
  const unsigned want_epoch = a.epoch ^ (a.wait_bias ? 0x8000u : 0u);
  {
    const int2 tk = a.tasks[task];
    const int grp = tk.x, tile = tk.y;
    const int tx = tile % a.tiles_x, ty = tile / a.tiles_x;
    const int d = a.group_dirs[grp * a.kd + kslot];
    const bool dir_ok = d >= 0;
    const int dd = dir_ok ? d : 0;
    const int flip = a.group_flip[grp];
    const real wX = a.abs_omega[dd * 3 + 0];
    const real wY = DIM == 3 ? a.abs_omega[dd * 3 + 1] : real(0);
    const real wS = a.abs_omega[dd * 3 + AS];
    real bX = 0, bY = 0, bS = 0;
    if (a.bnd) {
      bX = a.bnd[dd * 3 + 0];
      if (DIM == 3) bY = a.bnd[dd * 3 + 1];
      bS = a.bnd[dd * 3 + AS];
    }
    real w0 = 0, w1 = 0;  // M2D row (moment-fused form)
    if (FM >= 1) w0 = a.m2d[(size_t)dd * a.n_mom + 0];
    if (FM >= 2) w1 = a.m2d[(size_t)dd * a.n_mom + 1];
    const int dcls = a.dir_class[dd];
    // mirrored local dof offsets: phys(i') = base + c0*s0 + c1*s1 + c2*s2
    int base = 0, st0 = 1, st1 = P1, st2 = P1 * P1;
    if (flip & 1) { base += (P1 - 1); st0 = -1; }
    if (flip & 2) { base += (P1 - 1) * P1; st1 = -P1; }
    if (DIM == 3 && (flip & 4)) { base += (P1 - 1) * P1 * P1; st2 = -P1 * P1; }
    // Q1 cells: mirroring an axis flips one bit of the local index, so the
    // physical position of canonical dof i is i ^ fmask and a cell's values
    // move as whole 16-byte pieces
    constexpr bool VEC = Stream<real, FM, N>::VEC;
    static_assert(!VEC || P1 == 2, "the 16-byte path relies on the XOR form of Q1 mirroring");
    const int fmask = flip & (N - 1);
    auto off = [&](int i) {
      return C::comp(i, 0) * st0 + C::comp(i, 1) * st1 + (DIM == 3 ? C::comp(i, 2) * st2 : 0);
    };

    const int xc = tx * a.wx + lx;  // canonical transverse coordinates
    const int yc = ty * a.wy + ly;
    const bool col_ok = dir_ok && xc < NX && (DIM == 2 || yc < NY);
    const int xp = (flip & 1) ? NX - 1 - xc : xc;  // physical
    const int yp = DIM == 3 ? ((flip & 2) ? NY - 1 - yc : yc) : 0;
    const int sflip = DIM == 3 ? (flip & 4) : (flip & 2);
    const long colbase = DIM == 2 ? (long)xp : (long)xp + (long)NX * yp;
    const long plane = DIM == 2 ? (long)NX : (long)NX * NY;  // cells per sweep-axis layer
    auto cell_of = [&](int sc) { return colbase + plane * (sflip ? NS - 1 - sc : sc); };
    const size_t dirbase = (size_t)dd * a.n_dofs;
    const bool pub_x = tx + 1 < a.tiles_x && lx == a.wx - 1;
    const bool pub_y = DIM == 3 && ty + 1 < a.tiles_y && ly == a.wy - 1;

    // stream the source of plane pl into ring slot pl % kRing (one cp.async
    // group per plane).  With shared slots lane half h copies the dofs 2k + h
    // (offsets computed once per task)
    const int slot = kShare ? cell_lane : lane;
    const int part = kShare ? half : 0;
    constexpr int NH = (N + HS - 1) / HS;
    int hoff[NH];
#pragma unroll
    for (int k = 0; k < NH; ++k) hoff[k] = (HS * k + part < N) ? off(HS * k + part) : 0;
    auto issue = [&](int pl) {
      if (col_ok && pl < NS) {
        real* v = ring + ((pl % kRing) * SL + slot) * NVP;
        const long cell = cell_of(pl);
        const long cb = cell * N + base;
        if (part == 0) {
          const unsigned cdst = (unsigned)__cvta_generic_to_shared(cring + (pl % kRing) * SL + slot);
          asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(cdst), "l"(a.cell_class + cell)
                       : "memory");
        }
        if (VEC) {  // the cell's values in physical order, 16 bytes at a time
          const long c0 = cell * N;
          if (FM == 0) {
            cp_async_cell<real, N>(v, a.q + dirbase + c0);
          } else {
            cp_async_cell<real, N>(v, a.src + c0);
            if (FM >= 2) cp_async_cell<real, N>(v + N, a.src + a.n_dofs + c0);
            if (a.iso) {
              cp_async_cell<real, N>(v + FM * N, a.iso + c0);
            } else {
#pragma unroll
              for (int i = 0; i < N; ++i) v[FM * N + i] = real(0);
            }
          }
        } else if (FM == 0) {
          const real* Q = a.q + dirbase + cb;
#pragma unroll
          for (int k = 0; k < NH; ++k) {
            const int i = HS * k + part;
            if (HS == 1 || i < N) cp_async_elem(v + i, Q + hoff[k]);
          }
        } else {
          const real* T = a.src + cb;
#pragma unroll
          for (int k = 0; k < NH; ++k) {
            const int i = HS * k + part;
            if (HS == 1 || i < N) {
              cp_async_elem(v + i, T + hoff[k]);
              if (FM >= 2) cp_async_elem(v + N + i, T + a.n_dofs + hoff[k]);
              if (a.iso)
                cp_async_elem(v + FM * N + i, a.iso + cb + hoff[k]);
              else
                v[FM * N + i] = real(0);
            }
          }
        }
      }
      cp_async_commit();
    };
#pragma unroll
    for (int pl = 0; pl < kPrefetch; ++pl) issue(pl);

    real psiS[FD], psiX[FD], psiY[FD];
#pragma unroll
    for (int t = 0; t < FD; ++t) psiS[t] = psiX[t] = psiY[t] = real(0);
    // Edge words of the upwind tile are loaded one step ahead (the load
    // overlaps a step's work); their tags are checked when they are used, and
    // words that were not yet published are polled for as before.  For 8-byte
    // values and in 3-D (where shared memory, not registers, bounds the
    // resident blocks: 64^3 FP32 1.91 -> 1.86 ms); not for FP32 in 2-D, where
    // the extra registers cost more than the hidden load latency saves
    constexpr bool kAhead = sizeof(real) == 8 || DIM == 3;
    const bool recv_x = col_ok && lx == 0 && tx > 0;
    const bool recv_y = DIM == 3 && col_ok && ly == 0 && ty > 0;
    auto edge_x_at = [&](int r) {
      return a.edge_x + ((((size_t)d * tiles + tile - 1) * NS + r) * a.wy + ly) * (FD * W);
    };
    auto edge_y_at = [&](int r) {
      return a.edge_y + ((((size_t)d * tiles + tile - a.tiles_x) * NS + r) * a.wx + lx) * (FD * W);
    };
    unsigned long long rX[FD * W], rY[FD * W];
    bool hX = false, hY = false;  // rX / rY hold the words of this step's row

    for (int s = 0; s < nsteps; ++s) {
      const int sc = s - lx - ly;
      const bool act = col_ok && sc >= 0 && sc < NS;

      // ---- upwind face values.  Edge-buffer polls run first (divergent), the
      // shuffles after them (converged), and the boundary / edge / neighbour
      // choice is a branch-free select.
      real eX[FD], eY[FD];
#pragma unroll
      for (int t = 0; t < FD; ++t) eX[t] = eY[t] = real(0);
      bool failed = false;
      const unsigned tag = (want_epoch << 16) | ((unsigned)sc & 0xffffu);
      if (act && recv_x) {
        bool ok = hX;
#pragma unroll
        for (int t = 0; t < FD; ++t) ok &= Tagged<real>::decode(rX + t * W, tag, eX[t]);
        if (!ok) failed |= !fetch_edge<real, FD>(edge_x_at(sc), tag, eX, a.status, a.wait_limit_ns);
      }
      if (DIM == 3 && act && recv_y) {
        bool ok = hY;
#pragma unroll
        for (int t = 0; t < FD; ++t) ok &= Tagged<real>::decode(rY + t * W, tag, eY[t]);
        if (!ok) failed |= !fetch_edge<real, FD>(edge_y_at(sc), tag, eY, a.status, a.wait_limit_ns);
      }
      // the next step's row (sc + 1): load its words now
      hX = kAhead && recv_x && sc + 1 >= 0 && sc + 1 < NS;
      if (hX) {
        const unsigned long long* e = edge_x_at(sc + 1);
#pragma unroll
        for (int k = 0; k < FD * W; ++k) rX[k] = ld_relaxed_u64(e + k);
      }
      hY = kAhead && recv_y && sc + 1 >= 0 && sc + 1 < NS;
      if (DIM == 3 && hY) {
        const unsigned long long* e = edge_y_at(sc + 1);
#pragma unroll
        for (int k = 0; k < FD * W; ++k) rY[k] = ld_relaxed_u64(e + k);
      }
      if (__any_sync(FULL, failed)) {  // status is set; drain own copies, leave
        cp_async_wait<0>();
        break;
      }
      const bool x_edge = lx == 0;
      const bool y_edge = ly == 0;
      real upX[FD], upY[FD], upS[FD];
#pragma unroll
      for (int t = 0; t < FD; ++t) {
        const real sx = A::shfl_up(psiX[t], H);
        upX[t] = x_edge ? (tx == 0 ? bX : eX[t]) : sx;
        if (DIM == 3) {
          const real sy = A::shfl_up(psiY[t], a.wx * H);
          upY[t] = y_edge ? (ty == 0 ? bY : eY[t]) : sy;
        }
        upS[t] = sc == 0 ? bS : psiS[t];
      }

      real xr[NR];
#pragma unroll
      for (int k = 0; k < NR; ++k) xr[k] = real(0);
      constexpr bool kHoist = sizeof(real) == 4;
      constexpr int NP = pad4(N), FDP = pad4(FD);  // padded row strides of the tables
      real b[N];
      const real* Ai = a.ainv;
      real arow[kHoist ? NR : 1][kHoist ? N : 1];
      // inflow-face dot products F_a psi_up,a of the x and sweep-axis faces;
      // with two lanes per cell each lane of the pair computes one of the two
      // (lane half 0 the x face, half 1 the sweep-axis face) and the pair
      // exchanges them with a converged shuffle
      real faceX[FD], faceS[FD];
#pragma unroll
      for (int t = 0; t < FD; ++t) faceX[t] = faceS[t] = real(0);
      if (act) {
        cp_async_wait<kPrefetch - 1>();  // plane sc has landed (this lane's copies)
        if (kShare) __syncwarp(pair_mask);  // and the partner's (both lanes of a pair share act)
        const real* v = ring + ((sc % kRing) * SL + slot) * NVP;
        const int cls = cring[(sc % kRing) * SL + slot];
        if (VEC) {  // 16-byte loads of the slot (physical order), then canonical order
          real t0v[N], t1v[N], isv[N];
          load_cell<real, N>(v, t0v);
          xor_permute<real, N>(t0v, fmask);
          if (FM >= 2) {
            load_cell<real, N>(v + N, t1v);
            xor_permute<real, N>(t1v, fmask);
          }
          if (FM >= 1) {
            load_cell<real, N>(v + FM * N, isv);
            xor_permute<real, N>(isv, fmask);
          }
#pragma unroll
          for (int i = 0; i < N; ++i) {
            if (FM == 0) {
              b[i] = t0v[i];
            } else {  // sum_m M2D(d, m) T_m + isotropic source
              typename A::acc s = A::from(isv[i]);
              A::fma(s, w0, t0v[i]);
              if (FM >= 2) A::fma(s, w1, t1v[i]);
              b[i] = A::raw(s);
            }
          }
        } else {
#pragma unroll
          for (int i = 0; i < N; ++i) {
            if (FM == 0) {
              b[i] = v[i];
            } else {  // sum_m M2D(d, m) T_m + isotropic source
              typename A::acc s = A::from(v[FM * N + i]);
              A::fma(s, w0, v[i]);
              if (FM >= 2) A::fma(s, w1, v[N + i]);
              b[i] = A::raw(s);
            }
          }
        }
        issue(sc + kPrefetch);  // refills the slot consumed one step ago
        // FP32: this lane's rows of A'^-1 into registers now, so their loads
        // overlap the right-hand side below (for 8-byte values the longer
        // arithmetic hides them and the registers are better spent elsewhere)
        Ai = a.ainv + ((size_t)cls * a.n_dir_class + dcls) * (N * NP);
        if constexpr (kHoist) {
#pragma unroll
          for (int k = 0; k < NR; ++k) {
            const int i = k * H + half;
            if (H == 1 || i < N) {
              load_row<real, N>(Ai + i * NP, arow[k]);
            } else {
#pragma unroll
              for (int j = 0; j < N; ++j) arow[k][j] = real(0);
            }
          }
        }
        const real* FX = a.face_mass + 0 * FD * FDP;
        const real* FS = a.face_mass + AS * FD * FDP;
        if (H == 1) {
#pragma unroll
          for (int t = 0; t < FD; ++t) {
            real fx[FD], fs[FD];
            load_row<real, FD>(FX + t * FDP, fx);
            load_row<real, FD>(FS + t * FDP, fs);
            typename A::acc accx = A::prod(fx[0], upX[0]), accs = A::prod(fs[0], upS[0]);
#pragma unroll
            for (int u = 1; u < FD; ++u) {
              A::fma(accx, fx[u], upX[u]);
              A::fma(accs, fs[u], upS[u]);
            }
            faceX[t] = A::raw(accx);
            faceS[t] = A::raw(accs);
          }
        } else {  // one instruction stream: the face is selected by data, not by a branch
          const real* FF = half ? FS : FX;
          real upF[FD];
#pragma unroll
          for (int u = 0; u < FD; ++u) upF[u] = half ? upS[u] : upX[u];
#pragma unroll
          for (int t = 0; t < FD; ++t) {
            real f[FD];
            load_row<real, FD>(FF + t * FDP, f);
            typename A::acc acc = A::prod(f[0], upF[0]);
#pragma unroll
            for (int u = 1; u < FD; ++u) A::fma(acc, f[u], upF[u]);
            faceX[t] = A::raw(acc);  // this lane's face; sorted out after the exchange
          }
        }
      }
      if (H == 2) {  // every lane: exchange with the pair's partner (lane ^ 1)
#pragma unroll
        for (int t = 0; t < FD; ++t) {
          const real mine = faceX[t];
          const real other = A::shfl_xor(mine, 1);
          faceX[t] = half ? other : mine;
          faceS[t] = half ? mine : other;
        }
      }
      if (act) {
        // inflow faces: b_face += |Omega_a| F_a psi_up, one face after the
        // other (the two inflow faces share the corner dof)
#pragma unroll
        for (int t = 0; t < FD; ++t) {
          typename A::acc bx = A::from(b[C::x_in(t)]);
          A::fma(bx, wX, faceX[t]);
          b[C::x_in(t)] = A::raw(bx);
          typename A::acc bs = A::from(b[C::s_in(t)]);
          A::fma(bs, wS, faceS[t]);
          b[C::s_in(t)] = A::raw(bs);
        }
        if (DIM == 3) {
          const real* FY = a.face_mass + 1 * FD * FDP;
#pragma unroll
          for (int t = 0; t < FD; ++t) {
            real fy[FD];
            load_row<real, FD>(FY + t * FDP, fy);
            typename A::acc acc = A::prod(fy[0], upY[0]);
#pragma unroll
            for (int u = 1; u < FD; ++u) A::fma(acc, fy[u], upY[u]);
            typename A::acc by = A::from(b[C::y_in(t)]);
            A::fma(by, wY, A::raw(acc));
            b[C::y_in(t)] = A::raw(by);
          }
        }
        // x = A'^-1 b: this lane's rows i = k H + half
#pragma unroll
        for (int k = 0; k < NR; ++k) {
          const int i = k * H + half;
          typename A::acc acc = A::zero();
          if (H == 1 || i < N) {
            if constexpr (kHoist) {
              acc = A::prod(arow[k][0], b[0]);
#pragma unroll
              for (int j = 1; j < N; ++j) A::fma(acc, arow[k][j], b[j]);
            } else {
              real row[N];
              load_row<real, N>(Ai + i * NP, row);
              acc = A::prod(row[0], b[0]);
#pragma unroll
              for (int j = 1; j < N; ++j) A::fma(acc, row[j], b[j]);
            }
          }
          xr[k] = A::get(acc);
        }
      }
      // outflow values (converged: with H = 2 the partner lane holds half the rows)
#pragma unroll
      for (int t = 0; t < FD; ++t) {
        const real vx = cell_row<real, H>(xr, C::x_out(t), half);
        const real vs = cell_row<real, H>(xr, C::s_out(t), half);
        real vy = real(0);
        if (DIM == 3) vy = cell_row<real, H>(xr, C::y_out(t), half);
        if (act) {
          psiX[t] = vx;
          psiS[t] = vs;
          if (DIM == 3) psiY[t] = vy;
        }
      }
      if (act) {
        // edge values first, so the downwind tile can start; then the angular flux
        const unsigned ptag = (a.epoch << 16) | ((unsigned)sc & 0xffffu);
        if (pub_x && half == 0) {
          unsigned long long* e =
              a.edge_x + ((((size_t)d * tiles + tile) * NS + sc) * a.wy + ly) * (FD * W);
#pragma unroll
          for (int t = 0; t < FD; ++t) Tagged<real>::put(e + t * W, psiX[t], ptag);
        }
        if (pub_y && half == 0) {
          unsigned long long* e =
              a.edge_y + ((((size_t)d * tiles + tile) * NS + sc) * a.wx + lx) * (FD * W);
#pragma unroll
          for (int t = 0; t < FD; ++t) Tagged<real>::put(e + t * W, psiY[t], ptag);
        }
        if constexpr (VEC) {  // physical order by swaps, then 16-byte stores (H = 1: xr holds the cell)
          real o[N];
#pragma unroll
          for (int i = 0; i < N; ++i) o[i] = xr[i];
          xor_permute<real, N>(o, fmask);
          store_cell<real, N>(a.psi + dirbase + cell_of(sc) * N, o);
        } else {
          real* P = a.psi + dirbase + cell_of(sc) * N + base;
#pragma unroll
          for (int k = 0; k < NR; ++k) {
            const int i = k * H + half;
            if (H == 1 || i < N) store_stream(P + off(i), xr[k]);
          }
        }
      }
    }
  }
}

// Single problem: warps take tasks in ticket order (level-major), so every
// task a warp waits on was taken earlier by a running warp -- any grid is
// deadlock-free.
template <typename real, int DIM, int P1, int FM, int H>
__global__ void __launch_bounds__(128) sweep_kernel(const SweepArgs<real> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr unsigned FULL = 0xffffffffu;
  for (;;) {
    int task = 0, stop = 0;
    if ((threadIdx.x & 31) == 0) {
      task = atomicAdd(a.ticket, 1);
      stop = *(volatile int*)a.status;
    }
    task = __shfl_sync(FULL, task, 0);
    stop = __shfl_sync(FULL, stop, 0);
    if (task >= a.n_tasks || stop) return;
    sweep_task<real, DIM, P1, FM, H>(a, task, smem_raw);
  }
}

// Many problems in one persistent launch.  Ticket t names (problem, task) =
// tmap[t]; the map lists each problem's tasks in its own order, interleaved
// across problems, so the in-order argument above still holds.  A warp copies
// its task's problem arguments into its shared slot before the task; the
// edge-word epoch comes from device memory, so a captured launch replays with
// the epoch of the moment.
template <typename real, int DIM, int P1, int FM, int H>
__global__ void __launch_bounds__(128) sweep_batch_kernel(const SweepArgs<real>* __restrict__ args,
                                                          const int2* __restrict__ tmap, int n_total,
                                                          int* ticket, const int* status,
                                                          const unsigned* epoch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SweepArgs<real> s_args[4];
  static_assert(sizeof(SweepArgs<real>) % 4 == 0, "argument block is copied by words");
  constexpr int WORDS = (int)(sizeof(SweepArgs<real>) / 4);
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  for (;;) {
    int t = 0, stop = 0;
    if (lane == 0) {
      t = atomicAdd(ticket, 1);
      stop = *(volatile const int*)status;
    }
    t = __shfl_sync(FULL, t, 0);
    stop = __shfl_sync(FULL, stop, 0);
    if (t >= n_total || stop) return;
    const int2 pt = tmap[t];
    const unsigned* src = reinterpret_cast<const unsigned*>(args + pt.x);
    unsigned* dst = reinterpret_cast<unsigned*>(&s_args[warp]);
    for (int i = lane; i < WORDS; i += 32) dst[i] = src[i];
    __syncwarp();
    if (lane == 0) s_args[warp].epoch = *epoch;  // set on the device before the launch
    __syncwarp();
    sweep_task<real, DIM, P1, FM, H>(s_args[warp], pt.y, smem_raw);
    __syncwarp();  // the slot is rewritten by the next task
  }
}

// Shared-memory carveout for a launch: as much as the blocks that can be
// resident need, but at most what leaves keep_kb of the SM's on-chip memory
// to L1, where the cell-solve tables of the running directions live.  The
// kernels that stream their sources element by element (cp.async.ca, which
// allocates in L1) keep 144 KB: fewer resident warps with their tables in L1
// beat more warps missing it (2-D Q2 S16 double-float sweep: 4 blocks per SM
// 1.63 ms, 3 blocks 1.40 ms, 2 blocks 1.35 ms); the 16-byte kernels (Q1 cells,
// cp.async.cg past L1) keep 32 KB (3-D Q1 GLC S12 FP32: 5 blocks 2.30 ms,
// 3 or 4 blocks 2.10 ms).
inline int carveout_percent(int grid, size_t smem_per_block, int max_blocks_per_sm, int keep_kb) {
  static int sms = 0, smem_sm = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (sms < 1 || smem_sm < 1) return -1;  // leave the driver's choice
  }
  const size_t per_block = smem_per_block + 1024;  // + the runtime's reserve per block
  int per_sm = (grid + sms - 1) / sms;
  if (per_sm > max_blocks_per_sm) per_sm = max_blocks_per_sm;
  const long room = (long)smem_sm - (long)keep_kb * 1024;
  const int fit = room >= (long)per_block ? (int)(room / (long)per_block) : 1;
  if (per_sm > fit) per_sm = fit;
  const size_t need = (size_t)per_sm * per_block;
  const int pct = (int)((need * 100 + smem_sm - 1) / smem_sm);
  return pct < 100 ? pct : 100;
}
template <typename real, int FM, int N>
constexpr int l1_keep_kb() { return Stream<real, FM, N>::VEC ? 32 : 144; }

template <typename real, int DIM, int P1, int FM, int H>
cudaError_t launch_sweep_fm(const SweepArgs<real>& a, int grid, int block, cudaStream_t s) {
  constexpr int N = Cell<DIM, P1>::N;
  const size_t smem = (size_t)(block / 32) * Stream<real, FM, N>::template warp_bytes<H>;
  static bool configured = false;  // opt in to > 48 KB once per instantiation
  static int max_per_sm = 0, carve = -2;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(sweep_kernel<real, DIM, P1, FM, H>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_per_sm, sweep_kernel<real, DIM, P1, FM, H>, block, smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const int pct = carveout_percent(grid, smem, max_per_sm > 0 ? max_per_sm : 1, l1_keep_kb<real, FM, N>());
  if (pct >= 0 && pct != carve) {
    cudaError_t e = cudaFuncSetAttribute(sweep_kernel<real, DIM, P1, FM, H>,
                                         cudaFuncAttributePreferredSharedMemoryCarveout, pct);
    if (e != cudaSuccess) return e;
    carve = pct;
  }
  sweep_kernel<real, DIM, P1, FM, H><<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename real, int DIM, int P1, int FM, int H>
cudaError_t launch_sweep_batch_fm(const SweepArgs<real>* args, const int2* tmap, int n_total, int* ticket,
                                  const int* status, const unsigned* epoch, int grid, int block,
                                  cudaStream_t s) {
  constexpr int N = Cell<DIM, P1>::N;
  const size_t smem = (size_t)(block / 32) * Stream<real, FM, N>::template warp_bytes<H>;
  static bool configured = false;
  static int max_per_sm = 0, carve = -2;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(sweep_batch_kernel<real, DIM, P1, FM, H>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_per_sm, sweep_batch_kernel<real, DIM, P1, FM, H>, block,
                                                      smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  // static shared memory (the argument slots) counts too
  const int pct = carveout_percent(grid, smem + 4 * sizeof(SweepArgs<real>), max_per_sm > 0 ? max_per_sm : 1,
                                   l1_keep_kb<real, FM, N>());
  if (pct >= 0 && pct != carve) {
    cudaError_t e = cudaFuncSetAttribute(sweep_batch_kernel<real, DIM, P1, FM, H>,
                                         cudaFuncAttributePreferredSharedMemoryCarveout, pct);
    if (e != cudaSuccess) return e;
    carve = pct;
  }
  sweep_batch_kernel<real, DIM, P1, FM, H><<<grid, block, smem, s>>>(args, tmap, n_total, ticket, status, epoch);
  return cudaGetLastError();
}

template <typename real, int DIM, int P1, int H>
cudaError_t launch_sweep_batch_h(int fm, const SweepArgs<real>* args, const int2* tmap, int n_total, int* ticket,
                                 const int* status, const unsigned* epoch, int grid, int block, cudaStream_t s) {
  if (fm == 0) return launch_sweep_batch_fm<real, DIM, P1, 0, H>(args, tmap, n_total, ticket, status, epoch, grid, block, s);
  if (fm == 1) return launch_sweep_batch_fm<real, DIM, P1, 1, H>(args, tmap, n_total, ticket, status, epoch, grid, block, s);
  if (fm == 2) return launch_sweep_batch_fm<real, DIM, P1, 2, H>(args, tmap, n_total, ticket, status, epoch, grid, block, s);
  return cudaErrorInvalidValue;
}

// lanes per cell: 1, or 2 for cells of 9 or more dofs
template <typename real, int DIM, int P1>
cudaError_t launch_sweep_batch_impl(int fm, int lpc, const SweepArgs<real>* args, const int2* tmap, int n_total,
                                    int* ticket, const int* status, const unsigned* epoch, int grid,
                                    int block, cudaStream_t s) {
  if (lpc == 2) {
    if constexpr (Cell<DIM, P1>::N >= 9)
      return launch_sweep_batch_h<real, DIM, P1, 2>(fm, args, tmap, n_total, ticket, status, epoch, grid, block, s);
    return cudaErrorInvalidValue;
  }
  if (lpc != 1) return cudaErrorInvalidValue;
  return launch_sweep_batch_h<real, DIM, P1, 1>(fm, args, tmap, n_total, ticket, status, epoch, grid, block, s);
}

template <typename real, int DIM, int P1, int H>
cudaError_t launch_sweep_h(int fm, const SweepArgs<real>& a, int grid, int block, cudaStream_t s) {
  if (fm == 0) return launch_sweep_fm<real, DIM, P1, 0, H>(a, grid, block, s);
  if (fm == 1) return launch_sweep_fm<real, DIM, P1, 1, H>(a, grid, block, s);
  if (fm == 2) return launch_sweep_fm<real, DIM, P1, 2, H>(a, grid, block, s);
  return cudaErrorInvalidValue;
}

// a.lpc lanes per cell: 1, or 2 for cells of 9 or more dofs
template <typename real, int DIM, int P1>
cudaError_t launch_sweep_impl(int fm, const SweepArgs<real>& a, int grid, int block,
                              cudaStream_t s) {
  if (a.lpc == 2) {
    if constexpr (Cell<DIM, P1>::N >= 9) return launch_sweep_h<real, DIM, P1, 2>(fm, a, grid, block, s);
    return cudaErrorInvalidValue;
  }
  if (a.lpc != 1) return cudaErrorInvalidValue;
  return launch_sweep_h<real, DIM, P1, 1>(fm, a, grid, block, s);
}

}  // namespace ouranos
