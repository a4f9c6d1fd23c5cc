// Vector kernels around the sweep: scattering source, fixed source, the
// residual form of Apply, layout permutations and the FP64 BLAS-1 pieces of
// the Krylov drivers.  All are HBM-streaming, one grid-stride loop each.
#include <algorithm>
#include <mutex>
#include <type_traits>
#include <unordered_map>

#include "df64.cuh"
#include "internal.h"

namespace ouranos {
namespace {

constexpr int kBlock = 256;

inline int grid_for(long n) {
  long g = (n + kBlock - 1) / kBlock;
  if (g > 152L * 32) g = 152L * 32;  // 152 SMs x 32 resident blocks of 256 threads at most
  return g < 1 ? 1 : (int)g;
}

// Grid of the direction-axis contractions: no more blocks than can be
// resident at once, so the grid-stride loop runs in balanced rounds (one
// thread per dof left a nearly empty last wave: 2304 blocks over 760-912
// resident slots).  Resident blocks per SM are queried once per kernel.
template <typename K>
int resident_grid(K kernel, long n, size_t smem) {
  static std::mutex mu;
  static std::unordered_map<const void*, int> per_sm_cache;
  static int sms = 0;
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!sms) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (sms < 1) sms = 152;
    }
    auto it = per_sm_cache.find((const void*)kernel);
    if (it != per_sm_cache.end()) {
      per_sm = it->second;
    } else {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
      }
      per_sm_cache[(const void*)kernel] = per_sm;
    }
  }
  const long need = (n + kBlock - 1) / kBlock;
  const long g = std::min(need, (long)per_sm * sms);
  return g < 1 ? 1 : (int)g;
}

// compute_scattering_source (src/RadiativeTransfer.cc:811-843) and, for the
// right-hand side, compute_outer_scattering_source (:845-876):
//   T_m[c] = s(mat_c, g->g, l(m)) M x_m[c] + sum_{g' != g} s(mat_c, g'->g, l(m)) M phi_{g',m}[c]
// One thread per (moment, cell, local dof i).
template <typename real>
__global__ void scatter_source_kernel(const double* __restrict__ x, const double* __restrict__ gf,
                                      real* __restrict__ src, const double* __restrict__ M,
                                      const double* __restrict__ sscale,
                                      const double* __restrict__ oscale,
                                      const int* __restrict__ material, int n_groups, int group,
                                      long n_cells, int n, int n_mom, long n_dofs) {
  const long total = (long)n_mom * n_cells * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const int i = e % n;
    const long c = (e / n) % n_cells;
    const int m = e / ((long)n * n_cells);
    const int mat = material[c];
    const double* row = M + i * n;
    double acc = 0.0;
    if (x) {
      const double* xc = x + (size_t)m * n_dofs + c * n;
      double r = 0.0;
      for (int j = 0; j < n; ++j) r += row[j] * xc[j];
      acc = sscale[(size_t)mat * n_mom + m] * r;
    }
    if (gf) {
      for (int g = 0; g < n_groups; ++g) {
        if (g == group) continue;
        const double* xg = gf + ((size_t)g * n_mom + m) * n_dofs + c * n;
        double r = 0.0;
        for (int j = 0; j < n; ++j) r += row[j] * xg[j];
        acc += oscale[((size_t)mat * n_groups + g) * n_mom + m] * r;
      }
    }
    src[(size_t)m * n_dofs + c * n + i] = real_from_double<real>(acc);
  }
}

// b += M q/ws for the right-hand side (src/RadiativeTransfer.cc:914-922):
// iso[c*n+i] = (q_{src(c)}/ws) * sum_j M_ij.
template <typename real>
__global__ void iso_source_kernel(real* iso, const double* qcell, const double* rowsum,
                                  const int* source_id, long n_cells, int n) {
  const long total = n_cells * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const long c = e / n;
    const int i = e % n;
    const int sid = source_id ? source_id[c] : 0;
    iso[e] = real_from_double<real>(qcell[sid] * rowsum[i]);
  }
}

// y = sx * x + sp * phi; Apply uses (1, -1): y = x - D L^-1 M2D S x
// (src/RadiativeTransfer.cc:805-806); the driver's sweep uses (1, 1).
template <typename real>
__global__ void combine_kernel(const double* x, const real* phi, double* y, long len, double sx,
                               double sp) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < len;
       e += (long)gridDim.x * blockDim.x)
    y[e] = (x ? sx * x[e] : 0.0) + sp * (double)phi[e];
}

// y = sx x + sp phi on rows x len elements of row stride `stride` (one dof
// range of every moment)
template <typename real>
__global__ void combine_rows_kernel(const double* x, const real* phi, double* y, int rows, long len,
                                    long stride, double sx, double sp) {
  const long total = (long)rows * len;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < total; k += (long)gridDim.x * blockDim.x) {
    const long e = (k / len) * stride + k % len;
    y[e] = (x ? sx * x[e] : 0.0) + sp * (double)phi[e];
  }
}

// Gather between the caller's cell numbering and the lexicographic one.
__global__ void permute_kernel(const double* in, double* out, const long* order, long n_cells,
                               int n, int n_vec, int to_internal) {
  const long total = (long)n_vec * n_cells * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const int i = e % n;
    const long c = (e / n) % n_cells;
    const long v = e / ((long)n * n_cells);
    const long ext = (v * n_cells + order[c]) * n + i;
    if (to_internal)
      out[e] = in[ext];
    else
      out[ext] = in[e];
  }
}

// w += scale * sum_j coef[j] V[j]; pointers and coefficients staged in shared
// memory.  GB300's FP64 pipe runs at 1/64 of the FP32 rate and binds these
// FP64 vector kernels, so they issue exactly k multiply-adds per element: the
// k vectors go in chunks of 8, 4, 2 and 1 (a predicated-off multiply-add of a
// wider unrolled loop still takes its FP64 issue slot).  Fixed order, so the
// result is deterministic.
template <int W>
__device__ __forceinline__ double axpy_chunk(const double* const* sv, const double* sc, int j0, long e) {
  double a0 = 0.0, a1 = 0.0;
#pragma unroll
  for (int jj = 0; jj < W; ++jj) {
    const double t = sc[j0 + jj] * __ldg(sv[j0 + jj] + e);
    if (jj & 1) a1 += t;
    else a0 += t;
  }
  return a0 + a1;
}
template <int KMAX>
__global__ void multi_axpy_kernel(const double* const* V, int k, const double* coef, double scale,
                                  double* w, long len) {
  __shared__ const double* sv[KMAX];
  __shared__ double sc[KMAX];
  for (int j = threadIdx.x; j < KMAX; j += blockDim.x) {
    sv[j] = j < k ? V[j] : nullptr;
    sc[j] = j < k ? coef[j] * scale : 0.0;
  }
  __syncthreads();
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < len;
       e += (long)gridDim.x * blockDim.x) {
    double acc = 0.0;
    int j0 = 0;
    for (; j0 + 8 <= k; j0 += 8) acc += axpy_chunk<8>(sv, sc, j0, e);
    if (j0 + 4 <= k) {
      acc += axpy_chunk<4>(sv, sc, j0, e);
      j0 += 4;
    }
    if (j0 + 2 <= k) {
      acc += axpy_chunk<2>(sv, sc, j0, e);
      j0 += 2;
    }
    if (j0 < k) acc += axpy_chunk<1>(sv, sc, j0, e);
    w[e] += acc;
  }
}

__global__ void axpby_kernel(double a, const double* x, double b, double* y, long len) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < len;
       e += (long)gridDim.x * blockDim.x)
    y[e] = b == 0.0 ? a * x[e] : a * x[e] + b * y[e];  // y may be uninitialised when b == 0
}

// out[j] = sum_i xs[j][i] * y[i], j < k, in two launches.  Block b reduces its
// grid-stride slice into partial[j * gridDim.x + b], taking the vectors in
// chunks of 8, 4, 2 and 1 (W accumulators and W + 1 loads in flight per
// element, y re-read once per chunk; exactly k FP64 multiply-adds per element,
// see multi_axpy_kernel); then one warp per output sums the partials in a
// fixed order (deterministic, no atomics).
constexpr int kDotChunk = 8;
template <int W>
__device__ __forceinline__ void dots_chunk(const double* const* sx, const double* y, int j0, long len,
                                           double* partial, double (*red)[kBlock / 32]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double acc[W];
#pragma unroll
  for (int jj = 0; jj < W; ++jj) acc[jj] = 0.0;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < len; e += (long)gridDim.x * blockDim.x) {
    const double yv = __ldg(y + e);
#pragma unroll
    for (int jj = 0; jj < W; ++jj) acc[jj] += __ldg(sx[j0 + jj] + e) * yv;
  }
#pragma unroll
  for (int jj = 0; jj < W; ++jj) {
    double v = acc[jj];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[jj][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < W) {
    double v = 0.0;
    for (int w = 0; w < kBlock / 32; ++w) v += red[threadIdx.x][w];
    partial[(size_t)(j0 + threadIdx.x) * gridDim.x + blockIdx.x] = v;
  }
  __syncthreads();
}
__global__ void __launch_bounds__(kBlock) dots_partial_kernel(const double* const* xs, const double* y, int k,
                                                              long len, double* partial) {
  __shared__ const double* sx[32];
  __shared__ double red[kDotChunk][kBlock / 32];
  for (int j = threadIdx.x; j < 32; j += blockDim.x) sx[j] = j < k ? xs[j] : nullptr;
  __syncthreads();
  int j0 = 0;
  for (; j0 + 8 <= k; j0 += 8) dots_chunk<8>(sx, y, j0, len, partial, red);
  if (j0 + 4 <= k) {
    dots_chunk<4>(sx, y, j0, len, partial, red);
    j0 += 4;
  }
  if (j0 + 2 <= k) {
    dots_chunk<2>(sx, y, j0, len, partial, red);
    j0 += 2;
  }
  if (j0 < k) dots_chunk<1>(sx, y, j0, len, partial, red);
}
__global__ void __launch_bounds__(kBlock) dots_final_kernel(const double* partial, int k, int nblocks,
                                                            double* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = warp; j < k; j += kBlock / 32) {
    const double* pj = partial + (size_t)j * nblocks;
    double v = 0.0;
    for (int b = lane; b < nblocks; b += 32) v += pj[b];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) out[j] = v;
  }
}

// Moment <-> direction contractions over the direction axis.  Both are
// HBM-streaming: each thread owns one dof column e and loops over the short
// axis with the coefficient table in shared memory.
//   expand:  q[d][e] (+)= sum_{m<nm} m2d[d*ld + m] T[m][e] (+ iso[e])
//   reduce:  phi[m][e]   = sum_d d2m_t[d*ld + m] psi[d][e],  m < nm
template <typename real, int NM>
__global__ void expand_kernel(const real* __restrict__ T, const real* __restrict__ iso,
                              const real* __restrict__ m2d, int ld, real* __restrict__ q,
                              int n_dir, int nm, long n_dofs, long len, int accumulate) {
  extern __shared__ unsigned char smem_raw[];
  real* sm = reinterpret_cast<real*>(smem_raw);
  for (int k = threadIdx.x; k < n_dir * nm; k += blockDim.x) sm[k] = m2d[(k / nm) * ld + k % nm];
  __syncthreads();
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < len;
       e += (long)gridDim.x * blockDim.x) {
    real t[NM];
#pragma unroll
    for (int m = 0; m < NM; ++m) t[m] = m < nm ? T[(size_t)m * n_dofs + e] : real(0);
    const real is = iso ? iso[e] : real(0);
    for (int d = 0; d < n_dir; ++d) {
      real acc = accumulate ? q[(size_t)d * n_dofs + e] : is;
#pragma unroll
      for (int m = 0; m < NM; ++m)
        if (m < nm) acc += sm[d * nm + m] * t[m];
      q[(size_t)d * n_dofs + e] = acc;
    }
  }
}

template <typename real, int NM>
__global__ void reduce_kernel(const real* __restrict__ psi, const real* __restrict__ d2m_t, int ld,
                              real* __restrict__ phi, int n_dir, int nm, long n_dofs, long len) {
  extern __shared__ unsigned char smem_raw[];
  real* sm = reinterpret_cast<real*>(smem_raw);
  for (int k = threadIdx.x; k < n_dir * nm; k += blockDim.x) sm[k] = d2m_t[(k / nm) * ld + k % nm];
  __syncthreads();
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < len;
       e += (long)gridDim.x * blockDim.x) {
    real acc[NM];
#pragma unroll
    for (int m = 0; m < NM; ++m) acc[m] = real(0);
    for (int d = 0; d < n_dir; ++d) {
      const real v = psi[(size_t)d * n_dofs + e];
#pragma unroll
      for (int m = 0; m < NM; ++m)
        if (m < nm) acc[m] += sm[d * nm + m] * v;
    }
#pragma unroll
    for (int m = 0; m < NM; ++m)
      if (m < nm) phi[(size_t)m * n_dofs + e] = acc[m];
  }
}

// FP64 contractions in double-float arithmetic on the FP32 pipes (see df64.cuh):
// same inputs and outputs as expand_kernel<double> / reduce_kernel<double>.
// result of a double-float contraction in the storage type: double (rounded)
// or df64 (kept as the pair)
template <typename S>
__device__ __forceinline__ S store_df64(df64 v);
template <>
__device__ __forceinline__ double store_df64<double>(df64 v) { return df64_to(v); }
template <>
__device__ __forceinline__ df64 store_df64<df64>(df64 v) { return v; }

template <int NM, typename S>
__global__ void expand_df64_kernel(const S* __restrict__ T, const S* __restrict__ iso,
                                   const double* __restrict__ m2d, int ld, S* __restrict__ q,
                                   int n_dir, int nm, long n_dofs, long len, int accumulate) {
  extern __shared__ unsigned char smem_raw[];
  df64* sm = reinterpret_cast<df64*>(smem_raw);
  for (int k = threadIdx.x; k < n_dir * nm; k += blockDim.x) sm[k] = df64_from(m2d[(k / nm) * ld + k % nm]);
  __syncthreads();
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < len;
       e += (long)gridDim.x * blockDim.x) {
    df64 t[NM];
#pragma unroll
    for (int m = 0; m < NM; ++m) t[m] = m < nm ? to_df64(T[(size_t)m * n_dofs + e]) : df64(0.f);
    const df64 is = iso ? to_df64(iso[e]) : df64(0.f);
    for (int d = 0; d < n_dir; ++d) {
      df64_acc acc = acc_from(accumulate ? to_df64(q[(size_t)d * n_dofs + e]) : is);
#pragma unroll
      for (int m = 0; m < NM; ++m)
        if (m < nm) acc_fma(acc, sm[d * nm + m], t[m]);
      q[(size_t)d * n_dofs + e] = store_df64<S>(acc_result(acc));
    }
  }
}

template <int NM, typename S>
__global__ void reduce_df64_kernel(const S* __restrict__ psi, const double* __restrict__ d2m_t,
                                   int ld, double* __restrict__ phi, int n_dir, int nm, long n_dofs, long len) {
  extern __shared__ unsigned char smem_raw[];
  df64* sm = reinterpret_cast<df64*>(smem_raw);
  for (int k = threadIdx.x; k < n_dir * nm; k += blockDim.x) sm[k] = df64_from(d2m_t[(k / nm) * ld + k % nm]);
  __syncthreads();
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < len;
       e += (long)gridDim.x * blockDim.x) {
    df64_acc acc[NM];
#pragma unroll
    for (int m = 0; m < NM; ++m) acc[m] = acc_zero();
#pragma unroll 4  // several directions' loads in flight
    for (int d = 0; d < n_dir; ++d) {
      const df64 v = to_df64(psi[(size_t)d * n_dofs + e]);
#pragma unroll
      for (int m = 0; m < NM; ++m)
        if (m < nm) acc_fma(acc[m], sm[d * nm + m], v);
    }
#pragma unroll
    for (int m = 0; m < NM; ++m)
      if (m < nm) phi[(size_t)m * n_dofs + e] = df64_to(acc_result(acc[m]));
  }
}

}  // namespace

template <typename S>
static cudaError_t expand_df64_any(const S* T, const S* iso, const double* m2d, S* q, int n_dir, int n_mom,
                                   long n_dofs, cudaStream_t s, long len) {
  for (int m0 = 0; m0 < n_mom; m0 += 16) {
    const int nm = n_mom - m0 < 16 ? n_mom - m0 : 16;
    const size_t sh = sizeof(df64) * (size_t)n_dir * nm;
    const S* Tm = T + (size_t)m0 * n_dofs;
    const int acc = m0 > 0;
    const S* is = m0 == 0 ? iso : nullptr;
    if (nm <= 4)
      expand_df64_kernel<4, S><<<resident_grid(expand_df64_kernel<4, S>, len, sh), kBlock, sh, s>>>(Tm, is, m2d + m0, n_mom, q, n_dir, nm, n_dofs, len, acc);
    else if (nm <= 10)
      expand_df64_kernel<10, S><<<resident_grid(expand_df64_kernel<10, S>, len, sh), kBlock, sh, s>>>(Tm, is, m2d + m0, n_mom, q, n_dir, nm, n_dofs, len, acc);
    else
      expand_df64_kernel<16, S><<<resident_grid(expand_df64_kernel<16, S>, len, sh), kBlock, sh, s>>>(Tm, is, m2d + m0, n_mom, q, n_dir, nm, n_dofs, len, acc);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename S>
static cudaError_t reduce_df64_any(const S* psi, const double* d2m_t, double* phi, int n_dir, int n_mom,
                                   long n_dofs, cudaStream_t s, long len) {
  for (int m0 = 0; m0 < n_mom; m0 += 16) {
    const int nm = n_mom - m0 < 16 ? n_mom - m0 : 16;
    const size_t sh = sizeof(df64) * (size_t)n_dir * nm;
    double* ph = phi + (size_t)m0 * n_dofs;
    if (nm <= 1)
      reduce_df64_kernel<1, S><<<resident_grid(reduce_df64_kernel<1, S>, len, sh), kBlock, sh, s>>>(psi, d2m_t + m0, n_mom, ph, n_dir, nm, n_dofs, len);
    else if (nm <= 4)
      reduce_df64_kernel<4, S><<<resident_grid(reduce_df64_kernel<4, S>, len, sh), kBlock, sh, s>>>(psi, d2m_t + m0, n_mom, ph, n_dir, nm, n_dofs, len);
    else if (nm <= 10)
      reduce_df64_kernel<10, S><<<resident_grid(reduce_df64_kernel<10, S>, len, sh), kBlock, sh, s>>>(psi, d2m_t + m0, n_mom, ph, n_dir, nm, n_dofs, len);
    else
      reduce_df64_kernel<16, S><<<resident_grid(reduce_df64_kernel<16, S>, len, sh), kBlock, sh, s>>>(psi, d2m_t + m0, n_mom, ph, n_dir, nm, n_dofs, len);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

namespace {
// Shared-memory images of the symmetry tables: representative M2D or D2M rows
// as double-float [class][nm], members [class][P], groups [nm], signs [G].
template <int P>
__device__ __forceinline__ void load_sym(const SymTables& st, const double* rep, int nm, df64* srep, int* sdir,
                                         int* sgrp, unsigned* ssign) {
  for (int k = threadIdx.x; k < st.n_class * nm; k += blockDim.x) srep[k] = df64_from(rep[k]);
  for (int k = threadIdx.x; k < st.n_class * P; k += blockDim.x) sdir[k] = st.cls_dir[k];
  for (int k = threadIdx.x; k < nm; k += blockDim.x) sgrp[k] = st.mom_group[k];
  for (int k = threadIdx.x; k < st.G; k += blockDim.x) ssign[k] = st.sign[k];
  __syncthreads();
}
__device__ __forceinline__ df64 neg_if(df64 v, bool neg) { return neg ? df64(-v.hi, -v.lo) : v; }

// The parity groups of the real spherical-harmonic moments under the octant
// reflections, in the moment order of the quadrature tables (for l, then
// m = l..0 cosine parts, then m = 1..l sine parts), numbered by first
// appearance; a lower scattering order uses a prefix.  PAT 2: 2-D (P = 4,
// moments up to P3), PAT 3: 3-D (P = 8, up to P3); sign of group g on member
// f: bit f of the group's sign word.  PAT 0: the tables' own, read at run time.
// With PAT set, each moment's product goes to its group's accumulator and each
// member's signs are constants once the loops are unrolled (a run-time group
// index made the compiler predicate one multiply-add per possible group).
__host__ __device__ constexpr int sym_group(int pat, int m) {
  return pat == 2 ? (int)((0x12258088ull >> (3 * m)) & 7u)
                  : (int)((0x7da28ea20688ull >> (3 * m)) & 7u);
}
constexpr bool sym_pattern_is(int pat, const int* g, int n) {
  for (int m = 0; m < n; ++m)
    if (sym_group(pat, m) != g[m]) return false;
  return true;
}
constexpr int kSymGroups2[10] = {0, 1, 2, 0, 0, 3, 1, 1, 2, 2};
constexpr int kSymGroups3[16] = {0, 1, 2, 3, 0, 4, 0, 5, 6, 1, 2, 1, 2, 3, 7, 3};
static_assert(sym_pattern_is(2, kSymGroups2, 10) && sym_pattern_is(3, kSymGroups3, 16), "packed group tables");
__host__ __device__ constexpr bool sym_first_in_group(int pat, int m) {
  for (int k = 0; k < m; ++k)
    if (sym_group(pat, k) == sym_group(pat, m)) return false;
  return true;
}
__host__ __device__ constexpr unsigned sym_sign(int pat, int g) {
  return pat == 2 ? (g == 0 ? 0u : g == 1 ? 10u : g == 2 ? 12u : 6u)
                  : (g == 0 ? 0u : g == 1 ? 170u : g == 2 ? 240u : g == 3 ? 204u
                     : g == 4 ? 90u : g == 5 ? 60u : g == 6 ? 102u : 150u);
}

// Member f's sign in group g is (-1)^popcount(f & mask(g)): the groups are
// rows of the Hadamard matrix of order P, so the P signed sums of a class
// are one Walsh-Hadamard transform (log2 P butterfly levels of P additions)
__host__ __device__ constexpr int sym_mask(int pat, int g) {
  return pat == 2 ? g : (int)((0x73652410u >> (4 * g)) & 7u);  // 3-D: 0 1 4 2 5 6 3 7
}
constexpr bool sym_masks_match(int pat, int P) {
  for (int g = 0; g < P; ++g)
    for (int f = 0; f < P; ++f) {
      int par = 0;
      for (int b = f & sym_mask(pat, g); b; b >>= 1) par ^= b & 1;
      if ((int)((sym_sign(pat, g) >> f) & 1u) != par) return false;
    }
  return true;
}
static_assert(sym_masks_match(2, 4) && sym_masks_match(3, 8), "parity groups are Hadamard rows");
// compensated sums without renormalisation: a + b and a - b
__device__ __forceinline__ df64_acc acc_plus(df64_acc a, df64_acc b) {
  const float s = a.s + b.s;
  const float bb = s - a.s;
  return {s, (a.c + b.c) + ((a.s - (s - bb)) + (b.s - bb))};
}
__device__ __forceinline__ df64_acc acc_minus(df64_acc a, df64_acc b) {
  return acc_plus(a, df64_acc{-b.s, -b.c});
}
// in place: w[m] <- sum_f (-1)^popcount(f & m) w[f]
template <int P>
__device__ __forceinline__ void hadamard(df64_acc (&w)[P]) {
#pragma unroll
  for (int bit = 1; bit < P; bit <<= 1)
#pragma unroll
    for (int f = 0; f < P; ++f)
      if (!(f & bit)) {
        const df64_acc u = w[f], v = w[f | bit];
        w[f] = acc_plus(u, v);
        w[f | bit] = acc_minus(u, v);
      }
}

// q[d][e] for the P members d of each class: the class's products
// M2D_rep[m] T_m are summed per parity group once, then each member adds the
// group sums with its signs (+ iso)
template <int NM, int P, int PAT>
__global__ void __launch_bounds__(256) expand_sym_kernel(const df64* __restrict__ T, const df64* __restrict__ iso,
                                                         SymTables st, df64* __restrict__ q, int nm, long n_dofs, long len) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  df64* srep = reinterpret_cast<df64*>(smem_raw);
  int* sdir = reinterpret_cast<int*>(srep + st.n_class * nm);
  int* sgrp = sdir + st.n_class * P;
  unsigned* ssign = reinterpret_cast<unsigned*>(sgrp + 16);
  load_sym<P>(st, st.m2d_rep, nm, srep, sdir, sgrp, ssign);
  const int G = st.G;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < len; e += (long)gridDim.x * blockDim.x) {
    df64 t[NM];
#pragma unroll
    for (int m = 0; m < NM; ++m) t[m] = m < nm ? T[(size_t)m * n_dofs + e] : df64(0.f);
    const df64 is = iso ? iso[e] : df64(0.f);
    for (int c = 0; c < st.n_class; ++c) {
      df64_acc S[P];
#pragma unroll
      for (int g = 0; g < P; ++g) S[g] = acc_zero();
      const df64* rep = srep + c * nm;
#pragma unroll
      for (int m = 0; m < NM; ++m) {
        if (m >= nm) break;
        const df64 r = rep[m];
        if (PAT) {
          // a group's first moment starts its sum with the exact product
          // (the value a zero accumulator would give)
          if (sym_first_in_group(PAT, m)) S[sym_group(PAT, m)] = acc_prod(r, t[m]);
          else acc_fma(S[sym_group(PAT, m)], r, t[m]);
        } else {
          const int grp = sgrp[m];  // the same for every thread: uniform branches
#pragma unroll
          for (int g = 0; g < P; ++g)
            if (grp == g) acc_fma(S[g], r, t[m]);
        }
      }
      if constexpr (PAT != 0) {  // the members' signed sums by one Hadamard transform
        df64_acc w[P];
#pragma unroll
        for (int m = 0; m < P; ++m) w[m] = acc_zero();
#pragma unroll
        for (int g = 0; g < P; ++g)
          if (g < G) w[sym_mask(PAT, g)] = S[g];
        hadamard<P>(w);
#pragma unroll
        for (int f = 0; f < P; ++f) {
          if (iso) acc_add(w[f], is);
          q[(size_t)sdir[c * P + f] * n_dofs + e] = acc_result(w[f]);
        }
      } else {
        df64 sg[P];
#pragma unroll
        for (int g = 0; g < P; ++g) sg[g] = acc_result(S[g]);
#pragma unroll
        for (int f = 0; f < P; ++f) {
          df64_acc o = acc_from(is);
#pragma unroll
          for (int g = 0; g < P; ++g)
            if (g < G) acc_add(o, neg_if(sg[g], (ssign[g] >> f) & 1u));
          q[(size_t)sdir[c * P + f] * n_dofs + e] = acc_result(o);
        }
      }
    }
  }
}

// phi[m][e]: each class's P values of psi are combined into one signed sum
// per parity group, then every moment takes D2M_rep[m] times its group's sum
// With xc, the kernel writes out = xc - phi instead of phi (the Apply's
// y = x - phi, rounded once, as the combine kernel would).
template <int NM, int P, int PAT>
__global__ void __launch_bounds__(256) reduce_sym_kernel(const df64* __restrict__ psi, SymTables st,
                                                         double* __restrict__ phi, int nm, long n_dofs, long len,
                                                         const double* __restrict__ xc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  df64* srep = reinterpret_cast<df64*>(smem_raw);
  int* sdir = reinterpret_cast<int*>(srep + st.n_class * nm);
  int* sgrp = sdir + st.n_class * P;
  unsigned* ssign = reinterpret_cast<unsigned*>(sgrp + 16);
  load_sym<P>(st, st.d2m_rep, nm, srep, sdir, sgrp, ssign);
  const int G = st.G;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < len; e += (long)gridDim.x * blockDim.x) {
    df64_acc acc[NM];
#pragma unroll
    for (int m = 0; m < NM; ++m) acc[m] = acc_zero();
    // the next class's values are loaded while this class is combined (the
    // loads of one class no longer wait for the arithmetic of the one before)
    df64 pn[P];
#pragma unroll
    for (int f = 0; f < P; ++f) pn[f] = psi[(size_t)sdir[f] * n_dofs + e];
    for (int c = 0; c < st.n_class; ++c) {
      df64 ps[P];
#pragma unroll
      for (int f = 0; f < P; ++f) ps[f] = pn[f];
      if (c + 1 < st.n_class) {
#pragma unroll
        for (int f = 0; f < P; ++f) pn[f] = psi[(size_t)sdir[(c + 1) * P + f] * n_dofs + e];
      }
      df64 C[P];
      if constexpr (PAT != 0) {  // the P signed sums by one Hadamard transform
        df64_acc w[P];
#pragma unroll
        for (int f = 0; f < P; ++f) w[f] = acc_from(ps[f]);
        hadamard<P>(w);
        // (the sums feed compensated multiply-adds, which take any hi + lo
        // pair with a small low part: no renormalisation)
#pragma unroll
        for (int g = 0; g < P; ++g) C[g] = g < G ? df64(w[sym_mask(PAT, g)].s, w[sym_mask(PAT, g)].c) : df64(0.f);
      } else {
#pragma unroll
        for (int g = 0; g < P; ++g) {
          C[g] = df64(0.f);
          if (g < G) {
            const unsigned sg = ssign[g];
            df64_acc o = acc_from(neg_if(ps[0], sg & 1u));
#pragma unroll
            for (int f = 1; f < P; ++f) acc_add(o, neg_if(ps[f], (sg >> f) & 1u));
            C[g] = acc_result(o);
          }
        }
      }
      const df64* rep = srep + c * nm;
#pragma unroll
      for (int m = 0; m < NM; ++m) {
        if (m >= nm) break;
        df64 cg = C[0];
        if (PAT) {
          cg = C[sym_group(PAT, m)];
        } else {
          const int grp = sgrp[m];
#pragma unroll
          for (int g = 1; g < P; ++g)
            if (grp == g) cg = C[g];
        }
        acc_fma(acc[m], rep[m], cg);
      }
    }
#pragma unroll
    for (int m = 0; m < NM; ++m)
      if (m < nm) {
        const size_t i = (size_t)m * n_dofs + e;
        const double p = df64_to(acc_result(acc[m]));
        phi[i] = xc ? xc[i] - p : p;
      }
  }
}

template <int P, int PAT>
cudaError_t expand_sym_any(const df64* T, const df64* iso, const SymTables& st, df64* q, int nm, long n_dofs,
                           cudaStream_t s, long len) {
  const size_t sh = sizeof(df64) * st.n_class * nm + sizeof(int) * (st.n_class * P + 16) + sizeof(unsigned) * 8;
  if (nm <= 4)
    expand_sym_kernel<4, P, PAT><<<resident_grid(expand_sym_kernel<4, P, PAT>, len, sh), kBlock, sh, s>>>(T, iso, st, q, nm, n_dofs, len);
  else if (nm <= 10)
    expand_sym_kernel<10, P, PAT><<<resident_grid(expand_sym_kernel<10, P, PAT>, len, sh), kBlock, sh, s>>>(T, iso, st, q, nm, n_dofs, len);
  else
    expand_sym_kernel<16, P, PAT><<<resident_grid(expand_sym_kernel<16, P, PAT>, len, sh), kBlock, sh, s>>>(T, iso, st, q, nm, n_dofs, len);
  return cudaGetLastError();
}
template <int P, int PAT>
cudaError_t reduce_sym_any(const df64* psi, const SymTables& st, double* phi, int nm, long n_dofs, cudaStream_t s,
                           long len, const double* xc) {
  const size_t sh = sizeof(df64) * st.n_class * nm + sizeof(int) * (st.n_class * P + 16) + sizeof(unsigned) * 8;
  if (nm <= 1)
    reduce_sym_kernel<1, P, PAT><<<resident_grid(reduce_sym_kernel<1, P, PAT>, len, sh), kBlock, sh, s>>>(psi, st, phi, nm, n_dofs, len, xc);
  else if (nm <= 4)
    reduce_sym_kernel<4, P, PAT><<<resident_grid(reduce_sym_kernel<4, P, PAT>, len, sh), kBlock, sh, s>>>(psi, st, phi, nm, n_dofs, len, xc);
  else if (nm <= 10)
    reduce_sym_kernel<10, P, PAT><<<resident_grid(reduce_sym_kernel<10, P, PAT>, len, sh), kBlock, sh, s>>>(psi, st, phi, nm, n_dofs, len, xc);
  else
    reduce_sym_kernel<16, P, PAT><<<resident_grid(reduce_sym_kernel<16, P, PAT>, len, sh), kBlock, sh, s>>>(psi, st, phi, nm, n_dofs, len, xc);
  return cudaGetLastError();
}
}  // namespace

// the canonical pattern (2 or 3) the tables follow for their moments, else 0
int sym_canonical_pattern(int P, int nm, int G, const int* mom_group, const unsigned* sign) {
  const int pat = P == 4 ? 2 : P == 8 ? 3 : 0;
  if (!pat || nm > (pat == 2 ? 10 : 16)) return 0;
  for (int m = 0; m < nm; ++m)
    if (mom_group[m] != sym_group(pat, m)) return 0;
  for (int g = 0; g < G; ++g)
    if (sign[g] != sym_sign(pat, g)) return 0;
  return pat;
}

cudaError_t launch_expand_sym_pairs(const df64* T, const df64* iso, const SymTables& st, df64* q, int n_mom,
                                    long n_dofs, cudaStream_t s, long len) {
  if (n_mom > 16 || st.G > st.P) return cudaErrorInvalidValue;
  if (len < 0) len = n_dofs;
  if (st.P == 4) return st.pattern == 2 ? expand_sym_any<4, 2>(T, iso, st, q, n_mom, n_dofs, s, len)
                                        : expand_sym_any<4, 0>(T, iso, st, q, n_mom, n_dofs, s, len);
  if (st.P == 8) return st.pattern == 3 ? expand_sym_any<8, 3>(T, iso, st, q, n_mom, n_dofs, s, len)
                                        : expand_sym_any<8, 0>(T, iso, st, q, n_mom, n_dofs, s, len);
  return cudaErrorInvalidValue;
}
cudaError_t launch_reduce_sym_pairs(const df64* psi, const SymTables& st, double* phi, int n_mom, long n_dofs,
                                    cudaStream_t s, long len, const double* xc) {
  if (n_mom > 16 || st.G > st.P) return cudaErrorInvalidValue;
  if (len < 0) len = n_dofs;
  if (st.P == 4) return st.pattern == 2 ? reduce_sym_any<4, 2>(psi, st, phi, n_mom, n_dofs, s, len, xc)
                                        : reduce_sym_any<4, 0>(psi, st, phi, n_mom, n_dofs, s, len, xc);
  if (st.P == 8) return st.pattern == 3 ? reduce_sym_any<8, 3>(psi, st, phi, n_mom, n_dofs, s, len, xc)
                                        : reduce_sym_any<8, 0>(psi, st, phi, n_mom, n_dofs, s, len, xc);
  return cudaErrorInvalidValue;
}

cudaError_t launch_expand_source_df64(const double* T, const double* iso, const double* m2d,
                                      double* q, int n_dir, int n_mom, long n_dofs,
                                      cudaStream_t s, long len) {
  return expand_df64_any<double>(T, iso, m2d, q, n_dir, n_mom, n_dofs, s, len < 0 ? n_dofs : len);
}
cudaError_t launch_reduce_moments_df64(const double* psi, const double* d2m_t, double* phi,
                                       int n_dir, int n_mom, long n_dofs, cudaStream_t s, long len) {
  return reduce_df64_any<double>(psi, d2m_t, phi, n_dir, n_mom, n_dofs, s, len < 0 ? n_dofs : len);
}
cudaError_t launch_expand_source_pairs(const df64* T, const df64* iso, const double* m2d, df64* q,
                                       int n_dir, int n_mom, long n_dofs, cudaStream_t s, long len) {
  return expand_df64_any<df64>(T, iso, m2d, q, n_dir, n_mom, n_dofs, s, len < 0 ? n_dofs : len);
}
cudaError_t launch_reduce_moments_pairs(const df64* psi, const double* d2m_t, double* phi, int n_dir,
                                        int n_mom, long n_dofs, cudaStream_t s, long len) {
  return reduce_df64_any<df64>(psi, d2m_t, phi, n_dir, n_mom, n_dofs, s, len < 0 ? n_dofs : len);
}

template <typename real>
cudaError_t launch_expand_source(const real* T, const real* iso, const real* m2d, real* q,
                                 int n_dir, int n_mom, long n_dofs, cudaStream_t s, long len) {
  if (len < 0) len = n_dofs;
  // moments in chunks of at most 16 (Galerkin sets have n_mom = n_dir)
  for (int m0 = 0; m0 < n_mom; m0 += 16) {
    const int nm = n_mom - m0 < 16 ? n_mom - m0 : 16;
    const size_t sh = sizeof(real) * (size_t)n_dir * nm;
    const real* Tm = T + (size_t)m0 * n_dofs;
    const int acc = m0 > 0;
    const real* is = m0 == 0 ? iso : nullptr;
    if (nm <= 4)
      expand_kernel<real, 4><<<resident_grid(expand_kernel<real, 4>, len, sh), kBlock, sh, s>>>(Tm, is, m2d + m0, n_mom, q, n_dir, nm, n_dofs, len, acc);
    else if (nm <= 10)
      expand_kernel<real, 10><<<resident_grid(expand_kernel<real, 10>, len, sh), kBlock, sh, s>>>(Tm, is, m2d + m0, n_mom, q, n_dir, nm, n_dofs, len, acc);
    else
      expand_kernel<real, 16><<<resident_grid(expand_kernel<real, 16>, len, sh), kBlock, sh, s>>>(Tm, is, m2d + m0, n_mom, q, n_dir, nm, n_dofs, len, acc);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}
template cudaError_t launch_expand_source<double>(const double*, const double*, const double*,
                                                  double*, int, int, long, cudaStream_t, long);
template cudaError_t launch_expand_source<float>(const float*, const float*, const float*, float*,
                                                 int, int, long, cudaStream_t, long);

template <typename real>
cudaError_t launch_reduce_moments(const real* psi, const real* d2m_t, real* phi, int n_dir,
                                  int n_mom, long n_dofs, cudaStream_t s, long len) {
  if (len < 0) len = n_dofs;
  for (int m0 = 0; m0 < n_mom; m0 += 16) {
    const int nm = n_mom - m0 < 16 ? n_mom - m0 : 16;
    const size_t sh = sizeof(real) * (size_t)n_dir * nm;
    real* ph = phi + (size_t)m0 * n_dofs;
    if (nm <= 1)
      reduce_kernel<real, 1><<<resident_grid(reduce_kernel<real, 1>, len, sh), kBlock, sh, s>>>(psi, d2m_t + m0, n_mom, ph, n_dir, nm, n_dofs, len);
    else if (nm <= 4)
      reduce_kernel<real, 4><<<resident_grid(reduce_kernel<real, 4>, len, sh), kBlock, sh, s>>>(psi, d2m_t + m0, n_mom, ph, n_dir, nm, n_dofs, len);
    else if (nm <= 10)
      reduce_kernel<real, 10><<<resident_grid(reduce_kernel<real, 10>, len, sh), kBlock, sh, s>>>(psi, d2m_t + m0, n_mom, ph, n_dir, nm, n_dofs, len);
    else
      reduce_kernel<real, 16><<<resident_grid(reduce_kernel<real, 16>, len, sh), kBlock, sh, s>>>(psi, d2m_t + m0, n_mom, ph, n_dir, nm, n_dofs, len);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}
template cudaError_t launch_reduce_moments<double>(const double*, const double*, double*, int, int,
                                                   long, cudaStream_t, long);
template cudaError_t launch_reduce_moments<float>(const float*, const float*, float*, int, int,
                                                  long, cudaStream_t, long);

// Arithmetic of the per-cell scattering source: FP32 for the FP32 sweep,
// double-float for the FP64 sweep's pair storage
template <typename real>
struct SrcArith;
template <>
struct SrcArith<float> {
  using T = float;
  using Acc = float;
  __device__ static T from(double v) { return (float)v; }
  __device__ static Acc zero() { return 0.f; }
  __device__ static void fma(Acc& a, T u, T v) { a = __fmaf_rn(u, v, a); }
  __device__ static Acc prod(T u, T v) { return __fmul_rn(u, v); }
  __device__ static float out(Acc a, T sc) { return a * sc; }
};
template <>
struct SrcArith<df64> {
  using T = df64;
  using Acc = df64_acc;
  __device__ static T from(double v) { return df64_from(v); }
  __device__ static Acc zero() { return acc_zero(); }
  __device__ static void fma(Acc& a, T u, T v) { acc_fma(a, u, v); }
  __device__ static Acc prod(T u, T v) { return acc_prod(u, v); }
  __device__ static df64 out(Acc a, T sc) {
    df64_acc r = acc_zero();
    acc_fma(r, acc_result(a), sc);
    return acc_result(r);
  }
};

// The scattering source of one (moment, cell) per thread, without
// other-group terms: the cell's N values of x are converted once and the
// N x N mass-matrix products run on the FP32 pipes.  (One thread per output
// in FP64 spent N FP64 multiply-adds per value on GB300's 1/64-rate FP64
// pipe.)  Cells are the fastest index, so a warp reads and writes 32 * N
// consecutive values.
template <typename real, int N>
__global__ void __launch_bounds__(kBlock) scatter_cell_kernel(const double* __restrict__ x, real* __restrict__ src,
                                                              const double* __restrict__ M,
                                                              const double* __restrict__ sscale,
                                                              const int* __restrict__ material, long n_cells,
                                                              int n_mom, long n_dofs) {
  using A = SrcArith<real>;
  __shared__ typename A::T sM[N * N];
  for (int k = threadIdx.x; k < N * N; k += blockDim.x) sM[k] = A::from(M[k]);
  __syncthreads();
  const long total = (long)n_mom * n_cells;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const long c = t % n_cells;
    const int m = (int)(t / n_cells);
    const double* xc = x + (size_t)m * n_dofs + c * N;
    typename A::T xv[N];
#pragma unroll
    for (int j = 0; j < N; ++j) xv[j] = A::from(__ldg(xc + j));
    const typename A::T sc = A::from(__ldg(sscale + (size_t)material[c] * n_mom + m));
    real* out = src + (size_t)m * n_dofs + c * N;
#pragma unroll 1
    for (int i = 0; i < N; ++i) {
      typename A::Acc acc = A::prod(sM[i * N], xv[0]);
#pragma unroll
      for (int j = 1; j < N; ++j) A::fma(acc, sM[i * N + j], xv[j]);
      out[i] = A::out(acc, sc);
    }
  }
}

template <typename real, int N>
static cudaError_t scatter_cell(const double* x, real* src, const double* M, const double* sscale,
                                const int* material, long n_cells, int n_mom, long n_dofs, cudaStream_t s) {
  long g = ((long)n_mom * n_cells + kBlock - 1) / kBlock;
  if (g > 152L * 8) g = 152L * 8;  // each block converts the mass matrix once
  scatter_cell_kernel<real, N><<<(int)(g < 1 ? 1 : g), kBlock, 0, s>>>(x, src, M, sscale, material, n_cells, n_mom,
                                                                       n_dofs);
  return cudaGetLastError();
}
template <typename real>
static cudaError_t scatter_cell_any(const double* x, real* src, const double* M, const double* sscale,
                                    const int* material, long n_cells, int n, int n_mom, long n_dofs,
                                    cudaStream_t s, bool* done) {
  *done = true;
  switch (n) {
    case 4: return scatter_cell<real, 4>(x, src, M, sscale, material, n_cells, n_mom, n_dofs, s);
    case 8: return scatter_cell<real, 8>(x, src, M, sscale, material, n_cells, n_mom, n_dofs, s);
    case 9: return scatter_cell<real, 9>(x, src, M, sscale, material, n_cells, n_mom, n_dofs, s);
    case 16: return scatter_cell<real, 16>(x, src, M, sscale, material, n_cells, n_mom, n_dofs, s);
    case 25: return scatter_cell<real, 25>(x, src, M, sscale, material, n_cells, n_mom, n_dofs, s);
    case 27: return scatter_cell<real, 27>(x, src, M, sscale, material, n_cells, n_mom, n_dofs, s);
    default: *done = false; return cudaSuccess;
  }
}

template <typename real>
cudaError_t launch_scatter_source(const double* x, const double* gf, real* src,
                                  const double* M, const double* sscale, const double* oscale,
                                  const int* material, int n_mat, int n_groups, int group,
                                  long n_cells, int n, int n_mom, long n_dofs, cudaStream_t s) {
  (void)n_mat;
  if constexpr (!std::is_same<real, double>::value) {
    if (x && !gf) {  // the Apply's form: per-cell kernel on the FP32 pipes
      bool done = false;
      const cudaError_t e = scatter_cell_any<real>(x, src, M, sscale, material, n_cells, n, n_mom, n_dofs, s, &done);
      if (done) return e;
    }
  }
  scatter_source_kernel<real><<<grid_for((long)n_mom * n_cells * n), kBlock, 0, s>>>(
      x, gf, src, M, sscale, oscale, material, n_groups, group, n_cells, n, n_mom, n_dofs);
  return cudaGetLastError();
}
template cudaError_t launch_scatter_source<double>(const double*, const double*, double*,
                                                   const double*, const double*, const double*,
                                                   const int*, int, int, int, long, int, int,
                                                   long, cudaStream_t);
template cudaError_t launch_scatter_source<float>(const double*, const double*, float*,
                                                  const double*, const double*, const double*,
                                                  const int*, int, int, int, long, int, int, long,
                                                  cudaStream_t);
template cudaError_t launch_scatter_source<df64>(const double*, const double*, df64*, const double*,
                                                 const double*, const double*, const int*, int, int, int,
                                                 long, int, int, long, cudaStream_t);

template <typename real>
cudaError_t launch_iso_source(real* iso, const double* qcell, const double* rowsum,
                              const int* source_id, long n_cells, int n, cudaStream_t s) {
  iso_source_kernel<real><<<grid_for(n_cells * n), kBlock, 0, s>>>(iso, qcell, rowsum, source_id,
                                                                   n_cells, n);
  return cudaGetLastError();
}
template cudaError_t launch_iso_source<double>(double*, const double*, const double*, const int*,
                                               long, int, cudaStream_t);
template cudaError_t launch_iso_source<float>(float*, const double*, const double*, const int*,
                                              long, int, cudaStream_t);
template cudaError_t launch_iso_source<df64>(df64*, const double*, const double*, const int*, long, int,
                                             cudaStream_t);

template <typename real>
cudaError_t launch_combine(const double* x, const real* phi, double* y, long len, double sx,
                           double sp, cudaStream_t s) {
  combine_kernel<real><<<grid_for(len), kBlock, 0, s>>>(x, phi, y, len, sx, sp);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_combine_rows(const double* x, const real* phi, double* y, int rows, long len, long stride,
                                double sx, double sp, cudaStream_t s) {
  combine_rows_kernel<real><<<grid_for((long)rows * len), kBlock, 0, s>>>(x, phi, y, rows, len, stride, sx, sp);
  return cudaGetLastError();
}
template cudaError_t launch_combine_rows<double>(const double*, const double*, double*, int, long, long, double,
                                                 double, cudaStream_t);
template cudaError_t launch_combine_rows<float>(const double*, const float*, double*, int, long, long, double,
                                                double, cudaStream_t);
template cudaError_t launch_combine<double>(const double*, const double*, double*, long, double,
                                            double, cudaStream_t);
template cudaError_t launch_combine<float>(const double*, const float*, double*, long, double,
                                           double, cudaStream_t);

cudaError_t launch_permute(const double* in, double* out, const long* order, long n_cells, int n,
                           int n_vec, int to_internal, cudaStream_t s) {
  permute_kernel<<<grid_for((long)n_vec * n_cells * n), kBlock, 0, s>>>(in, out, order, n_cells,
                                                                        n, n_vec, to_internal);
  return cudaGetLastError();
}

cudaError_t launch_multi_axpy(const double* const* V, int k, const double* coef, double scale,
                              double* w, long len, cudaStream_t s) {
  if (k <= 8)
    multi_axpy_kernel<8><<<grid_for(len), kBlock, 0, s>>>(V, k, coef, scale, w, len);
  else if (k <= 32)
    multi_axpy_kernel<32><<<grid_for(len), kBlock, 0, s>>>(V, k, coef, scale, w, len);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

namespace {
// edge-word epochs cycle through [1, 0x7fff] (0 marks a never-written word)
__global__ void bump_epoch_kernel(unsigned* e) { *e = *e % 0x7fffu + 1u; }
// v *= 1/sqrt(*nrm2) (0 when the norm is 0)
__global__ void scale_inv_norm_kernel(const double* nrm2, double* v, long len) {
  const double n2 = *nrm2;
  const double sc = n2 > 0.0 ? 1.0 / sqrt(n2) : 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < len; i += (long)gridDim.x * blockDim.x)
    v[i] *= sc;
}
}  // namespace

namespace {
// One thread per (direction, cell): the cell's n values of psi^n are read
// once and q[d][c n + i] += sum_j (inv_vdt M)_ij psi^n_j is formed in
// double-float (FP64 storage) or FP32 -- no FP64 instruction, whose rate on
// GB300 is 1/64 of FP32.
template <typename real, int N>
__global__ void __launch_bounds__(256) angular_source_kernel(real* __restrict__ q, const float* __restrict__ psi,
                                                             const double* __restrict__ M, double inv_vdt,
                                                             long n_cells, int n_dir) {
  constexpr bool F32 = sizeof(real) == 4;
  __shared__ df64 sd[N * N];
  __shared__ float sf[N * N];
  for (int k = threadIdx.x; k < N * N; k += blockDim.x) {
    const double m = inv_vdt * M[k];
    sd[k] = df64_from(m);
    sf[k] = (float)m;
  }
  __syncthreads();
  const long total = (long)n_dir * n_cells;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const float* pc = psi + t * N;  // [dir][cell][N]: (direction, cell) t is contiguous
    float p[N];
    if constexpr (N % 4 == 0) {
#pragma unroll
      for (int k = 0; k < N / 4; ++k) {
        const float4 v = reinterpret_cast<const float4*>(pc)[k];
        p[4 * k] = v.x;
        p[4 * k + 1] = v.y;
        p[4 * k + 2] = v.z;
        p[4 * k + 3] = v.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < N; ++j) p[j] = pc[j];
    }
    real* qc = q + t * N;
#pragma unroll 1
    for (int i = 0; i < N; ++i) {
      if constexpr (F32) {
        float acc = (float)real_to_double(qc[i]);
#pragma unroll
        for (int j = 0; j < N; ++j) acc = __fmaf_rn(sf[i * N + j], p[j], acc);
        qc[i] = (real)acc;
      } else {
        df64_acc acc = acc_from(to_df64(qc[i]));
#pragma unroll
        for (int j = 0; j < N; ++j) acc_fma(acc, sd[i * N + j], df64(p[j]));
        qc[i] = store_df64<real>(acc_result(acc));
      }
    }
  }
}
}  // namespace

template <typename real>
cudaError_t launch_angular_source(real* q, const float* psi, const double* cell_mass, double inv_vdt,
                                  int n, long n_cells, int n_dir, cudaStream_t s) {
  const long total = (long)n_dir * n_cells;
  const int grid = grid_for(total);
  switch (n) {
#define CASE(NN)                                                                                             \
  case NN:                                                                                                   \
    angular_source_kernel<real, NN><<<grid, 256, 0, s>>>(q, psi, cell_mass, inv_vdt, n_cells, n_dir);         \
    break;
    CASE(4) CASE(8) CASE(9) CASE(16) CASE(25) CASE(27)
#undef CASE
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}
template cudaError_t launch_angular_source<double>(double*, const float*, const double*, double, int, long,
                                                   int, cudaStream_t);
template cudaError_t launch_angular_source<float>(float*, const float*, const double*, double, int, long,
                                                  int, cudaStream_t);
template cudaError_t launch_angular_source<df64>(df64*, const float*, const double*, double, int, long, int,
                                                 cudaStream_t);

namespace {
__global__ void to_f32_kernel(const double* in, float* out, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}
}  // namespace

namespace {
__global__ void pairs_to_f32_kernel(const df64* in, float* out, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = in[i].hi + in[i].lo;
}
}  // namespace

cudaError_t launch_to_f32_pairs(const df64* in, float* out, long n, cudaStream_t s) {
  pairs_to_f32_kernel<<<grid_for(n), kBlock, 0, s>>>(in, out, n);
  return cudaGetLastError();
}

cudaError_t launch_to_f32(const double* in, float* out, long n, cudaStream_t s) {
  to_f32_kernel<<<grid_for(n), kBlock, 0, s>>>(in, out, n);
  return cudaGetLastError();
}

cudaError_t launch_bump_epoch(unsigned* epoch, cudaStream_t s) {
  bump_epoch_kernel<<<1, 1, 0, s>>>(epoch);
  return cudaGetLastError();
}

cudaError_t launch_scale_inv_norm(const double* nrm2, double* v, long len, cudaStream_t s) {
  scale_inv_norm_kernel<<<grid_for(len), kBlock, 0, s>>>(nrm2, v, len);
  return cudaGetLastError();
}

cudaError_t launch_axpby(double a, const double* x, double b, double* y, long len,
                         cudaStream_t s) {
  axpby_kernel<<<grid_for(len), kBlock, 0, s>>>(a, x, b, y, len);
  return cudaGetLastError();
}

// xs: device array of k (<= 32) device pointers; out: k doubles; partial:
// k * kDotGrid doubles.  (`done` is not used by this two-launch form.)
cudaError_t launch_dots(const double* const* xs, const double* y, int k, long len, double* out,
                        double* partial, cudaStream_t s) {
  if (k < 1 || k > 32) return cudaErrorInvalidValue;
  dots_partial_kernel<<<kDotGrid, kBlock, 0, s>>>(xs, y, k, len, partial);
  dots_final_kernel<<<1, kBlock, 0, s>>>(partial, k, kDotGrid, out);
  return cudaGetLastError();
}

}  // namespace ouranos
