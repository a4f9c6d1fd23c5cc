// Diffusion synthetic acceleration (DSA) of the scalar flux for DG Q_p
// meshes, used as the right preconditioner of FGMRES and as the acceleration
// step of source iteration.
//
// The reference's Krylov solves run unpreconditioned (src/ouranos.cc:160-171),
// and its source iteration (src/ouranos.cc:72-95) is plain.  In optically
// thick, highly scattering cells both converge slowly: the slow error modes of
// the transport iteration are continuous scalar-flux fields that obey a
// diffusion equation.  For a residual v ([mom][dof]) the preconditioner is
//   P v = v + f,   (-div D grad + sigma_a) f = sigma_s0 v_0,
// f continuous trilinear (bilinear in 2-D) on the mesh vertices (for every
// DG order: the right-hand side takes the Q_p residual through the mixed
// mass matrix, the correction is f interpolated at the Q_p nodes), with the
// Marshak condition D df/dn + f/2 = 0 on vacuum and inflow boundaries and a
// zero current on reflective ones; D = 1 / (3 (sigma_t' - sigma_s1)),
// sigma_a = sigma_t' - sigma_s0, sigma_t' = sigma_t + 1/(v dt) in time steps.
// f is added to the scalar moment's nodal values of every cell (the DG Q_p
// space contains the continuous Q1 one), the higher moments pass unchanged.
// This is the continuous-finite-element DSA of the source-iteration error
// equation; as a right preconditioner of a Krylov method it stays effective at
// the material discontinuities where the same correction used inside plain
// source iteration can lose its efficiency.
//
// The diffusion system (one unknown per vertex, 27-point stencil in 3-D, its
// coefficients assembled once per table rebuild) is solved approximately by
// a fixed number of Jacobi-preconditioned conjugate-gradient steps, in FP32
// with FP64 scalars, all in one cooperative launch (the vertex vectors of a
// 64^3 mesh, 1.1 MB each, stay in L2) with two grid barriers per step:
//   matvec : w = C z, p = z + beta p, q = w + beta q, pq = p.q, alpha = rz/pq
//   update : x += alpha p, r -= alpha q, z = r / diag, rz' = r.z, beta = rz'/rz
// (q = C p is carried by recurrence, so the matrix is applied once per step).
// A caller may start the CG from a guess of f (the learned preconditioner's
// prediction): it is first scaled to its energy-norm-optimal multiple, one
// more grid barrier, so a poor guess can never start the CG farther from the
// solution than zero does.
// Every block sums the per-block partials of a dot product in block order, so
// all blocks hold the same, deterministic scalars.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "internal.h"

using namespace ouranos;

namespace {

constexpr int kThreads = 256;     // setup kernels
constexpr int kCgThreads = 1024;  // the CG kernel: one block per multiprocessor
constexpr int kMaxNodes = 27;     // DG Q_p nodes per cell the tables hold (3-D Q2, 2-D Q4: 25)

struct DsaGeom {
  int nx, ny, nz;      // cells per axis (nz = 1 in 2-D)
  int vx, vy, vz;      // vertices per axis (vz = 1 in 2-D)
  int nv;              // vertices (< 2^31)
  float ks[3];         // stiffness scale of axis a: (measure of the cell) / h_a^2
  float vol;           // measure of a cell
  float face[3];       // (measure of a face normal to axis a) / 2
  int robin;           // bit 2a+s: Marshak term on side s (0 low, 1 high) of axis a
  int off[27];         // index offset of stencil entry (dz*3 + dy)*3 + dx: vertex (I-1+dx, J-1+dy, K-1+dz)
};
// stencil entries of a vertex row: 27 in 3-D, 9 in 2-D (dz = 1)
template <int DIM>
constexpr int kStencil = DIM == 3 ? 27 : 9;

// 1-D Q1 factors between the basis functions of local corners u and w of a
// cell of unit length: mass (1/3 on, 1/6 off the diagonal) and stiffness
__device__ __forceinline__ float m1(int u, int w) { return u == w ? (1.f / 3.f) : (1.f / 6.f); }
__device__ __forceinline__ float s1(int u, int w) { return u == w ? 1.f : -1.f; }

// Row of the diffusion matrix at vertex (I, J, K) applied to the values
// nb[dz][dy][dx] of vertices (I-1+dx, J-1+dy, K-1+dz), 0 outside the mesh
// (2-D: only dz = 1 is read).  cell[c] = (D, sigma_a, sigma_s0, -).
template <int DIM>
__device__ __forceinline__ float row_apply(const DsaGeom& g, const float4* __restrict__ cell, int I, int J, int K,
                                           const float (&nb)[3][3][3]) {
  constexpr int NC = DIM == 3 ? 2 : 1;
  float acc = 0.f;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int kz = DIM == 3 ? K - 1 + c : 0;
    if (kz < 0 || kz >= g.nz) continue;
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const int ky = J - 1 + b;
      if (ky < 0 || ky >= g.ny) continue;
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const int kx = I - 1 + a;
        if (kx < 0 || kx >= g.nx) continue;
        const float4 cp = __ldg(cell + (kz * g.ny + ky) * g.nx + kx);
        float sm = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
        for (int c2 = 0; c2 < NC; ++c2)
#pragma unroll
          for (int b2 = 0; b2 < 2; ++b2)
#pragma unroll
            for (int a2 = 0; a2 < 2; ++a2) {
              const float val = nb[DIM == 3 ? c + c2 : 1][b + b2][a + a2];
              const float mx = m1(1 - a, a2), my = m1(1 - b, b2);
              const float mz = DIM == 3 ? m1(1 - c, c2) : 1.f;
              sm += mx * my * mz * val;
              sx += s1(1 - a, a2) * my * mz * val;
              sy += mx * s1(1 - b, b2) * mz * val;
              if (DIM == 3) sz += mx * my * s1(1 - c, c2) * val;
            }
        acc += cp.x * (g.ks[0] * sx + g.ks[1] * sy + (DIM == 3 ? g.ks[2] * sz : 0.f)) + cp.y * g.vol * sm;
      }
    }
  }
  // Marshak terms: (1/2) f w over the boundary faces through this vertex
  if (((I == 0 && (g.robin & 1)) || (I == g.vx - 1 && (g.robin & 2)))) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const int kz = DIM == 3 ? K - 1 + c : 0;
      if (kz < 0 || kz >= g.nz) continue;
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        const int ky = J - 1 + b;
        if (ky < 0 || ky >= g.ny) continue;
#pragma unroll
        for (int c2 = 0; c2 < NC; ++c2)
#pragma unroll
          for (int b2 = 0; b2 < 2; ++b2)
            acc += g.face[0] * m1(1 - b, b2) * (DIM == 3 ? m1(1 - c, c2) : 1.f) *
                   nb[DIM == 3 ? c + c2 : 1][b + b2][1];
      }
    }
  }
  if (((J == 0 && (g.robin & 4)) || (J == g.vy - 1 && (g.robin & 8)))) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const int kz = DIM == 3 ? K - 1 + c : 0;
      if (kz < 0 || kz >= g.nz) continue;
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const int kx = I - 1 + a;
        if (kx < 0 || kx >= g.nx) continue;
#pragma unroll
        for (int c2 = 0; c2 < NC; ++c2)
#pragma unroll
          for (int a2 = 0; a2 < 2; ++a2)
            acc += g.face[1] * m1(1 - a, a2) * (DIM == 3 ? m1(1 - c, c2) : 1.f) *
                   nb[DIM == 3 ? c + c2 : 1][1][a + a2];
      }
    }
  }
  if (DIM == 3 && ((K == 0 && (g.robin & 16)) || (K == g.vz - 1 && (g.robin & 32)))) {
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const int ky = J - 1 + b;
      if (ky < 0 || ky >= g.ny) continue;
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const int kx = I - 1 + a;
        if (kx < 0 || kx >= g.nx) continue;
#pragma unroll
        for (int b2 = 0; b2 < 2; ++b2)
#pragma unroll
          for (int a2 = 0; a2 < 2; ++a2)
            acc += g.face[2] * m1(1 - a, a2) * m1(1 - b, b2) * nb[1][b + b2][a + a2];
      }
    }
  }
  return acc;
}

__device__ __forceinline__ void vertex_ijk(const DsaGeom& g, int v, int& I, int& J, int& K) {
  const int t = v / g.vx;
  I = v - t * g.vx;
  K = t / g.vy;
  J = t - K * g.vy;
}

__device__ __forceinline__ void delta_nb(float (&nb)[3][3][3], int ex, int ey, int ez) {
#pragma unroll
  for (int dz = 0; dz < 3; ++dz)
#pragma unroll
    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
      for (int dx = 0; dx < 3; ++dx) nb[dz][dy][dx] = (dx == ex && dy == ey && dz == ez) ? 1.f : 0.f;
}

// Fixed-order sum over a block of kCgThreads; thread 0 returns the total.
__device__ __forceinline__ double block_sum(double t) {
  __shared__ double red[kCgThreads / 32];
  for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x < 32) {
    double u = red[threadIdx.x];
    for (int o = 16; o; o >>= 1) u += __shfl_xor_sync(0xffffffffu, u, o);
    t = u;
  }
  __syncthreads();
  return t;
}

// Sum of the nb per-block partials of a phase, in block order (every block
// of the problem gets the same value).
__device__ __forceinline__ double all_sum(const double* part, int nb) {
  __shared__ double total;
  double u = 0.0;
  for (int i = threadIdx.x; i < nb; i += kCgThreads) u += part[i];
  u = block_sum(u);
  if (threadIdx.x == 0) total = u;
  __syncthreads();
  return total;
}

struct DsaSync {
  unsigned count;  // blocks arrived at the current barrier
  unsigned gen;    // barriers completed
};
constexpr int kStatusBarrier = 2;  // status bit: a barrier wait gave up

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier of a cooperative launch (all blocks co-resident).
// Thread 0 of each block arrives with a release (after the block's bar.sync)
// and leaves with an acquire, so every write of any block before the barrier
// is visible to every thread after it.  The wait is bounded by limit_ns: a
// block that gives up sets the status bit and returns false, and blocks still
// waiting elsewhere see the bit and give up too.  bias (a test hook) makes the
// generation the waiters wait for one that never comes.  (Per-block epoch
// words polled by every block, in place of the shared counter, measured
// slower: 34.8 against 21.5 us per CG step at 152 blocks.)
__device__ __forceinline__ bool grid_barrier(DsaSync* s, int* status, long long limit_ns, unsigned bias = 0) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    const unsigned g = ld_acquire(&s->gen);
    if (atom_add_acq_rel(&s->count, 1u) == gridDim.x - 1 && !bias) {
      s->count = 0u;  // ordered before the release below; nobody arrives until it
      atom_add_acq_rel(&s->gen, 1u);
    } else {
      const unsigned long long t0 = global_ns();
      unsigned polls = 0;
      while (ld_acquire(&s->gen) == g) {
        if ((++polls & 255u) == 0 &&
            ((long long)(global_ns() - t0) > limit_ns || (*(volatile int*)status & kStatusBarrier))) {
          atomicOr(status, kStatusBarrier);
          ok = 0;
          break;
        }
      }
    }
  }
  __syncthreads();
  return ok != 0;
}

// The matrix row of every vertex as stencil coefficients coef[s][vertex]
// (entries that reach outside the mesh are 0), and 1 / diagonal.
template <int DIM>
__global__ void __launch_bounds__(kThreads) dsa_stencil_kernel(DsaGeom g, const float4* __restrict__ cell,
                                                               float* __restrict__ coef, float* __restrict__ dinv) {
  const int v = blockIdx.x * kThreads + threadIdx.x;
  if (v >= g.nv) return;
  int I, J, K;
  vertex_ijk(g, v, I, J, K);
  for (int s = 0; s < kStencil<DIM>; ++s) {
    const int dx = s % 3, dy = (s / 3) % 3, dz = DIM == 3 ? s / 9 : 1;
    float nb[3][3][3];
    delta_nb(nb, dx, dy, dz);
    const float c = row_apply<DIM>(g, cell, I, J, K, nb);
    if (dx == 1 && dy == 1 && dz == 1) dinv[v] = c > 0.f ? 1.f / c : 0.f;
    coef[(long)s * g.nv + v] = c;
  }
}

// assembled sigma_s0 M v_0 at vertex (I, J, K): for each cell around the
// vertex, the cell's nodal values times the row of the mixed mass matrix
// (vertex hat function x the cell's DG Q_p basis, cell measure folded in) of
// the corner the vertex is for that cell
template <int DIM>
__device__ __forceinline__ float assemble_rhs(const DsaGeom& g, const float4* __restrict__ cell,
                                              const double* __restrict__ v, int I, int J, int K,
                                              const float* __restrict__ smix, int n) {
  constexpr int NC = DIM == 3 ? 2 : 1;
  float acc = 0.f;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int kz = DIM == 3 ? K - 1 + c : 0;
    if (kz < 0 || kz >= g.nz) continue;
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const int ky = J - 1 + b;
      if (ky < 0 || ky >= g.ny) continue;
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const int kx = I - 1 + a;
        if (kx < 0 || kx >= g.nx) continue;
        const int cid = (kz * g.ny + ky) * g.nx + kx;
        const double* vc = v + (long)cid * n;
        const float* row = smix + ((1 - a) + 2 * (1 - b) + (DIM == 3 ? 4 * (1 - c) : 0)) * n;
        float sm = 0.f;
        for (int j = 0; j < n; ++j) sm += row[j] * (float)vc[j];
        acc += __ldg(&cell[cid].z) * sm;
      }
    }
  }
  return acc;
}

// The whole preconditioner of one problem: assemble the right-hand side,
// `iters` Jacobi-CG steps, and out = v + f on the scalar moment's nodes, run
// by the nb blocks lb = 0..nb-1 of a cooperative launch (the whole grid for
// one problem, a slice of it in a batch).  Each thread owns the same vertices
// (stride over the problem's blocks) in every phase, so its own x, r, p, q
// need no synchronisation; z of the neighbours and the partials cross
// blocks, and the barrier's release/acquire fences order them (plain loads
// after it see every write made before it).  Every block of the grid passes
// the same 2 iters grid barriers.  Dot products: FP32 per thread, FP64 from
// the block sums on; part_a/part_b hold the problem's nb partials.
template <int DIM>
__device__ __forceinline__ void cg_body(const DsaGeom& g, const float4* __restrict__ cell,
                                        const float* __restrict__ coef, const double* v, double* out, long len,
                                        long n0, const float* __restrict__ dinv, float* x, float* r, float* z,
                                        float* p, float* q, double* part_a, double* part_b, int lb, int nb,
                                        DsaSync* sync, int* status, long long limit_ns, int iters,
                                        const float* __restrict__ fe, int n, const float* __restrict__ x0,
                                        double* part_c, unsigned wait_bias) {
  constexpr int NCORNER = DIM == 3 ? 8 : 4;
  // the cell tables: mixed mass [corner][n] (measure folded in), then the
  // interpolation of the vertex values at the nodes [n][corner]
  __shared__ float smix[NCORNER * kMaxNodes], sipl[kMaxNodes * NCORNER];
  for (int k = threadIdx.x; k < NCORNER * n; k += kCgThreads) {
    smix[k] = fe[k];
    sipl[k] = fe[NCORNER * n + k];
  }
  __syncthreads();
  const int stride = nb * kCgThreads;
  const int first = lb * kCgThreads + threadIdx.x;
  // x = 0, r = rhs without a guess.  With a guess g (x0, written before the
  // launch with a zero halo like z, so every block reads its neighbours'
  // values without a barrier) the start is the multiple of g closest to the
  // solution in the energy norm, x = a g with a = (g, rhs) / (g, C g) (a
  // Galerkin step on span{g}: never farther from the solution than x = 0,
  // whatever the guess), and r = rhs - a C g (C g kept in q meanwhile).
  float t = 0.f;
  float a0 = 0.f;
  if (x0) {
    float t1 = 0.f, t2 = 0.f;
    for (int vid = first; vid < g.nv; vid += stride) {
      int I, J, K;
      vertex_ijk(g, vid, I, J, K);
      const float rr = assemble_rhs<DIM>(g, cell, v, I, J, K, smix, n);
      float w = 0.f;
#pragma unroll
      for (int s = 0; s < kStencil<DIM>; ++s) w += coef[(long)s * g.nv + vid] * x0[vid + g.off[s]];
      r[vid] = rr;
      q[vid] = w;
      t1 += x0[vid] * rr;
      t2 += x0[vid] * w;
    }
    // part_c is written here only, so no later phase overwrites it while a
    // slower block still reads it; part_a is next written after a barrier
    const double b1 = block_sum(t1), b2 = block_sum(t2);
    if (threadIdx.x == 0) {
      part_a[lb] = b1;
      part_c[lb] = b2;
    }
    if (!grid_barrier(sync, status, limit_ns, wait_bias)) return;
    const double gb = all_sum(part_a, nb), gcg = all_sum(part_c, nb);
    a0 = gcg > 0.0 ? (float)(gb / gcg) : 0.f;
  }
  for (int vid = first; vid < g.nv; vid += stride) {
    float rr, xx = 0.f;
    if (x0) {
      xx = a0 * x0[vid];
      rr = r[vid] - a0 * q[vid];
    } else {
      int I, J, K;
      vertex_ijk(g, vid, I, J, K);
      rr = assemble_rhs<DIM>(g, cell, v, I, J, K, smix, n);
    }
    const float zz = rr * dinv[vid];
    r[vid] = rr;
    z[vid] = zz;
    x[vid] = xx;
    t += rr * zz;
  }
  double bt = block_sum(t);
  if (threadIdx.x == 0) part_b[lb] = bt;
  if (!grid_barrier(sync, status, limit_ns, wait_bias)) return;
  double rz = all_sum(part_b, nb), beta = 0.0, alpha = 0.0;
  for (int it = 0; it < iters; ++it) {
    // w = C z; p = z + beta p; q = w + beta q
    const float fb = (float)beta;
    t = 0.f;
    for (int vid = first; vid < g.nv; vid += stride) {
      // z has a zero halo: every stencil offset stays inside the buffer, and
      // entries that wrap to another row have coefficient 0
      float w = 0.f;
#pragma unroll
      for (int s = 0; s < kStencil<DIM>; ++s) w += coef[(long)s * g.nv + vid] * z[vid + g.off[s]];
      const float zz = z[vid];
      const float pn = it ? zz + fb * p[vid] : zz;
      const float qn = it ? w + fb * q[vid] : w;
      p[vid] = pn;
      q[vid] = qn;
      t += pn * qn;
    }
    bt = block_sum(t);
    if (threadIdx.x == 0) part_a[lb] = bt;
    if (!grid_barrier(sync, status, limit_ns, wait_bias)) return;
    const double pq = all_sum(part_a, nb);
    alpha = pq > 0.0 ? rz / pq : 0.0;
    if (it == iters - 1) break;  // the last update folds into the output
    // x += alpha p; r -= alpha q; z = r / diag
    const float fa = (float)alpha;
    t = 0.f;
    for (int vid = first; vid < g.nv; vid += stride) {
      x[vid] += fa * p[vid];
      const float rn = r[vid] - fa * q[vid];
      const float zn = rn * dinv[vid];
      r[vid] = rn;
      z[vid] = zn;
      t += rn * zn;
    }
    bt = block_sum(t);
    if (threadIdx.x == 0) part_b[lb] = bt;
    if (!grid_barrier(sync, status, limit_ns, wait_bias)) return;
    const double rzn = all_sum(part_b, nb);
    beta = rz > 0.0 ? rzn / rz : 0.0;
    rz = rzn;
  }
  // out = v + f, f = x + alpha p interpolated from the cell's corner vertices
  // at each scalar-moment node (Q1: the node is the vertex); x and p of other
  // blocks' vertices are complete at the last barrier
  const float fa = (float)alpha;
  for (long e = first; e < len; e += stride) {
    double val = v[e];
    if (e < n0) {
      const long cid = e / n;
      const int k = (int)(e % n);
      const int kx = (int)(cid % g.nx);
      const long tt = cid / g.nx;
      const int ky = (int)(tt % g.ny), kz = (int)(tt / g.ny);
      const long v0 = ((long)kz * g.vy + ky) * g.vx + kx;  // the cell's corner (0, 0, 0)
      float f = 0.f;
      if (n == NCORNER) {
        const long vid = v0 + (DIM == 3 ? (long)(k >> 2) * g.vy * g.vx : 0) + ((k >> 1) & 1) * g.vx + (k & 1);
        f = x[vid] + fa * p[vid];
      } else {
#pragma unroll
        for (int cr = 0; cr < NCORNER; ++cr) {
          const long vid = v0 + (DIM == 3 ? (long)(cr >> 2) * g.vy * g.vx : 0) + ((cr >> 1) & 1) * g.vx + (cr & 1);
          f += sipl[k * NCORNER + cr] * (x[vid] + fa * p[vid]);
        }
      }
      val += (double)f;
    }
    out[e] = val;
  }
}

template <int DIM>
__global__ void __launch_bounds__(kCgThreads, 1) dsa_cg_kernel(DsaGeom g, const float4* __restrict__ cell,
                                                          const float* __restrict__ coef, const double* v,
                                                          double* out, long len, long n0,
                                                          const float* __restrict__ dinv, float* x, float* r,
                                                          float* z, float* p, float* q, double* part_a,
                                                          double* part_b, DsaSync* sync, int* status,
                                                          long long limit_ns, int iters,
                                                          const float* __restrict__ fe, int n,
                                                          const float* __restrict__ x0, double* part_c,
                                                          unsigned wait_bias) {
  cg_body<DIM>(g, cell, coef, v, out, len, n0, dinv, x, r, z, p, q, part_a, part_b, (int)blockIdx.x,
               (int)gridDim.x, sync, status, limit_ns, iters, fe, n, x0, part_c, wait_bias);
}

// One problem of a batched diffusion solve: its tables, vectors and the
// blocks [block0, block0 + nblk) of the batched grid
struct DsaProb {
  DsaGeom g;
  const float4* cell;
  const float* coef;
  const float* dinv;
  float *x, *r, *z, *p, *q;
  const float* fe;
  const double* v;
  double* out;
  long len, n0;
  int n, block0, nblk;
};

// Every problem of a batch in one cooperative launch: block b works on
// problem block_prob[b]; all problems run the same number of CG steps, so
// all blocks meet at the same grid barriers.  part_a/part_b: one partial per
// block of the grid, each problem using its slice.
template <int DIM>
__global__ void __launch_bounds__(kCgThreads, 1) dsa_cg_batch_kernel(const DsaProb* __restrict__ probs,
                                                                const int* __restrict__ block_prob,
                                                                double* part_a, double* part_b, DsaSync* sync,
                                                                int* status, long long limit_ns, int iters) {
  __shared__ DsaProb P;
  if (threadIdx.x == 0) P = probs[block_prob[blockIdx.x]];
  __syncthreads();
  const int lb = (int)blockIdx.x - P.block0;
  cg_body<DIM>(P.g, P.cell, P.coef, P.v, P.out, P.len, P.n0, P.dinv, P.x, P.r, P.z, P.p, P.q,
               part_a + P.block0, part_b + P.block0, lb, P.nblk, sync, status, limit_ns, iters, P.fe, P.n,
               nullptr, nullptr, 0u);
}

int dfail(ouranos_rt* rt, cudaError_t e, const char* what) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "diffusion acceleration, %s: %s", what, cudaGetErrorString(e));
  rt->err = buf;
  return OURANOS_ERR_CUDA;
}
#define DC(expr, what)                                  \
  do {                                                  \
    cudaError_t _e = (expr);                            \
    if (_e != cudaSuccess) return dfail(rt, _e, what);  \
  } while (0)

DsaGeom geom(const ouranos_rt* rt) {
  DsaGeom g{};
  g.nx = rt->nx[0];
  g.ny = rt->nx[1];
  g.nz = rt->dim == 3 ? rt->nx[2] : 1;
  g.vx = g.nx + 1;
  g.vy = g.ny + 1;
  g.vz = rt->dim == 3 ? g.nz + 1 : 1;
  g.nv = (int)((long)g.vx * g.vy * g.vz);
  const double hx = rt->h[0], hy = rt->h[1], hz = rt->dim == 3 ? rt->h[2] : 1.0;
  const double vol = hx * hy * hz;
  g.vol = (float)vol;
  g.ks[0] = (float)(vol / (hx * hx));
  g.ks[1] = (float)(vol / (hy * hy));
  g.ks[2] = (float)(rt->dim == 3 ? vol / (hz * hz) : 0.0);
  g.face[0] = (float)(0.5 * vol / hx);
  g.face[1] = (float)(0.5 * vol / hy);
  g.face[2] = (float)(rt->dim == 3 ? 0.5 * vol / hz : 0.0);
  g.robin = 0;
  for (int f = 0; f < 2 * rt->dim; ++f)
    if (rt->bc[f] != OURANOS_BC_REFLECTIVE) g.robin |= 1 << f;
  for (int s = 0; s < 27; ++s) {
    const int dx = s % 3 - 1, dy = (s / 3) % 3 - 1, dz = rt->dim == 3 ? s / 9 - 1 : 0;
    g.off[s] = (dz * g.vy + dy) * g.vx + dx;
  }
  return g;
}

// zero halo on each side of the z vector: the largest stencil offset
long halo(const DsaGeom& g) { return (long)g.vx * g.vy + g.vx + 1; }

inline int nblocks(long n) { return (int)((n + kThreads - 1) / kThreads); }

// per-cell coefficients and the Jacobi diagonal, rebuilt when the group or
// the time step changes
// Gauss-Legendre rule with m points on [0, 1] (Newton on P_m from the
// Chebyshev-like initial guesses)
void gauss01(int m, std::vector<double>& x, std::vector<double>& w) {
  x.assign(m, 0.0);
  w.assign(m, 0.0);
  for (int i = 0; i < m; ++i) {
    double t = std::cos(3.14159265358979323846 * (i + 0.75) / (m + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = t;
      for (int k = 2; k <= m; ++k) {
        const double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = m * (t * p1 - p0) / (t * t - 1.0);
      const double dt = p1 / dp;
      t -= dt;
      if (std::fabs(dt) < 1e-16) break;
    }
    x[i] = 0.5 * (1.0 - t);
    w[i] = 1.0 / ((1.0 - t * t) * dp * dp);  // (2 / ((1-t^2) P'^2)) / 2
  }
}

// The cell tables for DG Q_p nodes on the equidistant points j/p: the mixed
// mass matrix of the vertex hat functions against the Q_p basis, [corner][n]
// with the cell measure folded in, then the values of the hat functions at
// the nodes, [n][corner].  Both are tensor products of 1-D factors.  Q1: the
// Q1 mass matrix and the identity.
std::vector<float> fe_tables(const ouranos_rt* rt, double vol) {
  const int p = rt->p, p1 = p + 1, dim = rt->dim, nc = 1 << dim, n = rt->n;
  std::vector<double> gx, gw;
  gauss01(p + 2, gx, gw);
  auto lag = [&](int k, double x) {
    double v = 1.0;
    for (int j = 0; j <= p; ++j)
      if (j != k) v *= (x - (double)j / p) / ((double)(k - j) / p);
    return v;
  };
  auto hat = [](int a, double x) { return a ? x : 1.0 - x; };
  std::vector<double> m1(2 * p1), i1(p1 * 2);
  for (int a = 0; a < 2; ++a)
    for (int k = 0; k < p1; ++k) {
      double s = 0.0;
      for (size_t q = 0; q < gx.size(); ++q) s += gw[q] * hat(a, gx[q]) * lag(k, gx[q]);
      m1[a * p1 + k] = s;
      i1[k * 2 + a] = hat(a, (double)k / p);
    }
  std::vector<float> out(2 * (size_t)nc * n);
  for (int cr = 0; cr < nc; ++cr)
    for (int j = 0; j < n; ++j) {
      double mm = vol, ip = 1.0;
      for (int ax = 0; ax < dim; ++ax) {
        const int bit = (cr >> ax) & 1;
        const int comp = ax == 0 ? j % p1 : (ax == 1 ? (j / p1) % p1 : j / (p1 * p1));
        mm *= m1[bit * p1 + comp];
        ip *= i1[comp * 2 + bit];
      }
      out[(size_t)cr * n + j] = (float)mm;
      out[(size_t)nc * n + (size_t)j * nc + cr] = (float)ip;
    }
  return out;
}

int ensure_tables(ouranos_rt* rt) {
  if (rt->n > kMaxNodes) {
    rt->err = "diffusion acceleration: cells of at most 27 dofs";
    return OURANOS_ERR_UNSUPPORTED;
  }
  if ((long)(rt->nx[0] + 1) * (rt->nx[1] + 1) * (rt->dim == 3 ? rt->nx[2] + 1 : 1) >= (1L << 31)) {
    rt->err = "diffusion acceleration: at most 2^31 - 1 mesh vertices";
    return OURANOS_ERR_UNSUPPORTED;
  }
  if (rt->dsa_group == rt->group && rt->dsa_inv_vdt == rt->inv_vdt && rt->d_dsa_cell.p) return OURANOS_OK;
  const DsaGeom g = geom(rt);
  std::vector<float4> cell(rt->n_cells);
  const int G = rt->G, L = rt->l_max;
  for (long c = 0; c < rt->n_cells; ++c) {
    const int m = rt->material_id[c];
    const double st = rt->sigma_t[(size_t)m * G + rt->group] + rt->inv_vdt;
    const size_t base = (size_t)rt->group * (L + 1) + (size_t)rt->group * G * (L + 1) + (size_t)m * G * G * (L + 1);
    const double s0 = rt->sigma_s[base];
    const double s1v = L >= 1 ? rt->sigma_s[base + 1] : 0.0;
    double tr = st - s1v;
    if (!(tr > 1e-8)) tr = st > 1e-8 ? st : 1e-8;  // void cells: keep D finite
    const double sa = st - s0;
    cell[c] = make_float4((float)(1.0 / (3.0 * tr)), (float)(sa > 0.0 ? sa : 0.0), (float)s0, 0.f);
  }
  const long nv = g.nv;
  const int nb = nblocks(nv);
  DC(rt->d_dsa_cell.alloc(sizeof(float4) * rt->n_cells), "tables");
  const int ns = rt->dim == 3 ? kStencil<3> : kStencil<2>;
  // x, r, p, q, 1/diag, z and the initial guess x0, the last two with zero halos
  DC(rt->d_dsa_vec.alloc(sizeof(float) * (7 * nv + 4 * halo(g))), "vectors");
  DC(rt->d_dsa_coef.alloc(sizeof(float) * ns * nv), "stencil");
  DC(cudaMemsetAsync(rt->d_dsa_vec.p, 0, sizeof(float) * (7 * nv + 4 * halo(g)), rt->stream), "vectors");
  // partials of the two phases (one per block of the cooperative grid) and the barrier
  int per_sm = 0, sms = 0;
  DC(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, rt->device), "device");
  DC(rt->dim == 3 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dsa_cg_kernel<3>, kCgThreads, 0)
                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dsa_cg_kernel<2>, kCgThreads, 0),
     "occupancy");
  if (per_sm < 1) {
    rt->err = "diffusion acceleration: the CG kernel does not fit on a multiprocessor";
    return OURANOS_ERR_CUDA;
  }
  // one block per multiprocessor keeps the grid barrier to a few participants
  rt->dsa_grid = (int)std::min<long>(sms, (nv + kCgThreads - 1) / kCgThreads);
  // partials a, b, the barrier words, partials c (the guess's second sum)
  DC(rt->d_dsa_red.alloc(sizeof(double) * (3 * rt->dsa_grid + 2)), "reductions");
  DC(cudaMemcpyAsync(rt->d_dsa_cell.p, cell.data(), sizeof(float4) * rt->n_cells, cudaMemcpyHostToDevice,
                     rt->stream),
     "tables");
  const std::vector<float> fe = fe_tables(rt, (double)g.vol);
  DC(rt->d_dsa_fe.alloc(sizeof(float) * fe.size()), "tables");
  DC(cudaMemcpyAsync(rt->d_dsa_fe.p, fe.data(), sizeof(float) * fe.size(), cudaMemcpyHostToDevice, rt->stream),
     "tables");
  DC(cudaMemsetAsync(rt->d_dsa_red.as<double>() + 2 * rt->dsa_grid, 0, sizeof(DsaSync), rt->stream),
     "barrier");
  float* dinv = rt->d_dsa_vec.as<float>() + 4 * nv;
  if (rt->dim == 3)
    dsa_stencil_kernel<3><<<nb, kThreads, 0, rt->stream>>>(g, rt->d_dsa_cell.as<float4>(),
                                                           rt->d_dsa_coef.as<float>(), dinv);
  else
    dsa_stencil_kernel<2><<<nb, kThreads, 0, rt->stream>>>(g, rt->d_dsa_cell.as<float4>(),
                                                           rt->d_dsa_coef.as<float>(), dinv);
  DC(cudaGetLastError(), "stencil");
  DC(cudaStreamSynchronize(rt->stream), "tables");
  rt->dsa_group = rt->group;
  rt->dsa_inv_vdt = rt->inv_vdt;
  return OURANOS_OK;
}

template <int DIM>
int dsa_run(ouranos_rt* rt, const double* v, double* out, int iters, bool guess) {
  DsaGeom g = geom(rt);
  const long nv = g.nv;
  // x, r, p, q, 1/diag, then z with its halo
  float* base = rt->d_dsa_vec.as<float>();
  float *x = base, *r = base + nv, *p = base + 2 * nv, *q = base + 3 * nv;
  const float* dinv = base + 4 * nv;
  float* z = base + 5 * nv + halo(g);
  const float* x0 = guess ? base + 6 * nv + 3 * halo(g) : nullptr;
  const float* coef = rt->d_dsa_coef.as<float>();
  double* part_a = rt->d_dsa_red.as<double>();
  double* part_b = part_a + rt->dsa_grid;
  DsaSync* sync = reinterpret_cast<DsaSync*>(part_b + rt->dsa_grid);
  double* part_c = part_b + rt->dsa_grid + 2;
  int* status = rt->d_ctrl.as<int>() + 1;
  const float4* cell = rt->d_dsa_cell.as<float4>();
  long len = (long)rt->n_mom * rt->n_dofs, n0 = rt->n_cells * (long)rt->n;
  // a barrier that gave up in an earlier call leaves its counters behind
  DC(cudaMemsetAsync(sync, 0, sizeof(DsaSync), rt->stream), "barrier");
  long long limit = rt->wait_limit_ns;
  const float* fe = rt->d_dsa_fe.as<float>();
  int n = rt->n;
  unsigned bias = rt->wait_bias ? 1u : 0u;  // the test hook of ouranos_rt_debug_wait_bias
  void* args[] = {&g, &cell, &coef, &v, &out, &len, &n0, &dinv, &x, &r, &z, &p, &q, &part_a, &part_b, &sync, &status,
                  &limit, &iters, &fe, &n, &x0, &part_c, &bias};
  DC(cudaLaunchCooperativeKernel((const void*)dsa_cg_kernel<DIM>, dim3(rt->dsa_grid), dim3(kCgThreads), args, 0,
                                 rt->stream),
     "solve");
  return OURANOS_OK;
}

// One batched launch of the problems idx[0..count) (same mesh dimension DIM,
// count <= the cooperative grid's capacity).  Blocks go to the problems by
// their vertex counts: every problem gets one, then each further block goes to
// the problem with the most vertices per block, up to one vertex per thread.
template <int DIM>
int dsa_batch_launch(ouranos_rt* const* rts, const double* const* v, double* const* out, const int* idx, int count,
                     cudaStream_t stream, int* status, DsaBatchScratch& sc, int grid_cap, std::string& err) {
  std::vector<int> nblk(count, 1);
  std::vector<long> nv(count);
  for (int i = 0; i < count; ++i) nv[i] = geom(rts[idx[i]]).nv;
  int total = count;
  while (total < grid_cap) {
    int best = -1;
    double work = 0.0;
    for (int i = 0; i < count; ++i) {
      const double w = (double)nv[i] / nblk[i];
      if (nblk[i] * (long)kCgThreads < nv[i] && w > work) {
        work = w;
        best = i;
      }
    }
    if (best < 0) break;
    ++nblk[best];
    ++total;
  }
  const size_t probs_bytes = (sizeof(DsaProb) * count + 15) / 16 * 16;
  const size_t map_bytes = (sizeof(int) * total + 15) / 16 * 16;
  const size_t host_bytes = probs_bytes + map_bytes;
  const size_t dev_bytes = host_bytes + sizeof(double) * 2 * total + sizeof(DsaSync);
  if (sc.dev.alloc(dev_bytes) != cudaSuccess) {
    err = "diffusion acceleration: batch scratch allocation failed";
    return OURANOS_ERR_CUDA;
  }
  if (sc.host_bytes < host_bytes) {
    if (sc.host) cudaFreeHost(sc.host);
    sc.host = nullptr;
    sc.host_bytes = 0;
    if (cudaMallocHost(&sc.host, host_bytes) != cudaSuccess) {
      err = "diffusion acceleration: batch staging allocation failed";
      return OURANOS_ERR_CUDA;
    }
    sc.host_bytes = host_bytes;
  }
  DsaProb* hp = reinterpret_cast<DsaProb*>(sc.host);
  int* hmap = reinterpret_cast<int*>(static_cast<char*>(sc.host) + probs_bytes);
  int b0 = 0;
  for (int i = 0; i < count; ++i) {
    ouranos_rt* rt = rts[idx[i]];
    DsaProb& P = hp[i];
    P.g = geom(rt);
    const long n = P.g.nv;
    float* base = rt->d_dsa_vec.as<float>();
    P.x = base;
    P.r = base + n;
    P.p = base + 2 * n;
    P.q = base + 3 * n;
    P.dinv = base + 4 * n;
    P.z = base + 5 * n + halo(P.g);
    P.cell = rt->d_dsa_cell.as<float4>();
    P.coef = rt->d_dsa_coef.as<float>();
    P.fe = rt->d_dsa_fe.as<float>();
    P.v = v[idx[i]];
    P.out = out[idx[i]];
    P.len = (long)rt->n_mom * rt->n_dofs;
    P.n0 = rt->n_cells * (long)rt->n;
    P.n = rt->n;
    P.block0 = b0;
    P.nblk = nblk[i];
    for (int k = 0; k < nblk[i]; ++k) hmap[b0 + k] = i;
    b0 += nblk[i];
  }
  char* dbase = sc.dev.as<char>();
  const DsaProb* dprobs = reinterpret_cast<const DsaProb*>(dbase);
  const int* dmap = reinterpret_cast<const int*>(dbase + probs_bytes);
  double* part_a = reinterpret_cast<double*>(dbase + host_bytes);
  double* part_b = part_a + total;
  DsaSync* sync = reinterpret_cast<DsaSync*>(part_b + total);
  // the staging block is rewritten by the next call only after the caller has
  // synchronised the stream (one batched application per solver step)
  cudaError_t e = cudaMemcpyAsync(dbase, sc.host, host_bytes, cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(sync, 0, sizeof(DsaSync), stream);
  long long limit = rts[idx[0]]->wait_limit_ns;
  int iters = rts[idx[0]]->dsa_iters;
  void* args[] = {&dprobs, &dmap, &part_a, &part_b, &sync, &status, &limit, &iters};
  if (e == cudaSuccess)
    e = cudaLaunchCooperativeKernel((const void*)dsa_cg_batch_kernel<DIM>, dim3(total), dim3(kCgThreads), args, 0,
                                    stream);
  if (e != cudaSuccess) {
    err = std::string("diffusion acceleration, batched solve: ") + cudaGetErrorString(e);
    return OURANOS_ERR_CUDA;
  }
  return OURANOS_OK;
}

}  // namespace

namespace ouranos {
DsaBatchScratch::~DsaBatchScratch() {
  if (host) cudaFreeHost(host);
}

int rt_dsa_apply_batch(ouranos_rt* const* rts, const double* const* v, double* const* out, int count,
                       cudaStream_t stream, int* status, DsaBatchScratch& sc, std::string& err) {
  if (count <= 0) return OURANOS_OK;
  const int iters = rts[0]->dsa_iters;
  for (int i = 0; i < count; ++i) {
    if (rts[i]->dsa_iters < 1 || rts[i]->dsa_iters != iters) {
      err = "diffusion acceleration: every problem of a batch needs the same CG step count (>= 1)";
      return OURANOS_ERR_BAD_INPUT;
    }
    const int rc = ensure_tables(rts[i]);
    if (rc) {
      err = rts[i]->err;
      return rc;
    }
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, rts[0]->device) != cudaSuccess) {
    err = "diffusion acceleration: device query failed";
    return OURANOS_ERR_CUDA;
  }
  int launches = 0;
  for (int dim = 2; dim <= 3; ++dim) {
    int per_sm = 0;
    const cudaError_t e =
        dim == 3 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dsa_cg_batch_kernel<3>, kCgThreads, 0)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dsa_cg_batch_kernel<2>, kCgThreads, 0);
    if (e != cudaSuccess || per_sm < 1) {
      err = "diffusion acceleration: the batched CG kernel does not fit on a multiprocessor";
      return OURANOS_ERR_CUDA;
    }
    // one block per multiprocessor keeps the grid barrier to a few participants
    const int cap = sms;
    std::vector<int> idx;
    for (int i = 0; i < count; ++i)
      if (rts[i]->dim == dim) idx.push_back(i);
    for (size_t s0 = 0; s0 < idx.size(); s0 += cap) {  // at most one block per problem and SM per launch
      const int cnt = (int)std::min<size_t>(cap, idx.size() - s0);
      // a further launch rewrites the page-locked staging block: the copy
      // queued by the previous one must have run
      if (launches++ > 0 && cudaStreamSynchronize(stream) != cudaSuccess) {
        err = "diffusion acceleration: batch synchronisation failed";
        return OURANOS_ERR_CUDA;
      }
      const int rc = dim == 3 ? dsa_batch_launch<3>(rts, v, out, idx.data() + s0, cnt, stream, status, sc, cap, err)
                              : dsa_batch_launch<2>(rts, v, out, idx.data() + s0, cnt, stream, status, sc, cap, err);
      if (rc) return rc;
    }
  }
  return OURANOS_OK;
}

// out = P v on the handle's stream (device vectors, internal cell order);
// out may equal v
int rt_dsa_apply(ouranos_rt* rt, const double* v, double* out) {
  if (rt->dsa_iters < 1) {
    rt->err = "diffusion acceleration is off (ouranos_rt_set_dsa)";
    return OURANOS_ERR_BAD_INPUT;
  }
  int rc = ensure_tables(rt);
  if (rc) return rc;
  return rt->dim == 3 ? dsa_run<3>(rt, v, out, rt->dsa_iters, false) : dsa_run<2>(rt, v, out, rt->dsa_iters, false);
}
// The initial-guess buffer of the diffusion solve ([vertex], FP32, zero halo
// outside): a caller writes a guess of f there before rt_dsa_apply_guess.
int rt_dsa_guess_buffer(ouranos_rt* rt, float** guess, long* n_vertices) {
  int rc = ensure_tables(rt);
  if (rc) return rc;
  const DsaGeom g = geom(rt);
  *guess = rt->d_dsa_vec.as<float>() + 6L * g.nv + 3 * halo(g);
  *n_vertices = g.nv;
  return OURANOS_OK;
}
// out = v + f with the CG started from the guess in the guess buffer
int rt_dsa_apply_guess(ouranos_rt* rt, const double* v, double* out) {
  if (rt->dsa_iters < 1) {
    rt->err = "diffusion acceleration is off (ouranos_rt_set_dsa)";
    return OURANOS_ERR_BAD_INPUT;
  }
  int rc = ensure_tables(rt);
  if (rc) return rc;
  return rt->dim == 3 ? dsa_run<3>(rt, v, out, rt->dsa_iters, true) : dsa_run<2>(rt, v, out, rt->dsa_iters, true);
}
}  // namespace ouranos

extern "C" {

int ouranos_rt_set_dsa(ouranos_rt* rt, int cg_iterations) {
  if (!rt) return OURANOS_ERR_BAD_INPUT;
  if (cg_iterations < 0 || cg_iterations > 10000) {
    rt->err = "diffusion acceleration: CG steps must be in [0, 10000]";
    return OURANOS_ERR_BAD_INPUT;
  }
  if (cg_iterations > 0) {
    cudaSetDevice(rt->device);
    const int rc = ensure_tables(rt);
    if (rc) return rc;
  }
  rt->dsa_iters = cg_iterations;
  return OURANOS_OK;
}

int ouranos_rt_dsa_apply(ouranos_rt* rt, const double* v, double* z) {
  if (!rt || !v || !z) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  int rc = rt_clear_status(rt);
  if (rc) return rc;
  const double* dv = nullptr;
  rc = rt_stage_in(rt, v, rt->d_x, 1, &dv);
  if (rc) return rc;
  DC(rt->d_y.alloc(sizeof(double) * (long)rt->n_mom * rt->n_dofs), "output");
  if ((rc = rt_dsa_apply(rt, dv, rt->d_y.as<double>()))) return rc;
  if ((rc = rt_stage_out(rt, rt->d_y.as<double>(), z))) return rc;
  return rt_check_status(rt);
}

}  // extern "C"
