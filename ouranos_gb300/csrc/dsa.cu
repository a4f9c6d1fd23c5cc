// Diffusion synthetic acceleration (DSA) of the scalar flux for DG Q1 meshes,
// used as the right preconditioner of FGMRES and as the acceleration step of
// source iteration.
//
// The reference's Krylov solves run unpreconditioned (src/ouranos.cc:160-171),
// and its source iteration (src/ouranos.cc:72-95) is plain.  In optically
// thick, highly scattering cells both converge slowly: the slow error modes of
// the transport iteration are continuous scalar-flux fields that obey a
// diffusion equation.  For a residual v ([mom][dof]) the preconditioner is
//   P v = v + f,   (-div D grad + sigma_a) f = sigma_s0 v_0,
// f continuous trilinear (bilinear in 2-D) on the mesh vertices, with the
// Marshak condition D df/dn + f/2 = 0 on vacuum and inflow boundaries and a
// zero current on reflective ones; D = 1 / (3 (sigma_t' - sigma_s1)),
// sigma_a = sigma_t' - sigma_s0, sigma_t' = sigma_t + 1/(v dt) in time steps.
// f is added to the scalar moment's nodal values of every cell (the DG Q1
// space contains the continuous one), the higher moments pass unchanged.
// This is the continuous-finite-element DSA of the source-iteration error
// equation; as a right preconditioner of a Krylov method it stays effective at
// the material discontinuities where the same correction used inside plain
// source iteration can lose its efficiency.
//
// The diffusion system (one unknown per vertex, 27-point stencil in 3-D) is
// assembled on the fly from per-cell coefficients and solved approximately by
// a fixed number of Jacobi-preconditioned conjugate-gradient steps, in FP32
// with FP64 scalars, each step two launches and no host synchronisation:
//   update : x += alpha p, r -= alpha q, z = r / diag, rz' = r.z, beta = rz'/rz
//   matvec : w = C z, p = z + beta p, q = w + beta q, pq = p.q, alpha = rz/pq
// (q = C p is carried by recurrence, so the matrix is applied once per step).
// The dot products end in the last block of each launch, which sums the
// per-block partials in a fixed order: the result is deterministic.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "internal.h"

using namespace ouranos;

namespace {

constexpr int kThreads = 256;

struct DsaGeom {
  int nx, ny, nz;      // cells per axis (nz = 1 in 2-D)
  int vx, vy, vz;      // vertices per axis (vz = 1 in 2-D)
  long nv;             // vertices
  float ks[3];         // stiffness scale of axis a: (measure of the cell) / h_a^2
  float vol;           // measure of a cell
  float face[3];       // (measure of a face normal to axis a) / 2
  int robin;           // bit 2a+s: Marshak term on side s (0 low, 1 high) of axis a
};

// coefficients of CG's scalars, on the device
struct DsaScalars {
  double rz, alpha, beta, pq;
  unsigned count;  // blocks done in the current launch
};

// 1-D Q1 factors between the basis functions of local corners u and w of a
// cell of unit length: mass (1/3 on, 1/6 off the diagonal) and stiffness
__device__ __forceinline__ float m1(int u, int w) { return u == w ? (1.f / 3.f) : (1.f / 6.f); }
__device__ __forceinline__ float s1(int u, int w) { return u == w ? 1.f : -1.f; }

// Row of the diffusion matrix at vertex (I, J, K) applied to the values that
// ld(dx, dy, dz) returns for vertex (I-1+dx, J-1+dy, K-1+dz), dx..dz in 0..2
// (2-D: dz = 1 always).  cell[c] = (D, sigma_a, sigma_s0, -).
template <int DIM, class Load>
__device__ __forceinline__ float row_apply(const DsaGeom& g, const float4* __restrict__ cell, int I, int J,
                                           int K, Load ld) {
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
        const float4 cp = cell[((long)kz * g.ny + ky) * g.nx + kx];
        float sm = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
        for (int c2 = 0; c2 < NC; ++c2)
#pragma unroll
          for (int b2 = 0; b2 < 2; ++b2)
#pragma unroll
            for (int a2 = 0; a2 < 2; ++a2) {
              const float val = ld(a + a2, b + b2, DIM == 3 ? c + c2 : 1);
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
                   ld(1, b + b2, DIM == 3 ? c + c2 : 1);
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
                   ld(a + a2, 1, DIM == 3 ? c + c2 : 1);
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
            acc += g.face[2] * m1(1 - a, a2) * m1(1 - b, b2) * ld(a + a2, b + b2, 1);
      }
    }
  }
  return acc;
}

__device__ __forceinline__ void vertex_ijk(const DsaGeom& g, long v, int& I, int& J, int& K) {
  I = (int)(v % g.vx);
  const long t = v / g.vx;
  J = (int)(t % g.vy);
  K = (int)(t / g.vy);
}

struct VecLoad {
  const float* p;
  const DsaGeom* g;
  int I, J, K;
  __device__ __forceinline__ float operator()(int dx, int dy, int dz) const {
    const int i = I - 1 + dx, j = J - 1 + dy, k = K - 1 + dz;
    if (i < 0 || i >= g->vx || j < 0 || j >= g->vy || k < 0 || k >= g->vz) return 0.f;
    return p[((long)k * g->vy + j) * g->vx + i];
  }
};
struct DeltaLoad {
  __device__ __forceinline__ float operator()(int dx, int dy, int dz) const {
    return (dx == 1 && dy == 1 && dz == 1) ? 1.f : 0.f;
  }
};

// Fixed-order block sum; thread 0 returns the block total.
__device__ __forceinline__ double block_sum(double t) {
  __shared__ double red[kThreads / 32];
  for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / 32; ++w) s += red[w];
  __syncthreads();
  return s;
}

// Every block stores its partial; the last block to finish sums the partials
// in block order and returns true in thread 0 with the total in *total.
__device__ __forceinline__ bool grid_sum(double t, double* part, unsigned* count, double* total) {
  __shared__ bool last;
  const double s = block_sum(t);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = s;
    __threadfence();
    last = atomicAdd(count, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double u = 0.0;
  for (unsigned i = threadIdx.x; i < gridDim.x; i += kThreads) u += __ldcg(part + i);
  u = block_sum(u);
  if (threadIdx.x == 0) {
    *total = u;
    *count = 0u;
  }
  return threadIdx.x == 0;
}

template <int DIM>
__global__ void __launch_bounds__(kThreads) dsa_diag_kernel(DsaGeom g, const float4* __restrict__ cell,
                                                            float* __restrict__ dinv) {
  const long v = blockIdx.x * (long)kThreads + threadIdx.x;
  if (v >= g.nv) return;
  int I, J, K;
  vertex_ijk(g, v, I, J, K);
  const float d = row_apply<DIM>(g, cell, I, J, K, DeltaLoad{});
  dinv[v] = d > 0.f ? 1.f / d : 0.f;
}

// r = assembled sigma_s0 M v_0, z = r / diag, x = 0, rz = r.z
template <int DIM>
__global__ void __launch_bounds__(kThreads) dsa_init_kernel(DsaGeom g, const float4* __restrict__ cell,
                                                            const double* __restrict__ v,
                                                            const float* __restrict__ dinv, float* r, float* z,
                                                            float* x, double* part, DsaScalars* s) {
  constexpr int NC = DIM == 3 ? 2 : 1;
  constexpr int NODES = DIM == 3 ? 8 : 4;
  const long vid = blockIdx.x * (long)kThreads + threadIdx.x;
  double rz = 0.0;
  if (vid < g.nv) {
    int I, J, K;
    vertex_ijk(g, vid, I, J, K);
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
          const long cid = ((long)kz * g.ny + ky) * g.nx + kx;
          const double* vc = v + cid * NODES;
          float sm = 0.f;
#pragma unroll
          for (int c2 = 0; c2 < NC; ++c2)
#pragma unroll
            for (int b2 = 0; b2 < 2; ++b2)
#pragma unroll
              for (int a2 = 0; a2 < 2; ++a2)
                sm += m1(1 - a, a2) * m1(1 - b, b2) * (DIM == 3 ? m1(1 - c, c2) : 1.f) *
                      (float)vc[a2 + 2 * b2 + 4 * c2];
          acc += cell[cid].z * g.vol * sm;
        }
      }
    }
    const float zz = acc * dinv[vid];
    r[vid] = acc;
    z[vid] = zz;
    x[vid] = 0.f;
    rz = (double)acc * (double)zz;
  }
  double tot;
  if (grid_sum(rz, part, &s->count, &tot)) s->rz = tot;
}

// w = C z; p = z + beta p; q = w + beta q; alpha = rz / p.q
template <int DIM>
__global__ void __launch_bounds__(kThreads) dsa_matvec_kernel(DsaGeom g, const float4* __restrict__ cell,
                                                              const float* __restrict__ z, float* p, float* q,
                                                              double* part, DsaScalars* s, int first) {
  const long vid = blockIdx.x * (long)kThreads + threadIdx.x;
  double pq = 0.0;
  if (vid < g.nv) {
    int I, J, K;
    vertex_ijk(g, vid, I, J, K);
    const float w = row_apply<DIM>(g, cell, I, J, K, VecLoad{z, &g, I, J, K});
    const float beta = first ? 0.f : (float)s->beta;
    const float pn = z[vid] + beta * (first ? 0.f : p[vid]);
    const float qn = w + beta * (first ? 0.f : q[vid]);
    p[vid] = pn;
    q[vid] = qn;
    pq = (double)pn * (double)qn;
  }
  double tot;
  if (grid_sum(pq, part, &s->count, &tot)) {
    s->pq = tot;
    s->alpha = tot > 0.0 ? s->rz / tot : 0.0;
  }
}

// x += alpha p; r -= alpha q; z = r / diag; beta = r.z / rz
__global__ void __launch_bounds__(kThreads) dsa_update_kernel(long nv, const float* __restrict__ p,
                                                              const float* __restrict__ q,
                                                              const float* __restrict__ dinv, float* x, float* r,
                                                              float* z, double* part, DsaScalars* s) {
  const long vid = blockIdx.x * (long)kThreads + threadIdx.x;
  double rz = 0.0;
  if (vid < nv) {
    const float alpha = (float)s->alpha;
    x[vid] += alpha * p[vid];
    const float rn = r[vid] - alpha * q[vid];
    const float zn = rn * dinv[vid];
    r[vid] = rn;
    z[vid] = zn;
    rz = (double)rn * (double)zn;
  }
  double tot;
  if (grid_sum(rz, part, &s->count, &tot)) {
    const double old = s->rz;
    s->beta = old > 0.0 ? tot / old : 0.0;
    s->rz = tot;
  }
}

// out = v, plus f = x + alpha p at the vertices of each cell on the scalar
// moment's nodes (the last CG step's update folded in)
template <int DIM>
__global__ void dsa_correct_kernel(DsaGeom g, const double* v, double* out, long len, long n0,
                                   const float* __restrict__ x, const float* __restrict__ p,
                                   const DsaScalars* __restrict__ s) {
  constexpr int NODES = DIM == 3 ? 8 : 4;
  const float alpha = (float)s->alpha;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < len; e += (long)gridDim.x * blockDim.x) {
    double val = v[e];
    if (e < n0) {
      const long cid = e / NODES;
      const int k = (int)(e % NODES);
      const int kx = (int)(cid % g.nx);
      const long t = cid / g.nx;
      const int ky = (int)(t % g.ny), kz = (int)(t / g.ny);
      const long vid = ((long)(kz + (DIM == 3 ? (k >> 2) : 0)) * g.vy + (ky + ((k >> 1) & 1))) * g.vx +
                       (kx + (k & 1));
      val += (double)(x[vid] + alpha * p[vid]);
    }
    out[e] = val;
  }
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
  g.nv = (long)g.vx * g.vy * g.vz;
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
  return g;
}

inline int nblocks(long n) { return (int)((n + kThreads - 1) / kThreads); }

// per-cell coefficients and the Jacobi diagonal, rebuilt when the group or
// the time step changes
int ensure_tables(ouranos_rt* rt) {
  if (rt->n != (rt->dim == 3 ? 8 : 4) || rt->p != 1) {
    rt->err = "diffusion acceleration needs a DG Q1 mesh";
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
  DC(rt->d_dsa_vec.alloc(sizeof(float) * 6 * nv), "vectors");
  DC(rt->d_dsa_red.alloc(sizeof(double) * (nb + 8)), "reductions");
  DC(cudaMemcpyAsync(rt->d_dsa_cell.p, cell.data(), sizeof(float4) * rt->n_cells, cudaMemcpyHostToDevice,
                     rt->stream),
     "tables");
  DsaScalars* s = reinterpret_cast<DsaScalars*>(rt->d_dsa_red.as<double>() + nb);
  DC(cudaMemsetAsync(s, 0, sizeof(DsaScalars), rt->stream), "reductions");
  float* dinv = rt->d_dsa_vec.as<float>() + 5 * nv;
  if (rt->dim == 3)
    dsa_diag_kernel<3><<<nb, kThreads, 0, rt->stream>>>(g, rt->d_dsa_cell.as<float4>(), dinv);
  else
    dsa_diag_kernel<2><<<nb, kThreads, 0, rt->stream>>>(g, rt->d_dsa_cell.as<float4>(), dinv);
  DC(cudaGetLastError(), "diagonal");
  DC(cudaStreamSynchronize(rt->stream), "tables");
  rt->dsa_group = rt->group;
  rt->dsa_inv_vdt = rt->inv_vdt;
  return OURANOS_OK;
}

template <int DIM>
int dsa_run(ouranos_rt* rt, const double* v, double* out, int iters) {
  const DsaGeom g = geom(rt);
  const long nv = g.nv;
  const int nb = nblocks(nv);
  float* base = rt->d_dsa_vec.as<float>();
  float *x = base, *r = base + nv, *z = base + 2 * nv, *p = base + 3 * nv, *q = base + 4 * nv,
        *dinv = base + 5 * nv;
  double* part = rt->d_dsa_red.as<double>();
  DsaScalars* s = reinterpret_cast<DsaScalars*>(part + nb);
  const float4* cell = rt->d_dsa_cell.as<float4>();
  cudaStream_t st = rt->stream;
  dsa_init_kernel<DIM><<<nb, kThreads, 0, st>>>(g, cell, v, dinv, r, z, x, part, s);
  dsa_matvec_kernel<DIM><<<nb, kThreads, 0, st>>>(g, cell, z, p, q, part, s, 1);
  for (int it = 1; it < iters; ++it) {
    dsa_update_kernel<<<nb, kThreads, 0, st>>>(nv, p, q, dinv, x, r, z, part, s);
    dsa_matvec_kernel<DIM><<<nb, kThreads, 0, st>>>(g, cell, z, p, q, part, s, 0);
  }
  const long len = (long)rt->n_mom * rt->n_dofs;
  const long blocks = std::min<long>((len + kThreads - 1) / kThreads, 152L * 16);
  dsa_correct_kernel<DIM><<<(int)blocks, kThreads, 0, st>>>(g, v, out, len, rt->n_cells * (long)rt->n, x, p, s);
  DC(cudaGetLastError(), "solve");
  return OURANOS_OK;
}

}  // namespace

namespace ouranos {
// out = P v on the handle's stream (device vectors, internal cell order);
// out may equal v
int rt_dsa_apply(ouranos_rt* rt, const double* v, double* out) {
  if (rt->dsa_iters < 1) {
    rt->err = "diffusion acceleration is off (ouranos_rt_set_dsa)";
    return OURANOS_ERR_BAD_INPUT;
  }
  int rc = ensure_tables(rt);
  if (rc) return rc;
  return rt->dim == 3 ? dsa_run<3>(rt, v, out, rt->dsa_iters) : dsa_run<2>(rt, v, out, rt->dsa_iters);
}
int rt_dsa_kernels(const ouranos_rt* rt) { return rt->dsa_iters > 0 ? 2 * rt->dsa_iters + 1 : 0; }
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
  const double* dv = nullptr;
  int rc = rt_stage_in(rt, v, rt->d_x, 1, &dv);
  if (rc) return rc;
  DC(rt->d_y.alloc(sizeof(double) * (long)rt->n_mom * rt->n_dofs), "output");
  if ((rc = rt_dsa_apply(rt, dv, rt->d_y.as<double>()))) return rc;
  if ((rc = rt_stage_out(rt, rt->d_y.as<double>(), z))) return rc;
  DC(cudaStreamSynchronize(rt->stream), "apply");
  return OURANOS_OK;
}

}  // extern "C"
