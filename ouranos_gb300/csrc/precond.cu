// Learned preconditioner glue: per-cell features of a residual vector, the
// network's training target, and the correction it applies.
//
// For a residual v ([mom][dof], FP64) on a 3-D DG Q1 mesh (8 nodes per cell):
//   s          = sqrt(mean over all scalar-moment dofs of v_0^2)  (kept on the device)
//   c_c        = sigma_s0,c / sigma_t,c,   g_c = 1 / (1 - min(c_c, 1 - 1e-6))
//   feature[c] = (v_0[c,0..7]/s, log(sigma_t,c)/log(100), c_c)
// The network predicts y[c,i] ~ (A^-1 v - v)_0[c,i] / (s g_c), and the
// preconditioner returns z = v + s g_c y on the scalar moment's nodal values --
// a learned synthetic acceleration of the scalar flux.  g_c is the
// infinite-medium gain of source iteration in cell c (sum_k c^k); dividing it
// out keeps the regression targets O(1) although A^-1 amplifies the slow modes
// of thick, scattering cells by up to ~g_c.  The correction is per node, not
// per cell: in optically thick cells the slow error modes are continuous
// across faces, and a piecewise-constant correction of them leaves intra-cell
// residuals larger than the one it corrects.
#include <cmath>
#include <cstdio>
#include <vector>

#include "cnn_kernels.cuh"
#include "internal.h"

using namespace ouranos;

namespace {

constexpr int kNodes = OURANOS_CNN_OUTPUTS;
constexpr int kFeat = OURANOS_CNN_FEATURES;
constexpr int kPartials = 304;  // fixed grid of the deterministic sum of squares
constexpr double kGain = 64.0;  // output scale K of the correction

// partial sums of v[0..n) squared, one per block (fixed grid, fixed order)
__global__ void __launch_bounds__(256) sumsq_partial_kernel(const double* v, long n, double* partial) {
  __shared__ double red[8];
  double local = 0.0;
  for (long e = blockIdx.x * 256L + threadIdx.x; e < n; e += 256L * kPartials) local += v[e] * v[e];
  for (int o = 16; o; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w];
    partial[blockIdx.x] = t;
  }
}
// partial[kPartials] -> scale = sqrt(sum / n)
__global__ void __launch_bounds__(32) sumsq_final_kernel(double* partial, long n) {
  double t = 0.0;
  for (int i = threadIdx.x; i < kPartials; i += 32) t += partial[i];
  for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (threadIdx.x == 0) partial[kPartials] = n > 0 ? sqrt(t / (double)n) : 0.0;
}

__global__ void features_kernel(const double* v, const double* scale, long n_cells, const float2* prop,
                                float* feat) {
  const double s = *scale;
  const double inv = s > 0 ? 1.0 / s : 0.0;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n_cells * kFeat;
       e += (long)gridDim.x * blockDim.x) {
    const long c = e / kFeat;
    const int k = (int)(e % kFeat);
    float f;
    if (k < kNodes) f = (float)(v[c * kNodes + k] * inv);
    else f = k == kNodes ? prop[c].x : prop[c].y;
    feat[e] = f;
  }
}

// d[c,i] = (e_0 - v_0)[c,i] / (s K)  (before the continuity projection)
__global__ void target_kernel(const double* v, const double* e, const double* scale, long n, float* d) {
  const double s = *scale;
  const double inv = s > 0 ? 1.0 / (s * kGain) : 0.0;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
    d[k] = (float)((e[k] - v[k]) * inv);
}

// z = v; z_0[c,i] += s K y[c,i]
__global__ void correct_kernel(const double* v, double* z, long len, const float* y, const double* scale,
                               long n0) {
  const double sk = *scale * kGain;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < len; e += (long)gridDim.x * blockDim.x) {
    double val = v[e];
    if (e < n0) val += sk * (double)y[e];
    z[e] = val;
  }
}

// guess[vertex] = s K (mean of the network's nodal outputs y at the vertex):
// the network's prediction of the diffusion correction f as a vertex field
__global__ void vertex_guess_kernel(cnn::Grid g, const float* y, const double* scale, float* guess) {
  const float sk = (float)(*scale * kGain);
  const long nv = cnn::n_vertices(g);
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < nv; v += (long)gridDim.x * blockDim.x) {
    const int vx = (int)(v % (g.nx + 1)), vy = (int)((v / (g.nx + 1)) % (g.ny + 1));
    const int vz = (int)(v / ((long)(g.nx + 1) * (g.ny + 1)));
    float s = 0.f;
    int n = 0;
    for (int k = 0; k < kNodes; ++k) {
      const int cx = vx - (k & 1), cy = vy - ((k >> 1) & 1), cz = vz - (k >> 2);
      if (cx < 0 || cy < 0 || cz < 0 || cx >= g.nx || cy >= g.ny || cz >= g.nz) continue;
      s += y[(cx + (long)g.nx * (cy + (long)g.ny * cz)) * kNodes + k];
      ++n;
    }
    guess[v] = n ? sk * s / (float)n : 0.f;
  }
}

inline int blocks(long n) {
  long b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152L * 16 ? 152L * 16 : b));
}

int pfail(ouranos_rt* rt, cudaError_t e, const char* what) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  rt->err = buf;
  return OURANOS_ERR_CUDA;
}
#define PC(expr, what)                                  \
  do {                                                  \
    cudaError_t _e = (expr);                            \
    if (_e != cudaSuccess) return pfail(rt, _e, what);  \
  } while (0)

cnn::Grid pc_grid(const ouranos_rt* rt) { return cnn::Grid{rt->nx[0], rt->nx[1], rt->nx[2]}; }

// per-cell properties (uploaded once per handle/group) and the work area
int ensure_tables(ouranos_rt* rt) {
  if (rt->dim != 3 || rt->n != kNodes) {
    rt->err = "learned preconditioner: needs a 3-D DG Q1 mesh (8 nodes per cell)";
    return OURANOS_ERR_UNSUPPORTED;
  }
  if (rt->pc_group == rt->group && rt->d_pc_prop.p) return OURANOS_OK;
  std::vector<float2> prop(rt->n_cells);
  const int G = rt->G, L = rt->l_max;
  for (long c = 0; c < rt->n_cells; ++c) {
    const int m = rt->material_id[c];
    const double st = rt->sigma_t[(size_t)m * G + rt->group];
    const double ss = rt->sigma_s[(size_t)rt->group * (L + 1) + (size_t)rt->group * G * (L + 1) +
                                  (size_t)m * G * G * (L + 1)];
    prop[c] = make_float2((float)(std::log(st > 0 ? st : 1e-30) / std::log(100.0)),
                          (float)(st > 0 ? ss / st : 0.0));
  }
  PC(rt->d_pc_prop.alloc(sizeof(float2) * rt->n_cells), "preconditioner tables");
  PC(rt->d_pc_nodal.alloc(sizeof(float) * kNodes * rt->n_cells), "preconditioner work");
  PC(rt->d_pc_vert.alloc(sizeof(float) * cnn::n_vertices(pc_grid(rt))), "preconditioner work");
  PC(rt->d_pc_work.alloc(sizeof(double) * (kPartials + 8)), "preconditioner work");
  PC(cudaMemcpyAsync(rt->d_pc_prop.p, prop.data(), sizeof(float2) * rt->n_cells, cudaMemcpyHostToDevice, rt->stream), "tables");
  PC(cudaStreamSynchronize(rt->stream), "tables");
  rt->pc_group = rt->group;
  return OURANOS_OK;
}

// normalisation of v into work[kPartials]
int pc_scale(ouranos_rt* rt, const double* v) {
  double* work = rt->d_pc_work.as<double>();
  const long n0 = rt->n_cells * kNodes;
  sumsq_partial_kernel<<<kPartials, 256, 0, rt->stream>>>(v, n0, work);
  sumsq_final_kernel<<<1, 32, 0, rt->stream>>>(work, n0);
  PC(cudaGetLastError(), "scale");
  return OURANOS_OK;
}

}  // namespace

namespace ouranos {
// features of v into feat ([cells][OURANOS_CNN_FEATURES] FP32, device); the
// normalisation stays in the handle's work area for rt_pc_correct
int rt_pc_features(ouranos_rt* rt, const double* v, float* feat) {
  int rc = ensure_tables(rt);
  if (rc) return rc;
  if ((rc = pc_scale(rt, v))) return rc;
  features_kernel<<<blocks(rt->n_cells * kFeat), 256, 0, rt->stream>>>(
      v, rt->d_pc_work.as<double>() + kPartials, rt->n_cells, rt->d_pc_prop.as<float2>(), feat);
  PC(cudaGetLastError(), "features");
  return OURANOS_OK;
}

// The learned preconditioner inside the diffusion acceleration: the
// network's output on v (trained to predict the diffusion correction f of
// v) starts the diffusion CG, whose rt->dsa_iters steps then remove the
// network's error; out = v + f.  The CG converges to the same f from any
// guess, so a poor prediction costs CG progress, never a wrong correction.
int rt_pc_dsa_apply(ouranos_rt* rt, const double* v, double* out) {
  if (!rt->cnn) {
    rt->err = "no preconditioner installed (ouranos_rt_set_preconditioner)";
    return OURANOS_ERR_BAD_INPUT;
  }
  PC(rt->d_pc_feat.alloc(sizeof(float) * (kFeat + kNodes) * rt->n_cells), "preconditioner");
  float* feat = rt->d_pc_feat.as<float>();
  float* y = feat + (long)kFeat * rt->n_cells;
  int rc;
  if ((rc = rt_pc_features(rt, v, feat))) return rc;
  // no host synchronisation: the forward (a CUDA graph after its first two
  // calls) runs in the order of the handle's stream, and its status word is
  // read with the handle's own status
  rt->cnn_pending = true;
  if ((rc = cnn_forward_on(rt->cnn, feat, y, rt->stream))) {
    rt->err = "network forward failed";
    return rc;
  }
  float* guess = nullptr;
  long nv = 0;
  if ((rc = rt_dsa_guess_buffer(rt, &guess, &nv))) return rc;
  const cnn::Grid g = pc_grid(rt);
  vertex_guess_kernel<<<blocks(nv), 256, 0, rt->stream>>>(g, y, rt->d_pc_work.as<double>() + kPartials, guess);
  PC(cudaGetLastError(), "guess");
  return rt_dsa_apply_guess(rt, v, out);
}

// z = v + s * y with the normalisation of the last rt_pc_features call
int rt_pc_correct(ouranos_rt* rt, const double* v, const float* y, double* z) {
  const long len = (long)rt->n_mom * rt->n_dofs;
  correct_kernel<<<blocks(len), 256, 0, rt->stream>>>(v, z, len, y, rt->d_pc_work.as<double>() + kPartials,
                                                      rt->n_cells * kNodes);
  PC(cudaGetLastError(), "correction");
  return OURANOS_OK;
}
}  // namespace ouranos

extern "C" {

int ouranos_rt_set_preconditioner(ouranos_rt* rt, ouranos_cnn* cnn) {
  if (!rt) return OURANOS_ERR_BAD_INPUT;
  if (cnn) {
    int nx, ny, nz;
    cnn_grid(cnn, &nx, &ny, &nz);
    if (rt->dim != 3 || rt->n != kNodes) {
      rt->err = "learned preconditioner: needs a 3-D DG Q1 mesh (8 nodes per cell)";
      return OURANOS_ERR_UNSUPPORTED;
    }
    if (nx != rt->nx[0] || ny != rt->nx[1] || nz != rt->nx[2]) {
      rt->err = "learned preconditioner: network grid differs from the mesh";
      return OURANOS_ERR_BAD_INPUT;
    }
  }
  // a graph of the network's forward refers to the handle's feature buffers;
  // a timeout of forwards not yet checked is reported here, after the change
  int rc = OURANOS_OK;
  if (rt->cnn) {
    cudaSetDevice(rt->device);
    cudaStreamSynchronize(rt->stream);
    if (rt->cnn_pending && cnn_forward_status(rt->cnn)) {
      rt->err = "learned preconditioner: a convolution's tensor-core wait timed out";
      rc = OURANOS_ERR_TIMEOUT;
    }
    rt->cnn_pending = false;
    cnn_forward_release(rt->cnn);
  }
  if (cnn) cnn_forward_release(cnn);
  rt->cnn = cnn;
  return rc;
}

int ouranos_rt_pc_features(ouranos_rt* rt, const double* v, float* features, double* scale) {
  if (!rt || !v || !features) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  int rc = rt_pc_features(rt, v, features);
  if (rc) return rc;
  if (scale)
    PC(cudaMemcpyAsync(scale, rt->d_pc_work.as<double>() + kPartials, sizeof(double), cudaMemcpyDeviceToHost,
                       rt->stream),
       "scale");
  PC(cudaStreamSynchronize(rt->stream), "features");
  return OURANOS_OK;
}

int ouranos_rt_pc_target(ouranos_rt* rt, const double* v, const double* e, float* target) {
  if (!rt || !v || !e || !target) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  int rc = ensure_tables(rt);
  if (rc) return rc;
  if ((rc = pc_scale(rt, v))) return rc;
  const long n0 = rt->n_cells * kNodes;
  float* d = rt->d_pc_nodal.as<float>();
  float* vert = rt->d_pc_vert.as<float>();
  const cnn::Grid g = pc_grid(rt);
  target_kernel<<<blocks(n0), 256, 0, rt->stream>>>(v, e, rt->d_pc_work.as<double>() + kPartials, n0, d);
  cnn::vertex_average_kernel<<<blocks(cnn::n_vertices(g)), 256, 0, rt->stream>>>(g, d, kNodes, 1.f, vert);
  cnn::vertex_scatter_kernel<<<blocks(rt->n_cells), 256, 0, rt->stream>>>(g, vert, target);
  PC(cudaGetLastError(), "target");
  PC(cudaStreamSynchronize(rt->stream), "target");
  return OURANOS_OK;
}

int ouranos_rt_pc_dsa_apply(ouranos_rt* rt, const double* v, double* z) {
  if (!rt || !v || !z) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  int rc = rt_clear_status(rt);
  if (rc || (rc = rt_pc_dsa_apply(rt, v, z))) return rc;
  return rt_check_status(rt);
}

int ouranos_rt_pc_apply(ouranos_rt* rt, const double* v, double* z) {
  if (!rt || !v || !z || !rt->cnn) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  PC(rt->d_pc_feat.alloc(sizeof(float) * (kFeat + kNodes) * rt->n_cells), "preconditioner");
  float* feat = rt->d_pc_feat.as<float>();
  float* y = feat + (long)kFeat * rt->n_cells;
  int rc;
  if ((rc = rt_pc_features(rt, v, feat))) return rc;
  PC(cudaStreamSynchronize(rt->stream), "preconditioner");
  if ((rc = ouranos_cnn_forward(rt->cnn, feat, y))) {
    rt->err = "network forward failed";
    return rc;
  }
  if ((rc = rt_pc_correct(rt, v, y, z))) return rc;
  PC(cudaStreamSynchronize(rt->stream), "preconditioner");
  return OURANOS_OK;
}

}  // extern "C"
