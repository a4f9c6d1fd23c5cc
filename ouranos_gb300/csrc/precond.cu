// Learned preconditioner glue: per-cell features of a residual vector, the
// network's training target, and the correction it applies.
//
// For a residual v ([mom][dof], FP64) on a handle's mesh:
//   a[c]  = cell average of the scalar moment, sum_i (sum_j M_ij / |cell|) v_0[c,i]
//   s     = sqrt(mean_c a[c]^2)  (normalisation, kept on the device)
//   feature[c] = (a[c]/s, log(sigma_t,c)/log(100), sigma_s0,c/sigma_t,c)
// The network predicts y[c] ~ cell average of (A^-1 v - v)[c] / s, and the
// preconditioner returns z = v + s*y on the scalar moment (piecewise constant
// per cell) -- a learned synthetic acceleration of the scalar flux.
#include <cmath>
#include <cstdio>
#include <vector>

#include "internal.h"

using namespace ouranos;

namespace {

__global__ void cell_avg_kernel(const double* v, const double* wavg, int n, long n_cells, double* avg,
                                double* sumsq) {
  double local = 0.0;
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n_cells; c += (long)gridDim.x * blockDim.x) {
    double a = 0.0;
    for (int i = 0; i < n; ++i) a += wavg[i] * v[c * n + i];
    avg[c] = a;
    local += a * a;
  }
  for (int o = 16; o; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0 && sumsq) atomicAdd(sumsq, local);
}

__global__ void features_kernel(const double* avg, const double* sumsq, long n_cells, const float2* prop,
                                float* feat) {
  const double s = sqrt(*sumsq / (double)n_cells);
  const double inv = s > 0 ? 1.0 / s : 0.0;
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n_cells; c += (long)gridDim.x * blockDim.x) {
    feat[c * 3 + 0] = (float)(avg[c] * inv);
    feat[c * 3 + 1] = prop[c].x;
    feat[c * 3 + 2] = prop[c].y;
  }
}

// target[c] = (avg(e)[c] - avg(v)[c]) / s
__global__ void target_kernel(const double* avg_e, const double* avg_v, const double* sumsq, long n_cells,
                              float* target) {
  const double s = sqrt(*sumsq / (double)n_cells);
  const double inv = s > 0 ? 1.0 / s : 0.0;
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n_cells; c += (long)gridDim.x * blockDim.x)
    target[c] = (float)((avg_e[c] - avg_v[c]) * inv);
}

// z = v; z_0[c,i] += s * y[c]
__global__ void correct_kernel(const double* v, double* z, long len, const float* y, const double* sumsq,
                               int n, long n_cells) {
  const double s = sqrt(*sumsq / (double)n_cells);
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < len; e += (long)gridDim.x * blockDim.x) {
    double val = v[e];
    if (e < n_cells * n) val += s * (double)y[e / n];
    z[e] = val;
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

// per-cell properties and averaging weights (uploaded once per handle/group)
int ensure_tables(ouranos_rt* rt) {
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
  double vol = 1.0;
  for (int a = 0; a < rt->dim; ++a) vol *= rt->h[a];
  std::vector<double> w(rt->n, 0.0);
  for (int i = 0; i < rt->n; ++i)
    for (int j = 0; j < rt->n; ++j) w[i] += rt->fe.mass[j * rt->n + i] / vol;
  PC(rt->d_pc_prop.alloc(sizeof(float2) * rt->n_cells), "preconditioner tables");
  PC(rt->d_pc_wavg.alloc(sizeof(double) * rt->n), "preconditioner tables");
  PC(rt->d_pc_work.alloc(sizeof(double) * (2 * rt->n_cells + 8)), "preconditioner work");
  PC(cudaMemcpyAsync(rt->d_pc_prop.p, prop.data(), sizeof(float2) * rt->n_cells, cudaMemcpyHostToDevice, rt->stream), "tables");
  PC(cudaMemcpyAsync(rt->d_pc_wavg.p, w.data(), sizeof(double) * rt->n, cudaMemcpyHostToDevice, rt->stream), "tables");
  PC(cudaStreamSynchronize(rt->stream), "tables");
  rt->pc_group = rt->group;
  return OURANOS_OK;
}

}  // namespace

namespace ouranos {
// features of v into feat ([cells][3] FP32, device); the normalisation stays
// in the handle's work area (work[2*n_cells])
int rt_pc_features(ouranos_rt* rt, const double* v, float* feat) {
  int rc = ensure_tables(rt);
  if (rc) return rc;
  double* avg = rt->d_pc_work.as<double>();
  double* sumsq = avg + 2 * rt->n_cells;
  PC(cudaMemsetAsync(sumsq, 0, sizeof(double), rt->stream), "features");
  cell_avg_kernel<<<blocks(rt->n_cells), 256, 0, rt->stream>>>(v, rt->d_pc_wavg.as<double>(), rt->n,
                                                               rt->n_cells, avg, sumsq);
  features_kernel<<<blocks(rt->n_cells), 256, 0, rt->stream>>>(avg, sumsq, rt->n_cells,
                                                               rt->d_pc_prop.as<float2>(), feat);
  PC(cudaGetLastError(), "features");
  return OURANOS_OK;
}

// z = v + s * expand(y) with the normalisation of the last rt_pc_features call
int rt_pc_correct(ouranos_rt* rt, const double* v, const float* y, double* z) {
  const double* sumsq = rt->d_pc_work.as<double>() + 2 * rt->n_cells;
  const long len = (long)rt->n_mom * rt->n_dofs;
  correct_kernel<<<blocks(len), 256, 0, rt->stream>>>(v, z, len, y, sumsq, rt->n, rt->n_cells);
  PC(cudaGetLastError(), "correction");
  return OURANOS_OK;
}
}  // namespace ouranos

extern "C" {

int ouranos_rt_set_preconditioner(ouranos_rt* rt, ouranos_cnn* cnn) {
  if (!rt) return OURANOS_ERR_BAD_INPUT;
  rt->cnn = cnn;
  return OURANOS_OK;
}

int ouranos_rt_pc_features(ouranos_rt* rt, const double* v, float* features, double* scale) {
  if (!rt || !v || !features) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  int rc = rt_pc_features(rt, v, features);
  if (rc) return rc;
  if (scale) {
    double ss = 0.0;
    PC(cudaMemcpyAsync(&ss, rt->d_pc_work.as<double>() + 2 * rt->n_cells, sizeof(double),
                       cudaMemcpyDeviceToHost, rt->stream), "scale");
    PC(cudaStreamSynchronize(rt->stream), "scale");
    *scale = std::sqrt(ss / (double)rt->n_cells);
  }
  PC(cudaStreamSynchronize(rt->stream), "features");
  return OURANOS_OK;
}

int ouranos_rt_pc_target(ouranos_rt* rt, const double* v, const double* e, float* target) {
  if (!rt || !v || !e || !target) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  int rc = ensure_tables(rt);
  if (rc) return rc;
  double* avg = rt->d_pc_work.as<double>();
  double* avg_e = avg + rt->n_cells;
  double* sumsq = avg + 2 * rt->n_cells;
  PC(cudaMemsetAsync(sumsq, 0, sizeof(double), rt->stream), "target");
  cell_avg_kernel<<<blocks(rt->n_cells), 256, 0, rt->stream>>>(v, rt->d_pc_wavg.as<double>(), rt->n,
                                                               rt->n_cells, avg, sumsq);
  cell_avg_kernel<<<blocks(rt->n_cells), 256, 0, rt->stream>>>(e, rt->d_pc_wavg.as<double>(), rt->n,
                                                               rt->n_cells, avg_e, nullptr);
  target_kernel<<<blocks(rt->n_cells), 256, 0, rt->stream>>>(avg_e, avg, sumsq, rt->n_cells, target);
  PC(cudaGetLastError(), "target");
  PC(cudaStreamSynchronize(rt->stream), "target");
  return OURANOS_OK;
}

int ouranos_rt_pc_apply(ouranos_rt* rt, const double* v, double* z) {
  if (!rt || !v || !z || !rt->cnn) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  PC(rt->d_pc_feat.alloc(sizeof(float) * 4 * rt->n_cells), "preconditioner");
  float* feat = rt->d_pc_feat.as<float>();
  float* y = feat + 3 * rt->n_cells;
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
