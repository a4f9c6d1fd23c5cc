// The learned preconditioner's network: a three-level 3-D U-Net on the cell
// grid, BF16 activations, FP32 master weights, Adam.  No counterpart in the
// reference (its Krylov solves are unpreconditioned, src/ouranos.cc:160-171).
//
//   level 0 (n^3):   x0(16) -a0-> h_a0(16) -b0-> s0(16)
//   level 1 (n/2):   pool(s0) -a1-> h_a1(32) -b1-> s1(32)
//   level 2 (n/4):   pool(s1) -a2-> h_a2(32) -b2-> h_b2(32)
//   level 1:         up(h_b2)+s1 -c1-> h_c1(32) -d1-> h_d1(16)
//   level 0:         up(h_d1)+s0 -c0-> h_c0(16) -out-> o (channels 0..7 used)
//   continuity:      y = S o, S the projection onto continuous nodal fields
//                    (values at a shared mesh vertex averaged)
// Every layer is gated-linear: h = (W * x) . gamma, a 3x3x3 convolution with
// no bias followed by a per-voxel, per-channel gate gamma = a0 + a1 m0 + a2 m1
// that is affine in the local material features m = (log(sigma_t)/log(100),
// scattering ratio), average-pooled to the layer's level.  The network is
// therefore linear in the residual it is given -- like A^-1 itself -- while
// its coefficients follow the material map, and it answers consistently on
// any mix of the error modes it was fitted on.
// Inputs: channels 0..7 of x0 the residual's normalised scalar-flux values at
// the cell's eight Q1 nodes (features 0..7) rounded to BF16, channels 8..15
// the rounding remainders; features 8 and 9 are m.  Outputs: the eight nodal values of the continuous correction.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "cnn_kernels.cuh"
#include "internal.h"

using namespace ouranos;
using ouranos::cnn::Grid;

namespace {

constexpr int kCin0 = 16;  // padded input channels
constexpr int kFeatures = OURANOS_CNN_FEATURES;
constexpr int kNodal = 8;  // features 0..7: the residual's nodal values; 8, 9: materials
constexpr int kOut = OURANOS_CNN_OUTPUTS;
static_assert(kFeatures == kNodal + 2 && 2 * kNodal == kCin0 && kOut == 8,
              "features are 8 nodal values + 2 material fields; outputs are the 8 Q1 corners");

// one voxel per thread: channels 0..7 the BF16 of the nodal values, 8..15
// the BF16 of what that rounding lost (the first layer sees the residual to
// ~16 bits), two 16-byte stores
__global__ void features_kernel(const float* feat, __nv_bfloat16* x0, float2* mat, long V) {
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < V; v += (long)gridDim.x * blockDim.x) {
    const float* f = feat + v * kFeatures;
    uint32_t hi[4], lo[4];
#pragma unroll
    for (int c = 0; c < kNodal; c += 2) {
      const __nv_bfloat162 h = __floats2bfloat162_rn(f[c], f[c + 1]);
      const __nv_bfloat162 l = __floats2bfloat162_rn(f[c] - __low2float(h), f[c + 1] - __high2float(h));
      hi[c / 2] = *reinterpret_cast<const uint32_t*>(&h);
      lo[c / 2] = *reinterpret_cast<const uint32_t*>(&l);
    }
    uint4* o = reinterpret_cast<uint4*>(x0 + v * kCin0);
    o[0] = make_uint4(hi[0], hi[1], hi[2], hi[3]);
    o[1] = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    mat[v] = make_float2(f[kNodal], f[kNodal + 1]);
  }
}
// 2x2x2 average pool of the material features
__global__ void mat_pool_kernel(Grid fine, const float2* in, float2* out) {
  const Grid co{fine.nx / 2, fine.ny / 2, fine.nz / 2};
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < co.voxels(); v += (long)gridDim.x * blockDim.x) {
    const int x = (int)(v % co.nx), y = (int)((v / co.nx) % co.ny), z = (int)(v / ((long)co.nx * co.ny));
    float sx = 0.f, sy = 0.f;
    for (int k = 0; k < 8; ++k) {
      const float2 m = in[(2 * x + (k & 1)) + (long)fine.nx * ((2 * y + ((k >> 1) & 1)) + (long)fine.ny * (2 * z + (k >> 2)))];
      sx += m.x;
      sy += m.y;
    }
    out[v] = make_float2(0.125f * sx, 0.125f * sy);
  }
}
// gate: x[v,c] = o[v,c] * (a[3c] + a[3c+1] m[v].x + a[3c+2] m[v].y)
template <typename T>
__device__ __forceinline__ float to_f(T v);
template <>
__device__ __forceinline__ float to_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <typename T>
__device__ __forceinline__ T from_f(float v);
template <>
__device__ __forceinline__ float from_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16(v); }

__device__ __forceinline__ float gate_of(const float* a, int c, float2 m) {
  return a[3 * c] + a[3 * c + 1] * m.x + a[3 * c + 2] * m.y;
}
// backward of the gate: g_o = g . gamma (BF16, may alias g) and
// da[3c+j] += sum_v g[v,c] o[v,c] (1, m0, m1)_j
template <typename T>
__global__ void __launch_bounds__(256) gate_bwd_kernel(const __nv_bfloat16* g, const T* o, const float2* mat,
                                                       const float* a, int C, long V, __nv_bfloat16* g_o,
                                                       float* da) {
  __shared__ float s_da[3 * 32];
  for (int i = threadIdx.x; i < 3 * C; i += blockDim.x) s_da[i] = 0.f;
  __syncthreads();
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < V * C; e += (long)gridDim.x * blockDim.x) {
    const int c = (int)(e % C);
    const float2 m = mat[e / C];
    const float gv = __bfloat162float(g[e]);
    const float go = gv * to_f<T>(o[e]);
    g_o[e] = __float2bfloat16(gv * gate_of(a, c, m));
    atomicAdd(&s_da[3 * c], go);
    atomicAdd(&s_da[3 * c + 1], go * m.x);
    atomicAdd(&s_da[3 * c + 2], go * m.y);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 3 * C; i += blockDim.x) atomicAdd(da + i, s_da[i]);
}
__global__ void add_kernel(const __nv_bfloat16* a, const __nv_bfloat16* b, __nv_bfloat16* out, long n) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
    out[e] = __float2bfloat16(__bfloat162float(a[e]) + __bfloat162float(b[e]));
}
// 2x2x2 average pool (fine -> coarse) and its adjoint
// 8 channels of one coarse voxel per thread (16-byte loads and store)
__global__ void pool_kernel(Grid fine, const __nv_bfloat16* in, __nv_bfloat16* out, int C) {
  const Grid co{fine.nx / 2, fine.ny / 2, fine.nz / 2};
  const int C8 = C / 8;
  const long n = co.voxels() * C8;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const long v = e / C8;
    const int c = (int)(e % C8) * 8;
    const int x = (int)(v % co.nx), y = (int)((v / co.nx) % co.ny), z = (int)(v / ((long)co.nx * co.ny));
    float s[8] = {};
    for (int k = 0; k < 8; ++k) {
      const long fv = (2 * x + (k & 1)) + (long)fine.nx * ((2 * y + ((k >> 1) & 1)) + (long)fine.ny * (2 * z + (k >> 2)));
      const uint4 u = *reinterpret_cast<const uint4*>(in + fv * C + c);
      const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        s[2 * j] += __low2float(h[j]);
        s[2 * j + 1] += __high2float(h[j]);
      }
    }
    uint32_t r[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const __nv_bfloat162 q = __floats2bfloat162_rn(0.125f * s[2 * j], 0.125f * s[2 * j + 1]);
      r[j] = *reinterpret_cast<const uint32_t*>(&q);
    }
    *reinterpret_cast<uint4*>(out + v * C + c) = make_uint4(r[0], r[1], r[2], r[3]);
  }
}
__global__ void pool_bwd_kernel(Grid fine, const __nv_bfloat16* gco, __nv_bfloat16* gfine, int C) {
  const Grid co{fine.nx / 2, fine.ny / 2, fine.nz / 2};
  const long n = fine.voxels() * C;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const long v = e / C;
    const int c = (int)(e % C);
    const int x = (int)(v % fine.nx) / 2, y = (int)((v / fine.nx) % fine.ny) / 2,
              z = (int)(v / ((long)fine.nx * fine.ny)) / 2;
    gfine[e] = __float2bfloat16(0.125f * __bfloat162float(gco[(x + (long)co.nx * (y + (long)co.ny * z)) * C + c]));
  }
}
// nearest upsample (coarse -> fine) plus a skip tensor on the fine grid
// nearest upsample (coarse -> fine) plus a skip tensor on the fine grid,
// 8 channels of one fine voxel per thread
__global__ void up_add_kernel(Grid fine, const __nv_bfloat16* co_in, const __nv_bfloat16* skip,
                              __nv_bfloat16* out, int C) {
  const Grid co{fine.nx / 2, fine.ny / 2, fine.nz / 2};
  const int C8 = C / 8;
  const long n = fine.voxels() * C8;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const long v = e / C8;
    const int c = (int)(e % C8) * 8;
    const int x = (int)(v % fine.nx) / 2, y = (int)((v / fine.nx) % fine.ny) / 2,
              z = (int)(v / ((long)fine.nx * fine.ny)) / 2;
    const uint4 a = *reinterpret_cast<const uint4*>(co_in + (x + (long)co.nx * (y + (long)co.ny * z)) * C + c);
    const uint4 b = *reinterpret_cast<const uint4*>(skip + v * C + c);
    const __nv_bfloat162* ha = reinterpret_cast<const __nv_bfloat162*>(&a);
    const __nv_bfloat162* hb = reinterpret_cast<const __nv_bfloat162*>(&b);
    uint32_t r[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const __nv_bfloat162 q = __floats2bfloat162_rn(__low2float(ha[j]) + __low2float(hb[j]),
                                                     __high2float(ha[j]) + __high2float(hb[j]));
      r[j] = *reinterpret_cast<const uint32_t*>(&q);
    }
    *reinterpret_cast<uint4*>(out + v * C + c) = make_uint4(r[0], r[1], r[2], r[3]);
  }
}
// adjoint of nearest upsample: sum the 8 children
__global__ void up_bwd_kernel(Grid fine, const __nv_bfloat16* gfine, __nv_bfloat16* gco, int C) {
  const Grid co{fine.nx / 2, fine.ny / 2, fine.nz / 2};
  const long n = co.voxels() * C;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const long v = e / C;
    const int c = (int)(e % C);
    const int x = (int)(v % co.nx), y = (int)((v / co.nx) % co.ny), z = (int)(v / ((long)co.nx * co.ny));
    float s = 0.f;
    for (int k = 0; k < 8; ++k) {
      const long fv = (2 * x + (k & 1)) + (long)fine.nx * ((2 * y + ((k >> 1) & 1)) + (long)fine.ny * (2 * z + (k >> 2)));
      s += __bfloat162float(gfine[fv * C + c]);
    }
    gco[e] = __float2bfloat16(s);
  }
}
// residual r = y - target over all V*kOut entries, loss = mean(r^2)
__global__ void resid_kernel(const float* y, const float* target, long n, float* resid, float* loss_acc) {
  float local = 0.f;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const float d = y[e] - target[e];
    resid[e] = d;
    local += d * d;
  }
  for (int o = 16; o; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss_acc, local / (float)n);
}
// d loss / d o = S (2 r / n): the vertex averages of 2r/n scattered to channels
// 0..7 of the output layer's gradient (BF16), zero on channels 8..15
__global__ void grad_scatter_kernel(Grid g, const float* vert, __nv_bfloat16* grad) {
  const long n = g.voxels() * 16;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const int c = (int)(e & 15);
    grad[e] = __float2bfloat16(c < kOut ? vert[ouranos::cnn::corner_vertex(g, e >> 4, c)] : 0.f);
  }
}
__global__ void adam_kernel(float* w, const float* g, float* m, float* v, long n, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const float gg = g[e];
    m[e] = b1 * m[e] + (1.f - b1) * gg;
    v[e] = b2 * v[e] + (1.f - b2) * gg * gg;
    w[e] -= lr * (m[e] / c1) / (sqrtf(v[e] / c2) + eps);
  }
}
// master [tap][cin][cout] -> forward copy [tap][cout][cin] and mirrored-tap copy [26-tap][cin][cout]
__global__ void weight_copies_kernel(const float* w, int cin, int cout, __nv_bfloat16* fwd,
                                     __nv_bfloat16* bwd) {
  const long n = 27L * cin * cout;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const int tap = (int)(e / ((long)cin * cout));
    const int ci = (int)((e / cout) % cin), co = (int)(e % cout);
    const __nv_bfloat16 b = __float2bfloat16(w[e]);
    fwd[((long)tap * cout + co) * cin + ci] = b;
    bwd[((long)(26 - tap) * cin + ci) * cout + co] = b;
  }
}

inline int blocks_for(long n) {
  long b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152L * 16 ? 152L * 16 : b));
}

struct Layer {
  int cin, cout;
  int level;          // 0, 1, 2: grid n, n/2, n/4
  Grid grid;
  size_t woff, goff;  // offsets into the weight and gate arrays
};

}  // namespace

struct ouranos_cnn {
  Grid g0, g1, g2;
  std::vector<Layer> L;  // a0 b0 a1 b1 a2 b2 c1 d1 c0 out
  size_t n_w = 0, n_g = 0;  // conv weights, gate coefficients (3 per output channel)
  float *w = nullptr, *gt = nullptr, *dw = nullptr, *dgt = nullptr;
  float *mw = nullptr, *vw = nullptr, *mg = nullptr, *vg = nullptr;
  __nv_bfloat16 *wf = nullptr, *wb = nullptr;  // BF16 forward / mirrored copies (n_w each)
  // gated activations (inputs of the next layer) and the pre-gate conv outputs
  __nv_bfloat16 *x0, *ha0, *s0, *p0, *ha1, *s1, *p1, *ha2, *hb2, *u1, *hc1, *hd1, *u0, *hc0;
  __nv_bfloat16 *o[9];                                    // pre-gate outputs of a0 .. c0
  float2 *mat[3];                                         // material features per level
  __nv_bfloat16 *ga, *gb_, *gc, *gskip0, *gskip1, *gout;  // gradients
  float* out = nullptr;    // output layer before its gate, [voxel][16]
  float* outg = nullptr;   // output layer after its gate, [voxel][16]
  float* outp = nullptr;   // projected output y = S outg, [voxel][kOut]
  float* resid = nullptr;  // y - target, [voxel][kOut]
  float* vert = nullptr;   // one value per mesh vertex
  float* dloss = nullptr;
  int* status = nullptr;   // bit 0: a convolution's bounded wait ran out
  int* status_host = nullptr;  // page-locked copy, read after each synchronisation
  long step = 0;
  cudaStream_t stream = nullptr;
  // the forward as a CUDA graph on a caller's stream (cnn_forward_on): the
  // buffers it was recorded with, and the calls seen with them
  cudaGraphExec_t fwd_exec = nullptr;
  const float* fwd_in = nullptr;
  float* fwd_out = nullptr;
  int fwd_calls = 0;
  cudaEvent_t fwd_ev[2] = {nullptr, nullptr};
  std::string err;
  std::vector<void*> allocs;
};

namespace {

enum { A0, B0, A1, B1, A2, B2, C1, D1, C0, OUT };

int cnn_fail(ouranos_cnn* n, cudaError_t e, const char* what) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  n->err = buf;
  return OURANOS_ERR_CUDA;
}
#define CN(expr, what)                                      \
  do {                                                      \
    cudaError_t _e = (expr);                                \
    if (_e != cudaSuccess) return cnn_fail(net, _e, what);  \
  } while (0)

template <class T>
cudaError_t dalloc(ouranos_cnn* net, T** p, size_t count) {
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
  if (e == cudaSuccess) {
    net->allocs.push_back(*p);
    cudaMemset(*p, 0, sizeof(T) * (count ? count : 1));
  }
  return e;
}

const __nv_bfloat16* wf_of(const ouranos_cnn* n, int l) { return n->wf + n->L[l].woff; }
const __nv_bfloat16* wb_of(const ouranos_cnn* n, int l) { return n->wb + n->L[l].woff; }

int refresh_copies(ouranos_cnn* net) {
  for (const Layer& l : net->L)
    weight_copies_kernel<<<blocks_for(27L * l.cin * l.cout), 256, 0, net->stream>>>(
        net->w + l.woff, l.cin, l.cout, net->wf + l.woff, net->wb + l.woff);
  CN(cudaGetLastError(), "weight copies");
  return OURANOS_OK;
}

constexpr long long kConvWaitNs = 2000000000LL;  // bound of a convolution's waits

int conv_call(ouranos_cnn* net, cudaError_t e, const std::string& what) {
  if (e == cudaSuccess) return OURANOS_OK;
  if (net->err.empty() || net->err.compare(0, 12, "convolution:") != 0) net->err = what;
  return cnn_fail(net, e, net->err.c_str());
}

// layer l on `in`: o_l = W_l * in and the gated activation into `out`, one launch
int conv_layer(ouranos_cnn* net, int l, const __nv_bfloat16* in, __nv_bfloat16* out) {
  const Layer& L = net->L[l];
  net->err.clear();
  return conv_call(net,
                   cnn::conv3_tc(L.cin, L.cout, L.grid, in, wf_of(net, l), net->mat[L.level], net->gt + L.goff,
                                 net->o[l], out, nullptr, nullptr, net->status, kConvWaitNs, net->stream, &net->err),
                   "conv forward");
}

// bounded waits of the convolutions since the last call: the status word
// travels with the caller's final copy, one synchronisation for both
int conv_status(ouranos_cnn* net, bool sync = true) {
  if (sync) {
    CN(cudaMemcpyAsync(net->status_host, net->status, sizeof(int), cudaMemcpyDeviceToHost, net->stream), "status");
    CN(cudaStreamSynchronize(net->stream), "status");
  }
  const int st = *net->status_host;
  if (st) {
    *net->status_host = 0;
    CN(cudaMemsetAsync(net->status, 0, sizeof(int), net->stream), "status");
    net->err = "convolution: a tensor-core wait timed out";
    return OURANOS_ERR_TIMEOUT;
  }
  return OURANOS_OK;
}

int forward(ouranos_cnn* net, const float* feat) {
  cudaStream_t s = net->stream;
  const long V0 = net->g0.voxels();
  features_kernel<<<blocks_for(V0), 256, 0, s>>>(feat, net->x0, net->mat[0], V0);
  mat_pool_kernel<<<blocks_for(net->g1.voxels()), 256, 0, s>>>(net->g0, net->mat[0], net->mat[1]);
  mat_pool_kernel<<<blocks_for(net->g2.voxels()), 256, 0, s>>>(net->g1, net->mat[1], net->mat[2]);
  int rc;
  if ((rc = conv_layer(net, A0, net->x0, net->ha0)) || (rc = conv_layer(net, B0, net->ha0, net->s0)))
    return rc;
  pool_kernel<<<blocks_for(net->g1.voxels() * 2), 256, 0, s>>>(net->g0, net->s0, net->p0, 16);
  if ((rc = conv_layer(net, A1, net->p0, net->ha1)) || (rc = conv_layer(net, B1, net->ha1, net->s1)))
    return rc;
  pool_kernel<<<blocks_for(net->g2.voxels() * 4), 256, 0, s>>>(net->g1, net->s1, net->p1, 32);
  if ((rc = conv_layer(net, A2, net->p1, net->ha2)) || (rc = conv_layer(net, B2, net->ha2, net->hb2)))
    return rc;
  up_add_kernel<<<blocks_for(net->g1.voxels() * 4), 256, 0, s>>>(net->g1, net->hb2, net->s1, net->u1, 32);
  if ((rc = conv_layer(net, C1, net->u1, net->hc1)) || (rc = conv_layer(net, D1, net->hc1, net->hd1)))
    return rc;
  up_add_kernel<<<blocks_for(V0 * 2), 256, 0, s>>>(net->g0, net->hd1, net->s0, net->u0, 16);
  if ((rc = conv_layer(net, C0, net->u0, net->hc0))) return rc;
  const Layer& LO = net->L[OUT];
  if ((rc = conv_call(net,
                      cnn::conv3_tc(LO.cin, LO.cout, LO.grid, net->hc0, wf_of(net, OUT), net->mat[0],
                                    net->gt + LO.goff, nullptr, nullptr, net->out, net->outg, net->status,
                                    kConvWaitNs, s, &net->err),
                      "conv forward")))
    return rc;
  const long NV = ouranos::cnn::n_vertices(net->g0);
  ouranos::cnn::vertex_average_kernel<<<blocks_for(NV), 256, 0, s>>>(net->g0, net->outg, 16, 1.f, net->vert);
  ouranos::cnn::vertex_scatter_kernel<<<blocks_for(V0), 256, 0, s>>>(net->g0, net->vert, net->outp);
  CN(cudaGetLastError(), "forward");
  return OURANOS_OK;
}

// gradient of conv layer l: given the gradient g_o of its pre-gate output,
// accumulate its weight gradients and, if g_in is not NULL, produce the input
// gradient
int conv_backward(ouranos_cnn* net, int l, const __nv_bfloat16* in, const __nv_bfloat16* g_o,
                  __nv_bfloat16* g_in) {
  const Layer& L = net->L[l];
  net->err.clear();
  int rc = conv_call(net,
                     cnn::conv3_wgrad_tc(L.cin, L.cout, L.grid, in, g_o, net->dw + L.woff, net->status, kConvWaitNs,
                                         net->stream),
                     "weight gradient");
  if (rc) return rc;
  if (g_in) {
    rc = conv_call(net,
                   cnn::conv3_tc(L.cout, L.cin, L.grid, g_o, wb_of(net, l), nullptr, nullptr, g_in, nullptr, nullptr,
                                 nullptr, net->status, kConvWaitNs, net->stream, &net->err),
                   "data gradient");
    if (rc) return rc;
  }
  return OURANOS_OK;
}

// gate backward of layer l in place: g (gradient of the gated activation)
// becomes the gradient of the pre-gate output; gate gradients accumulate
int gate_backward(ouranos_cnn* net, int l, __nv_bfloat16* g) {
  const Layer& L = net->L[l];
  gate_bwd_kernel<__nv_bfloat16><<<blocks_for(L.grid.voxels() * L.cout), 256, 0, net->stream>>>(
      g, net->o[l], net->mat[L.level], net->gt + L.goff, L.cout, L.grid.voxels(), g, net->dgt + L.goff);
  CN(cudaGetLastError(), "gate gradient");
  return OURANOS_OK;
}

int backward(ouranos_cnn* net, const float* target, float* loss_host) {
  cudaStream_t s = net->stream;
  const long V0 = net->g0.voxels(), V1 = net->g1.voxels(), V2 = net->g2.voxels();
  CN(cudaMemsetAsync(net->dw, 0, sizeof(float) * net->n_w, s), "zero grads");
  CN(cudaMemsetAsync(net->dgt, 0, sizeof(float) * net->n_g, s), "zero grads");
  CN(cudaMemsetAsync(net->dloss, 0, sizeof(float), s), "zero loss");
  const long n_out = V0 * kOut;
  resid_kernel<<<blocks_for(n_out), 256, 0, s>>>(net->outp, target, n_out, net->resid, net->dloss);
  ouranos::cnn::vertex_average_kernel<<<blocks_for(ouranos::cnn::n_vertices(net->g0)), 256, 0, s>>>(
      net->g0, net->resid, kOut, 2.f / (float)n_out, net->vert);
  grad_scatter_kernel<<<blocks_for(V0 * 16), 256, 0, s>>>(net->g0, net->vert, net->gout);  // d outg
  const Layer& LO = net->L[OUT];
  gate_bwd_kernel<float><<<blocks_for(V0 * 16), 256, 0, s>>>(net->gout, net->out, net->mat[0],
                                                             net->gt + LO.goff, 16, V0, net->gout,
                                                             net->dgt + LO.goff);
  int rc;
  __nv_bfloat16 *ga = net->ga, *gb = net->gb_, *gc = net->gc;
  if ((rc = conv_backward(net, OUT, net->hc0, net->gout, ga))) return rc;     // ga = d hc0
  if ((rc = gate_backward(net, C0, ga))) return rc;
  if ((rc = conv_backward(net, C0, net->u0, ga, gb))) return rc;              // gb = d u0
  CN(cudaMemcpyAsync(net->gskip0, gb, sizeof(__nv_bfloat16) * V0 * 16, cudaMemcpyDeviceToDevice, s), "skip");
  up_bwd_kernel<<<blocks_for(V1 * 16), 256, 0, s>>>(net->g0, gb, ga, 16);     // ga = d hd1
  if ((rc = gate_backward(net, D1, ga))) return rc;
  if ((rc = conv_backward(net, D1, net->hc1, ga, gb))) return rc;             // gb = d hc1
  if ((rc = gate_backward(net, C1, gb))) return rc;
  if ((rc = conv_backward(net, C1, net->u1, gb, ga))) return rc;              // ga = d u1
  CN(cudaMemcpyAsync(net->gskip1, ga, sizeof(__nv_bfloat16) * V1 * 32, cudaMemcpyDeviceToDevice, s), "skip");
  up_bwd_kernel<<<blocks_for(V2 * 32), 256, 0, s>>>(net->g1, ga, gb, 32);     // gb = d hb2
  if ((rc = gate_backward(net, B2, gb))) return rc;
  if ((rc = conv_backward(net, B2, net->ha2, gb, ga))) return rc;             // ga = d ha2
  if ((rc = gate_backward(net, A2, ga))) return rc;
  if ((rc = conv_backward(net, A2, net->p1, ga, gb))) return rc;              // gb = d p1
  pool_bwd_kernel<<<blocks_for(V1 * 32), 256, 0, s>>>(net->g1, gb, gc, 32);   // gc = d s1 (pool path)
  add_kernel<<<blocks_for(V1 * 32), 256, 0, s>>>(gc, net->gskip1, gc, V1 * 32);
  if ((rc = gate_backward(net, B1, gc))) return rc;
  if ((rc = conv_backward(net, B1, net->ha1, gc, ga))) return rc;             // ga = d ha1
  if ((rc = gate_backward(net, A1, ga))) return rc;
  if ((rc = conv_backward(net, A1, net->p0, ga, gb))) return rc;              // gb = d p0
  pool_bwd_kernel<<<blocks_for(V0 * 16), 256, 0, s>>>(net->g0, gb, gc, 16);   // gc = d s0 (pool path)
  add_kernel<<<blocks_for(V0 * 16), 256, 0, s>>>(gc, net->gskip0, gc, V0 * 16);
  if ((rc = gate_backward(net, B0, gc))) return rc;
  if ((rc = conv_backward(net, B0, net->ha0, gc, ga))) return rc;             // ga = d ha0
  if ((rc = gate_backward(net, A0, ga))) return rc;
  if ((rc = conv_backward(net, A0, net->x0, ga, nullptr))) return rc;
  CN(cudaGetLastError(), "backward");
  // the convolutions' status travels with the loss (one synchronisation)
  CN(cudaMemcpyAsync(net->status_host, net->status, sizeof(int), cudaMemcpyDeviceToHost, s), "status");
  if (loss_host) {
    CN(cudaMemcpyAsync(loss_host, net->dloss, sizeof(float), cudaMemcpyDeviceToHost, s), "loss");
    CN(cudaStreamSynchronize(s), "loss");
  }
  return OURANOS_OK;
}

}  // namespace

namespace ouranos {
void cnn_grid(const ouranos_cnn* net, int* nx, int* ny, int* nz) {
  *nx = net->g0.nx;
  *ny = net->g0.ny;
  *nz = net->g0.nz;
}

void cnn_forward_release(ouranos_cnn* net) {
  if (!net) return;
  if (net->fwd_exec) {
    cudaEventSynchronize(net->fwd_ev[1]);  // the last launch of the graph has ended
    cudaGraphExecDestroy(net->fwd_exec);
  }
  net->fwd_exec = nullptr;
  net->fwd_in = nullptr;
  net->fwd_out = nullptr;
  net->fwd_calls = 0;
}

int cnn_forward_on(ouranos_cnn* net, const float* features, float* out, cudaStream_t s) {
  if (!net || !features || !out) return OURANOS_ERR_BAD_INPUT;
  if (features != net->fwd_in || out != net->fwd_out) {
    cnn_forward_release(net);
    net->fwd_in = features;
    net->fwd_out = out;
  }
  if (!net->fwd_exec && net->fwd_calls > 0) {
    // second call with these buffers: every kernel is configured, record the
    // launches and the two copies (nothing runs during the recording)
    CN(cudaStreamBeginCapture(net->stream, cudaStreamCaptureModeThreadLocal), "forward capture");
    int rc = forward(net, features);
    if (!rc) {
      const cudaError_t e1 = cudaMemcpyAsync(out, net->outp, sizeof(float) * kOut * net->g0.voxels(),
                                             cudaMemcpyDeviceToDevice, net->stream);
      const cudaError_t e2 = cudaMemcpyAsync(net->status_host, net->status, sizeof(int), cudaMemcpyDeviceToHost,
                                             net->stream);
      if (e1 != cudaSuccess || e2 != cudaSuccess) rc = cnn_fail(net, e1 != cudaSuccess ? e1 : e2, "forward capture");
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(net->stream, &graph);
    if (!rc && e == cudaSuccess) {
      const cudaError_t ei = cudaGraphInstantiate(&net->fwd_exec, graph, 0);
      if (ei != cudaSuccess) {
        net->fwd_exec = nullptr;
        rc = cnn_fail(net, ei, "forward graph");
      }
    } else if (!rc) {
      rc = cnn_fail(net, e, "forward capture");
    }
    if (graph) cudaGraphDestroy(graph);
    if (rc) return rc;
  }
  if (net->fwd_exec) {
    CN(cudaGraphLaunch(net->fwd_exec, s), "forward graph");
    CN(cudaEventRecord(net->fwd_ev[1], s), "forward graph");
  } else {
    // first call: the launches run (and configure their kernels) on the
    // network's stream, between events that order them after and before s
    for (cudaEvent_t& ev : net->fwd_ev)
      if (!ev) CN(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "forward");
    CN(cudaEventRecord(net->fwd_ev[0], s), "forward");
    CN(cudaStreamWaitEvent(net->stream, net->fwd_ev[0], 0), "forward");
    int rc = forward(net, features);
    if (rc) return rc;
    CN(cudaMemcpyAsync(out, net->outp, sizeof(float) * kOut * net->g0.voxels(), cudaMemcpyDeviceToDevice,
                       net->stream),
       "output");
    CN(cudaMemcpyAsync(net->status_host, net->status, sizeof(int), cudaMemcpyDeviceToHost, net->stream), "status");
    CN(cudaEventRecord(net->fwd_ev[1], net->stream), "forward");
    CN(cudaStreamWaitEvent(s, net->fwd_ev[1], 0), "forward");
  }
  ++net->fwd_calls;
  return OURANOS_OK;
}

int cnn_forward_status(ouranos_cnn* net) { return net ? conv_status(net, false) : OURANOS_OK; }
}  // namespace ouranos

// ---------------------------------------------------------------- C-ABI
extern "C" {

int ouranos_cnn_create(int nx, int ny, int nz, unsigned long long seed, ouranos_cnn** out) {
  if (!out) return OURANOS_ERR_BAD_INPUT;
  *out = nullptr;
  if (nx < 4 || ny < 4 || nz < 4 || nx % 4 || ny % 4 || nz % 4) return OURANOS_ERR_BAD_INPUT;
  ouranos_cnn* net = new ouranos_cnn();
  *out = net;
  net->g0 = {nx, ny, nz};
  net->g1 = {nx / 2, ny / 2, nz / 2};
  net->g2 = {nx / 4, ny / 4, nz / 4};
  struct Spec { int cin, cout, level; };
  const Spec spec[] = {{16, 16, 0}, {16, 16, 0}, {16, 32, 1}, {32, 32, 1}, {32, 32, 2},
                       {32, 32, 2}, {32, 32, 1}, {32, 16, 1}, {16, 16, 0}, {16, 16, 0}};
  const Grid grids[3] = {net->g0, net->g1, net->g2};
  for (const Spec& sp : spec) {
    Layer l{sp.cin, sp.cout, sp.level, grids[sp.level], net->n_w, net->n_g};
    net->n_w += 27L * sp.cin * sp.cout;
    net->n_g += 3L * sp.cout;
    net->L.push_back(l);
  }
  // blocking: ordered against the legacy default stream the caller's tensors
  // are usually written on
  if (cudaStreamCreateWithFlags(&net->stream, cudaStreamDefault) != cudaSuccess)
    return cnn_fail(net, cudaGetLastError(), "stream");
  const long V0 = net->g0.voxels(), V1 = net->g1.voxels(), V2 = net->g2.voxels();
  CN(dalloc(net, &net->status, 1), "status");
  CN(cudaMallocHost((void**)&net->status_host, sizeof(int)), "status");
  *net->status_host = 0;
  CN(dalloc(net, &net->w, net->n_w), "params");
  CN(dalloc(net, &net->gt, net->n_g), "params");
  CN(dalloc(net, &net->dw, net->n_w), "grads");
  CN(dalloc(net, &net->dgt, net->n_g), "grads");
  CN(dalloc(net, &net->mw, net->n_w), "adam");
  CN(dalloc(net, &net->vw, net->n_w), "adam");
  CN(dalloc(net, &net->mg, net->n_g), "adam");
  CN(dalloc(net, &net->vg, net->n_g), "adam");
  CN(dalloc(net, &net->wf, net->n_w), "weights");
  CN(dalloc(net, &net->wb, net->n_w), "weights");
  __nv_bfloat16** a16[] = {&net->x0, &net->ha0, &net->s0, &net->u0, &net->hc0};
  for (auto p : a16) CN(dalloc(net, p, V0 * 16), "activations");
  CN(dalloc(net, &net->p0, V1 * 16), "activations");
  CN(dalloc(net, &net->hd1, V1 * 16), "activations");
  __nv_bfloat16** a1[] = {&net->ha1, &net->s1, &net->u1, &net->hc1};
  for (auto p : a1) CN(dalloc(net, p, V1 * 32), "activations");
  CN(dalloc(net, &net->p1, V2 * 32), "activations");
  CN(dalloc(net, &net->ha2, V2 * 32), "activations");
  CN(dalloc(net, &net->hb2, V2 * 32), "activations");
  for (int l = A0; l < OUT; ++l) CN(dalloc(net, &net->o[l], net->L[l].grid.voxels() * net->L[l].cout), "activations");
  for (int k = 0; k < 3; ++k) CN(dalloc(net, &net->mat[k], grids[k].voxels()), "materials");
  const long gmax = V0 * 16 > V1 * 32 ? V0 * 16 : V1 * 32;
  CN(dalloc(net, &net->ga, gmax), "gradients");
  CN(dalloc(net, &net->gb_, gmax), "gradients");
  CN(dalloc(net, &net->gc, gmax), "gradients");
  CN(dalloc(net, &net->gskip0, V0 * 16), "gradients");
  CN(dalloc(net, &net->gskip1, V1 * 32), "gradients");
  CN(dalloc(net, &net->gout, V0 * 16), "gradients");
  CN(dalloc(net, &net->out, V0 * 16), "output");
  CN(dalloc(net, &net->outg, V0 * 16), "output");
  CN(dalloc(net, &net->outp, V0 * kOut), "output");
  CN(dalloc(net, &net->resid, V0 * kOut), "output");
  CN(dalloc(net, &net->vert, ouranos::cnn::n_vertices(net->g0)), "output");
  CN(dalloc(net, &net->dloss, 1), "loss");
  // weights: normal with variance 1/fan_in (a linear network keeps the signal
  // scale), the output layer 0.1x so the initial correction is small; gates
  // start at gamma = 1.  SplitMix64 stream, Box-Muller.
  std::vector<float> w(net->n_w, 0.f), gt(net->n_g, 0.f);
  unsigned long long st = seed;
  auto next = [&]() {
    st += 0x9E3779B97F4A7C15ull;
    unsigned long long z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  };
  for (size_t li = 0; li < net->L.size(); ++li) {
    const Layer& l = net->L[li];
    const double sd = std::sqrt(1.0 / (27.0 * l.cin)) * (li == OUT ? 0.1 : 1.0);
    for (long k = 0; k < 27L * l.cin * l.cout; ++k) {
      const double u1 = next(), u2 = next();
      w[l.woff + k] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2));
    }
    for (int c = 0; c < l.cout; ++c) gt[l.goff + 3 * c] = 1.f;
  }
  CN(cudaMemcpy(net->w, w.data(), sizeof(float) * net->n_w, cudaMemcpyHostToDevice), "params");
  CN(cudaMemcpy(net->gt, gt.data(), sizeof(float) * net->n_g, cudaMemcpyHostToDevice), "params");
  int rc = refresh_copies(net);
  if (rc) return rc;
  CN(cudaStreamSynchronize(net->stream), "init");
  return OURANOS_OK;
}

int ouranos_cnn_destroy(ouranos_cnn* net) {
  if (!net) return OURANOS_OK;
  if (net->stream) cudaStreamSynchronize(net->stream);
  cnn_forward_release(net);
  for (cudaEvent_t ev : net->fwd_ev)
    if (ev) cudaEventDestroy(ev);
  for (void* p : net->allocs) cudaFree(p);
  if (net->status_host) cudaFreeHost(net->status_host);
  if (net->stream) cudaStreamDestroy(net->stream);
  delete net;
  return OURANOS_OK;
}

int ouranos_cnn_n_params(const ouranos_cnn* net, long* n) {
  if (!net || !n) return OURANOS_ERR_BAD_INPUT;
  *n = (long)(net->n_w + net->n_g);
  return OURANOS_OK;
}

// parameter vector: all conv weights ([tap][cin][cout] per layer, layers in
// order), then all gate coefficients ([cout][3] per layer)
int ouranos_cnn_get_params(const ouranos_cnn* cnet, float* host) {
  ouranos_cnn* net = const_cast<ouranos_cnn*>(cnet);
  if (!net || !host) return OURANOS_ERR_BAD_INPUT;
  CN(cudaStreamSynchronize(net->stream), "params");
  CN(cudaMemcpy(host, net->w, sizeof(float) * net->n_w, cudaMemcpyDeviceToHost), "params");
  CN(cudaMemcpy(host + net->n_w, net->gt, sizeof(float) * net->n_g, cudaMemcpyDeviceToHost), "params");
  return OURANOS_OK;
}

int ouranos_cnn_set_params(ouranos_cnn* net, const float* host) {
  if (!net || !host) return OURANOS_ERR_BAD_INPUT;
  CN(cudaStreamSynchronize(net->stream), "params");
  CN(cudaMemcpy(net->w, host, sizeof(float) * net->n_w, cudaMemcpyHostToDevice), "params");
  CN(cudaMemcpy(net->gt, host + net->n_w, sizeof(float) * net->n_g, cudaMemcpyHostToDevice), "params");
  int rc = refresh_copies(net);
  if (rc) return rc;
  CN(cudaStreamSynchronize(net->stream), "params");
  return OURANOS_OK;
}

// features: device [voxel][kFeatures] FP32; out: device [voxel][kOut] FP32
int ouranos_cnn_forward(ouranos_cnn* net, const float* features, float* out) {
  if (!net || !features || !out) return OURANOS_ERR_BAD_INPUT;
  int rc = forward(net, features);
  if (rc) return rc;
  CN(cudaMemcpyAsync(out, net->outp, sizeof(float) * kOut * net->g0.voxels(), cudaMemcpyDeviceToDevice,
                     net->stream),
     "output");
  CN(cudaMemcpyAsync(net->status_host, net->status, sizeof(int), cudaMemcpyDeviceToHost, net->stream), "status");
  CN(cudaStreamSynchronize(net->stream), "forward");
  return conv_status(net, false);
}

// loss and gradients without an update; grads_host (may be NULL) receives [n_params]
int ouranos_cnn_gradients(ouranos_cnn* net, const float* features, const float* target,
                          float* grads_host, float* loss) {
  if (!net || !features || !target) return OURANOS_ERR_BAD_INPUT;
  int rc;
  if ((rc = forward(net, features)) || (rc = backward(net, target, loss)) || (rc = conv_status(net, !loss)))
    return rc;
  if (grads_host) {
    CN(cudaStreamSynchronize(net->stream), "grads");
    CN(cudaMemcpy(grads_host, net->dw, sizeof(float) * net->n_w, cudaMemcpyDeviceToHost), "grads");
    CN(cudaMemcpy(grads_host + net->n_w, net->dgt, sizeof(float) * net->n_g, cudaMemcpyDeviceToHost), "grads");
  }
  return OURANOS_OK;
}

// one Adam step on the MSE loss of (features -> target)
int ouranos_cnn_train_step(ouranos_cnn* net, const float* features, const float* target, float lr,
                           float* loss) {
  if (!net || !features || !target || !(lr > 0)) return OURANOS_ERR_BAD_INPUT;
  int rc;
  if ((rc = forward(net, features)) || (rc = backward(net, target, loss))) return rc;
  ++net->step;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - std::pow(b1, (float)net->step), c2 = 1.f - std::pow(b2, (float)net->step);
  adam_kernel<<<blocks_for(net->n_w), 256, 0, net->stream>>>(net->w, net->dw, net->mw, net->vw, net->n_w, lr, b1, b2, eps, c1, c2);
  // gates multiply through all ten layers: a tenth of the weights' step
  adam_kernel<<<blocks_for(net->n_g), 256, 0, net->stream>>>(net->gt, net->dgt, net->mg, net->vg, net->n_g, 0.1f * lr, b1, b2, eps, c1, c2);
  CN(cudaGetLastError(), "adam");
  if ((rc = refresh_copies(net))) return rc;
  // with a loss the stream was synchronised inside backward; without one the
  // status is read at the next synchronising call
  return loss ? conv_status(net, false) : OURANOS_OK;
}

int ouranos_cnn_last_error(const ouranos_cnn* net, char* buf, size_t len) {
  if (!net || !buf || !len) return OURANOS_ERR_BAD_INPUT;
  std::snprintf(buf, len, "%s", net->err.c_str());
  return OURANOS_OK;
}

}  // extern "C"
