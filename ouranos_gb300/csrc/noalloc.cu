// Apply without device allocation.
//
// Some callers cannot allocate device memory at the moment they apply the
// operator: a solver framework that owns the device memory pool and forbids
// allocations inside its operator callbacks, or a driver that allows
// allocations only during set-up.  ouranos_rt_apply allocates its work buffers
// lazily on first use; this entry point instead places every scratch buffer of
// one Apply -- the scattering source, the expanded source, the angular flux,
// the flux moments, the tile edge buffers, the ticket/status words and (for a
// caller cell order) the permuted vectors -- in one file-scope device array of
// kNoAllocScratchBytes.  Every GPU that loads the library holds that array
// until the process exits.
//
// Host code may not use the array's name as a device address: set-up looks
// the address up with cudaGetSymbolAddress, once per device, with that device
// current, and caches it.  Set-up runs inside ouranos_rt_create (under CUDA's
// lazy module loading that lookup is also what places the array on the
// device), so the entry point itself only reads the cached address.  It runs
// the kernels of ouranos_rt_apply for the handle's arithmetic, with the same
// launch shapes, so its result is the same bit for bit.  All calls share the
// array and it keeps the previous call's contents: the ticket/status words
// and the edge buffers are cleared at the start of every call, everything
// else is fully overwritten before it is read.  Calls whose GPU work overlaps
// (two streams, two threads, two handles) race on the array.
#include <algorithm>
#include <cstdio>
#include <mutex>
#include <type_traits>

#include "internal.h"

using namespace ouranos;

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;  // 32 MiB
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

int fail(ouranos_rt* rt, int code, const char* msg) {
  rt->err = msg;
  return code;
}
int cfail(ouranos_rt* rt, cudaError_t e, const char* what) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  rt->err = buf;
  return OURANOS_ERR_CUDA;
}
#define NA_CU(expr, what)                               \
  do {                                                  \
    cudaError_t _e = (expr);                            \
    if (_e != cudaSuccess) return cfail(rt, _e, what);  \
  } while (0)

bool on_device(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Byte layout of one Apply's scratch inside the array.
struct Layout {
  size_t ctrl, T, q, psi, phi, edge_x, edge_y, xin, yout, total;
  size_t edge_x_bytes, edge_y_bytes;
};

Layout layout_for(const ouranos_rt* rt, size_t real_bytes, bool expand) {
  Layout L;
  const size_t nd = rt->n_dofs;
  const size_t tiles = (size_t)rt->tiles_x * rt->tiles_y;
  const size_t NS = rt->nx[rt->dim - 1];
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off += round256(bytes);
    return at;
  };
  L.ctrl = take(256);
  L.T = take(real_bytes * rt->n_mom * nd);
  L.q = expand ? take(real_bytes * rt->n_dir * nd) : 0;
  L.psi = take(real_bytes * rt->n_dir * nd);
  L.phi = take(real_bytes * rt->n_mom * nd);
  // two tagged 64-bit words per edge value cover both precisions
  L.edge_x_bytes = 16 * (size_t)rt->n_dir * tiles * NS * rt->wy * rt->fd;
  L.edge_y_bytes = rt->dim == 3 ? 16 * (size_t)rt->n_dir * tiles * NS * rt->wx * rt->fd : 16;
  L.edge_x = take(L.edge_x_bytes);
  L.edge_y = take(L.edge_y_bytes);
  const bool perm = !rt->cell_order.empty();
  L.xin = perm ? take(8 * (size_t)rt->n_mom * nd) : 0;
  L.yout = perm ? take(8 * (size_t)rt->n_mom * nd) : 0;
  L.total = off;
  return L;
}

// the table of the sweep's arithmetic type (as the regular Apply reads them)
template <typename real>
const real* tbl(const DevBuf& b64, const DevBuf& b32, const DevBuf& bdf) {
  if constexpr (std::is_same<real, float>::value) return (const real*)b32.p;
  else if constexpr (std::is_same<real, df64>::value) return (const real*)bdf.p;
  else return (const real*)b64.p;
}

// q = M2D T in the contraction form of the regular Apply for this arithmetic
template <typename real>
cudaError_t expand(const ouranos_rt* rt, const real* T, real* q, int* status, cudaStream_t st) {
  const long nd = rt->n_dofs;
  if constexpr (std::is_same<real, df64>::value) {
    if (rt->fp64_contract == OURANOS_FP64_DF64_SWEEP_TC)
      return launch_expand_oz(T, nullptr, rt->oz, q, nd, status, rt->wait_limit_ns, st);
    if (rt->sym.n_class) return launch_expand_sym_pairs(T, nullptr, rt->sym, q, rt->n_mom, nd, st);
    return launch_expand_source_pairs(T, nullptr, rt->d_m2d64.as<double>(), q, rt->n_dir, rt->n_mom, nd, st);
  } else if constexpr (std::is_same<real, double>::value) {
    if (rt->fp64_contract != OURANOS_FP64_NATIVE)
      return launch_expand_source_df64(T, nullptr, rt->d_m2d64.as<double>(), q, rt->n_dir, rt->n_mom, nd, st);
    return launch_expand_source<double>(T, nullptr, rt->d_m2d64.as<double>(), q, rt->n_dir, rt->n_mom, nd, st);
  } else {
    if (rt->fp32_contract == OURANOS_FP32_CONTRACT_TENSOR)
      return launch_expand_tc(T, nullptr, rt->tc, q, nd, status, rt->wait_limit_ns, st);
    return launch_expand_source<float>(T, nullptr, rt->d_m2d32.as<float>(), q, rt->n_dir, rt->n_mom, nd, st);
  }
}

// phi = D2M psi, likewise; phi is float for the FP32 sweep, double otherwise
template <typename real>
cudaError_t reduce(const ouranos_rt* rt, const real* psi, void* phi, int* status, cudaStream_t st) {
  const long nd = rt->n_dofs;
  if constexpr (std::is_same<real, df64>::value) {
    if (rt->fp64_contract == OURANOS_FP64_DF64_SWEEP_TC)
      return launch_reduce_oz(psi, rt->oz, (double*)phi, nd, status, rt->wait_limit_ns, st);
    if (rt->sym.n_class) return launch_reduce_sym_pairs(psi, rt->sym, (double*)phi, rt->n_mom, nd, st);
    return launch_reduce_moments_pairs(psi, rt->d_d2m64.as<double>(), (double*)phi, rt->n_dir, rt->n_mom, nd, st);
  } else if constexpr (std::is_same<real, double>::value) {
    if (rt->fp64_contract != OURANOS_FP64_NATIVE)
      return launch_reduce_moments_df64(psi, rt->d_d2m64.as<double>(), (double*)phi, rt->n_dir, rt->n_mom, nd,
                                        st);
    return launch_reduce_moments<double>(psi, rt->d_d2m64.as<double>(), (double*)phi, rt->n_dir, rt->n_mom, nd,
                                         st);
  } else {
    if (rt->fp32_contract == OURANOS_FP32_CONTRACT_TENSOR)
      return launch_reduce_tc(psi, rt->tc, (float*)phi, nd, status, rt->wait_limit_ns, st);
    return launch_reduce_moments<float>(psi, rt->d_d2m32.as<float>(), (float*)phi, rt->n_dir, rt->n_mom, nd, st);
  }
}

// real: float (FP32 sweep), double (FP64 sweep) or df64 (double-float sweep,
// sources and angular fluxes stored as pairs)
template <typename real>
int apply_noalloc(ouranos_rt* rt, unsigned char* base, const Layout& L, bool expand_source,
                  const double* x, double* y) {
  const long len = (long)rt->n_mom * rt->n_dofs;
  cudaStream_t st = rt->stream;
  int* ctrl = reinterpret_cast<int*>(base + L.ctrl);
  real* T = reinterpret_cast<real*>(base + L.T);
  real* q = expand_source ? reinterpret_cast<real*>(base + L.q) : nullptr;
  real* psi = reinterpret_cast<real*>(base + L.psi);
  void* phi = base + L.phi;
  // the array keeps the last call's contents: clear what must start at zero
  NA_CU(cudaMemsetAsync(ctrl, 0, 256, st), "clear control words");
  NA_CU(cudaMemsetAsync(base + L.edge_x, 0, L.edge_x_bytes, st), "clear edge buffer");
  NA_CU(cudaMemsetAsync(base + L.edge_y, 0, L.edge_y_bytes, st), "clear edge buffer");
  const double* xd = x;
  double* yd = y;
  if (!rt->cell_order.empty()) {
    double* xin = reinterpret_cast<double*>(base + L.xin);
    NA_CU(launch_permute(x, xin, rt->d_cell_order.as<long>(), rt->n_cells, rt->n, rt->n_mom, 1, st),
          "permute in");
    xd = xin;
    yd = reinterpret_cast<double*>(base + L.yout);
  }
  NA_CU(launch_scatter_source<real>(xd, nullptr, T, rt->d_cell_mass.as<double>(),
                                    rt->d_sscale.as<double>(), rt->d_oscale.as<double>(),
                                    rt->d_material.as<int>(), rt->n_mat, rt->G, rt->group,
                                    rt->n_cells, rt->n, rt->n_mom, rt->n_dofs, st),
        "scattering source");
  if (expand_source) NA_CU(expand<real>(rt, T, q, ctrl + 1, st), "source expansion");
  SweepArgs<real> a;
  a.nx = rt->nx[0];
  a.ny = rt->nx[1];
  a.nz = rt->nx[2];
  a.n_sweep = rt->nx[rt->dim - 1];
  a.n_dofs = rt->n_dofs;
  a.n_mom = rt->n_mom;
  a.wx = rt->wx;
  a.wy = rt->wy;
  a.kd = rt->kd;
  a.lpc = rt->lpc;
  a.tiles_x = rt->tiles_x;
  a.tiles_y = rt->tiles_y;
  a.n_tasks = rt->n_tasks;
  a.tasks = rt->d_tasks.as<int2>();
  a.group_dirs = rt->d_group_dirs.as<int>();
  a.group_flip = rt->d_group_flip.as<int>();
  a.dir_class = rt->d_dir_class.as<int>();
  a.n_dir_class = rt->n_dir_class;
  a.abs_omega = tbl<real>(rt->d_abs64, rt->d_abs32, rt->d_absdf);
  a.m2d = tbl<real>(rt->d_m2d64, rt->d_m2d32, rt->d_m2ddf);
  a.ainv = tbl<real>(rt->d_ainv64, rt->d_ainv32, rt->d_ainvdf);
  a.cell_class = rt->d_cell_class.as<int>();
  a.face_mass = tbl<real>(rt->d_face64, rt->d_face32, rt->d_facedf);
  a.src = T;
  a.iso = nullptr;
  a.q = q;
  a.bnd = nullptr;
  a.psi = psi;
  a.edge_x = reinterpret_cast<unsigned long long*>(base + L.edge_x);
  a.edge_y = reinterpret_cast<unsigned long long*>(base + L.edge_y);
  a.epoch = 1;  // the edge buffers were cleared above, so any nonzero epoch is fresh
  a.ticket = ctrl;
  a.status = ctrl + 1;
  a.wait_limit_ns = rt->wait_limit_ns;
  a.wait_bias = rt->wait_bias;
  int sms = 0;
  NA_CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, rt->device), "device query");
  const int grid = std::min((rt->n_tasks + 3) / 4, std::max(1, sms * 8));
  NA_CU(launch_sweep<real>(rt->dim, rt->p1, expand_source ? 0 : rt->n_mom, a, grid, 128, st), "sweep");
  NA_CU(reduce<real>(rt, psi, phi, ctrl + 1, st), "moment reduction");
  if constexpr (std::is_same<real, float>::value)
    NA_CU(launch_combine<float>(xd, (const float*)phi, yd, len, 1.0, -1.0, st), "combine");
  else
    NA_CU(launch_combine<double>(xd, (const double*)phi, yd, len, 1.0, -1.0, st), "combine");
  if (!rt->cell_order.empty())
    NA_CU(launch_permute(yd, y, rt->d_cell_order.as<long>(), rt->n_cells, rt->n, rt->n_mom, 0, st),
          "permute out");
  NA_CU(cudaStreamSynchronize(st), "apply");
  int status = 0;
  NA_CU(cudaMemcpy(&status, ctrl + 1, sizeof(int), cudaMemcpyDeviceToHost), "status");
  if (status)
    return fail(rt, OURANOS_ERR_TIMEOUT,
                (status & 4) ? "tensor-core contraction: MMA completion wait timed out" : "sweep dependency wait timed out");
  return OURANOS_OK;
}

}  // namespace

namespace ouranos {
// Set-up of the allocation-free Apply on the current device (ouranos_rt_create
// calls it once the handle's device is current): look the scratch array's
// device address up once per device and keep it.
int noalloc_setup(int device) {
  if (device < 0 || device >= kMaxDevices) return OURANOS_ERR_BAD_INPUT;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_ptr[device]) return OURANOS_OK;
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return OURANOS_ERR_CUDA;
  g_scratch_ptr[device] = p;
  return OURANOS_OK;
}
}  // namespace ouranos

extern "C" int ouranos_rt_apply_noalloc(ouranos_rt* rt, const double* x, double* y) {
  if (!rt || !x || !y) return OURANOS_ERR_BAD_INPUT;
  if (cudaSetDevice(rt->device) != cudaSuccess) return cfail(rt, cudaGetLastError(), "set device");
  if (!on_device(x) || !on_device(y))
    return fail(rt, OURANOS_ERR_BAD_INPUT,
                "ouranos_rt_apply_noalloc takes device pointers only (no staging buffers)");
  // same form choice as the regular Apply: expand the source when it has more
  // moments than the sweep applies in place
  const bool expand_source = !(rt->n_mom <= 2 && rt->n * (rt->n_mom + 1) <= 32) || rt->lpc == 32;
  // double, and the double-float pairs, take 8 bytes a value
  const size_t rb = rt->precision == OURANOS_FP64 ? 8 : 4;
  const Layout L = layout_for(rt, rb, expand_source);
  if (L.total > kNoAllocScratchBytes) {
    char buf[256];
    std::snprintf(buf, sizeof buf,
                  "problem needs %zu bytes of scratch; the allocation-free Apply holds at most %zu "
                  "(use ouranos_rt_apply)",
                  L.total, kNoAllocScratchBytes);
    return fail(rt, OURANOS_ERR_BAD_INPUT, buf);
  }
  if (rt->device < 0 || rt->device >= kMaxDevices)
    return fail(rt, OURANOS_ERR_BAD_INPUT, "device ordinal out of range");
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    base = g_scratch_ptr[rt->device];
  }
  if (!base)
    return fail(rt, OURANOS_ERR_CUDA, "the scratch array was not set up on this device at handle creation");
  unsigned char* b = (unsigned char*)base;
  if (rt->precision == OURANOS_FP32) return apply_noalloc<float>(rt, b, L, expand_source, x, y);
  if (rt->fp64_contract == OURANOS_FP64_DF64_SWEEP || rt->fp64_contract == OURANOS_FP64_DF64_SWEEP_TC)
    return apply_noalloc<df64>(rt, b, L, expand_source, x, y);
  return apply_noalloc<double>(rt, b, L, expand_source, x, y);
}
