// The transport operator behind the C-ABI: setup (RadiativeTransfer::setup,
// src/RadiativeTransfer.cc:50-78), the sweep launch (the task loop of
// src/RadiativeTransfer.cc:797-803) and Apply (:780-809).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <type_traits>
#include <vector>

#include "internal.h"

using namespace ouranos;

namespace {

#define OK_OR_RETURN(expr)                 \
  do {                                     \
    int _rc = (expr);                      \
    if (_rc != OURANOS_OK) return _rc;     \
  } while (0)

int cuda_fail(ouranos_rt* rt, cudaError_t e, const char* what) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  rt->err = buf;
  return OURANOS_ERR_CUDA;
}
#define CU(expr, what)                                  \
  do {                                                  \
    cudaError_t _e = (expr);                            \
    if (_e != cudaSuccess) return cuda_fail(rt, _e, what); \
  } while (0)

int bad(ouranos_rt* rt, const char* msg) {
  rt->err = msg;
  return OURANOS_ERR_BAD_INPUT;
}

template <class T>
int upload(ouranos_rt* rt, DevBuf& buf, const std::vector<T>& v, const char* what) {
  CU(buf.alloc(sizeof(T) * std::max<size_t>(v.size(), 1)), what);
  if (!v.empty())
    CU(cudaMemcpyAsync(buf.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, rt->stream),
       what);
  return OURANOS_OK;
}

template <class T>
std::vector<float> to_f32(const std::vector<T>& v) {
  return std::vector<float>(v.begin(), v.end());
}

// tables of the double-float sweep: each value as its (hi, lo) float pair
std::vector<df64> to_df(const std::vector<double>& v) {
  std::vector<df64> out(v.size());
  for (size_t k = 0; k < v.size(); ++k) out[k] = df64_split(v[k]);
  return out;
}

// rows x cols -> rows x pad4(cols), zero padding: the sweep's cell tables are
// read a row at a time in 16-byte pieces
std::vector<double> pad_rows(const std::vector<double>& v, long rows, int cols) {
  const int pc = (cols + 3) & ~3;
  std::vector<double> out((size_t)rows * pc, 0.0);
  for (long r = 0; r < rows; ++r)
    for (int c = 0; c < cols; ++c) out[(size_t)r * pc + c] = v[(size_t)r * cols + c];
  return out;
}

// the sweep runs in double-float with pair storage
bool df64_sweep(const ouranos_rt* rt) {
  return rt->precision == OURANOS_FP64 &&
         (rt->fp64_contract == OURANOS_FP64_DF64_SWEEP || rt->fp64_contract == OURANOS_FP64_DF64_SWEEP_TC);
}

// the table of the sweep's arithmetic type
template <typename real>
const real* table(const DevBuf& b64, const DevBuf& b32, const DevBuf& bdf) {
  if (std::is_same<real, float>::value) return (const real*)b32.p;
  if (std::is_same<real, df64>::value) return (const real*)bdf.p;
  return (const real*)b64.p;
}

// page-locked host memory (the copies of it are asynchronous)
bool is_pinned_host_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

long vec_len(const ouranos_rt* rt) { return (long)rt->n_mom * rt->n_dofs; }

// --------------------------------------------------------- octant symmetry
// Classes of P = 2^dim directions with equal |Omega| (member f: Omega_a < 0
// for the bits a of f), and for every moment the sign pattern of its M2D and
// D2M entries over the members, which must be the same in every class (the
// parity of a real spherical harmonic under the axis reflections).  Entries
// count as equal or opposite within 32 ulps of the moment's largest entry
// (harmonics evaluated at reflected angles differ by a few ulps);
// anything else (a quadrature without full octant symmetry, directions on an
// axis plane) leaves the symmetric contractions off.
int build_symmetry(ouranos_rt* rt) {
  rt->sym = SymTables{};
  const int P = 1 << rt->dim, nd = rt->n_dir, nm = rt->n_mom, nc = rt->n_dir_class;
  if (nm > 16 || nd != nc * P) return OURANOS_OK;
  std::vector<int> cls(nc * P, -1);
  for (int d = 0; d < nd; ++d) {
    int f = 0;
    for (int a = 0; a < rt->dim; ++a) {
      if (rt->omega[3 * d + a] == 0.0) return OURANOS_OK;
      if (rt->omega[3 * d + a] < 0.0) f |= 1 << a;
    }
    int& slot = cls[rt->dir_class_h[d] * P + f];
    if (slot >= 0) return OURANOS_OK;
    slot = d;
  }
  for (int v : cls)
    if (v < 0) return OURANOS_OK;
  const double tol = 32.0 * 2.220446049250313e-16;
  auto m2d = [&](int d, int m) { return rt->m2d[(size_t)d * nm + m]; };
  auto d2m = [&](int d, int m) { return rt->d2m[(size_t)m * nd + d]; };
  std::vector<unsigned> group_sign;
  std::vector<int> mom_group(nm, 0);
  for (int m = 0; m < nm; ++m) {
    // bits whose sign some entry pins down (equal or opposite to member 0's
    // within the tolerance), and their values
    unsigned known = 0, value = 0;
    for (int which = 0; which < 2; ++which) {
      auto val = [&](int d) { return which ? d2m(d, m) : m2d(d, m); };
      double scale = 0.0;
      for (int d = 0; d < nd; ++d) scale = std::max(scale, std::fabs(val(d)));
      const double t = tol * scale;
      for (int c = 0; c < nc; ++c) {
        const double a = val(cls[c * P]);
        for (int f = 0; f < P; ++f) {
          const double b = val(cls[c * P + f]);
          const bool eq = std::fabs(b - a) <= t, opp = std::fabs(b + a) <= t;
          if (!eq && !opp) return OURANOS_OK;
          if (eq == opp) continue;  // |a|, |b| below the tolerance: either sign
          const unsigned bit = 1u << f;
          if ((known & bit) && ((value & bit) != 0) != opp) return OURANOS_OK;
          known |= bit;
          if (opp) value |= bit;
        }
      }
    }
    int g = 0;
    while (g < (int)group_sign.size() && group_sign[g] != value) ++g;
    if (g == (int)group_sign.size()) group_sign.push_back(value);
    mom_group[m] = g;
  }
  if ((int)group_sign.size() > P) return OURANOS_OK;
  std::vector<double> m2d_rep((size_t)nc * nm), d2m_rep((size_t)nc * nm);
  for (int c = 0; c < nc; ++c)
    for (int m = 0; m < nm; ++m) {
      m2d_rep[(size_t)c * nm + m] = m2d(cls[c * P], m);
      d2m_rep[(size_t)c * nm + m] = d2m(cls[c * P], m);
    }
  int rc;
  if ((rc = upload(rt, rt->d_sym_dir, cls, "symmetry")) || (rc = upload(rt, rt->d_sym_group, mom_group, "symmetry")) ||
      (rc = upload(rt, rt->d_sym_sign, group_sign, "symmetry")) ||
      (rc = upload(rt, rt->d_sym_m2d, m2d_rep, "symmetry")) || (rc = upload(rt, rt->d_sym_d2m, d2m_rep, "symmetry")))
    return rc;
  rt->sym.n_class = nc;
  rt->sym.P = P;
  rt->sym.G = (int)group_sign.size();
  rt->sym.pattern = sym_canonical_pattern(P, nm, rt->sym.G, mom_group.data(), group_sign.data());
  rt->sym.cls_dir = rt->d_sym_dir.as<int>();
  rt->sym.mom_group = rt->d_sym_group.as<int>();
  rt->sym.sign = rt->d_sym_sign.as<unsigned>();
  rt->sym.m2d_rep = rt->d_sym_m2d.as<double>();
  rt->sym.d2m_rep = rt->d_sym_d2m.as<double>();
  return OURANOS_OK;
}

// ------------------------------------------------------------------ schedule
// Directions of one octant (same sign pattern) are grouped kd at a time; each
// group crosses the transverse tiles in dependency order.
int build_schedule(ouranos_rt* rt) {
  const int dim = rt->dim;
  const int NX = rt->nx[0], NY = dim == 3 ? rt->nx[1] : 1, NS = rt->nx[dim - 1];
  rt->tiles_x = (NX + rt->wx - 1) / rt->wx;
  rt->tiles_y = dim == 3 ? (NY + rt->wy - 1) / rt->wy : 1;
  const int tiles = rt->tiles_x * rt->tiles_y;
  std::map<int, std::vector<int>> by_flip;
  for (int d = 0; d < rt->n_dir; ++d) {
    int f = 0;
    for (int a = 0; a < dim; ++a)
      if (rt->omega[3 * d + a] < 0.0) f |= 1 << a;
    by_flip[f].push_back(d);
  }
  std::vector<int> gdirs, gflip;
  for (auto& kv : by_flip) {
    const auto& ds = kv.second;
    for (size_t i = 0; i < ds.size(); i += rt->kd) {
      for (int k = 0; k < rt->kd; ++k) gdirs.push_back(i + k < ds.size() ? ds[i + k] : -1);
      gflip.push_back(kv.first);
    }
  }
  const int n_groups = (int)gflip.size();
  rt->n_groups_dir = n_groups;
  std::vector<int2> tasks;
  const int levels = rt->tiles_x + rt->tiles_y - 1;
  for (int L = 0; L < levels; ++L)
    for (int g = 0; g < n_groups; ++g)
      for (int ty = 0; ty < rt->tiles_y; ++ty) {
        const int tx = L - ty;
        if (tx < 0 || tx >= rt->tiles_x) continue;
        tasks.push_back(make_int2(g, tx + rt->tiles_x * ty));
      }
  rt->n_tasks = (int)tasks.size();
  OK_OR_RETURN(upload(rt, rt->d_tasks, tasks, "tasks"));
  OK_OR_RETURN(upload(rt, rt->d_group_dirs, gdirs, "group dirs"));
  OK_OR_RETURN(upload(rt, rt->d_group_flip, gflip, "group flips"));
  // control block: [0] ticket, [1] status (the rest is spare)
  CU(rt->d_ctrl.alloc(sizeof(int) * (64 + (size_t)n_groups * tiles)), "control block");
  CU(cudaMemsetAsync(rt->d_ctrl.p, 0, rt->d_ctrl.bytes, rt->stream), "control block");
  const size_t ex = (size_t)rt->n_dir * tiles * NS * rt->wy * rt->fd;
  const size_t ey = dim == 3 ? (size_t)rt->n_dir * tiles * NS * rt->wx * rt->fd : 1;
  const size_t esz = rt->precision == OURANOS_FP64 ? 8 : 4;
  // two 64-bit tagged words per value cover both precisions
  CU(rt->d_edge_x.alloc(ex * 16 > 0 ? ex * 16 : 16), "edge buffer x");
  CU(rt->d_edge_y.alloc(ey * 16 > 0 ? ey * 16 : 16), "edge buffer y");
  CU(cudaMemsetAsync(rt->d_edge_x.p, 0, rt->d_edge_x.bytes, rt->stream), "edge buffer x");
  CU(cudaMemsetAsync(rt->d_edge_y.p, 0, rt->d_edge_y.bytes, rt->stream), "edge buffer y");
  (void)esz;
  return OURANOS_OK;
}

// the per-lane sweep kernels are instantiated for 2-D Q1..Q4 and 3-D Q1..Q2;
// every order (up to Q5) also runs one warp per cell
static bool register_form(const ouranos_rt* rt) { return rt->dim == 2 ? rt->p1 <= 5 : rt->p1 <= 3; }

int default_tiling(ouranos_rt* rt) {
  // one direction per warp: every lane of a warp reads the same inverse table
  // (broadcast loads); 32 cells per warp (2-D: 32 x 1, 3-D: 4 x 8), or 16
  // cells solved by two lanes each for cells of 9 or more dofs (3-D: 4 x 4).
  // Measured on GB300, 64^3 Q1 GLC S12 FP32 sweep: 4 x 8 1.80 ms, 8 x 4 1.86,
  // 4 x 4 x 2 directions 1.94, 8 x 2 x 2 2.21.  Higher orders: one warp per cell.
  rt->kd = 1;
  if (!register_form(rt)) {
    rt->wx = rt->wy = 1;
    rt->lpc = 32;
    return OURANOS_OK;
  }
  rt->lpc = rt->n >= 9 ? 2 : 1;
  if (rt->dim == 2) {
    rt->wx = 32 / rt->lpc;
    rt->wy = 1;
  } else {
    rt->wx = 4;
    rt->wy = rt->lpc == 2 ? 4 : 8;
  }
  return OURANOS_OK;
}

// ------------------------------------------------------- per-group tables
int setup_group(ouranos_rt* rt) {
  const int g = rt->group, G = rt->G, nm = rt->n_mom, L = rt->l_max;
  const int n = rt->n;
  // sigma_t classes (A depends on the cell only through sigma_t)
  std::vector<double> cls_val;
  std::vector<int> mat_cls(rt->n_mat);
  for (int m = 0; m < rt->n_mat; ++m) {
    const double st = rt->sigma_t[(size_t)m * G + g] + rt->inv_vdt;  // implicit Euler shift
    auto it = std::find(cls_val.begin(), cls_val.end(), st);
    if (it == cls_val.end()) {
      mat_cls[m] = (int)cls_val.size();
      cls_val.push_back(st);
    } else {
      mat_cls[m] = (int)(it - cls_val.begin());
    }
  }
  rt->sigma_class_value = cls_val;
  std::vector<int> ccls(rt->n_cells);
  for (long c = 0; c < rt->n_cells; ++c) ccls[c] = mat_cls[rt->material_id[c]];
  OK_OR_RETURN(upload(rt, rt->d_cell_class, ccls, "cell classes"));
  // A'^-1 per (sigma class, |Omega| class)
  const size_t nn = (size_t)n * n;
  std::vector<double> ainv(cls_val.size() * rt->n_dir_class * nn);
  for (size_t s = 0; s < cls_val.size(); ++s)
    for (int dc = 0; dc < rt->n_dir_class; ++dc)
      canonical_inverse(rt->fe, cls_val[s], &rt->class_abs_omega[3 * dc],
                        &ainv[(s * rt->n_dir_class + dc) * nn]);
  // rows padded to whole 16-byte pieces in every precision (the per-lane sweep
  // loads them as vectors); one warp per cell reads the transpose, whose row j
  // holds entry (i, j) for consecutive i
  std::vector<double> ainv_p;
  if (rt->lpc == 32) {
    ainv_p.resize(ainv.size());
    const size_t mats = cls_val.size() * rt->n_dir_class;
    for (size_t m = 0; m < mats; ++m)
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) ainv_p[m * nn + (size_t)j * n + i] = ainv[m * nn + (size_t)i * n + j];
  } else {
    ainv_p = pad_rows(ainv, (long)cls_val.size() * rt->n_dir_class * n, n);
  }
  OK_OR_RETURN(upload(rt, rt->d_ainv64, ainv_p, "inverse tables"));
  OK_OR_RETURN(upload(rt, rt->d_ainv32, to_f32(ainv_p), "inverse tables"));
  OK_OR_RETURN(upload(rt, rt->d_ainvdf, to_df(ainv_p), "inverse tables"));
  // scattering scales: sigma_s(mat, g'->g, l(m)) (by Legendre order)
  auto sig_s = [&](int mat, int gf, int gt, int l) {
    if (l > L) return 0.0;
    return rt->sigma_s[(size_t)l + (size_t)gt * (L + 1) + (size_t)gf * G * (L + 1) +
                       (size_t)mat * G * G * (L + 1)];
  };
  std::vector<double> ss((size_t)rt->n_mat * nm), os((size_t)rt->n_mat * G * nm);
  for (int mat = 0; mat < rt->n_mat; ++mat)
    for (int q = 0; q < nm; ++q) {
      ss[(size_t)mat * nm + q] = sig_s(mat, g, g, rt->moment_l[q]);
      for (int gf = 0; gf < G; ++gf)
        os[((size_t)mat * G + gf) * nm + q] = sig_s(mat, gf, g, rt->moment_l[q]);
    }
  OK_OR_RETURN(upload(rt, rt->d_sscale, ss, "scattering scales"));
  OK_OR_RETURN(upload(rt, rt->d_oscale, os, "scattering scales"));
  // fixed source per source id: q/ws (src/RadiativeTransfer.cc:918-921)
  std::vector<double> q(std::max(rt->n_src, 1), 0.0);
  for (int s = 0; s < rt->n_src; ++s) q[s] = rt->source[(size_t)s * G + g] / rt->ws;
  OK_OR_RETURN(upload(rt, rt->d_qcell, q, "sources"));
  // boundary inflow per (direction, axis) (src/RadiativeTransfer.cc:958-975)
  std::vector<double> bnd((size_t)rt->n_dir * 3, 0.0);
  for (int d = 0; d < rt->n_dir; ++d)
    for (int a = 0; a < rt->dim; ++a) {
      const int f = rt->omega[3 * d + a] > 0.0 ? 2 * a : 2 * a + 1;  // entering face
      const int bt = rt->bc[f];
      const bool mn = !rt->most_normal.empty() && rt->most_normal[(size_t)f * rt->n_dir + d];
      double inc = 0.0;
      if ((bt == OURANOS_BC_MOST_NORMAL && mn) || bt == OURANOS_BC_ISOTROPIC)
        inc = rt->inc_flux.empty() ? 0.0 : rt->inc_flux[(size_t)f * G + g];
      bnd[3 * d + a] = inc / rt->ws;
    }
  OK_OR_RETURN(upload(rt, rt->d_bnd64, bnd, "boundary"));
  OK_OR_RETURN(upload(rt, rt->d_bnd32, to_f32(bnd), "boundary"));
  OK_OR_RETURN(upload(rt, rt->d_bnddf, to_df(bnd), "boundary"));
  return OURANOS_OK;
}

// --------------------------------------------------------------- the sweep
// Source moments with at most this many entries are applied inside the sweep;
// more are first expanded to per-direction sources (a dense contraction over
// the moment axis that streams better than a per-step loop over moments).
constexpr int kFusedMomentsMax = 2;

// Sweep arguments for one problem (pointers into the handle's buffers) and,
// when the source is expanded (fm = 0), the expansion launch.  Epoch, ticket
// and status are left for the caller.
// q = M2D src (+ iso) on the dofs [e0, e0 + len) into the expanded-source
// buffer, in the contraction form of the sweep's precision
template <typename real>
int sweep_expand(ouranos_rt* rt, const real* src, const real* iso, long e0, long len) {
  const long nd = rt->n_dofs;
  src += e0;
  if (iso) iso += e0;
  if (std::is_same<real, df64>::value && rt->fp64_contract == OURANOS_FP64_DF64_SWEEP_TC)  // tensor cores
    CU(launch_expand_oz((const df64*)src, (const df64*)iso, rt->oz, rt->d_q.as<df64>() + e0, nd,
                        rt->d_ctrl.as<int>() + 1, rt->wait_limit_ns, rt->stream, len),
       "source expansion");
  else if (std::is_same<real, df64>::value && rt->sym.n_class)  // pairs, through the octant symmetry
    CU(launch_expand_sym_pairs((const df64*)src, (const df64*)iso, rt->sym, rt->d_q.as<df64>() + e0, rt->n_mom,
                               nd, rt->stream, len),
       "source expansion");
  else if (std::is_same<real, df64>::value)  // pairs in, pairs out
    CU(launch_expand_source_pairs((const df64*)src, (const df64*)iso, rt->d_m2d64.as<double>(),
                                  rt->d_q.as<df64>() + e0, rt->n_dir, rt->n_mom, nd, rt->stream, len),
       "source expansion");
  else if (std::is_same<real, double>::value && rt->fp64_contract != OURANOS_FP64_NATIVE)
    CU(launch_expand_source_df64((const double*)src, (const double*)iso, rt->d_m2d64.as<double>(),
                                 rt->d_q.as<double>() + e0, rt->n_dir, rt->n_mom, nd, rt->stream, len),
       "source expansion");
  else if (std::is_same<real, float>::value && rt->fp32_contract == OURANOS_FP32_CONTRACT_TENSOR)
    CU(launch_expand_tc((const float*)src, (const float*)iso, rt->tc, rt->d_q.as<float>() + e0, nd,
                        rt->d_ctrl.as<int>() + 1, rt->wait_limit_ns, rt->stream, len),
       "source expansion");
  else
    CU(launch_expand_source<real>(src, iso, table<real>(rt->d_m2d64, rt->d_m2d32, rt->d_m2ddf),
                                  rt->d_q.as<real>() + e0, rt->n_dir, rt->n_mom, nd, rt->stream, len),
       "source expansion");
  return OURANOS_OK;
}

template <typename real>
int sweep_prepare(ouranos_rt* rt, const real* src, const real* iso, const real* bnd, SweepArgs<real>& a,
                  int& fm, int& kernels, bool expand = true) {
  const long len_dir = (long)rt->n_dir * rt->n_dofs;
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
  a.abs_omega = table<real>(rt->d_abs64, rt->d_abs32, rt->d_absdf);
  a.m2d = table<real>(rt->d_m2d64, rt->d_m2d32, rt->d_m2ddf);
  a.ainv = table<real>(rt->d_ainv64, rt->d_ainv32, rt->d_ainvdf);
  a.cell_class = rt->d_cell_class.as<int>();
  a.face_mass = table<real>(rt->d_face64, rt->d_face32, rt->d_facedf);
  a.src = src;
  a.iso = iso;
  a.q = nullptr;
  a.bnd = bnd;
  CU(rt->d_psi.alloc(sizeof(real) * len_dir), "angular flux");
  a.psi = rt->d_psi.as<real>();
  a.edge_x = rt->d_edge_x.as<unsigned long long>();
  a.edge_y = rt->d_edge_y.as<unsigned long long>();
  a.wait_limit_ns = rt->wait_limit_ns;
  a.wait_bias = rt->wait_bias;
  a.epoch = 0;
  a.ticket = nullptr;
  a.status = nullptr;
  kernels = 0;
  // (the fused form holds (moments + 1) prefetched values per dof in registers)
  fm = (rt->n_mom <= kFusedMomentsMax && rt->n * (rt->n_mom + 1) <= 32) ? rt->n_mom : 0;
  // a source sweep of a time step carries the per-direction psi^n term: expanded form
  const bool angular = iso && rt->inv_vdt > 0.0 && rt->d_psi_prev.p;
  if (angular || rt->lpc == 32) fm = 0;  // (one warp per cell reads the expanded source only)
  if (fm == 0) {
    CU(rt->d_q.alloc(sizeof(real) * len_dir), "expanded source");
    a.q = rt->d_q.as<real>();
    if (expand) {
      OK_OR_RETURN(sweep_expand<real>(rt, src, iso, 0, rt->n_dofs));
      kernels += (rt->n_mom + 15) / 16;
    }
    if (angular) {
      CU(launch_angular_source<real>(rt->d_q.as<real>(), rt->d_psi_prev.as<float>(), rt->d_cell_mass.as<double>(),
                                     rt->inv_vdt, rt->n, rt->n_cells, rt->n_dir, rt->stream),
         "time-step source");
      ++kernels;
    }
  }
  return OURANOS_OK;
}

// phi = D2M psi (the moment reduction after a sweep); phi is float for the
// FP32 sweep, double for the FP64 and double-float sweeps
// The double-float reductions can write the Apply's y = x - phi in phi's
// place (one rounding, as the combine kernel): one kernel and one pass over
// phi less per Apply
bool fused_combine(const ouranos_rt* rt) {
  return df64_sweep(rt) && (rt->fp64_contract == OURANOS_FP64_DF64_SWEEP_TC ? rt->oz.npad > 0 : rt->sym.n_class > 0);
}

template <typename real>
int sweep_reduce(ouranos_rt* rt, const real* psi, void* phi, long e0 = 0, long len = -1, const double* xc = nullptr) {
  // dofs [e0, e0 + len): psi and phi move by e0, their row stride stays n_dofs;
  // with xc (fused_combine only), phi receives xc - phi
  const long nd = rt->n_dofs;
  if (len < 0) len = nd;
  psi += e0;
  double* phi64 = (double*)phi + e0;
  if (xc) {
    if (!std::is_same<real, df64>::value || !fused_combine(rt)) return bad(rt, "no fused combination here");
    xc += e0;
  }
  if (std::is_same<real, df64>::value && rt->fp64_contract == OURANOS_FP64_DF64_SWEEP_TC)
    CU(launch_reduce_oz((const df64*)psi, rt->oz, phi64, nd, rt->d_ctrl.as<int>() + 1, rt->wait_limit_ns,
                        rt->stream, len, xc),
       "moment reduction");
  else if (std::is_same<real, df64>::value && rt->sym.n_class)
    CU(launch_reduce_sym_pairs((const df64*)psi, rt->sym, phi64, rt->n_mom, nd, rt->stream, len, xc),
       "moment reduction");
  else if (std::is_same<real, df64>::value)
    CU(launch_reduce_moments_pairs((const df64*)psi, rt->d_d2m64.as<double>(), phi64, rt->n_dir, rt->n_mom, nd,
                                   rt->stream, len),
       "moment reduction");
  else if (std::is_same<real, double>::value && rt->fp64_contract != OURANOS_FP64_NATIVE)
    CU(launch_reduce_moments_df64((const double*)psi, rt->d_d2m64.as<double>(), phi64, rt->n_dir, rt->n_mom,
                                  nd, rt->stream, len),
       "moment reduction");
  else if (std::is_same<real, double>::value)
    CU(launch_reduce_moments<double>((const double*)psi, rt->d_d2m64.as<double>(), phi64, rt->n_dir,
                                     rt->n_mom, nd, rt->stream, len),
       "moment reduction");
  else if (rt->fp32_contract == OURANOS_FP32_CONTRACT_TENSOR)
    CU(launch_reduce_tc((const float*)psi, rt->tc, (float*)phi + e0, nd, rt->d_ctrl.as<int>() + 1,
                        rt->wait_limit_ns, rt->stream, len),
       "moment reduction");
  else
    CU(launch_reduce_moments<float>((const float*)psi, rt->d_d2m32.as<float>(), (float*)phi + e0, rt->n_dir,
                                    rt->n_mom, nd, rt->stream, len),
       "moment reduction");
  return OURANOS_OK;
}

// The sweep launch of prepared arguments: a fresh epoch, the ticket reset,
// the kernel between the handle's timing events
template <typename real>
int sweep_launch(ouranos_rt* rt, SweepArgs<real>& a, int fm) {
  // epochs cycle through [1, 0x7fff]; every sweep rewrites every edge word it
  // reads, so a stale word carries the previous epoch and never matches
  rt->epoch = rt->epoch % 0x7fffu + 1u;
  a.epoch = rt->epoch;
  int* ctrl = rt->d_ctrl.as<int>();
  a.ticket = ctrl;
  a.status = ctrl + 1;
  // ticket -> 0.  The status word [1] is sticky: it is cleared at the start of
  // each C-ABI call (clear_status), so a timeout inside a solve (a sweep's
  // dependency wait, bit 1; a diffusion-solve barrier, bit 2) is seen at its
  // end and every later sweep of that call exits at once.
  CU(cudaMemsetAsync(ctrl, 0, sizeof(int), rt->stream), "reset sweep control");
  int sms = 0;
  CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, rt->device), "device query");
  const int block = 128;
  // tasks are handed out by ticket, so any grid is deadlock-free; 8 blocks of
  // 4 warps per SM covers every instantiation's register budget
  const int grid = std::min((rt->n_tasks + 3) / 4, std::max(1, sms * 8));
  CU(cudaEventRecord(rt->ev0, rt->stream), "event");
  CU(launch_sweep<real>(rt->dim, rt->p1, fm, a, grid, block, rt->stream), "sweep launch");
  CU(cudaEventRecord(rt->ev1, rt->stream), "event");
  return OURANOS_OK;
}

template <typename real>
int run_sweep(ouranos_rt* rt, const real* src, const real* iso, const real* bnd, void* phi,
              const double* xc = nullptr) {
  SweepArgs<real> a;
  int fm = 0, kernels = 0;
  OK_OR_RETURN(sweep_prepare<real>(rt, src, iso, bnd, a, fm, kernels));
  OK_OR_RETURN(sweep_launch<real>(rt, a, fm));
  ++kernels;
  OK_OR_RETURN(sweep_reduce<real>(rt, a.psi, phi, 0, -1, xc));
  kernels += (rt->n_mom + 15) / 16;
  rt->last_kernels = kernels;
  return OURANOS_OK;
}

int clear_status(ouranos_rt* rt) {
  CU(cudaMemsetAsync(rt->d_ctrl.as<int>() + 1, 0, sizeof(int), rt->stream), "reset status");
  return OURANOS_OK;
}

int finish(ouranos_rt* rt) {
  CU(cudaStreamSynchronize(rt->stream), "sweep");
  int st = 0;
  CU(cudaMemcpy(&st, rt->d_ctrl.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost), "status");
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, rt->ev0, rt->ev1) == cudaSuccess)
    rt->last_ms = ms;
  else
    (void)cudaGetLastError();  // no sweep recorded the events: not an error of this call
  if (st) {
    rt->err = (st & 2)   ? "diffusion acceleration: grid barrier wait timed out"
              : (st & 4) ? "tensor-core contraction: MMA completion wait timed out"
                         : "sweep dependency wait timed out";
    return OURANOS_ERR_TIMEOUT;
  }
  // the installed network's forwards on this stream (cnn_forward_on)
  const bool pending = rt->cnn_pending;
  rt->cnn_pending = false;
  if (pending && rt->cnn && cnn_forward_status(rt->cnn)) {
    rt->err = "learned preconditioner: a convolution's tensor-core wait timed out";
    return OURANOS_ERR_TIMEOUT;
  }
  return OURANOS_OK;
}

// Bring a caller vector (host or device, caller numbering) into a device
// buffer in lexicographic numbering.  Returns the device pointer to use.
int stage_in(ouranos_rt* rt, const double* v, DevBuf& buf, int n_vec, const double** out) {
  const long len = (long)n_vec * vec_len(rt) / rt->n_mom * rt->n_mom;
  const size_t bytes = sizeof(double) * (size_t)n_vec * rt->n_mom * rt->n_dofs;
  const bool dev = is_device_ptr(v);
  (void)len;
  if (dev && rt->cell_order.empty()) {
    *out = v;
    return OURANOS_OK;
  }
  CU(buf.alloc(bytes), "staging");
  if (!dev) {
    if (rt->cell_order.empty()) {
      CU(cudaMemcpyAsync(buf.p, v, bytes, cudaMemcpyHostToDevice, rt->stream), "copy in");
      *out = buf.as<double>();
      return OURANOS_OK;
    }
    CU(rt->d_tmp.alloc(bytes), "staging");
    CU(cudaMemcpyAsync(rt->d_tmp.p, v, bytes, cudaMemcpyHostToDevice, rt->stream), "copy in");
    v = rt->d_tmp.as<double>();
  }
  CU(launch_permute(v, buf.as<double>(), rt->d_cell_order.as<long>(), rt->n_cells, rt->n,
                    n_vec * rt->n_mom, 1, rt->stream),
     "permute in");
  *out = buf.as<double>();
  return OURANOS_OK;
}

// Copy a lexicographic device vector back to the caller's buffer.
int stage_out(ouranos_rt* rt, const double* dv, double* user) {
  const size_t bytes = sizeof(double) * vec_len(rt);
  const bool dev = is_device_ptr(user);
  if (rt->cell_order.empty()) {
    if (dv != user)
      CU(cudaMemcpyAsync(user, dv, bytes, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                         rt->stream),
         "copy out");
    return OURANOS_OK;
  }
  if (dev) {
    CU(launch_permute(dv, user, rt->d_cell_order.as<long>(), rt->n_cells, rt->n, rt->n_mom, 0,
                      rt->stream),
       "permute out");
    return OURANOS_OK;
  }
  CU(rt->d_tmp.alloc(bytes), "staging");
  CU(launch_permute(dv, rt->d_tmp.as<double>(), rt->d_cell_order.as<long>(), rt->n_cells, rt->n,
                    rt->n_mom, 0, rt->stream),
     "permute out");
  CU(cudaMemcpyAsync(user, rt->d_tmp.p, bytes, cudaMemcpyDeviceToHost, rt->stream), "copy out");
  return OURANOS_OK;
}

// Source moments T (precision of the sweep) from x (FP64, device) and the
// other groups' fluxes gf (device or NULL).
// (pairs: the double-float sweep's storage, in the same buffer as the FP64 source)
int build_source(ouranos_rt* rt, const double* x, const double* gf, bool pairs, long c0 = 0, long nc = -1) {
  const long len = vec_len(rt);
  const double* M = rt->d_cell_mass.as<double>();
  // cells [c0, c0 + nc): every per-cell pointer moves by c0 cells, the moment
  // stride stays n_dofs
  if (nc < 0) nc = rt->n_cells;
  const long o = c0 * rt->n;
  if (x) x += o;
  if (gf) gf += o;
  const int* mat = rt->d_material.as<int>() + c0;
  if (rt->precision == OURANOS_FP64 && pairs) {
    CU(rt->d_src64.alloc(sizeof(df64) * len), "source");
    CU(launch_scatter_source<df64>(x, gf, rt->d_src64.as<df64>() + o, M, rt->d_sscale.as<double>(),
                                   rt->d_oscale.as<double>(), mat, rt->n_mat, rt->G, rt->group, nc, rt->n,
                                   rt->n_mom, rt->n_dofs, rt->stream),
       "scattering source");
  } else if (rt->precision == OURANOS_FP64) {
    CU(rt->d_src64.alloc(sizeof(double) * len), "source");
    CU(launch_scatter_source<double>(x, gf, rt->d_src64.as<double>() + o, M, rt->d_sscale.as<double>(),
                                     rt->d_oscale.as<double>(), mat, rt->n_mat, rt->G, rt->group, nc, rt->n,
                                     rt->n_mom, rt->n_dofs, rt->stream),
       "scattering source");
  } else {
    CU(rt->d_src32.alloc(sizeof(float) * len), "source");
    CU(launch_scatter_source<float>(x, gf, rt->d_src32.as<float>() + o, M, rt->d_sscale.as<double>(),
                                    rt->d_oscale.as<double>(), mat, rt->n_mat, rt->G, rt->group, nc, rt->n,
                                    rt->n_mom, rt->n_dofs, rt->stream),
       "scattering source");
  }
  return OURANOS_OK;
}

// phi = D L^-1 (M2D T [+ iso + inflow]) into the precision's phi buffer.
int sweep_into_phi(ouranos_rt* rt, bool sources) {
  const long len = vec_len(rt);
  if (df64_sweep(rt)) {  // double-float sweep: sources as pairs
    CU(rt->d_phi64.alloc(sizeof(double) * len), "flux");
    const df64* iso = nullptr;
    if (sources) {
      CU(rt->d_iso64.alloc(sizeof(df64) * rt->n_dofs), "iso");
      CU(launch_iso_source<df64>(rt->d_iso64.as<df64>(), rt->d_qcell.as<double>(),
                                 rt->d_rowsum_mass.as<double>(), rt->d_source_id.as<int>(), rt->n_cells,
                                 rt->n, rt->stream),
         "iso source");
      iso = rt->d_iso64.as<df64>();
    }
    return run_sweep<df64>(rt, rt->d_src64.as<df64>(), iso, sources ? rt->d_bnddf.as<df64>() : nullptr,
                           rt->d_phi64.p);
  }
  if (rt->precision == OURANOS_FP64) {
    CU(rt->d_phi64.alloc(sizeof(double) * len), "flux");
    const double* iso = nullptr;
    if (sources) {
      CU(rt->d_iso64.alloc(sizeof(double) * rt->n_dofs), "iso");
      CU(launch_iso_source<double>(rt->d_iso64.as<double>(), rt->d_qcell.as<double>(),
                                   rt->d_rowsum_mass.as<double>(), rt->d_source_id.as<int>(),
                                   rt->n_cells, rt->n, rt->stream),
         "iso source");
      iso = rt->d_iso64.as<double>();
    }
    return run_sweep<double>(rt, rt->d_src64.as<double>(), iso,
                             sources ? rt->d_bnd64.as<double>() : nullptr, rt->d_phi64.p);
  }
  CU(rt->d_phi32.alloc(sizeof(float) * len), "flux");
  const float* iso = nullptr;
  if (sources) {
    CU(rt->d_iso32.alloc(sizeof(float) * rt->n_dofs), "iso");
    CU(launch_iso_source<float>(rt->d_iso32.as<float>(), rt->d_qcell.as<double>(),
                                rt->d_rowsum_mass.as<double>(), rt->d_source_id.as<int>(),
                                rt->n_cells, rt->n, rt->stream),
       "iso source");
    iso = rt->d_iso32.as<float>();
  }
  return run_sweep<float>(rt, rt->d_src32.as<float>(), iso,
                          sources ? rt->d_bnd32.as<float>() : nullptr, rt->d_phi32.p);
}

// y = sx * x + sp * phi  (x may be NULL)
int phi_combine(ouranos_rt* rt, const double* x, double* y, double sx, double sp) {
  const long len = vec_len(rt);
  if (rt->precision == OURANOS_FP64)
    CU(launch_combine<double>(x, rt->d_phi64.as<double>(), y, len, sx, sp, rt->stream), "combine");
  else
    CU(launch_combine<float>(x, rt->d_phi32.as<float>(), y, len, sx, sp, rt->stream), "combine");
  return OURANOS_OK;
}

// Apply for page-locked host vectors with the copies overlapped.  The cells
// are cut into OURANOS_OVERLAP_CHUNKS ranges.  Each range of x travels on the
// copy stream (one 2-D copy: the range's dofs of every moment) while the
// handle's stream builds the scattering source (and the expanded source) of
// the ranges that have landed; after the sweep each range is reduced and
// combined and travels back while the next one is reduced.  The kernels and
// their arithmetic per dof are those of the device Apply, so y is identical.
template <typename real>
int apply_overlapped(ouranos_rt* rt, const double* hx, double* hy) {
  constexpr int K = OURANOS_OVERLAP_CHUNKS;
  const long n = rt->n, nd = rt->n_dofs, nc = rt->n_cells;
  const int nm = rt->n_mom;
  const long len = vec_len(rt);
  const bool f64 = rt->precision == OURANOS_FP64;
  const bool pairs = std::is_same<real, df64>::value;
  CU(rt->d_x.alloc(sizeof(double) * len), "staging");
  CU(rt->d_y.alloc(sizeof(double) * len), "apply");
  DevBuf& sb = f64 ? rt->d_src64 : rt->d_src32;
  CU(sb.alloc(sizeof(real) * len), "source");
  DevBuf& pb = f64 ? rt->d_phi64 : rt->d_phi32;
  CU(pb.alloc((f64 ? sizeof(double) : sizeof(float)) * len), "flux");
  if (!rt->copy_stream) {
    CU(cudaStreamCreateWithFlags(&rt->copy_stream, cudaStreamNonBlocking), "copy stream");
    for (cudaEvent_t& e : rt->ev_chunk) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "copy events");
  }
  double* dx = rt->d_x.as<double>();
  double* dy = rt->d_y.as<double>();
  cudaEvent_t* ev = rt->ev_chunk;  // [0, K) in, [K, 2K) out, [2K] start, [2K + 1] done
  // the copies wait for the work already queued on the handle's stream
  CU(cudaEventRecord(ev[2 * K], rt->stream), "copy order");
  CU(cudaStreamWaitEvent(rt->copy_stream, ev[2 * K], 0), "copy order");
  SweepArgs<real> a;
  int fm = 0, kernels = 0;
  const real* src = sb.as<real>();
  OK_OR_RETURN(sweep_prepare<real>(rt, src, nullptr, nullptr, a, fm, kernels, false));
  // cell ranges of 1/8, 1/4, 1/4, 1/4, 1/8 of the cells: only the first
  // range's copy in and the last range's copy out wait with nothing to
  // overlap, so those two are the short ones (the middle copies hide behind
  // the per-cell kernels of the neighbouring ranges)
  static_assert(K == 5, "range weights below");
  constexpr int kWeight[K + 1] = {0, 1, 3, 5, 7, 8};  // cumulative eighths
  auto range = [&](int k, long& c0, long& cn) {
    c0 = nc * kWeight[k] / 8;
    cn = nc * kWeight[k + 1] / 8 - c0;
  };
  const size_t pitch = sizeof(double) * nd;
  for (int k = 0; k < K; ++k) {
    long c0 = 0, cn = 0;
    range(k, c0, cn);
    if (cn > 0) {
      CU(cudaMemcpy2DAsync(dx + c0 * n, pitch, hx + c0 * n, pitch, sizeof(double) * cn * n, nm,
                           cudaMemcpyHostToDevice, rt->copy_stream),
         "copy in");
    }
    CU(cudaEventRecord(ev[k], rt->copy_stream), "copy order");
    CU(cudaStreamWaitEvent(rt->stream, ev[k], 0), "copy order");
    if (cn == 0) continue;
    OK_OR_RETURN(build_source(rt, dx, nullptr, pairs, c0, cn));
    if (fm == 0) OK_OR_RETURN(sweep_expand<real>(rt, src, nullptr, c0 * n, cn * n));
  }
  OK_OR_RETURN(sweep_launch<real>(rt, a, fm));
  for (int k = 0; k < K; ++k) {
    long c0 = 0, cn = 0;
    range(k, c0, cn);
    if (cn > 0) {
      const long e0 = c0 * n;
      if (fused_combine(rt)) {  // the reduction writes the range of y = x - phi
        OK_OR_RETURN(sweep_reduce<real>(rt, a.psi, dy, e0, cn * n, dx));
      } else {
        OK_OR_RETURN(sweep_reduce<real>(rt, a.psi, pb.p, e0, cn * n));
      if (f64)
        CU(launch_combine_rows<double>(dx + e0, pb.as<double>() + e0, dy + e0, nm, cn * n, nd, 1.0, -1.0,
                                       rt->stream),
           "combine");
      else
        CU(launch_combine_rows<float>(dx + e0, pb.as<float>() + e0, dy + e0, nm, cn * n, nd, 1.0, -1.0,
                                      rt->stream),
           "combine");
      }
    }
    CU(cudaEventRecord(ev[K + k], rt->stream), "copy order");
    CU(cudaStreamWaitEvent(rt->copy_stream, ev[K + k], 0), "copy order");
    if (cn > 0)
      CU(cudaMemcpy2DAsync(hy + c0 * n, pitch, dy + c0 * n, pitch, sizeof(double) * cn * n, nm,
                           cudaMemcpyDeviceToHost, rt->copy_stream),
         "copy out");
  }
  // later work on the handle's stream (and its synchronisation) follows the copies
  CU(cudaEventRecord(ev[2 * K + 1], rt->copy_stream), "copy order");
  CU(cudaStreamWaitEvent(rt->stream, ev[2 * K + 1], 0), "copy order");
  // per range: scattering source, expansion (expanded form), reduction and
  // combination (unless fused); and the sweep
  rt->last_kernels = 2 * K + 1 + (fm == 0 ? K : 0) + (fused_combine(rt) ? 0 : K);
  return OURANOS_OK;
}

}  // namespace

// ============================================================== internal API
namespace ouranos {
// Device-side Apply for the solvers: y = x - D L^-1 M2D S x, x and y device,
// lexicographic numbering.  Does not synchronise.
int rt_apply_device(ouranos_rt* rt, const double* x, double* y) {
  OK_OR_RETURN(build_source(rt, x, nullptr, df64_sweep(rt)));
  if (fused_combine(rt)) {  // the reduction writes y = x - phi
    OK_OR_RETURN(run_sweep<df64>(rt, rt->d_src64.as<df64>(), nullptr, nullptr, y, x));
    rt->last_kernels += 1;  // the scattering source
    return OURANOS_OK;
  }
  OK_OR_RETURN(sweep_into_phi(rt, false));
  rt->last_kernels += 2;  // the scattering source and the combination
  return phi_combine(rt, x, y, 1.0, -1.0);
}
// rhs = D L^-1 (q + outer + inflow) with zero in-group scattering (device).
int rt_rhs_device(ouranos_rt* rt, const double* gf, double* rhs) {
  OK_OR_RETURN(build_source(rt, nullptr, gf, df64_sweep(rt)));
  OK_OR_RETURN(sweep_into_phi(rt, true));
  return phi_combine(rt, nullptr, rhs, 0.0, 1.0);
}
// Batched Apply pieces (batch.cu): the per-problem work before and after the
// batched sweep launch.  prepare: the source terms in the sweep precision --
// the scattering source of x, or with `sources` the fixed source and inflow
// (no scattering) -- and the problem's sweep arguments (plus the source
// expansion when the sweep reads expanded sources); finish: the moment
// reduction and y = x - phi, or y = phi with `sources`.
template <typename real>
static int batch_prepare(ouranos_rt* rt, const double* x, SweepArgs<real>* a, int* fm, bool sources) {
  const bool f64 = sizeof(real) == 8;
  rt->precision = f64 ? OURANOS_FP64 : OURANOS_FP32;
  OK_OR_RETURN(build_source(rt, sources ? nullptr : x, nullptr, false));  // batch: double sweep
  const long len = vec_len(rt);
  if (f64) CU(rt->d_phi64.alloc(sizeof(double) * len), "flux");
  else CU(rt->d_phi32.alloc(sizeof(float) * len), "flux");
  const real* iso = nullptr;
  const real* bnd = nullptr;
  if (sources) {
    DevBuf& ib = f64 ? rt->d_iso64 : rt->d_iso32;
    CU(ib.alloc(sizeof(real) * rt->n_dofs), "iso");
    CU(launch_iso_source<real>(ib.as<real>(), rt->d_qcell.as<double>(), rt->d_rowsum_mass.as<double>(),
                               rt->d_source_id.as<int>(), rt->n_cells, rt->n, rt->stream),
       "iso source");
    iso = ib.as<real>();
    bnd = (const real*)(f64 ? rt->d_bnd64.p : rt->d_bnd32.p);
  }
  int kernels = 0;
  const real* src = (const real*)(f64 ? rt->d_src64.p : rt->d_src32.p);
  return sweep_prepare<real>(rt, src, iso, bnd, *a, *fm, kernels);
}
int rt_batch_prepare(ouranos_rt* rt, const double* x, SweepArgs<double>* a, int* fm, bool sources) {
  return batch_prepare<double>(rt, x, a, fm, sources);
}
int rt_batch_prepare(ouranos_rt* rt, const double* x, SweepArgs<float>* a, int* fm, bool sources) {
  return batch_prepare<float>(rt, x, a, fm, sources);
}
int rt_batch_finish(ouranos_rt* rt, const double* x, double* y, bool sources) {
  if (rt->precision == OURANOS_FP64)
    OK_OR_RETURN(sweep_reduce<double>(rt, rt->d_psi.as<double>(), rt->d_phi64.p));
  else
    OK_OR_RETURN(sweep_reduce<float>(rt, rt->d_psi.as<float>(), rt->d_phi32.p));
  return sources ? phi_combine(rt, nullptr, y, 0.0, 1.0) : phi_combine(rt, x, y, 1.0, -1.0);
}
int rt_check_status(ouranos_rt* rt) { return finish(rt); }
int rt_clear_status(ouranos_rt* rt) { return clear_status(rt); }
int rt_stage_in(ouranos_rt* rt, const double* v, DevBuf& buf, int n_vec, const double** out) {
  return stage_in(rt, v, buf, n_vec, out);
}
int rt_stage_out(ouranos_rt* rt, const double* dv, double* user) { return stage_out(rt, dv, user); }
}  // namespace ouranos

// ===================================================================== C-ABI
extern "C" {

int ouranos_rt_create(const ouranos_problem_desc* D, int device, ouranos_rt** out) {
  if (!out) return OURANOS_ERR_BAD_INPUT;
  *out = nullptr;
  if (!D) return OURANOS_ERR_BAD_INPUT;
  ouranos_rt* rt = new (std::nothrow) ouranos_rt();
  if (!rt) return OURANOS_ERR_BAD_INPUT;
  auto fail = [&](int rc) {
    // keep the handle so the caller can read the message; it must destroy it
    *out = rt;
    return rc;
  };
  if (D->dim != 2 && D->dim != 3) return fail(bad(rt, "dim must be 2 or 3"));
  if (D->fe_order < 1 || D->fe_order > 5) {
    rt->err = "fe_order outside the range of DG Q1..Q5";
    return fail(OURANOS_ERR_UNSUPPORTED);
  }
  if (D->n_groups < 1 || D->n_dir < 1 || D->n_mom < 1 || D->n_materials < 1 || D->l_max < 0 ||
      !D->omega || !D->m2d || !D->d2m || !D->moment_l || !D->sigma_t || !D->sigma_s ||
      !D->material_id || !(D->weight_sum > 0.0))
    return fail(bad(rt, "incomplete problem description"));
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    rt->err = "no CUDA device";
    return fail(OURANOS_ERR_NO_DEVICE);
  }
  if (device < 0) cudaGetDevice(&device);
  rt->device = device;
  if (cudaSetDevice(device) != cudaSuccess) return fail(cuda_fail(rt, cudaGetLastError(), "set device"));
  rt->dim = D->dim;
  rt->p = D->fe_order;
  rt->p1 = rt->p + 1;
  rt->n_cells = 1;
  for (int a = 0; a < 3; ++a) {
    if (a < rt->dim) {
      if (D->n_cells[a] < 1 || !(D->upper[a] > D->lower[a])) return fail(bad(rt, "bad mesh box"));
      rt->nx[a] = D->n_cells[a];
      rt->h[a] = (D->upper[a] - D->lower[a]) / D->n_cells[a];
    } else {
      rt->nx[a] = 1;
      rt->h[a] = 1.0;
    }
    rt->n_cells *= rt->nx[a];
  }
  if (rt->nx[rt->dim - 1] > 0xffff) return fail(bad(rt, "at most 65535 cells along the sweep axis"));
  rt->fe = build_fe_tables(rt->dim, rt->p, rt->h);
  rt->n = rt->fe.n;
  rt->fd = rt->fe.fd;
  rt->n_dofs = rt->n_cells * rt->n;
  rt->G = D->n_groups;
  rt->n_dir = D->n_dir;
  rt->n_mom = D->n_mom;
  rt->n_mat = D->n_materials;
  rt->l_max = D->l_max;
  rt->ws = D->weight_sum;
  rt->omega.assign(D->omega, D->omega + 3 * (size_t)rt->n_dir);
  rt->m2d.assign(D->m2d, D->m2d + (size_t)rt->n_dir * rt->n_mom);
  rt->d2m.assign(D->d2m, D->d2m + (size_t)rt->n_dir * rt->n_mom);
  rt->moment_l.assign(D->moment_l, D->moment_l + rt->n_mom);
  if (D->most_normal)
    rt->most_normal.assign(D->most_normal, D->most_normal + (size_t)2 * rt->dim * rt->n_dir);
  rt->sigma_t.assign(D->sigma_t, D->sigma_t + (size_t)rt->n_mat * rt->G);
  rt->sigma_s.assign(D->sigma_s, D->sigma_s + (size_t)rt->n_mat * rt->G * rt->G * (rt->l_max + 1));
  rt->material_id.assign(D->material_id, D->material_id + rt->n_cells);
  for (long c = 0; c < rt->n_cells; ++c)
    if (rt->material_id[c] < 0 || rt->material_id[c] >= rt->n_mat)
      return fail(bad(rt, "material id out of range"));
  rt->n_src = D->source ? D->n_sources : 0;
  if (D->source) rt->source.assign(D->source, D->source + (size_t)rt->n_src * rt->G);
  if (D->source_id) {
    rt->source_id.assign(D->source_id, D->source_id + rt->n_cells);
    for (long c = 0; c < rt->n_cells; ++c)
      if (rt->source_id[c] < 0 || (rt->source_id[c] >= rt->n_src && rt->n_src > 0))
        return fail(bad(rt, "source id out of range"));
  }
  for (int f = 0; f < 6; ++f) rt->bc[f] = D->bc_type[f];
  if (D->inc_flux) rt->inc_flux.assign(D->inc_flux, D->inc_flux + (size_t)2 * rt->dim * rt->G);
  for (int q = 0; q < rt->n_mom; ++q)
    if (rt->moment_l[q] < 0) return fail(bad(rt, "negative moment order"));
  for (int d = 0; d < rt->n_dir; ++d)
    for (int a = 0; a < rt->dim; ++a)
      if (rt->omega[3 * d + a] == 0.0)
        return fail(bad(rt, "a direction is parallel to a mesh face (Omega_a == 0)"));
  if (D->cell_order) {
    rt->cell_order.assign(D->cell_order, D->cell_order + rt->n_cells);
    std::vector<char> seen(rt->n_cells, 0);
    for (long c = 0; c < rt->n_cells; ++c) {
      const long o = rt->cell_order[c];
      if (o < 0 || o >= rt->n_cells || seen[o]) return fail(bad(rt, "cell_order is not a permutation"));
      seen[o] = 1;
    }
  }
  // A blocking stream: work on it is ordered after work already issued to the
  // legacy default stream (and before work issued there later), so device
  // vectors a caller has just written on that stream are read complete.
  if (cudaStreamCreateWithFlags(&rt->own_stream, cudaStreamDefault) != cudaSuccess ||
      cudaEventCreate(&rt->ev0) != cudaSuccess || cudaEventCreate(&rt->ev1) != cudaSuccess)
    return fail(cuda_fail(rt, cudaGetLastError(), "stream"));
  rt->stream = rt->own_stream;
  // the allocation-free Apply's scratch array is placed on the device here,
  // at set-up, so that no call of ouranos_rt_apply_noalloc allocates
  if (noalloc_setup(device) != OURANOS_OK)
    return fail(cuda_fail(rt, cudaGetLastError(), "allocation-free Apply set-up"));

  // |Omega| classes (the canonical cell matrix depends on |Omega_a| only)
  std::vector<int> dcls(rt->n_dir);
  for (int d = 0; d < rt->n_dir; ++d) {
    double w[3] = {0, 0, 0};
    for (int a = 0; a < rt->dim; ++a) w[a] = std::fabs(rt->omega[3 * d + a]);
    int found = -1;
    for (int c = 0; c < rt->n_dir_class && found < 0; ++c)
      if (rt->class_abs_omega[3 * c] == w[0] && rt->class_abs_omega[3 * c + 1] == w[1] &&
          rt->class_abs_omega[3 * c + 2] == w[2])
        found = c;
    if (found < 0) {
      found = rt->n_dir_class++;
      rt->class_abs_omega.insert(rt->class_abs_omega.end(), w, w + 3);
    }
    dcls[d] = found;
  }
  rt->dir_class_h = dcls;
  std::vector<double> absw((size_t)rt->n_dir * 3), d2m_t((size_t)rt->n_dir * rt->n_mom);
  for (int d = 0; d < rt->n_dir; ++d)
    for (int a = 0; a < 3; ++a) absw[3 * d + a] = std::fabs(rt->omega[3 * d + a]);
  for (int q = 0; q < rt->n_mom; ++q)
    for (int d = 0; d < rt->n_dir; ++d)
      d2m_t[(size_t)d * rt->n_mom + q] = rt->d2m[(size_t)q * rt->n_dir + d];
  std::vector<double> rowsum(rt->n, 0.0);
  for (int i = 0; i < rt->n; ++i)
    for (int j = 0; j < rt->n; ++j) rowsum[i] += rt->fe.mass[i * rt->n + j];
  std::vector<int> sid = rt->source_id;
  if (sid.empty()) sid.assign(rt->n_cells, 0);
  int rc;
  if ((rc = upload(rt, rt->d_dir_class, dcls, "dir classes")) ||
      (rc = upload(rt, rt->d_abs64, absw, "omega")) ||
      (rc = upload(rt, rt->d_abs32, to_f32(absw), "omega")) ||
      (rc = upload(rt, rt->d_absdf, to_df(absw), "omega")) ||
      (rc = upload(rt, rt->d_m2d64, rt->m2d, "m2d")) ||
      (rc = upload(rt, rt->d_m2d32, to_f32(rt->m2d), "m2d")) ||
      (rc = upload(rt, rt->d_m2ddf, to_df(rt->m2d), "m2d")) ||
      (rc = upload(rt, rt->d_d2m64, d2m_t, "d2m")) ||
      (rc = upload(rt, rt->d_d2m32, to_f32(d2m_t), "d2m")) ||
      (rc = upload(rt, rt->d_face64, pad_rows(rt->fe.face_mass, 3L * rt->fd, rt->fd), "face mass")) ||
      (rc = upload(rt, rt->d_face32, to_f32(pad_rows(rt->fe.face_mass, 3L * rt->fd, rt->fd)), "face mass")) ||
      (rc = upload(rt, rt->d_facedf, to_df(pad_rows(rt->fe.face_mass, 3L * rt->fd, rt->fd)), "face mass")) ||
      (rc = upload(rt, rt->d_cell_mass, rt->fe.mass, "mass")) ||
      (rc = upload(rt, rt->d_rowsum_mass, rowsum, "mass")) ||
      (rc = upload(rt, rt->d_material, rt->material_id, "materials")) ||
      (rc = upload(rt, rt->d_source_id, sid, "source ids")))
    return fail(rc);
  if (!rt->cell_order.empty() && (rc = upload(rt, rt->d_cell_order, rt->cell_order, "cell order")))
    return fail(rc);
  if ((rc = build_symmetry(rt))) return fail(rc);
  if (tc_contractions_fit(rt->n_dir, rt->n_mom)) {
    std::vector<uint8_t> mi, di;
    tc_build_images(rt->m2d, rt->d2m, rt->n_dir, rt->n_mom, mi, di, rt->tc.npad, rt->tc.kpad);
    if ((rc = upload(rt, rt->d_tc_m2d, mi, "tensor-core tables")) ||
        (rc = upload(rt, rt->d_tc_d2m, di, "tensor-core tables")))
      return fail(rc);
    rt->tc.m2d_img = rt->d_tc_m2d.as<uint8_t>();
    rt->tc.d2m_img = rt->d_tc_d2m.as<uint8_t>();
    rt->tc.n_dir = rt->n_dir;
    rt->tc.n_mom = rt->n_mom;
  }
  if (oz_contractions_fit(rt->n_dir, rt->n_mom)) {
    OzHost h;
    oz_build_tables(rt->m2d, rt->d2m, rt->n_dir, rt->n_mom, h);
    if ((rc = upload(rt, rt->d_oz_m2d, h.m2d_img, "tensor-core FP64 tables")) ||
        (rc = upload(rt, rt->d_oz_d2m, h.d2m_img, "tensor-core FP64 tables")) ||
        (rc = upload(rt, rt->d_oz_m2d_exp, h.m2d_exp, "tensor-core FP64 tables")) ||
        (rc = upload(rt, rt->d_oz_d2m_exp, h.d2m_exp, "tensor-core FP64 tables")))
      return fail(rc);
    rt->oz.m2d_img = rt->d_oz_m2d.as<uint8_t>();
    rt->oz.d2m_img = rt->d_oz_d2m.as<uint8_t>();
    rt->oz.m2d_exp = rt->d_oz_m2d_exp.as<int>();
    rt->oz.d2m_exp = rt->d_oz_d2m_exp.as<int>();
    rt->oz.n_dir = h.n_dir;
    rt->oz.n_mom = h.n_mom;
    rt->oz.npad = h.npad;
    rt->oz.nch = h.nch;
  }
  if ((rc = default_tiling(rt)) || (rc = build_schedule(rt)) || (rc = setup_group(rt)))
    return fail(rc);
  if (cudaStreamSynchronize(rt->stream) != cudaSuccess)
    return fail(cuda_fail(rt, cudaGetLastError(), "setup"));
  *out = rt;
  return OURANOS_OK;
}

int ouranos_rt_destroy(ouranos_rt* rt) {
  if (!rt) return OURANOS_OK;
  if (rt->stream) {
    cudaSetDevice(rt->device);
    cudaStreamSynchronize(rt->stream);
  }
  if (rt->ev0) cudaEventDestroy(rt->ev0);
  if (rt->ev1) cudaEventDestroy(rt->ev1);
  for (cudaEvent_t e : rt->ev_chunk)
    if (e) cudaEventDestroy(e);
  if (rt->copy_stream) {
    cudaStreamSynchronize(rt->copy_stream);
    cudaStreamDestroy(rt->copy_stream);
  }
  if (rt->own_stream) cudaStreamDestroy(rt->own_stream);
  delete rt;
  return OURANOS_OK;
}

int ouranos_rt_set_group(ouranos_rt* rt, int g) {
  if (!rt) return OURANOS_ERR_BAD_INPUT;
  if (g < 0 || g >= rt->G) return bad(rt, "group out of range");
  cudaSetDevice(rt->device);
  rt->group = g;
  OK_OR_RETURN(setup_group(rt));
  CU(cudaStreamSynchronize(rt->stream), "set group");
  return OURANOS_OK;
}

int ouranos_rt_set_precision(ouranos_rt* rt, int precision) {
  if (!rt) return OURANOS_ERR_BAD_INPUT;
  if (precision != OURANOS_FP64 && precision != OURANOS_FP32) return bad(rt, "unknown precision");
  rt->precision = precision;
  return OURANOS_OK;
}

int ouranos_rt_set_fp64_contractions(ouranos_rt* rt, int mode) {
  if (!rt) return OURANOS_ERR_BAD_INPUT;
  if (mode != OURANOS_FP64_NATIVE && mode != OURANOS_FP64_DF64 && mode != OURANOS_FP64_DF64_SWEEP &&
      mode != OURANOS_FP64_DF64_SWEEP_TC)
    return bad(rt, "unknown FP64 mode");
  if (mode == OURANOS_FP64_DF64_SWEEP_TC && !rt->oz.npad) {
    rt->err = "tensor-core FP64 contractions take at most 192 directions and 16 moments";
    return OURANOS_ERR_UNSUPPORTED;
  }
  rt->fp64_contract = mode;
  return OURANOS_OK;
}

int ouranos_rt_set_fp32_contractions(ouranos_rt* rt, int mode) {
  if (!rt) return OURANOS_ERR_BAD_INPUT;
  if (mode != OURANOS_FP32_CONTRACT_CUDA_CORES && mode != OURANOS_FP32_CONTRACT_TENSOR)
    return bad(rt, "unknown FP32 contraction mode");
  if (mode == OURANOS_FP32_CONTRACT_TENSOR && !rt->tc.npad) {
    rt->err = "tensor-core contractions take at most 256 directions and 16 moments";
    return OURANOS_ERR_UNSUPPORTED;
  }
  rt->fp32_contract = mode;
  return OURANOS_OK;
}

int ouranos_rt_vector_length(const ouranos_rt* rt, long* length) {
  if (!rt || !length) return OURANOS_ERR_BAD_INPUT;
  *length = vec_len(rt);
  return OURANOS_OK;
}

int ouranos_rt_n_tasks(const ouranos_rt* rt, long* n_tasks) {
  if (!rt || !n_tasks) return OURANOS_ERR_BAD_INPUT;
  *n_tasks = rt->n_cells * rt->n_dir;
  return OURANOS_OK;
}

int ouranos_rt_scattering_source(ouranos_rt* rt, const double* x) {
  if (!rt || !x) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  // S = sigma_s M x is rebuilt from the stored argument at each sweep (it is
  // cheap next to the sweep and keeps one FP64 copy for both precisions)
  const double* dx = nullptr;
  OK_OR_RETURN(stage_in(rt, x, rt->d_x, 1, &dx));
  CU(rt->d_scatx.alloc(sizeof(double) * vec_len(rt)), "scattering source");
  CU(cudaMemcpyAsync(rt->d_scatx.p, dx, sizeof(double) * vec_len(rt), cudaMemcpyDeviceToDevice,
                     rt->stream),
     "scattering source");
  rt->scat_valid = true;
  CU(cudaStreamSynchronize(rt->stream), "scattering source");
  return OURANOS_OK;
}

int ouranos_rt_sweep(ouranos_rt* rt, double* flux, const double* group_flux) {
  if (!rt || !flux) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  OK_OR_RETURN(clear_status(rt));
  const double* dgf = nullptr;
  if (group_flux) OK_OR_RETURN(stage_in(rt, group_flux, rt->d_gf, rt->G, &dgf));
  OK_OR_RETURN(build_source(rt, rt->scat_valid ? rt->d_scatx.as<double>() : nullptr, dgf, df64_sweep(rt)));
  OK_OR_RETURN(sweep_into_phi(rt, group_flux != nullptr));
  const double* dflux = nullptr;
  OK_OR_RETURN(stage_in(rt, flux, rt->d_x, 1, &dflux));
  CU(rt->d_y.alloc(sizeof(double) * vec_len(rt)), "flux");
  OK_OR_RETURN(phi_combine(rt, dflux, rt->d_y.as<double>(), 1.0, 1.0));  // flux + phi
  OK_OR_RETURN(stage_out(rt, rt->d_y.as<double>(), flux));
  return finish(rt);
}

int ouranos_rt_apply(ouranos_rt* rt, const double* x, double* y) {
  if (!rt || !x || !y) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  OK_OR_RETURN(clear_status(rt));
  if (rt->cell_order.empty() && is_pinned_host_ptr(x) && is_pinned_host_ptr(y) &&
      rt->n_cells >= 64 * OURANOS_OVERLAP_CHUNKS) {
    if (df64_sweep(rt)) OK_OR_RETURN(apply_overlapped<df64>(rt, x, y));
    else if (rt->precision == OURANOS_FP64) OK_OR_RETURN(apply_overlapped<double>(rt, x, y));
    else OK_OR_RETURN(apply_overlapped<float>(rt, x, y));
    return finish(rt);
  }
  const double* dx = nullptr;
  OK_OR_RETURN(stage_in(rt, x, rt->d_x, 1, &dx));
  CU(rt->d_y.alloc(sizeof(double) * vec_len(rt)), "apply");
  OK_OR_RETURN(rt_apply_device(rt, dx, rt->d_y.as<double>()));
  OK_OR_RETURN(stage_out(rt, rt->d_y.as<double>(), y));
  return finish(rt);
}

int ouranos_rt_sweep_rhs(ouranos_rt* rt, const double* group_flux, double* rhs) {
  if (!rt || !rhs) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  OK_OR_RETURN(clear_status(rt));
  const double* dgf = nullptr;
  if (group_flux) OK_OR_RETURN(stage_in(rt, group_flux, rt->d_gf, rt->G, &dgf));
  OK_OR_RETURN(build_source(rt, nullptr, dgf, df64_sweep(rt)));
  OK_OR_RETURN(sweep_into_phi(rt, true));
  const double* drhs = nullptr;
  OK_OR_RETURN(stage_in(rt, rhs, rt->d_x, 1, &drhs));
  CU(rt->d_y.alloc(sizeof(double) * vec_len(rt)), "rhs");
  OK_OR_RETURN(phi_combine(rt, drhs, rt->d_y.as<double>(), 1.0, 1.0));
  OK_OR_RETURN(stage_out(rt, rt->d_y.as<double>(), rhs));
  return finish(rt);
}

int ouranos_rt_set_time_step(ouranos_rt* rt, double inv_vdt) {
  if (!rt) return OURANOS_ERR_BAD_INPUT;
  if (!(inv_vdt >= 0.0) || !std::isfinite(inv_vdt)) return bad(rt, "1/(v dt) must be finite and >= 0");
  cudaSetDevice(rt->device);
  CU(cudaStreamSynchronize(rt->stream), "time step");
  rt->inv_vdt = inv_vdt;
  OK_OR_RETURN(setup_group(rt));  // sigma_t classes and cell inverses with the shift
  if (inv_vdt > 0.0) {
    const size_t bytes = sizeof(float) * (size_t)rt->n_dir * rt->n_dofs;
    CU(rt->d_psi_prev.alloc(bytes), "angular flux of the previous step");
    CU(cudaMemsetAsync(rt->d_psi_prev.p, 0, bytes, rt->stream), "angular flux of the previous step");
  } else {
    rt->d_psi_prev.release();
  }
  CU(cudaStreamSynchronize(rt->stream), "time step");
  return OURANOS_OK;
}

int ouranos_rt_set_source(ouranos_rt* rt, const double* source) {
  if (!rt || (!source && rt->n_src > 0)) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  CU(cudaStreamSynchronize(rt->stream), "source");
  for (size_t k = 0; k < (size_t)rt->n_src * rt->G; ++k) {
    if (!std::isfinite(source[k])) return bad(rt, "source strengths must be finite");
    rt->source[k] = source[k];
  }
  // fixed source per source id: q/ws (src/RadiativeTransfer.cc:918-921)
  std::vector<double> q(std::max(rt->n_src, 1), 0.0);
  for (int s = 0; s < rt->n_src; ++s) q[s] = rt->source[(size_t)s * rt->G + rt->group] / rt->ws;
  OK_OR_RETURN(upload(rt, rt->d_qcell, q, "sources"));
  CU(cudaStreamSynchronize(rt->stream), "source");
  return OURANOS_OK;
}

// One implicit Euler step: phi^{n+1} from (I - T) phi = D L^-1 (q + inflow +
// inv_vdt M psi^n) with `solver` started from phi (e.g. phi^n), then psi^n <-
// psi^{n+1} by one FP64 source sweep of phi^{n+1}, stored in FP32.  psi^n is
// left as it was when the solve does not converge.
int ouranos_rt_time_advance(ouranos_rt* rt, int solver, int restart, int max_it, double tol, double* phi,
                            ouranos_solve_info* info) {
  if (!rt || !phi) return OURANOS_ERR_BAD_INPUT;
  if (!(rt->inv_vdt > 0.0) || !rt->d_psi_prev.p) return bad(rt, "no time step set (ouranos_rt_set_time_step)");
  const int rc = ouranos_solve(rt, solver | OURANOS_SOLVER_WARM_START, restart, max_it, tol, nullptr, phi,
                               nullptr, info);
  if (rc != OURANOS_OK) return rc;
  cudaSetDevice(rt->device);
  OK_OR_RETURN(clear_status(rt));
  const double* dphi = nullptr;
  OK_OR_RETURN(stage_in(rt, phi, rt->d_x, 1, &dphi));
  const int saved = rt->precision;
  rt->precision = OURANOS_FP64;
  int r2 = build_source(rt, dphi, nullptr, df64_sweep(rt));
  if (r2 == OURANOS_OK) r2 = sweep_into_phi(rt, true);
  rt->precision = saved;
  OK_OR_RETURN(r2);
  rt->precision = OURANOS_FP64;
  const bool pairs = df64_sweep(rt);
  rt->precision = saved;
  if (pairs)
    CU(launch_to_f32_pairs(rt->d_psi.as<df64>(), rt->d_psi_prev.as<float>(), (long)rt->n_dir * rt->n_dofs,
                           rt->stream),
       "angular flux");
  else
    CU(launch_to_f32(rt->d_psi.as<double>(), rt->d_psi_prev.as<float>(), (long)rt->n_dir * rt->n_dofs,
                     rt->stream),
       "angular flux");
  return finish(rt);
}

// psi^n as doubles ([dir][dof], lexicographic cells) -- a checkpoint's state
int ouranos_rt_get_angular_flux(ouranos_rt* rt, double* psi) {
  if (!rt || !psi) return OURANOS_ERR_BAD_INPUT;
  if (!rt->d_psi_prev.p) return bad(rt, "no time step set (ouranos_rt_set_time_step)");
  cudaSetDevice(rt->device);
  const size_t n = (size_t)rt->n_dir * rt->n_dofs;
  std::vector<float> h(n);
  CU(cudaMemcpyAsync(h.data(), rt->d_psi_prev.p, sizeof(float) * n, cudaMemcpyDeviceToHost, rt->stream),
     "angular flux");
  CU(cudaStreamSynchronize(rt->stream), "angular flux");
  for (size_t k = 0; k < n; ++k) psi[k] = h[k];
  return OURANOS_OK;
}

int ouranos_rt_set_angular_flux(ouranos_rt* rt, const double* psi) {
  if (!rt || !psi) return OURANOS_ERR_BAD_INPUT;
  if (!rt->d_psi_prev.p) return bad(rt, "no time step set (ouranos_rt_set_time_step)");
  cudaSetDevice(rt->device);
  const size_t n = (size_t)rt->n_dir * rt->n_dofs;
  std::vector<float> h(n);
  for (size_t k = 0; k < n; ++k) h[k] = (float)psi[k];
  CU(cudaMemcpyAsync(rt->d_psi_prev.p, h.data(), sizeof(float) * n, cudaMemcpyHostToDevice, rt->stream),
     "angular flux");
  CU(cudaStreamSynchronize(rt->stream), "angular flux");
  return OURANOS_OK;
}

int ouranos_wavefront_levels(int dim, const int* nx, int n_dir, const double* omega, int* levels) {
  if ((dim != 2 && dim != 3) || !nx || n_dir < 1 || !omega || !levels) return OURANOS_ERR_BAD_INPUT;
  long n_cells = 1;
  for (int a = 0; a < dim; ++a) {
    if (nx[a] < 1) return OURANOS_ERR_BAD_INPUT;
    n_cells *= nx[a];
  }
  // wavefront level of (direction, cell): its distance in cells from the
  // corner the direction enters through, sum_a (Omega_a > 0 ? i_a : N_a - 1 - i_a)
  // -- the longest upwind chain ending at the cell in the task graph of
  // src/RadiativeTransfer.cc:80-232
  for (int d = 0; d < n_dir; ++d)
    for (long c = 0; c < n_cells; ++c) {
      long r = c;
      int lev = 0;
      for (int a = 0; a < dim; ++a) {
        const int i = (int)(r % nx[a]);
        r /= nx[a];
        lev += omega[3 * d + a] > 0.0 ? i : nx[a] - 1 - i;
      }
      levels[(size_t)d * n_cells + c] = lev;
    }
  return OURANOS_OK;
}

int ouranos_rt_task_levels(const ouranos_rt* rt, int* levels) {
  if (!rt || !levels) return OURANOS_ERR_BAD_INPUT;
  return ouranos_wavefront_levels(rt->dim, rt->nx, rt->n_dir, rt->omega.data(), levels);
}

int ouranos_rt_set_stream(ouranos_rt* rt, void* stream) {
  if (!rt) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  CU(cudaStreamSynchronize(rt->stream), "set stream");
  rt->stream = stream ? (cudaStream_t)stream : rt->own_stream;
  return OURANOS_OK;
}

int ouranos_rt_last_error(const ouranos_rt* rt, char* buf, size_t len) {
  if (!rt || !buf || !len) return OURANOS_ERR_BAD_INPUT;
  std::snprintf(buf, len, "%s", rt->err.c_str());
  return OURANOS_OK;
}

int ouranos_rt_last_sweep_ms(const ouranos_rt* rt, double* ms, int* kernels) {
  if (!rt) return OURANOS_ERR_BAD_INPUT;
  if (ms) *ms = rt->last_ms;
  if (kernels) *kernels = rt->last_kernels;
  return OURANOS_OK;
}

int ouranos_rt_set_tiling(ouranos_rt* rt, int cells_x, int cells_y, int dirs) {
  if (!rt) return OURANOS_ERR_BAD_INPUT;
  cudaSetDevice(rt->device);
  const bool was_wide = rt->lpc == 32;
  if (cells_x == 0 && cells_y == 0 && dirs == 0) {
    OK_OR_RETURN(default_tiling(rt));
  } else {
    if (rt->dim == 2) cells_y = 1;
    const int lanes = cells_x * cells_y * dirs;
    const bool wide = lanes == 1;            // one warp per cell
    const bool two = lanes == 16 && rt->n >= 9;  // two lanes per cell
    if (cells_x < 1 || cells_y < 1 || dirs < 1 || (lanes != 32 && !two && !wide) || (dirs & (dirs - 1)))
      return bad(rt, "tiling must satisfy cells_x*cells_y*dirs == 32 (or 16, two lanes per cell, for cells "
                     "of 9 or more dofs; or 1 x 1 x 1, one warp per cell) with dirs a power of two");
    if (!wide && !register_form(rt))
      return bad(rt, "this DG order runs one warp per cell only (tiling 1 x 1 x 1): the per-lane sweep "
                     "covers 2-D Q1..Q4 and 3-D Q1..Q2");
    rt->wx = cells_x;
    rt->wy = cells_y;
    rt->kd = dirs;
    rt->lpc = wide ? 32 : (two ? 2 : 1);
  }
  OK_OR_RETURN(build_schedule(rt));
  if (was_wide != (rt->lpc == 32)) OK_OR_RETURN(setup_group(rt));  // the inverse tables change layout
  CU(cudaStreamSynchronize(rt->stream), "tiling");
  return OURANOS_OK;
}

int ouranos_rt_get_tiling(const ouranos_rt* rt, int* cx, int* cy, int* dirs) {
  if (!rt) return OURANOS_ERR_BAD_INPUT;
  if (cx) *cx = rt->wx;
  if (cy) *cy = rt->wy;
  if (dirs) *dirs = rt->kd;
  return OURANOS_OK;
}

int ouranos_rt_set_wait_limit(ouranos_rt* rt, double ns) {
  if (!rt || !(ns > 0)) return OURANOS_ERR_BAD_INPUT;
  rt->wait_limit_ns = (long long)ns;
  return OURANOS_OK;
}

int ouranos_rt_debug_wait_bias(ouranos_rt* rt, int extra) {
  if (!rt || extra < 0) return OURANOS_ERR_BAD_INPUT;
  rt->wait_bias = extra;
  return OURANOS_OK;
}

}  // extern "C"
