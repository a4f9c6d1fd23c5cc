// Drivers around the operator: the source iteration and Krylov solves of
// src/ouranos.cc:43-209 (the reference hands Apply to AztecOO through deal.II's
// TrilinosWrappers::SolverGMRES / SolverBicgstab; here the methods are written
// out on device vectors).  Gram-Schmidt, norms and dot products are FP64
// (classical Gram-Schmidt with one re-orthogonalisation pass); the small
// Hessenberg least-squares problem is solved on the host.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "internal.h"

using namespace ouranos;

namespace {

#define RC(expr)                       \
  do {                                 \
    int _rc = (expr);                  \
    if (_rc != OURANOS_OK) return _rc; \
  } while (0)

int cfail(ouranos_rt* rt, cudaError_t e, const char* what) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  rt->err = buf;
  return OURANOS_ERR_CUDA;
}
#define CUC(expr, what)                                \
  do {                                                 \
    cudaError_t _e = (expr);                           \
    if (_e != cudaSuccess) return cfail(rt, _e, what); \
  } while (0)

struct Work {
  ouranos_rt* rt;
  long len;
  int nvec;
  double* base = nullptr;
  double** dptrs = nullptr;   // device array of vector pointers (scratch, 64)
  double** vptrs = nullptr;   // device array of every basis vector's pointer (64)
  double* dres = nullptr;     // device results (64) + partials
  std::vector<double*> vec;   // host copy of vector pointers
  double* v(int i) const { return vec[i]; }
};

int make_work(ouranos_rt* rt, int nvec, Work& w) {
  w.rt = rt;
  w.len = (long)rt->n_mom * rt->n_dofs;
  w.nvec = nvec;
  const size_t vbytes = sizeof(double) * (size_t)w.len;
  const size_t ptr_bytes = sizeof(double*) * 128;
  const size_t res_bytes = sizeof(double) * (64 + 64 * (size_t)kDotGrid);
  const size_t total = vbytes * nvec + ptr_bytes + res_bytes + 256;
  CUC(rt->d_krylov.alloc(total), "solver workspace");
  char* p = (char*)rt->d_krylov.p;
  w.base = (double*)p;
  w.vec.resize(nvec);
  for (int i = 0; i < nvec; ++i) w.vec[i] = w.base + (size_t)i * w.len;
  p += vbytes * nvec;
  w.dptrs = (double**)p;
  w.vptrs = w.dptrs + 64;
  p += ptr_bytes;
  w.dres = (double*)p;
  return OURANOS_OK;
}

int dot_pair(Work& w, const double* a, const double* b, double* out) {
  ouranos_rt* rt = w.rt;
  const double* ptrs[1] = {a};
  CUC(cudaMemcpyAsync(w.dptrs, ptrs, sizeof(double*), cudaMemcpyHostToDevice, rt->stream), "dot");
  CUC(launch_dots((const double* const*)w.dptrs, b, 1, w.len, w.dres, w.dres + 64,
                  rt->stream),
      "dot");
  CUC(cudaMemcpyAsync(out, w.dres, sizeof(double), cudaMemcpyDeviceToHost, rt->stream), "dot");
  CUC(cudaStreamSynchronize(rt->stream), "dot");
  return OURANOS_OK;
}

double nrm(Work& w, const double* a, int* rc) {
  double v = 0.0;
  *rc = dot_pair(w, a, a, &v);
  return std::sqrt(std::fmax(v, 0.0));
}

// op(x) -> y : FP64 or FP32 sweep Apply
int apply_prec(ouranos_rt* rt, int precision, const double* x, double* y) {
  const int saved = rt->precision;
  rt->precision = precision;
  int rc = rt_apply_device(rt, x, y);
  rt->precision = saved;
  return rc;
}

// x += sum_j y_j Z_{first+j}
int update(Work& w, int first, const std::vector<double>& y, double* x) {
  ouranos_rt* rt = w.rt;
  const int k = (int)y.size();
  if (!k) return OURANOS_OK;
  CUC(cudaMemcpyAsync(w.dptrs, &w.vec[first], sizeof(double*) * k, cudaMemcpyHostToDevice,
                      rt->stream),
      "update");
  CUC(cudaMemcpyAsync(w.dres, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, rt->stream),
      "update");
  CUC(launch_multi_axpy((const double* const*)w.dptrs, k, w.dres, 1.0, x, w.len, rt->stream),
      "update");
  CUC(cudaStreamSynchronize(rt->stream), "update");
  return OURANOS_OK;
}

// Restarted (F)GMRES.  Arnoldi applies use `inner_prec`; each cycle starts
// from the FP64 true residual.  mixed: the cycle stops once its own residual
// estimate has dropped by `inner_drop` (FP32 operator accuracy), and the FP64
// restart refines the solution (iterative refinement).
// dsa: the diffusion synthetic acceleration is the right preconditioner; with
// learned, the network's output starts its CG (and the plain diffusion
// correction is the fallback).
int gmres(ouranos_rt* rt, int m, int max_it, double tol, const double* b, double* x,
          double* hist, ouranos_solve_info* info, int inner_prec, double inner_drop,
          bool learned = false, bool warm = false, bool dsa = false) {
  m = std::max(1, std::min(m, 32));  // dot kernel handles up to 32 basis vectors
  const bool flexible = inner_prec != OURANOS_FP64 || dsa;
  // vectors: V[0..m], Z[0..m-1] (flexible), r
  Work w;
  const int nv = (m + 1) + (flexible ? m : 0) + 1;
  RC(make_work(rt, nv, w));
  const int V0 = 0, Z0 = m + 1, R = nv - 1;
  int rc = 0;
  // the basis pointers once, and a pinned block for each iteration's
  // Gram-Schmidt coefficients ([0,32) pass 1, [32,64) pass 2, [64] |w|^2)
  CUC(cudaMemcpyAsync(w.vptrs, &w.vec[V0], sizeof(double*) * (m + 1), cudaMemcpyHostToDevice, rt->stream),
      "gmres");
  struct Pinned {
    double* p = nullptr;
    ~Pinned() {
      if (p) cudaFreeHost(p);
    }
  } hb;
  CUC(cudaMallocHost((void**)&hb.p, sizeof(double) * 128), "gmres");
  const double bnorm = nrm(w, b, &rc);
  RC(rc);
  if (!warm) CUC(cudaMemsetAsync(x, 0, sizeof(double) * w.len, rt->stream), "gmres");
  int total = 0, cycles = 0;
  bool use_pc = learned && rt->cnn;
  enum { kPcTrial, kPcCompare, kPcOn, kPcOff };
  int pc_state = kPcTrial;
  double pc_rate = 0.0, plain_rate = 0.0;
  double rel = bnorm > 0 ? 1.0 : 0.0;
  if (hist) hist[0] = rel;
  bool converged = bnorm == 0.0;
  if (converged && warm) CUC(cudaMemsetAsync(x, 0, sizeof(double) * w.len, rt->stream), "gmres");  // b = 0: x = 0
  while (!converged && total < max_it) {
    // true residual r = b - A x in FP64
    if (cycles == 0 && !warm) {  // x = 0: r = b
      CUC(cudaMemcpyAsync(w.v(R), b, sizeof(double) * w.len, cudaMemcpyDeviceToDevice, rt->stream),
          "gmres");
    } else {
      RC(apply_prec(rt, OURANOS_FP64, x, w.v(R)));
      CUC(launch_axpby(1.0, b, -1.0, w.v(R), w.len, rt->stream), "gmres");
    }
    const double beta = nrm(w, w.v(R), &rc);
    RC(rc);
    rel = beta / bnorm;
    if (rel < tol) {
      converged = true;
      break;
    }
    ++cycles;
    CUC(launch_axpby(1.0 / beta, w.v(R), 0.0, w.v(V0), w.len, rt->stream), "gmres");
    Givens gv(m);
    gv.g[0] = beta;
    int k = 0;
    std::vector<double> col(m + 2);
    for (; k < m && total < max_it; ++k) {
      const double* vin = w.v(V0 + k);
      if (flexible) {
        // right preconditioner: z_k = P(v_k), learned correction, diffusion
        // correction or identity
        if (use_pc && dsa) {
          RC(rt_pc_dsa_apply(rt, vin, w.v(Z0 + k)));
        } else if (use_pc) {
          RC(ouranos_rt_pc_apply(rt, vin, w.v(Z0 + k)));
        } else if (dsa) {
          RC(rt_dsa_apply(rt, vin, w.v(Z0 + k)));
        } else {
          CUC(cudaMemcpyAsync(w.v(Z0 + k), vin, sizeof(double) * w.len, cudaMemcpyDeviceToDevice,
                              rt->stream),
              "fgmres");
        }
        vin = w.v(Z0 + k);
      }
      double* nxt = w.v(V0 + k + 1);
      RC(apply_prec(rt, inner_prec, vin, nxt));
      // CGS2 with the coefficients kept on the device, the norm and the
      // normalisation too: one host synchronisation per iteration
      for (int pass = 0; pass < 2; ++pass) {
        CUC(launch_dots((const double* const*)w.vptrs, nxt, k + 1, w.len, w.dres, w.dres + 64,
                        rt->stream),
            "orthogonalise");
        CUC(cudaMemcpyAsync(hb.p + 32 * pass, w.dres, sizeof(double) * (k + 1), cudaMemcpyDeviceToHost,
                            rt->stream),
            "orthogonalise");
        CUC(launch_multi_axpy((const double* const*)w.vptrs, k + 1, w.dres, -1.0, nxt, w.len, rt->stream),
            "orthogonalise");
      }
      CUC(launch_dots((const double* const*)(w.vptrs + k + 1), nxt, 1, w.len, w.dres, w.dres + 64,
                      rt->stream),
          "norm");
      CUC(cudaMemcpyAsync(hb.p + 64, w.dres, sizeof(double), cudaMemcpyDeviceToHost, rt->stream), "norm");
      CUC(launch_scale_inv_norm(w.dres, nxt, w.len, rt->stream), "normalise");
      CUC(cudaStreamSynchronize(rt->stream), "gmres");
      for (int j = 0; j <= k; ++j) col[j] = hb.p[j] + hb.p[32 + j];
      const double hn = std::sqrt(std::max(hb.p[64], 0.0));
      col[k + 1] = hn;
      const double est = gv.add_column(k, col.data()) / bnorm;
      ++total;
      if (hist) hist[total] = est;
      if (est < tol || (flexible && est < rel * inner_drop) || hn == 0.0) {
        ++k;
        break;
      }
    }
    std::vector<double> y = gv.solve(k);
    RC(update(w, flexible ? Z0 : V0, y, x));
    // Safeguard for the learned preconditioner (the plain method is its
    // fallback).  A preconditioned cycle that needed all m steps is suspect:
    // the next cycle runs unpreconditioned, and the solve keeps whichever of
    // the two reduced the residual estimate more per iteration.  While the
    // preconditioner stays on, every later full cycle is held to that plain
    // rate; one that falls behind switches it off for the rest of the solve.
    if (learned && rt->cnn && k > 0 && pc_state != kPcOff) {
      const double est = std::max(std::fabs(gv.g[k]) / bnorm, 1e-300);
      const double rate = std::log(est / rel) / k;  // < 0; more negative = faster
      if (pc_state == kPcTrial && use_pc && k == m) {
        pc_rate = rate;
        pc_state = kPcCompare;
        use_pc = false;
      } else if (pc_state == kPcCompare) {
        plain_rate = rate;
        use_pc = pc_rate < plain_rate;
        pc_state = use_pc ? kPcOn : kPcOff;
      } else if (pc_state == kPcOn && k == m && rate > plain_rate) {
        use_pc = false;
        pc_state = kPcOff;
      }
    }
  }
  // final FP64 true residual (already in hand when the loop ended on it)
  double fin = rel;
  if (!converged) {
    RC(apply_prec(rt, OURANOS_FP64, x, w.v(R)));
    CUC(launch_axpby(1.0, b, -1.0, w.v(R), w.len, rt->stream), "gmres");
    fin = nrm(w, w.v(R), &rc) / (bnorm > 0 ? bnorm : 1.0);
    RC(rc);
  }
  RC(rt_check_status(rt));
  info->iterations = total;
  info->restarts = cycles;
  info->residual = fin;
  info->converged = fin < tol;
  return OURANOS_OK;
}

int bicgstab(ouranos_rt* rt, int max_it, double tol, const double* b, double* x, double* hist,
             ouranos_solve_info* info) {
  Work w;
  RC(make_work(rt, 7, w));
  double *r = w.v(0), *r0 = w.v(1), *p = w.v(2), *v = w.v(3), *s = w.v(4), *t = w.v(5);
  int rc = 0;
  const double bnorm = nrm(w, b, &rc);
  RC(rc);
  CUC(cudaMemsetAsync(x, 0, sizeof(double) * w.len, rt->stream), "bicgstab");
  CUC(cudaMemcpyAsync(r, b, sizeof(double) * w.len, cudaMemcpyDeviceToDevice, rt->stream), "bicgstab");
  CUC(cudaMemcpyAsync(r0, b, sizeof(double) * w.len, cudaMemcpyDeviceToDevice, rt->stream), "bicgstab");
  CUC(cudaMemsetAsync(p, 0, sizeof(double) * w.len, rt->stream), "bicgstab");
  CUC(cudaMemsetAsync(v, 0, sizeof(double) * w.len, rt->stream), "bicgstab");
  double rho = 1.0, alpha = 1.0, om = 1.0;
  if (hist) hist[0] = 1.0;
  int it = 0;
  for (; it < max_it && bnorm > 0; ++it) {
    double rho1;
    RC(dot_pair(w, r0, r, &rho1));
    const double beta = (rho1 / rho) * (alpha / om);
    rho = rho1;
    // p = r + beta (p - om v)
    CUC(launch_axpby(-om, v, 1.0, p, w.len, rt->stream), "bicgstab");
    CUC(launch_axpby(1.0, r, beta, p, w.len, rt->stream), "bicgstab");
    RC(apply_prec(rt, OURANOS_FP64, p, v));
    double r0v;
    RC(dot_pair(w, r0, v, &r0v));
    alpha = rho / r0v;
    CUC(cudaMemcpyAsync(s, r, sizeof(double) * w.len, cudaMemcpyDeviceToDevice, rt->stream), "bicgstab");
    CUC(launch_axpby(-alpha, v, 1.0, s, w.len, rt->stream), "bicgstab");
    RC(apply_prec(rt, OURANOS_FP64, s, t));
    double ts, tt;
    RC(dot_pair(w, t, s, &ts));
    RC(dot_pair(w, t, t, &tt));
    om = tt > 0 ? ts / tt : 0.0;
    CUC(launch_axpby(alpha, p, 1.0, x, w.len, rt->stream), "bicgstab");
    CUC(launch_axpby(om, s, 1.0, x, w.len, rt->stream), "bicgstab");
    CUC(cudaMemcpyAsync(r, s, sizeof(double) * w.len, cudaMemcpyDeviceToDevice, rt->stream), "bicgstab");
    CUC(launch_axpby(-om, t, 1.0, r, w.len, rt->stream), "bicgstab");
    const double rel = nrm(w, r, &rc) / bnorm;
    RC(rc);
    if (hist) hist[it + 1] = rel;
    if (rel < tol) {
      ++it;
      break;
    }
  }
  RC(apply_prec(rt, OURANOS_FP64, x, t));
  CUC(launch_axpby(1.0, b, -1.0, t, w.len, rt->stream), "bicgstab");
  const double fin = nrm(w, t, &rc) / (bnorm > 0 ? bnorm : 1.0);
  RC(rc);
  RC(rt_check_status(rt));
  info->iterations = it;
  info->restarts = 0;
  info->residual = fin;
  info->converged = fin < tol;
  return OURANOS_OK;
}

// Source iteration phi <- D L^-1 (M2D S phi + q + inflow) (src/ouranos.cc:72-95,
// written as intended: a fresh sweep each iteration), relative-change test.
// With dsa, the change of each iteration is accelerated by the diffusion
// correction of its scalar moment: phi <- phi + P (T phi + rhs - phi).
int source_iteration(ouranos_rt* rt, int max_it, double tol, const double* gf, const double* b,
                     double* x, double* hist, ouranos_solve_info* info, bool warm, bool dsa) {
  Work w;
  RC(make_work(rt, 3, w));
  double *xn = w.v(0), *dlt = w.v(1), *rr = w.v(2);
  int rc = 0;
  if (!warm) CUC(cudaMemsetAsync(x, 0, sizeof(double) * w.len, rt->stream), "si");
  int it = 0;
  double rel = 1.0;
  for (; it < max_it; ++it) {
    // phi_new = T phi + rhs  (the rhs sweep is linear: sweep(S x + q) = T x + rhs)
    RC(rt_apply_device(rt, x, xn));                          // xn = x - T x
    CUC(launch_axpby(1.0, x, -1.0, xn, w.len, rt->stream), "si");  // xn = T x
    CUC(launch_axpby(1.0, b, 1.0, xn, w.len, rt->stream), "si");   // xn = T x + rhs
    CUC(cudaMemcpyAsync(dlt, xn, sizeof(double) * w.len, cudaMemcpyDeviceToDevice, rt->stream), "si");
    CUC(launch_axpby(-1.0, x, 1.0, dlt, w.len, rt->stream), "si");
    if (dsa) {
      RC(rt_dsa_apply(rt, dlt, dlt));
      CUC(cudaMemcpyAsync(xn, x, sizeof(double) * w.len, cudaMemcpyDeviceToDevice, rt->stream), "si");
      CUC(launch_axpby(1.0, dlt, 1.0, xn, w.len, rt->stream), "si");
    }
    const double num = nrm(w, dlt, &rc);
    RC(rc);
    const double den = nrm(w, xn, &rc);
    RC(rc);
    CUC(cudaMemcpyAsync(x, xn, sizeof(double) * w.len, cudaMemcpyDeviceToDevice, rt->stream), "si");
    rel = den > 0 ? num / den : 0.0;
    if (hist) hist[it] = rel;
    if (rel < tol) {
      ++it;
      break;
    }
  }
  (void)gf;
  RC(apply_prec(rt, OURANOS_FP64, x, rr));
  CUC(launch_axpby(1.0, b, -1.0, rr, w.len, rt->stream), "si");
  const double bn = nrm(w, b, &rc);
  RC(rc);
  const double fin = nrm(w, rr, &rc) / (bn > 0 ? bn : 1.0);
  RC(rc);
  RC(rt_check_status(rt));
  info->iterations = it;
  info->restarts = 0;
  info->residual = fin;
  info->converged = rel < tol;
  return OURANOS_OK;
}


// One group's solve on device vectors in the handle's numbering: dgf (may be
// NULL) the group fluxes of the other groups, sol the initial guess (with
// OURANOS_SOLVER_WARM_START) and the solution.  Flags as in ouranos_solve.
int solve_device(ouranos_rt* rt, int solver, int restart, int max_it, double tol, const double* dgf, double* sol,
                 double* hist, ouranos_solve_info* info) {
  const bool warm = (solver & OURANOS_SOLVER_WARM_START) != 0;
  const bool dsa = (solver & OURANOS_SOLVER_DSA) != 0;
  solver &= ~(OURANOS_SOLVER_WARM_START | OURANOS_SOLVER_DSA);
  if (dsa && (solver == OURANOS_SOLVER_BICGSTAB || rt->dsa_iters < 1)) {
    rt->err = solver == OURANOS_SOLVER_BICGSTAB ? "BiCGSTAB runs unpreconditioned"
                                                : "diffusion acceleration is off (ouranos_rt_set_dsa)";
    return OURANOS_ERR_BAD_INPUT;
  }
  if (warm && solver == OURANOS_SOLVER_BICGSTAB) {
    rt->err = "BiCGSTAB starts from zero";
    return OURANOS_ERR_UNSUPPORTED;
  }
  std::memset(info, 0, sizeof *info);
  // rhs and solution live in their own buffers while the solver workspace
  // holds the Krylov vectors
  const long len = (long)rt->n_mom * rt->n_dofs;
  DevBuf rhs, x;
  CUC(rhs.alloc(sizeof(double) * len), "rhs");
  CUC(x.alloc(sizeof(double) * len), "solution");
  RC(rt_rhs_device(rt, dgf, rhs.as<double>()));
  if (warm) CUC(cudaMemcpyAsync(x.p, sol, sizeof(double) * len, cudaMemcpyDeviceToDevice, rt->stream), "guess");
  const int saved = rt->precision;
  int rc;
  switch (solver) {
    case OURANOS_SOLVER_SI:
      rc = source_iteration(rt, max_it, tol, dgf, rhs.as<double>(), x.as<double>(), hist, info, warm, dsa);
      break;
    case OURANOS_SOLVER_GMRES:
      rc = gmres(rt, restart, max_it, tol, rhs.as<double>(), x.as<double>(), hist, info,
                 OURANOS_FP64, 0.0, false, warm, dsa);
      break;
    case OURANOS_SOLVER_BICGSTAB:
      rc = bicgstab(rt, max_it, tol, rhs.as<double>(), x.as<double>(), hist, info);
      break;
    case OURANOS_SOLVER_FGMRES_MIXED:
      rc = gmres(rt, restart, max_it, tol, rhs.as<double>(), x.as<double>(), hist, info,
                 OURANOS_FP32, 1e-5, false, warm, dsa);
      break;
    case OURANOS_SOLVER_FGMRES_LEARNED:
      if (!rt->cnn) {
        rt->err = "no preconditioner installed (ouranos_rt_set_preconditioner)";
        rc = OURANOS_ERR_BAD_INPUT;
        break;
      }
      rc = gmres(rt, restart, max_it, tol, rhs.as<double>(), x.as<double>(), hist, info,
                 OURANOS_FP32, 1e-5, true, warm, dsa);
      break;
    default:
      rt->err = "unknown solver";
      rc = OURANOS_ERR_BAD_INPUT;
  }
  rt->precision = saved;
  if (rc) return rc;
  CUC(cudaMemcpyAsync(sol, x.p, sizeof(double) * len, cudaMemcpyDeviceToDevice, rt->stream), "solution");
  return OURANOS_OK;
}

}  // namespace

extern "C" int ouranos_solve(ouranos_rt* rt, int solver, int restart, int max_it, double tol,
                             const double* group_flux, double* x, double* hist,
                             ouranos_solve_info* info) {
  if (!rt || !x || max_it < 1 || !(tol > 0)) return OURANOS_ERR_BAD_INPUT;
  ouranos_solve_info local;
  if (!info) info = &local;
  std::memset(info, 0, sizeof *info);
  cudaSetDevice(rt->device);
  RC(rt_clear_status(rt));
  const auto t0 = std::chrono::steady_clock::now();
  const double* dgf = nullptr;
  if (group_flux) RC(rt_stage_in(rt, group_flux, rt->d_gf, rt->G, &dgf));
  const long len = (long)rt->n_mom * rt->n_dofs;
  DevBuf sol;
  CUC(sol.alloc(sizeof(double) * len), "solution");
  if (solver & OURANOS_SOLVER_WARM_START) {
    const double* dx = nullptr;
    RC(rt_stage_in(rt, x, rt->d_x, 1, &dx));
    CUC(cudaMemcpyAsync(sol.p, dx, sizeof(double) * len, cudaMemcpyDeviceToDevice, rt->stream), "guess");
  }
  RC(solve_device(rt, solver, restart, max_it, tol, dgf, sol.as<double>(), hist, info));
  RC(rt_stage_out(rt, sol.as<double>(), x));
  CUC(cudaStreamSynchronize(rt->stream), "solve");
  info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return info->converged ? OURANOS_OK : OURANOS_ERR_NOT_CONVERGED;
}

// Gauss-Seidel over the groups (src/ouranos.cc:62-128, 141-207): each outer
// iteration solves every group in turn against the latest fluxes of the
// others, warm-started from its own last flux (BiCGSTAB from zero), and
// stops once the relative L2 change of all group fluxes is below outer_tol.
extern "C" int ouranos_solve_multigroup(ouranos_rt* rt, int solver, int restart, int max_inner_it,
                                        double inner_tol, int max_outer_it, double outer_tol,
                                        double* group_flux, ouranos_multigroup_info* info) {
  if (!rt || !group_flux || max_inner_it < 1 || max_outer_it < 1 || !(inner_tol > 0) || !(outer_tol > 0))
    return OURANOS_ERR_BAD_INPUT;
  ouranos_multigroup_info local;
  if (!info) info = &local;
  std::memset(info, 0, sizeof *info);
  cudaSetDevice(rt->device);
  RC(rt_clear_status(rt));
  const auto t0 = std::chrono::steady_clock::now();
  const int G = rt->G;
  const long len = (long)rt->n_mom * rt->n_dofs;
  const long all = (long)G * len;
  DevBuf cur, old, red;
  CUC(cur.alloc(sizeof(double) * all), "group fluxes");
  CUC(old.alloc(sizeof(double) * all), "group fluxes");
  CUC(red.alloc(sizeof(double) * (64 + 64 * (size_t)kDotGrid) + sizeof(double*) * 2), "reductions");
  {
    const double* in = nullptr;
    RC(rt_stage_in(rt, group_flux, cur, G, &in));
    if (in != cur.as<double>())
      CUC(cudaMemcpyAsync(cur.p, in, sizeof(double) * all, cudaMemcpyDeviceToDevice, rt->stream), "group fluxes");
  }
  const int kind = solver & ~OURANOS_SOLVER_WARM_START;
  const int inner = (kind & ~OURANOS_SOLVER_DSA) == OURANOS_SOLVER_BICGSTAB ? kind : kind | OURANOS_SOLVER_WARM_START;
  double* d_out = red.as<double>();
  double* partial = d_out + 64;
  const double** ptrs = reinterpret_cast<const double**>(partial + 64 * (size_t)kDotGrid);
  const double* host_ptrs[2] = {old.as<double>(), cur.as<double>()};
  CUC(cudaMemcpyAsync(ptrs, host_ptrs, sizeof host_ptrs, cudaMemcpyHostToDevice, rt->stream), "reductions");
  double change = 0.0;
  for (int out = 0; out < max_outer_it; ++out) {
    CUC(cudaMemcpyAsync(old.p, cur.p, sizeof(double) * all, cudaMemcpyDeviceToDevice, rt->stream), "group fluxes");
    for (int g = 0; g < G; ++g) {
      RC(ouranos_rt_set_group(rt, g));
      ouranos_solve_info gi;
      const int rc = solve_device(rt, inner, restart, max_inner_it, inner_tol, cur.as<double>(),
                                  cur.as<double>() + (size_t)g * len, nullptr, &gi);
      if (rc && rc != OURANOS_ERR_NOT_CONVERGED) return rc;
      info->inner_iterations += gi.iterations;
    }
    // change = |cur - old| / |cur| over all groups
    CUC(launch_axpby(1.0, cur.as<double>(), -1.0, old.as<double>(), all, rt->stream), "change");
    CUC(launch_dots(ptrs, old.as<double>(), 1, all, d_out, partial, rt->stream), "change");
    CUC(launch_dots(ptrs + 1, cur.as<double>(), 1, all, d_out + 1, partial, rt->stream), "change");
    double h[2] = {0.0, 0.0};
    CUC(cudaMemcpyAsync(h, d_out, sizeof h, cudaMemcpyDeviceToHost, rt->stream), "change");
    CUC(cudaStreamSynchronize(rt->stream), "change");
    change = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : std::sqrt(h[0]);
    info->outer_iterations = out + 1;
    info->change = change;
    if (change < outer_tol) {
      info->converged = 1;
      break;
    }
  }
  for (int g = 0; g < G; ++g)
    RC(rt_stage_out(rt, cur.as<double>() + (size_t)g * len, group_flux + (size_t)g * len));
  CUC(cudaStreamSynchronize(rt->stream), "multigroup");
  RC(rt_check_status(rt));
  info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return info->converged ? OURANOS_OK : OURANOS_ERR_NOT_CONVERGED;
}
