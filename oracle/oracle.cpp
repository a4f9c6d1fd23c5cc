/*
 * ORACLE -- test infrastructure only (see oracle.h for the parity anchoring).
 *
 * Plain FP64 C++ restatement of the reference's sweep path.  Each function
 * names the reference lines it follows.  Deliberate differences from the
 * reference, all documented reference defects:
 *   - 3-D: 8 octants are deployed (src/RTQuadrature.cc:58-95 only fills 4),
 *     the breadth-first ordering loop terminates (src/RadiativeTransfer.cc:149
 *     increments the wrong iterator) and the 3-D face map is {1,0,3,2,5,4}
 *     (src/FECell.cc:24 has {1,0,3,2,6,5}).
 *   - sigma_s is indexed by the Legendre order l(m) of moment m
 *     (src/RadiativeTransfer.cc:834-835,869-870 index it by m).
 *   - a task's missing-dof counter is initialised and a task is queued exactly
 *     once (src/Task.cc:10-19 leaves n_missing_dofs uninitialised).
 *   - the SI driver clears the flux before each sweep (src/ouranos.cc:74-84
 *     accumulates into the previous iterate).
 */
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <list>
#include <set>
#include <thread>
#include <vector>

namespace {

/* ------------------------------------------------------------------------ */
/* 1-D building blocks                                                      */
/* ------------------------------------------------------------------------ */

/* Gauss-Legendre rule with k points on [0,1] (deal.II QGauss<1>(k)), by
 * Newton iteration on P_k from the Chebyshev initial guess. */
void gauss_legendre01(int k, std::vector<double>& x, std::vector<double>& w) {
  x.assign(k, 0.0);
  w.assign(k, 0.0);
  auto legendre = [k](double z, double* pk, double* pk1) {
    double p0 = 1.0, p1 = z;
    for (int l = 2; l <= k; ++l) {
      double p2 = ((2.0 * l - 1.0) * z * p1 - (l - 1.0) * p0) / l;
      p0 = p1;
      p1 = p2;
    }
    *pk = p1;
    *pk1 = p0;
  };
  for (int i = 0; i < k; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (k + 0.5));  // descending in i
    double pk, pk1, dp;
    for (int it = 0; it < 100; ++it) {
      legendre(z, &pk, &pk1);
      dp = k * (z * pk - pk1) / (z * z - 1.0);
      double dz = pk / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    legendre(z, &pk, &pk1);
    dp = k * (z * pk - pk1) / (z * z - 1.0);
    x[i] = 0.5 * (1.0 - z);                 // ascending on [0,1]
    w[i] = 1.0 / ((1.0 - z * z) * dp * dp);  // half of the [-1,1] weight
  }
}

/* Lagrange basis on equidistant nodes j/p (deal.II FE_DGQ<dim>(p) support
 * points) -- value and derivative of basis k at xi. */
double lagrange(int p, int k, double xi) {
  double v = 1.0;
  for (int j = 0; j <= p; ++j)
    if (j != k) v *= (xi - double(j) / p) / (double(k) / p - double(j) / p);
  return v;
}
double lagrange_d(int p, int k, double xi) {
  double s = 0.0;
  for (int m = 0; m <= p; ++m) {
    if (m == k) continue;
    double t = 1.0 / (double(k) / p - double(m) / p);
    for (int j = 0; j <= p; ++j)
      if (j != k && j != m) t *= (xi - double(j) / p) / (double(k) / p - double(j) / p);
    s += t;
  }
  return s;
}

/* ------------------------------------------------------------------------ */
/* Crout LU with row pivoting, src/RadiativeTransfer.cc:1026-1105           */
/* ------------------------------------------------------------------------ */
void lu_decomposition(std::vector<double>& A, int n, std::vector<int>& piv) {
  for (int k = 0; k < n; ++k) {
    piv[k] = k;
    double mx = std::fabs(A[k * n + k]);
    for (int j = k + 1; j < n; ++j)
      if (mx < std::fabs(A[j * n + k])) {
        mx = std::fabs(A[j * n + k]);
        piv[k] = j;
      }
    if (piv[k] != k) {
      int r = piv[k];
      for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[r * n + j]);
    }
    for (int j = k + 1; j < n; ++j) A[k * n + j] /= A[k * n + k];
    for (int i = k + 1; i < n; ++i)
      for (int j = k + 1; j < n; ++j) A[i * n + j] -= A[i * n + k] * A[k * n + j];
  }
}
void lu_solve(const std::vector<double>& A, int n, std::vector<double>& b,
              std::vector<double>& x, const std::vector<int>& piv) {
  for (int k = 0; k < n; ++k) {
    if (piv[k] != k) std::swap(b[k], b[piv[k]]);
    x[k] = b[k];
    for (int i = 0; i < k; ++i) x[k] -= x[i] * A[k * n + i];
    x[k] /= A[k * n + k];
  }
  for (int k = n - 1; k >= 0; --k)
    for (int i = k + 1; i < n; ++i) x[k] -= x[i] * A[k * n + i];
}

}  // namespace

/* ------------------------------------------------------------------------ */
/* Problem                                                                  */
/* ------------------------------------------------------------------------ */
struct orc_problem {
  int dim, p, n, nx[3];
  long n_cells, n_dofs;
  double h[3], lower[3];
  int G, group, n_dir, n_mom, n_mat, l_max, n_src;
  std::vector<double> omega, m2d, d2m, sigma_t, sigma_s, source, inc_flux;
  std::vector<int> moment_l, most_normal, material_id, source_id;
  double ws;
  int bc[6];
  /* FE matrices of an interior cell (uniform Cartesian mesh: identical for every
   * cell). Upwind matrices of boundary faces are zero (src/FECell.cc:67). */
  std::vector<double> M, Gm, E, U, normals;
  /* task graph */
  std::vector<long> task_cell, task_id_of;     // task -> cell ; (dir,cell) -> task
  std::vector<int> task_dir;
  std::vector<std::vector<long>> required;     // task -> upwind tasks (sorted)
  std::vector<std::vector<long>> waiting;      // task -> downwind tasks (sorted)
  std::vector<long> last_order;
  bool tasks_built = false;  /* the graph is built on first use (build_tasks) */
  int scheduler = 0;         /* the order orc_apply / orc_solve sweep in */
  /* state */
  std::vector<double> scat;                    // [mom][dof]
  /* implicit Euler (an extension, see orc_set_time_step): sigma_t shift and psi^n */
  double inv_vdt = 0.0;
  std::vector<double> psi_prev;                // [dir][dof]
  std::vector<double>* psi_capture = nullptr;  // receives the next sweep's psi

  long cell_index(int i, int j, int k) const { return i + (long)nx[0] * (j + (long)nx[1] * k); }
  void cell_ijk(long c, int* ijk) const {
    ijk[0] = c % nx[0];
    ijk[1] = (c / nx[0]) % nx[1];
    ijk[2] = dim == 3 ? int(c / ((long)nx[0] * nx[1])) : 0;
  }
  /* neighbour across face f or -1 at the domain boundary */
  long neighbor(long c, int f) const {
    int ijk[3];
    cell_ijk(c, ijk);
    int a = f / 2;
    int s = (f % 2) ? 1 : -1;
    ijk[a] += s;
    if (ijk[a] < 0 || ijk[a] >= nx[a]) return -1;
    return cell_index(ijk[0], ijk[1], ijk[2]);
  }
  double sig_t(int mat) const { return sigma_t[mat * G + group] + inv_vdt; }
  double sig_s(int mat, int gf, int gt, int l) const {
    if (l > l_max) return 0.0;
    return sigma_s[l + gt * (l_max + 1) + gf * G * (l_max + 1) + (long)mat * G * G * (l_max + 1)];
  }
};

namespace {

/* FECell::FECell, src/FECell.cc:10-78: exact Gauss integration (p+1 points) of
 * the equidistant Lagrange basis on an h-scaled box. */
void build_fe(orc_problem* P) {
  const int p = P->p, dim = P->dim, n = P->n, q1 = p + 1;
  std::vector<double> xq, wq;
  gauss_legendre01(q1, xq, wq);
  auto idx = [&](int i, int* c) {
    c[0] = i % q1;
    c[1] = (i / q1) % q1;
    c[2] = dim == 3 ? i / (q1 * q1) : 0;
  };
  auto shape = [&](int i, const double* xi) {
    int c[3];
    idx(i, c);
    double v = 1.0;
    for (int a = 0; a < dim; ++a) v *= lagrange(p, c[a], xi[a]);
    return v;
  };
  auto shape_grad = [&](int i, const double* xi, int d) {
    int c[3];
    idx(i, c);
    double v = 1.0;
    for (int a = 0; a < dim; ++a)
      v *= (a == d) ? lagrange_d(p, c[a], xi[a]) / P->h[a] : lagrange(p, c[a], xi[a]);
    return v;
  };
  double vol = 1.0;
  for (int a = 0; a < dim; ++a) vol *= P->h[a];
  const int nq = dim == 2 ? q1 * q1 : q1 * q1 * q1;
  P->M.assign(n * n, 0.0);
  P->Gm.assign(dim * n * n, 0.0);
  P->E.assign(2 * dim * n * n, 0.0);
  P->U.assign(2 * dim * n * n, 0.0);
  P->normals.assign(2 * dim * 3, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int q = 0; q < nq; ++q) {
        int c[3];
        idx(q, c);
        double xi[3] = {xq[c[0]], xq[c[1]], dim == 3 ? xq[c[2]] : 0.0};
        double jxw = vol * wq[c[0]] * wq[c[1]] * (dim == 3 ? wq[c[2]] : 1.0);
        P->M[i * n + j] += shape(i, xi) * shape(j, xi) * jxw;
        for (int d = 0; d < dim; ++d)
          P->Gm[(d * n + i) * n + j] += shape(j, xi) * shape_grad(i, xi, d) * jxw;
      }
  /* faces: f = 2a + s, xi_a = s, outward normal (2s-1) e_a */
  const int face_map[6] = {1, 0, 3, 2, 5, 4};
  const int nfq = dim == 2 ? q1 : q1 * q1;
  for (int f = 0; f < 2 * dim; ++f) {
    int a = f / 2, s = f % 2;
    P->normals[f * 3 + a] = s ? 1.0 : -1.0;
    double area = vol / P->h[a];
    int g = face_map[f];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        for (int q = 0; q < nfq; ++q) {
          double xi[3] = {0, 0, 0}, xn[3] = {0, 0, 0};
          int t0 = q % q1, t1 = q / q1;
          int other[2], o = 0;
          for (int b = 0; b < dim; ++b)
            if (b != a) other[o++] = b;
          xi[other[0]] = xq[t0];
          double jxw = area * wq[t0];
          if (dim == 3) {
            xi[other[1]] = xq[t1];
            jxw *= wq[t1];
          }
          xi[a] = s;
          for (int b = 0; b < 3; ++b) xn[b] = xi[b];
          xn[g / 2] = g % 2;  // neighbour's reference coordinate on its face
          P->E[(f * n + i) * n + j] += shape(i, xi) * shape(j, xi) * jxw;
          P->U[(f * n + i) * n + j] += shape(i, xi) * shape(j, xn) * jxw;
        }
  }
}

/* compute_sweep_ordering, src/RadiativeTransfer.cc:80-232, single domain. The
 * waiting/required maps (:234-584) reduce, on one domain, to the upwind and
 * downwind neighbour tasks of the same direction. */
void build_tasks(orc_problem* P) {
  if (P->tasks_built) return;
  P->tasks_built = true;
  const int dim = P->dim;
  const long nc = P->n_cells;
  std::vector<std::set<long>> boundary(2 * dim);
  for (long c = 0; c < nc; ++c)
    for (int f = 0; f < 2 * dim; ++f)
      if (P->neighbor(c, f) < 0) boundary[f].insert(c);
  const long nt = nc * P->n_dir;
  P->task_cell.assign(nt, -1);
  P->task_dir.assign(nt, -1);
  P->task_id_of.assign(nt, -1);
  long task_id = 0;
  for (int d = 0; d < P->n_dir; ++d) {
    std::vector<int> down(dim), up(dim);
    for (int i = 0; i < dim; ++i) {
      if (P->omega[d * 3 + i] > 0.) {
        down[i] = 2 * i + 1;
        up[i] = 2 * i;
      } else {
        down[i] = 2 * i;
        up[i] = 2 * i + 1;
      }
    }
    std::set<long> uni;
    for (int i = 0; i < dim; ++i) uni.insert(boundary[up[i]].begin(), boundary[up[i]].end());
    std::list<long> cand(uni.begin(), uni.end());
    std::vector<char> used(nc, 0), in_cand(nc, 0);
    for (long c : cand) in_cand[c] = 1;
    while (!cand.empty()) {
      long c = cand.front();
      cand.pop_front();
      in_cand[c] = 0;
      used[c] = 1;
      for (int i = 0; i < dim; ++i) {
        long nb = P->neighbor(c, down[i]);
        if (nb >= 0 && !used[nb] && !in_cand[nb]) {
          cand.push_back(nb);
          in_cand[nb] = 1;
        }
      }
      P->task_cell[task_id] = c;
      P->task_dir[task_id] = d;
      P->task_id_of[(long)d * nc + c] = task_id;
      ++task_id;
    }
  }
  P->required.assign(nt, {});
  P->waiting.assign(nt, {});
  for (long t = 0; t < nt; ++t) {
    int d = P->task_dir[t];
    long c = P->task_cell[t];
    for (int i = 0; i < dim; ++i) {
      int f = P->omega[d * 3 + i] > 0. ? 2 * i : 2 * i + 1;
      long nb = P->neighbor(c, f);
      if (nb >= 0) {
        long u = P->task_id_of[(long)d * nc + nb];
        P->required[t].push_back(u);
        P->waiting[u].push_back(t);
      }
    }
  }
  for (long t = 0; t < nt; ++t) {
    std::sort(P->required[t].begin(), P->required[t].end());
    std::sort(P->waiting[t].begin(), P->waiting[t].end());
  }
}

struct SweepCtx {
  const double* group_flux;  // NULL => homogeneous (Apply) form
  std::vector<double> psi;   // [dir][cell][n] for the directions of this worker
  std::vector<double> A, b, x;
  std::vector<int> piv;
};

/* RadiativeTransfer::sweep, src/RadiativeTransfer.cc:878-1012, one task: the
 * cell c in direction d. */
void sweep_task(orc_problem* P, int d, long c, SweepCtx& ctx, double* phi, int dir_base) {
  const int n = P->n, dim = P->dim;
  const double* om = &P->omega[d * 3];
  const int mat = P->material_id[c];
  std::vector<double>& A = ctx.A;
  std::vector<double>& b = ctx.b;
  // volumetric terms, :898-905
  for (int k = 0; k < n * n; ++k) A[k] = P->M[k];
  const double st = P->sig_t(mat);
  for (int k = 0; k < n * n; ++k) A[k] *= st;
  for (int dd = 0; dd < dim; ++dd)
    for (int k = 0; k < n * n; ++k) A[k] += (-om[dd]) * P->Gm[dd * n * n + k];
  // scattering source, :908-913
  std::fill(b.begin(), b.end(), 0.0);
  for (int m = 0; m < P->n_mom; ++m) {
    const double m2d = P->m2d[d * P->n_mom + m];
    for (int j = 0; j < n; ++j) b[j] += m2d * P->scat[(long)m * P->n_dofs + c * n + j];
  }
  if (ctx.group_flux) {
    // fixed source, :914-922
    const int sid = P->source_id.empty() ? 0 : P->source_id[c];
    const double s = P->source.empty() ? 0.0 : P->source[sid * P->G + P->group] / P->ws;
    for (int i = 0; i < n; ++i) {
      double acc = 0.0;
      for (int j = 0; j < n; ++j) acc += P->M[i * n + j] * s;
      b[i] += acc;
    }
    // implicit Euler: + inv_vdt M psi^n of this direction
    if (!P->psi_prev.empty()) {
      const double* pp = &P->psi_prev[(long)d * P->n_dofs + c * n];
      for (int i = 0; i < n; ++i) {
        double acc = 0.0;
        for (int j = 0; j < n; ++j) acc += P->M[i * n + j] * pp[j];
        b[i] += P->inv_vdt * acc;
      }
    }
    // other-group scattering, compute_outer_scattering_source :845-876
    for (int g = 0; g < P->G; ++g) {
      if (g == P->group) continue;
      for (int m = 0; m < P->n_mom; ++m) {
        const double m2d = P->m2d[d * P->n_mom + m];
        const double* xg = ctx.group_flux + ((long)g * P->n_mom + m) * P->n_dofs + c * n;
        const double sc = m2d * P->sig_s(mat, g, P->group, P->moment_l[m]);
        for (int i = 0; i < n; ++i) {
          double acc = 0.0;
          for (int j = 0; j < n; ++j) acc += P->M[i * n + j] * xg[j];
          b[i] += acc * sc;
        }
      }
    }
  }
  // surface terms, :928-982
  for (int f = 0; f < 2 * dim; ++f) {
    double ndo = 0.0;
    for (int dd = 0; dd < dim; ++dd) ndo += om[dd] * P->normals[f * 3 + dd];
    if (ndo < 0.) {
      long nb = P->neighbor(c, f);
      if (nb >= 0) {
        const double* pn = &ctx.psi[((long)(d - dir_base) * P->n_cells + nb) * n];
        for (int i = 0; i < n; ++i) {
          double acc = 0.0;
          for (int j = 0; j < n; ++j) acc += P->U[(f * n + i) * n + j] * (-ndo * pn[j]);
          b[i] += acc;
        }
      } else if (ctx.group_flux) {
        double inc = 0.0;
        const int bt = P->bc[f];
        bool mn = P->most_normal.empty() ? false : P->most_normal[f * P->n_dir + d] != 0;
        if ((bt == ORC_BC_MOST_NORMAL && mn) || bt == ORC_BC_ISOTROPIC)
          inc = P->inc_flux.empty() ? 0.0 : P->inc_flux[f * P->G + P->group];
        inc /= P->ws;
        for (int i = 0; i < n; ++i) {
          double acc = 0.0;
          for (int j = 0; j < n; ++j) acc += P->E[(f * n + i) * n + j] * inc;
          b[i] += (-ndo) * acc;
        }
      }
    } else {
      for (int k = 0; k < n * n; ++k) A[k] += ndo * P->E[f * n * n + k];
    }
  }
  lu_decomposition(A, n, ctx.piv);
  lu_solve(A, n, b, ctx.x, ctx.piv);
  // flux moments, :991-996
  for (int m = 0; m < P->n_mom; ++m) {
    const double w = P->d2m[(long)m * P->n_dir + d];
    for (int j = 0; j < n; ++j) phi[(long)m * P->n_dofs + c * n + j] += w * ctx.x[j];
  }
  double* out = &ctx.psi[((long)(d - dir_base) * P->n_cells + c) * n];
  for (int j = 0; j < n; ++j) out[j] = ctx.x[j];
}

/* Scheduler over the tasks of directions [d0,d1): initialize_scheduler,
 * get_next_task, send_angular_flux (src/RadiativeTransfer.cc:605-692). */
void run_sweep(orc_problem* P, double* phi, const double* group_flux, int scheduler,
               int d0, int d1, std::vector<long>* order) {
  const long nc = P->n_cells;
  const long t0 = (long)d0 * nc, t1 = (long)d1 * nc;  // task ids are direction-major
  SweepCtx ctx;
  ctx.group_flux = group_flux;
  ctx.psi.assign((long)(d1 - d0) * nc * P->n, 0.0);
  ctx.A.assign(P->n * P->n, 0.0);
  ctx.b.assign(P->n, 0.0);
  ctx.x.assign(P->n, 0.0);
  ctx.piv.assign(P->n, 0);
  std::vector<long> missing(t1 - t0);
  std::deque<long> ready;
  for (long t = t0; t < t1; ++t) {
    missing[t - t0] = (long)P->required[t].size() * P->n;  // dofs, src/Task.cc:38-44
    if (P->required[t].empty()) ready.push_back(t);
  }
  long left = t1 - t0;
  while (left) {
    long t = ready.front();
    ready.pop_front();
    --left;
    sweep_task(P, P->task_dir[t], P->task_cell[t], ctx, phi, d0);
    if (order) order->push_back((long)P->task_dir[t] * nc + P->task_cell[t]);
    if (scheduler == 1) {
      // the reference's scan of every task after each completion (:673-689)
      for (long i = t0; i < t1; ++i) {
        const auto& rq = P->required[i];
        if (std::binary_search(rq.begin(), rq.end(), t)) {
          missing[i - t0] -= P->n;
          if (missing[i - t0] == 0) ready.push_back(i);
        }
      }
    } else {
      for (long w : P->waiting[t]) {
        missing[w - t0] -= P->n;
        if (missing[w - t0] == 0) ready.push_back(w);
      }
    }
  }
  // the angular flux of directions [d0, d1) for orc_advance_angular
  if (P->psi_capture)
    std::copy(ctx.psi.begin(), ctx.psi.end(), P->psi_capture->begin() + (long)d0 * P->n_dofs);
}

/* The same tasks in another topological order of the same graph, without
 * the graph: each direction of [d0, d1) in turn, its cells in lexicographic
 * order along the sweep (ascending along axis a when Omega_a > 0, descending
 * otherwise), so every upwind neighbour of a cell (src/RadiativeTransfer.cc:
 * 113-125) is solved before it.  Each task then sees the same inputs as under
 * the ready-list scheduler and computes the same values; only the order of
 * the additions into the flux moments differs.  The graph of a large mesh
 * costs O(tasks) memory (tens of GB at 10^8 tasks); this order needs one
 * direction's angular flux per worker. */
void run_sweep_cartesian(orc_problem* P, double* phi, const double* group_flux, int d0, int d1) {
  const long nc = P->n_cells;
  SweepCtx ctx;
  ctx.group_flux = group_flux;
  ctx.psi.assign(nc * P->n, 0.0);
  ctx.A.assign(P->n * P->n, 0.0);
  ctx.b.assign(P->n, 0.0);
  ctx.x.assign(P->n, 0.0);
  ctx.piv.assign(P->n, 0);
  for (int d = d0; d < d1; ++d) {
    int lo[3], step[3];
    for (int a = 0; a < 3; ++a) {
      const bool up = a < P->dim && P->omega[d * 3 + a] > 0.;
      lo[a] = up ? 0 : P->nx[a] - 1;
      step[a] = up ? 1 : -1;
    }
    for (int kk = 0; kk < P->nx[2]; ++kk)
      for (int jj = 0; jj < P->nx[1]; ++jj)
        for (int ii = 0; ii < P->nx[0]; ++ii) {
          const long c = P->cell_index(lo[0] + step[0] * ii, lo[1] + step[1] * jj, lo[2] + step[2] * kk);
          sweep_task(P, d, c, ctx, phi, d);
        }
    if (P->psi_capture)
      std::copy(ctx.psi.begin(), ctx.psi.end(), P->psi_capture->begin() + (long)d * P->n_dofs);
  }
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

}  // namespace

extern "C" {

orc_problem* orc_create(const orc_desc* D) {
  if (!D || (D->dim != 2 && D->dim != 3) || D->fe_order < 1 || D->fe_order > 5) return nullptr;
  orc_problem* P = new orc_problem();
  P->dim = D->dim;
  P->p = D->fe_order;
  P->n = 1;
  for (int a = 0; a < P->dim; ++a) P->n *= (P->p + 1);
  P->n_cells = 1;
  for (int a = 0; a < 3; ++a) {
    P->nx[a] = a < P->dim ? D->n_cells[a] : 1;
    P->lower[a] = D->lower[a];
    P->h[a] = a < P->dim ? (D->upper[a] - D->lower[a]) / P->nx[a] : 1.0;
    P->n_cells *= P->nx[a];
  }
  P->n_dofs = P->n_cells * P->n;
  P->G = D->n_groups;
  P->group = D->group;
  P->n_dir = D->n_dir;
  P->n_mom = D->n_mom;
  P->omega.assign(D->omega, D->omega + 3 * D->n_dir);
  P->m2d.assign(D->m2d, D->m2d + (long)D->n_dir * D->n_mom);
  P->d2m.assign(D->d2m, D->d2m + (long)D->n_dir * D->n_mom);
  P->moment_l.assign(D->moment_l, D->moment_l + D->n_mom);
  if (D->most_normal) P->most_normal.assign(D->most_normal, D->most_normal + 2 * P->dim * D->n_dir);
  P->ws = D->weight_sum;
  P->n_mat = D->n_materials;
  P->l_max = D->l_max;
  P->sigma_t.assign(D->sigma_t, D->sigma_t + P->n_mat * P->G);
  P->sigma_s.assign(D->sigma_s, D->sigma_s + (long)P->n_mat * P->G * P->G * (P->l_max + 1));
  P->material_id.assign(D->material_id, D->material_id + P->n_cells);
  if (D->source_id) P->source_id.assign(D->source_id, D->source_id + P->n_cells);
  P->n_src = D->n_sources;
  if (D->source) P->source.assign(D->source, D->source + P->n_src * P->G);
  for (int f = 0; f < 6; ++f) P->bc[f] = D->bc_type[f];
  if (D->inc_flux) P->inc_flux.assign(D->inc_flux, D->inc_flux + 2 * P->dim * P->G);
  build_fe(P);
  P->scat.assign((long)P->n_mom * P->n_dofs, 0.0);
  return P;
}

void orc_destroy(orc_problem* p) { delete p; }

/* Implicit Euler in time -- an extension: the reference operator is steady
 * (its TimeDiscretization class, src/TimeDiscretization.cc:10-82, is never
 * called).  inv_vdt = 1/(v dt) is added to sigma_t and source sweeps gain
 * inv_vdt M psi^n per direction; psi^n starts at 0. */
void orc_set_time_step(orc_problem* p, double inv_vdt) {
  p->inv_vdt = inv_vdt;
  if (inv_vdt > 0.0) p->psi_prev.assign((long)p->n_dir * p->n_dofs, 0.0);
  else p->psi_prev.clear();
}
void orc_set_source(orc_problem* p, const double* source) {
  p->source.assign(source, source + (long)p->n_src * p->G);
}
/* psi^n <- the angular flux of a source sweep of phi (the step's end) */
void orc_advance_angular(orc_problem* p, const double* phi, int n_threads) {
  std::vector<double> psi((long)p->n_dir * p->n_dofs, 0.0);
  std::vector<double> gf((long)p->G * p->n_mom * p->n_dofs, 0.0), out((long)p->n_mom * p->n_dofs, 0.0);
  orc_scattering_source(p, phi);
  p->psi_capture = &psi;
  orc_sweep(p, out.data(), gf.data(), p->scheduler, n_threads);
  p->psi_capture = nullptr;
  p->psi_prev.swap(psi);
}
void orc_get_angular(const orc_problem* p, double* psi) {
  std::copy(p->psi_prev.begin(), p->psi_prev.end(), psi);
}
void orc_set_angular(orc_problem* p, const double* psi) {
  std::copy(psi, psi + (long)p->n_dir * p->n_dofs, p->psi_prev.begin());
}
void orc_set_group(orc_problem* p, int g) { p->group = g; }
void orc_set_scheduler(orc_problem* p, int scheduler) { p->scheduler = scheduler; }
long orc_n_dofs(const orc_problem* p) { return p->n_dofs; }
long orc_n_tasks(const orc_problem* p) { return p->n_cells * p->n_dir; }

void orc_clear_scattering_source(orc_problem* P) { std::fill(P->scat.begin(), P->scat.end(), 0.0); }

void orc_scattering_source(orc_problem* P, const double* x) {
  const int n = P->n;
  std::fill(P->scat.begin(), P->scat.end(), 0.0);
  for (long c = 0; c < P->n_cells; ++c) {
    const int mat = P->material_id[c];
    for (int m = 0; m < P->n_mom; ++m) {
      const double* xc = x + (long)m * P->n_dofs + c * n;
      const double s = P->sig_s(mat, P->group, P->group, P->moment_l[m]);
      for (int i = 0; i < n; ++i) {
        double acc = 0.0;
        for (int j = 0; j < n; ++j) acc += P->M[i * n + j] * xc[j];
        P->scat[(long)m * P->n_dofs + c * n + i] += acc * s;
      }
    }
  }
}

void orc_sweep(orc_problem* P, double* phi, const double* group_flux, int scheduler,
               int n_threads) {
  if (scheduler != 2) build_tasks(P);
  if (n_threads <= 1) {
    P->last_order.clear();
    if (scheduler == 2)
      run_sweep_cartesian(P, phi, group_flux, 0, P->n_dir);
    else
      run_sweep(P, phi, group_flux, scheduler, 0, P->n_dir, &P->last_order);
    return;
  }
  const long len = (long)P->n_mom * P->n_dofs;
  std::vector<std::vector<double>> part(n_threads, std::vector<double>(len, 0.0));
  std::vector<std::thread> th;
  for (int w = 0; w < n_threads; ++w) {
    int d0 = (int)((long)P->n_dir * w / n_threads), d1 = (int)((long)P->n_dir * (w + 1) / n_threads);
    th.emplace_back([=, &part]() {
      if (scheduler == 2)
        run_sweep_cartesian(P, part[w].data(), group_flux, d0, d1);
      else
        run_sweep(P, part[w].data(), group_flux, scheduler, d0, d1, nullptr);
    });
  }
  for (auto& t : th) t.join();
  for (int w = 0; w < n_threads; ++w)
    for (long i = 0; i < len; ++i) phi[i] += part[w][i];
}

void orc_apply(orc_problem* P, const double* x, double* y, int n_threads) {
  const long len = (long)P->n_mom * P->n_dofs;
  orc_scattering_source(P, x);
  std::vector<double> phi(len, 0.0);
  orc_sweep(P, phi.data(), nullptr, P->scheduler, n_threads);
  for (long i = 0; i < len; ++i) y[i] = x[i] - phi[i];
}

void orc_last_order(const orc_problem* P, long* order) {
  std::copy(P->last_order.begin(), P->last_order.end(), order);
}

void orc_task_levels(orc_problem* P, int* levels) {
  build_tasks(P);
  const long nt = (long)P->n_cells * P->n_dir;
  std::vector<long> indeg(nt);
  std::vector<int> lev(nt, 0);
  std::deque<long> q;
  for (long t = 0; t < nt; ++t) {
    indeg[t] = P->required[t].size();
    if (!indeg[t]) q.push_back(t);
  }
  while (!q.empty()) {
    long t = q.front();
    q.pop_front();
    for (long w : P->waiting[t]) {
      lev[w] = std::max(lev[w], lev[t] + 1);
      if (--indeg[w] == 0) q.push_back(w);
    }
  }
  for (long t = 0; t < nt; ++t) levels[(long)P->task_dir[t] * P->n_cells + P->task_cell[t]] = lev[t];
}

void orc_task_ids(orc_problem* P, long* ids) {
  build_tasks(P);
  std::copy(P->task_id_of.begin(), P->task_id_of.end(), ids);
}

void orc_fecell(const orc_problem* P, long cell, double* mass, double* grad, double* downwind,
                double* upwind, double* normals) {
  const int n = P->n, dim = P->dim;
  if (mass) std::copy(P->M.begin(), P->M.end(), mass);
  if (grad) std::copy(P->Gm.begin(), P->Gm.end(), grad);
  if (downwind) std::copy(P->E.begin(), P->E.end(), downwind);
  if (upwind)
    for (int f = 0; f < 2 * dim; ++f)
      for (int k = 0; k < n * n; ++k)
        upwind[f * n * n + k] = P->neighbor(cell, f) >= 0 ? P->U[f * n * n + k] : 0.0;
  if (normals) std::copy(P->normals.begin(), P->normals.end(), normals);
}

/* src/ouranos.cc:43-209 with the SI branch written as intended (D6/D7) and
 * Krylov methods restated from their textbook forms (AztecOO is not part of
 * the reference tree). */
int orc_solve(orc_problem* P, int kind, int restart, int max_it, double tol,
              const double* group_flux, double* xout, double* hist, int n_threads) {
  const long len = (long)P->n_mom * P->n_dofs;
  std::vector<double> gf_zero;
  if (!group_flux) {
    gf_zero.assign((long)P->G * len, 0.0);
    group_flux = gf_zero.data();
  }
  // right-hand side: one sweep of the fixed sources with no in-group scattering
  std::vector<double> rhs(len, 0.0);
  orc_clear_scattering_source(P);
  orc_sweep(P, rhs.data(), group_flux, P->scheduler, n_threads);
  std::vector<double> x(len, 0.0);
  int it = 0;
  const double bnorm = std::sqrt(dot(rhs, rhs));
  if (kind == 0) {
    // source iteration: phi <- D L^-1 (M2D S phi + q), relative-change test
    std::vector<double> nx(len);
    for (it = 0; it < max_it; ++it) {
      orc_scattering_source(P, x.data());
      std::fill(nx.begin(), nx.end(), 0.0);
      orc_sweep(P, nx.data(), group_flux, P->scheduler, n_threads);
      double num = 0.0, den = 0.0;
      for (long i = 0; i < len; ++i) {
        num += (nx[i] - x[i]) * (nx[i] - x[i]);
        den += nx[i] * nx[i];
      }
      x = nx;
      double rel = std::sqrt(num / den);
      if (hist) hist[it] = rel;
      if (rel < tol) { ++it; break; }
    }
  } else if (kind == 1) {
    const int m = restart;
    std::vector<std::vector<double>> V(m + 1, std::vector<double>(len));
    std::vector<double> H((m + 1) * m), cs(m), sn(m), g(m + 1), w(len), y(m);
    int total = 0;
    bool done = false;
    if (hist) hist[0] = 1.0;
    while (!done && total < max_it) {
      orc_apply(P, x.data(), w.data(), n_threads);
      for (long i = 0; i < len; ++i) V[0][i] = rhs[i] - w[i];
      double beta = std::sqrt(dot(V[0], V[0]));
      if (beta / bnorm < tol) break;
      for (long i = 0; i < len; ++i) V[0][i] /= beta;
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int k = 0;
      for (; k < m && total < max_it; ++k) {
        orc_apply(P, V[k].data(), w.data(), n_threads);
        for (int j = 0; j <= k; ++j) {  // modified Gram-Schmidt
          double h = dot(w, V[j]);
          H[j * m + k] = h;
          for (long i = 0; i < len; ++i) w[i] -= h * V[j][i];
        }
        double hn = std::sqrt(dot(w, w));
        H[(k + 1) * m + k] = hn;
        for (long i = 0; i < len; ++i) V[k + 1][i] = hn > 0 ? w[i] / hn : 0.0;
        for (int j = 0; j < k; ++j) {
          double a = H[j * m + k], b2 = H[(j + 1) * m + k];
          H[j * m + k] = cs[j] * a + sn[j] * b2;
          H[(j + 1) * m + k] = -sn[j] * a + cs[j] * b2;
        }
        double a = H[k * m + k], b2 = H[(k + 1) * m + k];
        double r = std::sqrt(a * a + b2 * b2);
        cs[k] = a / r;
        sn[k] = b2 / r;
        H[k * m + k] = r;
        H[(k + 1) * m + k] = 0.0;
        g[k + 1] = -sn[k] * g[k];
        g[k] = cs[k] * g[k];
        ++total;
        double rel = std::fabs(g[k + 1]) / bnorm;
        if (hist) hist[total] = rel;
        if (rel < tol) { ++k; done = true; break; }
      }
      for (int i = k - 1; i >= 0; --i) {
        double s = g[i];
        for (int j = i + 1; j < k; ++j) s -= H[i * m + j] * y[j];
        y[i] = s / H[i * m + i];
      }
      for (int j = 0; j < k; ++j)
        for (long i = 0; i < len; ++i) x[i] += y[j] * V[j][i];
    }
    it = total;
  } else {
    // BiCGSTAB (van der Vorst 1992), unpreconditioned
    std::vector<double> r(len), r0(len), pv(len, 0.0), v(len, 0.0), s(len), t(len);
    orc_apply(P, x.data(), t.data(), n_threads);
    for (long i = 0; i < len; ++i) r[i] = rhs[i] - t[i];
    r0 = r;
    double rho = 1.0, alpha = 1.0, omg = 1.0;
    if (hist) hist[0] = 1.0;
    for (it = 0; it < max_it; ++it) {
      double rho1 = dot(r0, r);
      double beta = (rho1 / rho) * (alpha / omg);
      rho = rho1;
      for (long i = 0; i < len; ++i) pv[i] = r[i] + beta * (pv[i] - omg * v[i]);
      orc_apply(P, pv.data(), v.data(), n_threads);
      alpha = rho / dot(r0, v);
      for (long i = 0; i < len; ++i) s[i] = r[i] - alpha * v[i];
      orc_apply(P, s.data(), t.data(), n_threads);
      omg = dot(t, s) / dot(t, t);
      for (long i = 0; i < len; ++i) {
        x[i] += alpha * pv[i] + omg * s[i];
        r[i] = s[i] - omg * t[i];
      }
      double rel = std::sqrt(dot(r, r)) / bnorm;
      if (hist) hist[it + 1] = rel;
      if (rel < tol) { ++it; break; }
    }
  }
  std::copy(x.begin(), x.end(), xout);
  return it;
}

/* ------------------------------------------------------------------------ */
/* Quadrature, src/RTQuadrature.cc:10-238, src/LS.cc:667-682, src/GLC.cc:14-58 */
/* ------------------------------------------------------------------------ */
int orc_quadrature_sizes(int sn, int l_max, int galerkin, int dim, int* n_dir, int* n_mom) {
  if (sn < 2 || sn % 2) return -1;
  int per_oct = sn * (sn + 2) / 8;
  *n_dir = per_oct * (dim == 3 ? 8 : 4);
  if (galerkin)
    *n_mom = *n_dir;
  else
    *n_mom = dim == 3 ? (l_max + 1) * (l_max + 1) : (l_max + 1) * (l_max + 2) / 2;
  return 0;
}

static double assoc_legendre(int l, int m, double x) {
  // P_l^m(x) with the Condon-Shortley phase
  double pmm = 1.0;
  double s = std::sqrt(std::max(0.0, (1.0 - x) * (1.0 + x)));
  double fact = 1.0;
  for (int i = 1; i <= m; ++i) {
    pmm *= -fact * s;
    fact += 2.0;
  }
  if (l == m) return pmm;
  double pmmp1 = x * (2 * m + 1) * pmm;
  if (l == m + 1) return pmmp1;
  double pll = 0.0;
  for (int ll = m + 2; ll <= l; ++ll) {
    pll = (x * (2 * ll - 1) * pmmp1 - (ll + m - 1) * pmm) / (ll - m);
    pmm = pmmp1;
    pmmp1 = pll;
  }
  return pll;
}

static double harm_norm(int l, int m) {
  double r = (2.0 * l + 1.0) / (4.0 * M_PI);
  for (int k = l - m + 1; k <= l + m; ++k) r /= k;
  return std::sqrt(r);
}

int orc_quadrature_build(int type, int sn, int l_max, int galerkin, double ws, int dim,
                         int harmonics, const double* ta, const double* tb, double* omega,
                         double* weight, double* m2d, double* d2m, int* moment_l,
                         int* most_normal) {
  int n_dir, n_mom;
  if (orc_quadrature_sizes(sn, l_max, galerkin, dim, &n_dir, &n_mom)) return -1;
  if (galerkin && dim == 3) return -2;  // src/RTQuadrature.cc:30-31
  const int per_oct = sn * (sn + 2) / 8;
  const int half = sn / 2;
  std::vector<double> w(n_dir, 0.0);
  // first octant
  if (type == ORC_QUAD_LS) {
    // LS::compute_omega, src/LS.cc:667-682
    int off = 0;
    for (int j = 0; j < half; ++j) {
      for (int i = 0; i < half - j; ++i) {
        omega[(off + i) * 3 + 0] = ta[half - 1 - j - i];
        omega[(off + i) * 3 + 1] = ta[i];
        omega[(off + i) * 3 + 2] = ta[j];
      }
      off += half - j;
    }
    for (int k = 0; k < per_oct; ++k) w[k] = tb[k];
  } else {
    // GLC::build_octant + build_chebyshev_quadrature, src/GLC.cc:14-58
    int pos = 0;
    for (int i = 0; i < half; ++i) {
      const double jmax = half - i;
      const double st = std::sqrt(1. - ta[i] * ta[i]);
      for (int j = 0; j < half - i; ++j) {
        double az = M_PI_2 * j / jmax + M_PI_4 / jmax;
        double aw = M_PI_2 / jmax;
        omega[pos * 3 + 0] = st * std::cos(az);
        omega[pos * 3 + 1] = st * std::sin(az);
        omega[pos * 3 + 2] = ta[i];
        w[pos] = tb[i] * aw;
        ++pos;
      }
    }
  }
  // deploy_octant, src/RTQuadrature.cc:58-95 (3-D: z-reflected copies 4..7)
  const int n_oct = dim == 3 ? 8 : 4;
  const double sx[8] = {1, 1, -1, -1, 1, 1, -1, -1};
  const double sy[8] = {1, -1, -1, 1, 1, -1, -1, 1};
  const double sz[8] = {1, 1, 1, 1, -1, -1, -1, -1};
  for (int o = 1; o < n_oct; ++o)
    for (int j = 0; j < per_oct; ++j) {
      int k = o * per_oct + j;
      if (!galerkin) w[k] = w[j];
      omega[k * 3 + 0] = sx[o] * omega[j * 3 + 0];
      omega[k * 3 + 1] = sy[o] * omega[j * 3 + 1];
      omega[k * 3 + 2] = sz[o] * omega[j * 3 + 2];
    }
  if (!galerkin) {
    double s = 0.0;
    for (int i = 0; i < per_oct; ++i) s += w[i];
    for (int i = 0; i < n_dir; ++i) w[i] *= (1.0 / n_oct) / s;
  }
  if (weight)
    for (int i = 0; i < n_dir; ++i) weight[i] = w[i];
  // compute_harmonics, src/RTQuadrature.cc:97-198
  const double w_sph = std::sqrt(4. * M_PI / ws);
  const int Lx = galerkin ? sn : l_max;
  for (int d = 0; d < n_dir; ++d) {
    const double* o = &omega[d * 3];
    double phi = std::atan(o[1] / o[0]);
    if (o[0] < 0.) phi += M_PI;
    double x = harmonics == ORC_HARM_REFERENCE ? std::cos(o[2]) : o[2];
    int pos = 0;
    auto put = [&](int l, double v) {
      if (pos < n_mom) {
        m2d[d * n_mom + pos] = v;
        if (d == 0) moment_l[pos] = l;
      }
      ++pos;
    };
    for (int l = 0; l <= Lx; ++l) {
      for (int m = l; m >= 0; --m) {
        bool keep = dim == 3 ? true : ((m + l) % 2 == 0);
        if (galerkin) keep = keep && (l < sn);
        if (!keep) continue;
        double f = (harmonics == ORC_HARM_ORTHONORMAL && m > 0) ? std::sqrt(2.0) : 1.0;
        put(l, w_sph * f * harm_norm(l, m) * assoc_legendre(l, m, x) * std::cos(m * phi));
      }
      for (int m = 1; m <= l; ++m) {
        bool keep = dim == 3 ? true : ((m + l) % 2 == 0);
        if (galerkin) keep = keep && (l <= sn);
        if (!keep) continue;
        double f = harmonics == ORC_HARM_ORTHONORMAL ? std::sqrt(2.0) : 1.0;
        put(l, w_sph * f * harm_norm(l, m) * assoc_legendre(l, m, x) * std::sin(m * phi));
      }
    }
    if (pos < n_mom) return -3;
  }
  if (galerkin) {
    // D2M = M2D^-1 (Gauss-Jordan with partial pivoting)
    const int N = n_dir;
    std::vector<double> a(m2d, m2d + N * N), inv(N * N, 0.0);
    for (int i = 0; i < N; ++i) inv[i * N + i] = 1.0;
    for (int k = 0; k < N; ++k) {
      int pr = k;
      for (int i = k + 1; i < N; ++i)
        if (std::fabs(a[i * N + k]) > std::fabs(a[pr * N + k])) pr = i;
      for (int j = 0; j < N; ++j) {
        std::swap(a[k * N + j], a[pr * N + j]);
        std::swap(inv[k * N + j], inv[pr * N + j]);
      }
      double dv = a[k * N + k];
      for (int j = 0; j < N; ++j) {
        a[k * N + j] /= dv;
        inv[k * N + j] /= dv;
      }
      for (int i = 0; i < N; ++i)
        if (i != k) {
          double f = a[i * N + k];
          for (int j = 0; j < N; ++j) {
            a[i * N + j] -= f * a[k * N + j];
            inv[i * N + j] -= f * inv[k * N + j];
          }
        }
    }
    for (int i = 0; i < N * N; ++i) d2m[i] = inv[i];
  } else {
    for (int m = 0; m < n_mom; ++m)
      for (int d = 0; d < n_dir; ++d) d2m[m * n_dir + d] = m2d[d * n_mom + m] * ws * w[d];
  }
  // compute_most_normal_directions, src/RTQuadrature.cc:200-238
  if (most_normal) {
    double mx[6] = {0, 0, 0, 0, 0, 0};
    for (int d = 0; d < n_dir; ++d)
      for (int i = 0; i < dim; ++i) {
        double v = omega[d * 3 + i];
        if (v > mx[2 * i]) mx[2 * i] = v;
        if (v < mx[2 * i + 1]) mx[2 * i + 1] = v;
      }
    for (int f = 0; f < 2 * dim; ++f)
      for (int d = 0; d < n_dir; ++d) most_normal[f * n_dir + d] = omega[d * 3 + f / 2] == mx[f];
  }
  return 0;
}

}  // extern "C"
