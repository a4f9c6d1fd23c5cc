// Reference-cell DG tables.  Stand-in for FECell (src/FECell.cc:10-78), which
// integrates every matrix cell by cell with deal.II FEValues; on a uniform
// Cartesian mesh all cells share one set of matrices, built here from 1-D
// integrals by tensor products.
#include <cmath>
#include <vector>

#include "internal.h"

namespace ouranos {
namespace {

// Lagrange polynomial k on nodes j/p and its derivative.
double lag(int p, int k, double x) {
  double v = 1.0;
  for (int j = 0; j <= p; ++j)
    if (j != k) v *= (x * p - j) / double(k - j);
  return v;
}
double lag_d(int p, int k, double x) {
  double s = 0.0;
  for (int m = 0; m <= p; ++m) {
    if (m == k) continue;
    double t = double(p) / double(k - m);
    for (int j = 0; j <= p; ++j)
      if (j != k && j != m) t *= (x * p - j) / double(k - j);
    s += t;
  }
  return s;
}

// q-point Gauss rule on [0,1].
void gauss01(int q, std::vector<double>& x, std::vector<double>& w) {
  x.resize(q);
  w.resize(q);
  for (int i = 0; i < q; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (q + 0.5));
    double a = 1, b = z;
    for (int it = 0; it < 64; ++it) {
      a = 1.0;
      b = z;
      for (int l = 2; l <= q; ++l) {
        double c = ((2 * l - 1) * z * b - (l - 1) * a) / l;
        a = b;
        b = c;
      }
      double dp = q * (z * b - a) / (z * z - 1.0);
      double dz = b / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    a = 1.0;
    b = z;
    for (int l = 2; l <= q; ++l) {
      double c = ((2 * l - 1) * z * b - (l - 1) * a) / l;
      a = b;
      b = c;
    }
    double dp = q * (z * b - a) / (z * z - 1.0);
    x[i] = 0.5 * (1.0 - z);
    w[i] = 1.0 / ((1.0 - z * z) * dp * dp);
  }
}

}  // namespace

FETables build_fe_tables(int dim, int p, const double* h) {
  FETables t;
  t.dim = dim;
  t.p = p;
  t.p1 = p + 1;
  const int p1 = p + 1;
  t.n = dim == 2 ? p1 * p1 : p1 * p1 * p1;
  t.fd = dim == 2 ? p1 : p1 * p1;
  for (int a = 0; a < 3; ++a) t.h[a] = a < dim ? h[a] : 1.0;
  std::vector<double> xq, wq;
  gauss01(p1, xq, wq);  // exact for the degree-2p products below
  std::vector<double> m1(p1 * p1, 0.0), g1(p1 * p1, 0.0), e0(p1), e1(p1);
  for (int i = 0; i < p1; ++i) {
    e0[i] = lag(p, i, 0.0);
    e1[i] = lag(p, i, 1.0);
    for (int j = 0; j < p1; ++j)
      for (int q = 0; q < p1; ++q) {
        m1[i * p1 + j] += lag(p, i, xq[q]) * lag(p, j, xq[q]) * wq[q];
        g1[i * p1 + j] += lag(p, j, xq[q]) * lag_d(p, i, xq[q]) * wq[q];  // int L_j L_i'
      }
  }
  t.mass1d = m1;
  const int n = t.n;
  auto comp = [&](int i, int a) {
    return a == 0 ? i % p1 : (a == 1 ? (i / p1) % p1 : i / (p1 * p1));
  };
  double vol = 1.0;
  for (int a = 0; a < dim; ++a) vol *= t.h[a];
  t.mass.assign(n * n, 0.0);
  t.grad.assign(dim * n * n, 0.0);
  t.face.assign(2 * dim * n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double m = vol;
      for (int a = 0; a < dim; ++a) m *= m1[comp(i, a) * p1 + comp(j, a)];
      t.mass[i * n + j] = m;
      for (int a = 0; a < dim; ++a) {
        double area = vol / t.h[a];
        double trans = 1.0;
        for (int b = 0; b < dim; ++b)
          if (b != a) trans *= m1[comp(i, b) * p1 + comp(j, b)];
        const int ia = comp(i, a), ja = comp(j, a);
        t.grad[(a * n + i) * n + j] = area * g1[ia * p1 + ja] * trans;
        t.face[((2 * a) * n + i) * n + j] = area * e0[ia] * e0[ja] * trans;
        t.face[((2 * a + 1) * n + i) * n + j] = area * e1[ia] * e1[ja] * trans;
      }
    }
  // transverse face mass of axis a, transverse index over the other axes in
  // increasing order
  const int fd = t.fd;
  t.face_mass.assign(3 * fd * fd, 0.0);
  for (int a = 0; a < dim; ++a) {
    const double area = vol / t.h[a];
    for (int u = 0; u < fd; ++u)
      for (int v = 0; v < fd; ++v) {
        double m = area;
        if (dim == 2) {
          m *= m1[u * p1 + v];
        } else {
          m *= m1[(u % p1) * p1 + (v % p1)] * m1[(u / p1) * p1 + (v / p1)];
        }
        t.face_mass[(a * fd + u) * fd + v] = m;
      }
  }
  return t;
}

void canonical_inverse(const FETables& fe, double sigma_t, const double* aw, double* out) {
  const int n = fe.n;
  std::vector<double> A(n * n);
  for (int k = 0; k < n * n; ++k) A[k] = sigma_t * fe.mass[k];
  for (int a = 0; a < fe.dim; ++a)
    for (int k = 0; k < n * n; ++k)
      A[k] += -aw[a] * fe.grad[a * n * n + k] + aw[a] * fe.face[(2 * a + 1) * n * n + k];
  // pivoted Crout LU, unit upper U (src/RadiativeTransfer.cc:1026-1065)
  std::vector<int> piv(n);
  for (int k = 0; k < n; ++k) {
    piv[k] = k;
    double mx = std::fabs(A[k * n + k]);
    for (int j = k + 1; j < n; ++j)
      if (mx < std::fabs(A[j * n + k])) {
        mx = std::fabs(A[j * n + k]);
        piv[k] = j;
      }
    if (piv[k] != k)
      for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[piv[k] * n + j]);
    for (int j = k + 1; j < n; ++j) A[k * n + j] /= A[k * n + k];
    for (int i = k + 1; i < n; ++i)
      for (int j = k + 1; j < n; ++j) A[i * n + j] -= A[i * n + k] * A[k * n + j];
  }
  // column c of the inverse = solve with e_c (src/RadiativeTransfer.cc:1067-1105)
  std::vector<double> b(n), x(n);
  for (int c = 0; c < n; ++c) {
    for (int i = 0; i < n; ++i) b[i] = i == c ? 1.0 : 0.0;
    for (int k = 0; k < n; ++k) {
      if (piv[k] != k) std::swap(b[k], b[piv[k]]);
      x[k] = b[k];
      for (int i = 0; i < k; ++i) x[k] -= x[i] * A[k * n + i];
      x[k] /= A[k * n + k];
    }
    for (int k = n - 1; k >= 0; --k)
      for (int i = k + 1; i < n; ++i) x[k] -= x[i] * A[k * n + i];
    for (int i = 0; i < n; ++i) out[i * n + c] = x[i];
  }
}

}  // namespace ouranos
