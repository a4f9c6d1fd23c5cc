// Angular quadrature: direction sets, weights and the moment <-> discrete
// matrices.  Stands in for RTQuadrature / LS / GLC (src/RTQuadrature.cc:10-238,
// src/LS.cc:14-682, src/GLC.cc:14-1285).
//
// The level-symmetric tables are the published LS direction cosines and point
// weights (the values the reference tabulates in src/LS.cc).  They are stored
// here by weight class: a first-octant point with cosine indices (a, b, c),
// a+b+c = sn/2-1, has the weight of the sorted triple.  The reference's S14
// table carries w_1 = 1.0579... (src/LS.cc:172); the published value
// 0.0579970408969969964063611 is used instead.  Orders above S16 are not
// provided: the reference's S18 table assigns 44 of its 45 weights and its
// S20/S22 tables give one weight class two different values.
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

namespace ouranos {
namespace {

struct LSClass {
  int a, b, c;
  double w;
};
struct LSTable {
  int sn;
  int n_cos;
  double cosine[8];
  int n_class;
  LSClass cls[8];
};

const LSTable kLS[] = {
    {2, 1, {0.577350269189625764509149}, 1, {{0, 0, 0, 1.0}}},
    {4, 2, {0.350021174581540677777041, 0.868890300722201205229788}, 1,
     {{0, 0, 1, 1.0 / 3.0}}},
    {6, 3, {0.266635401516704720331535, 0.681507726536546927403750, 0.926180935517489107558380}, 2,
     {{0, 0, 2, 0.176126130863383433783565}, {0, 1, 1, 0.157207202469949899549768}}},
    {8, 4,
     {0.218217890235992381266097, 0.577350269189625764509149, 0.786795792469443145800830,
      0.951189731211341853132399},
     3,
     {{0, 0, 3, 0.120987654320987654320988},
      {0, 1, 2, 0.0907407407407407407407407},
      {1, 1, 1, 0.0925925925925925925925926}}},
    {10, 5,
     {0.189321326478010476671494, 0.508881755582618974382711, 0.694318887594384317279217,
      0.839759962236684758403029, 0.963490981110468484701598},
     4,
     {{0, 0, 4, 0.0893031479843567214704325},
      {0, 1, 3, 0.0725291517123655242296233},
      {0, 2, 2, 0.0450437674364086390490892},
      {1, 1, 2, 0.0539281144878369243545650}}},
    {12, 6,
     {0.167212652822713264084504, 0.459547634642594690016761, 0.628019096642130901034766,
      0.760021014833664062877138, 0.872270543025721502340662, 0.971637719251358378302376},
     5,
     {{0, 0, 5, 0.0707625899700910439766549},
      {0, 1, 4, 0.0558811015648888075828962},
      {0, 2, 3, 0.0373376737588285824652402},
      {1, 1, 3, 0.0502819010600571181385765},
      {1, 2, 2, 0.0258512916557503911218290}}},
    {14, 7,
     {0.151985861461031912404799, 0.422156982304796966896263, 0.577350269189625764509149,
      0.698892086775901338963210, 0.802226255231412057244328, 0.893691098874356784901111,
      0.976627152925770351762946},
     7,
     {{0, 0, 6, 0.0579970408969969964063611},
      {0, 1, 5, 0.0489007976368104874582568},
      {0, 2, 4, 0.0227935342411872473257345},
      {0, 3, 3, 0.0394132005950078294492985},
      {1, 1, 4, 0.0380990861440121712365891},
      {1, 2, 3, 0.0258394076418900119611012},
      {2, 2, 2, 0.00826957997262252825269908}}},
    {16, 8,
     {0.138956875067780344591732, 0.392289261444811712294197, 0.537096561300879079878296,
      0.650426450628771770509703, 0.746750573614681064580018, 0.831996556910044145168291,
      0.909285500943725291652116, 0.980500879011739882135849},
     8,
     {{0, 0, 7, 0.0489872391580385335008367},
      {0, 1, 6, 0.0413295978698440232405505},
      {0, 2, 5, 0.0203032007393652080748070},
      {0, 3, 4, 0.0265500757813498446015484},
      {1, 1, 5, 0.0379074407956004002099321},
      {1, 2, 4, 0.0135295047786756344371600},
      {1, 3, 3, 0.0326369372026850701318409},
      {2, 2, 3, 0.0103769578385399087825920}}},
};

const LSTable* find_ls(int sn) {
  for (const auto& t : kLS)
    if (t.sn == sn) return &t;
  return nullptr;
}

double ls_weight(const LSTable* t, int a, int b, int c) {
  int v[3] = {a, b, c};
  // sort three
  if (v[0] > v[1]) std::swap(v[0], v[1]);
  if (v[1] > v[2]) std::swap(v[1], v[2]);
  if (v[0] > v[1]) std::swap(v[0], v[1]);
  for (int k = 0; k < t->n_class; ++k)
    if (t->cls[k].a == v[0] && t->cls[k].b == v[1] && t->cls[k].c == v[2]) return t->cls[k].w;
  return -1.0;
}

// Positive Gauss-Legendre nodes (ascending) and weights of a k-point rule on
// [-1,1], k even: Newton iteration on P_k (Golub & Welsch would do as well).
void gauss_legendre_half(int k, std::vector<double>& nodes, std::vector<double>& weights) {
  const int half = k / 2;
  nodes.assign(half, 0.0);
  weights.assign(half, 0.0);
  for (int i = 0; i < half; ++i) {
    // i-th largest root
    double z = std::cos(M_PI * (i + 0.75) / (k + 0.5));
    double pk = 0.0, pkm1 = 0.0;
    for (int it = 0; it < 64; ++it) {
      double a = 1.0, b = z;
      for (int l = 2; l <= k; ++l) {
        double c = ((2 * l - 1) * z * b - (l - 1) * a) / l;
        a = b;
        b = c;
      }
      pk = b;
      pkm1 = a;
      double dp = k * (z * pk - pkm1) / (z * z - 1.0);
      double dz = pk / dp;
      z -= dz;
      if (std::fabs(dz) <= 1e-16 * std::fabs(z)) break;
    }
    double a = 1.0, b = z;
    for (int l = 2; l <= k; ++l) {
      double c = ((2 * l - 1) * z * b - (l - 1) * a) / l;
      a = b;
      b = c;
    }
    double dp = k * (z * b - a) / (z * z - 1.0);
    nodes[half - 1 - i] = z;
    weights[half - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// Fully normalised associated Legendre function
//   N_lm P_l^m(x),  N_lm = sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!),
// with the Condon-Shortley phase, by the standard stable recurrences in the
// normalised functions (no factorials).
double norm_legendre(int l, int m, double x) {
  const double s = std::sqrt(std::fmax(0.0, (1.0 - x) * (1.0 + x)));
  double pmm = std::sqrt(1.0 / (4.0 * M_PI));
  for (int k = 1; k <= m; ++k) pmm *= -std::sqrt((2.0 * k + 1.0) / (2.0 * k)) * s;
  if (l == m) return pmm;
  double pm1 = x * std::sqrt(2.0 * m + 3.0) * pmm;
  if (l == m + 1) return pm1;
  double pl = 0.0;
  for (int ll = m + 2; ll <= l; ++ll) {
    const double a = std::sqrt((4.0 * ll * ll - 1.0) / (double(ll) * ll - double(m) * m));
    const double b = std::sqrt(((ll - 1.0) * (ll - 1.0) - double(m) * m) / (4.0 * (ll - 1.0) * (ll - 1.0) - 1.0));
    pl = a * (x * pm1 - b * pmm);
    pmm = pm1;
    pm1 = pl;
  }
  return pl;
}

}  // namespace

int quadrature_sizes(int sn, int l_max, int galerkin, int dim, int* n_dir, int* n_mom) {
  if (sn < 2 || (sn & 1) || (dim != 2 && dim != 3) || l_max < 0) return OURANOS_ERR_BAD_INPUT;
  if (galerkin && dim == 3) return OURANOS_ERR_UNSUPPORTED;  // src/RTQuadrature.cc:30-31
  const int per_oct = sn * (sn + 2) / 8;
  const int nd = per_oct * (dim == 3 ? 8 : 4);
  int nm;
  if (galerkin)
    nm = nd;
  else
    nm = dim == 3 ? (l_max + 1) * (l_max + 1) : (l_max + 1) * (l_max + 2) / 2;
  if (n_dir) *n_dir = nd;
  if (n_mom) *n_mom = nm;
  return OURANOS_OK;
}

int quadrature_build(int type, int sn, int l_max, int galerkin, double ws, int dim,
                     int harmonics, double* omega_out, double* weight_out, double* m2d_out,
                     double* d2m_out, int* l_out, int* mn_out) {
  int nd, nm;
  int rc = quadrature_sizes(sn, l_max, galerkin, dim, &nd, &nm);
  if (rc) return rc;
  if (!(ws > 0.0)) return OURANOS_ERR_BAD_INPUT;
  const int half = sn / 2, per_oct = sn * (sn + 2) / 8;
  std::vector<double> om(3 * nd), w(nd);
  // ---- first octant
  if (type == OURANOS_QUAD_LS) {
    const LSTable* t = find_ls(sn);
    if (!t) return OURANOS_ERR_UNSUPPORTED;
    // points ordered by polar level j (Omega_z = cosine[j]), then i (Omega_y = cosine[i]),
    // Omega_x = cosine[half-1-i-j]: the order of LS::compute_omega (src/LS.cc:667-682)
    int k = 0;
    for (int j = 0; j < half; ++j)
      for (int i = 0; i < half - j; ++i, ++k) {
        const int ix = half - 1 - i - j;
        om[3 * k + 0] = t->cosine[ix];
        om[3 * k + 1] = t->cosine[i];
        om[3 * k + 2] = t->cosine[j];
        w[k] = ls_weight(t, ix, i, j);
        if (w[k] < 0) return OURANOS_ERR_UNSUPPORTED;
      }
  } else if (type == OURANOS_QUAD_GLC) {
    // Gauss-Legendre polar x Chebyshev azimuthal, triangular (src/GLC.cc:14-58)
    std::vector<double> mu, wmu;
    gauss_legendre_half(sn, mu, wmu);
    int k = 0;
    for (int i = 0; i < half; ++i) {
      const int na = half - i;
      const double st = std::sqrt(1.0 - mu[i] * mu[i]);
      for (int j = 0; j < na; ++j, ++k) {
        const double az = M_PI_2 * j / na + M_PI_4 / na;
        om[3 * k + 0] = st * std::cos(az);
        om[3 * k + 1] = st * std::sin(az);
        om[3 * k + 2] = mu[i];
        w[k] = wmu[i] * (M_PI_2 / na);
      }
    }
  } else {
    return OURANOS_ERR_BAD_INPUT;
  }
  // ---- reflect into the other octants: 2-D order (+,+),(+,-),(-,-),(-,+) as
  // src/RTQuadrature.cc:62-86; 3-D adds the same four with Omega_z < 0.
  const int n_oct = dim == 3 ? 8 : 4;
  static const int fx[8] = {1, 1, -1, -1, 1, 1, -1, -1};
  static const int fy[8] = {1, -1, -1, 1, 1, -1, -1, 1};
  static const int fz[8] = {1, 1, 1, 1, -1, -1, -1, -1};
  for (int o = 1; o < n_oct; ++o)
    for (int j = 0; j < per_oct; ++j) {
      const int k = o * per_oct + j;
      om[3 * k + 0] = fx[o] * om[3 * j + 0];
      om[3 * k + 1] = fy[o] * om[3 * j + 1];
      om[3 * k + 2] = fz[o] * om[3 * j + 2];
      w[k] = galerkin ? 0.0 : w[j];  // Galerkin weights stay unused and unreflected
    }
  if (!galerkin) {
    double wsum = 0.0;
    for (int j = 0; j < per_oct; ++j) wsum += w[j];
    for (int k = 0; k < nd; ++k) w[k] *= (1.0 / n_oct) / wsum;  // src/RTQuadrature.cc:87-94
  }
  // ---- moments: for l, cos part m = l..0, then sin part m = 1..l; 2-D keeps
  // even l+m (src/RTQuadrature.cc:136-197)
  struct Mom {
    int l, m;
    bool sine;
  };
  std::vector<Mom> moms;
  const int Lx = galerkin ? sn : l_max;
  for (int l = 0; l <= Lx; ++l) {
    for (int m = l; m >= 0; --m) {
      bool keep = dim == 3 || ((l + m) % 2 == 0);
      if (galerkin) keep = keep && l < sn;
      if (keep) moms.push_back({l, m, false});
    }
    for (int m = 1; m <= l; ++m) {
      bool keep = dim == 3 || ((l + m) % 2 == 0);
      if (galerkin) keep = keep && l <= sn;
      if (keep) moms.push_back({l, m, true});
    }
  }
  if ((int)moms.size() < nm) return OURANOS_ERR_BAD_INPUT;
  moms.resize(nm);
  const double wsph = std::sqrt(4.0 * M_PI / ws);
  std::vector<double> m2d((size_t)nd * nm);
  for (int d = 0; d < nd; ++d) {
    const double* o = &om[3 * d];
    double phi = std::atan(o[1] / o[0]);
    if (o[0] < 0.0) phi += M_PI;
    const double x = harmonics == OURANOS_HARM_REFERENCE ? std::cos(o[2]) : o[2];
    for (int q = 0; q < nm; ++q) {
      const Mom& mo = moms[q];
      double f = (harmonics == OURANOS_HARM_ORTHONORMAL && mo.m > 0) ? std::sqrt(2.0) : 1.0;
      double ang = mo.sine ? std::sin(mo.m * phi) : std::cos(mo.m * phi);
      m2d[(size_t)d * nm + q] = wsph * f * norm_legendre(mo.l, mo.m, x) * ang;
    }
  }
  std::vector<double> d2m((size_t)nm * nd);
  if (galerkin) {
    // D2M = M2D^-1 by Gauss-Jordan elimination with partial pivoting
    const int N = nd;
    std::vector<double> a(m2d), inv((size_t)N * N, 0.0);
    for (int i = 0; i < N; ++i) inv[(size_t)i * N + i] = 1.0;
    for (int c = 0; c < N; ++c) {
      int piv = c;
      for (int r = c + 1; r < N; ++r)
        if (std::fabs(a[(size_t)r * N + c]) > std::fabs(a[(size_t)piv * N + c])) piv = r;
      if (a[(size_t)piv * N + c] == 0.0) return OURANOS_ERR_BAD_INPUT;
      if (piv != c)
        for (int j = 0; j < N; ++j) {
          std::swap(a[(size_t)c * N + j], a[(size_t)piv * N + j]);
          std::swap(inv[(size_t)c * N + j], inv[(size_t)piv * N + j]);
        }
      const double dv = 1.0 / a[(size_t)c * N + c];
      for (int j = 0; j < N; ++j) {
        a[(size_t)c * N + j] *= dv;
        inv[(size_t)c * N + j] *= dv;
      }
      for (int r = 0; r < N; ++r) {
        if (r == c) continue;
        const double f = a[(size_t)r * N + c];
        if (f == 0.0) continue;
        for (int j = 0; j < N; ++j) {
          a[(size_t)r * N + j] -= f * a[(size_t)c * N + j];
          inv[(size_t)r * N + j] -= f * inv[(size_t)c * N + j];
        }
      }
    }
    d2m = inv;
  } else {
    for (int q = 0; q < nm; ++q)
      for (int d = 0; d < nd; ++d) d2m[(size_t)q * nd + d] = m2d[(size_t)d * nm + q] * ws * w[d];
  }
  if (omega_out) std::memcpy(omega_out, om.data(), sizeof(double) * 3 * nd);
  if (weight_out) std::memcpy(weight_out, w.data(), sizeof(double) * nd);
  if (m2d_out) std::memcpy(m2d_out, m2d.data(), sizeof(double) * nd * nm);
  if (d2m_out) std::memcpy(d2m_out, d2m.data(), sizeof(double) * nd * nm);
  if (l_out)
    for (int q = 0; q < nm; ++q) l_out[q] = moms[q].l;
  if (mn_out) {
    // most-normal direction sets (src/RTQuadrature.cc:200-238)
    double ext[6] = {0, 0, 0, 0, 0, 0};
    for (int d = 0; d < nd; ++d)
      for (int a = 0; a < dim; ++a) {
        ext[2 * a] = std::fmax(ext[2 * a], om[3 * d + a]);
        ext[2 * a + 1] = std::fmin(ext[2 * a + 1], om[3 * d + a]);
      }
    for (int f = 0; f < 2 * dim; ++f)
      for (int d = 0; d < nd; ++d) mn_out[f * nd + d] = om[3 * d + f / 2] == ext[f] ? 1 : 0;
  }
  return OURANOS_OK;
}

}  // namespace ouranos

extern "C" int ouranos_quadrature_sizes(int sn, int l_max, int galerkin, int dim, int* n_dir,
                                        int* n_mom) {
  return ouranos::quadrature_sizes(sn, l_max, galerkin, dim, n_dir, n_mom);
}

extern "C" int ouranos_quadrature_build(int type, int sn, int l_max, int galerkin,
                                        double weight_sum, int dim, int harmonics, double* omega,
                                        double* weight, double* m2d, double* d2m, int* moment_l,
                                        int* most_normal) {
  return ouranos::quadrature_build(type, sn, l_max, galerkin, weight_sum, dim, harmonics, omega,
                                   weight, m2d, d2m, moment_l, most_normal);
}
