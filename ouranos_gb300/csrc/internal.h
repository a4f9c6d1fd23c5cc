// Internal declarations of the GB300 transport-sweep operator.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/ouranos_gb300.h"
#include "df64.cuh"

namespace ouranos {

// ---------------------------------------------------------------- FE tables
// Reference-cell matrices of DG Q_p on equidistant Lagrange nodes, assembled
// by tensor products of 1-D integrals (exact Gauss integration), then scaled
// to an h_x x h_y (x h_z) box.  Local dof i = ix + P1*(iy + P1*iz).
struct FETables {
  int dim = 0, p = 0, p1 = 0, n = 0, fd = 0;
  double h[3] = {1, 1, 1};
  std::vector<double> mass;        // [n][n]
  std::vector<double> grad;        // [dim][n][n]: G_a[i][j] = int b_j d_a b_i
  std::vector<double> face;        // [2*dim][n][n]: E_f[i][j] = int_f b_i b_j
  std::vector<double> face_mass;   // [3][fd][fd]: transverse face mass, axis a
  std::vector<double> mass1d;      // [p1][p1] on [0,1]
};
FETables build_fe_tables(int dim, int p, const double* h);

// Inverse of the canonical-orientation cell matrix
//   A' = sigma_t M - sum_a |Omega_a| G_a + sum_a |Omega_a| E_{a,max}
// (every direction mapped to the all-positive octant, see sweep.cuh), computed
// with the reference's pivoted Crout LU (src/RadiativeTransfer.cc:1026-1105)
// applied to the unit vectors.  out: [n][n] row-major.
void canonical_inverse(const FETables& fe, double sigma_t, const double* abs_omega, double* out);

// --------------------------------------------------------------- quadrature
int quadrature_sizes(int sn, int l_max, int galerkin, int dim, int* n_dir, int* n_mom);
int quadrature_build(int type, int sn, int l_max, int galerkin, double ws, int dim,
                     int harmonics, double* omega, double* weight, double* m2d, double* d2m,
                     int* moment_l, int* most_normal);

// ------------------------------------------------------------ device buffer
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) {
    o.p = nullptr;
    o.bytes = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      bytes = o.bytes;
      o.p = nullptr;
      o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t alloc(size_t b) {
    if (b <= bytes && p) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p, b ? b : 16);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// ---------------------------------------------------------- sweep kernels
// Arguments of one sweep launch (see sweep.cuh for the algorithm).
template <typename real>
struct SweepArgs {
  int nx, ny, nz;              // cells per axis (physical)
  int n_sweep;                 // cells along the sweep axis (y in 2-D, z in 3-D)
  long n_dofs;                 // cells * n
  int n_mom;
  int wx, wy, kd;              // warp tiling: wx*wy cells x kd directions x lpc = 32 lanes
  int tiles_x, tiles_y;
  int n_tasks;
  const int2* tasks;           // (dir group, tile) in dependency order
  const int* group_dirs;       // [n_groups][kd] direction or -1
  const int* group_flip;       // [n_groups] bit a set: Omega_a < 0
  const int* dir_class;        // [n_dir] index of |Omega| class
  int n_dir_class;
  const real* abs_omega;       // [n_dir][3]
  const real* m2d;             // [n_dir][n_mom]      (moment-fused form)
  const real* ainv;            // [n_sigma_class][n_dir_class][n][pad4(n)]; lpc 32: [..][j][i] (transposed)
  const int* cell_class;       // [cells] sigma_t class
  const real* face_mass;       // [3][fd][pad4(fd)]
  const real* src;             // [n_mom][n_dofs] source moments T (moment-fused form)
  const real* iso;             // [n_dofs] isotropic fixed source or NULL (moment-fused form)
  const real* q;               // [n_dir][n_dofs] per-direction source (expanded form)
  const real* bnd;             // [n_dir][3] boundary inflow per axis or NULL
  real* psi;                   // [n_dir][n_dofs] angular flux out
  // edge buffers of tagged 64-bit words (1 per FP32 value, 2 per FP64 value)
  unsigned long long* edge_x;  // [n_dir][tiles][n_sweep][wy][fd][words]
  unsigned long long* edge_y;  // [n_dir][tiles][n_sweep][wx][fd][words]
  unsigned epoch;              // sweep epoch in [1, 0x7fff], tags edge words
  int* ticket;                 // task counter
  int* status;                 // 0 ok, 1 wait timeout
  long long wait_limit_ns;
  int wait_bias;
  int lpc;                     // lanes per cell: 1, 2 (cells of 9 or more dofs), or 32 (one warp
                               // per cell, sweep_wide.cuh; tiling 1 x 1 x 1, expanded source)
};

// fused_moments: 0 = read the expanded per-direction source q; 1 or 2 = apply
// M2D to that many source moments inside the sweep.
template <typename real>
cudaError_t launch_sweep(int dim, int p1, int fused_moments, const SweepArgs<real>& a, int grid,
                         int block, cudaStream_t s);
// One warp per cell (a.lpc == 32), every order of both dimensions: the form
// of the orders the per-lane kernels do not instantiate (sweep_wide.cuh)
template <typename real>
cudaError_t launch_sweep_wide(int dim, int p1, const SweepArgs<real>& a, int grid, int block, cudaStream_t s);
// Many problems in one persistent launch: args[p] per problem, tmap[t] =
// (problem, task) for ticket t, epoch read from the device (all problems of
// the launch share it), ticket reset to 0 by the caller.
template <typename real>
cudaError_t launch_sweep_batch(int dim, int p1, int fused_moments, int lanes_per_cell,
                               const SweepArgs<real>* args, const int2* tmap, int n_total, int* ticket,
                               const int* status, const unsigned* epoch, int grid, int block, cudaStream_t s);
// q[d][e] = sum_m M2D[d][m] T[m][e] (+ iso[e])  -- moment -> direction expansion.
// Every contraction below strides its rows by n_dofs and covers the dofs
// [0, len) of the pointers it gets (len < 0: all n_dofs), so a caller runs it
// on the dof range [e0, e0 + len) by offsetting each pointer by e0.
template <typename real>
cudaError_t launch_expand_source(const real* T, const real* iso, const real* m2d, real* q,
                                 int n_dir, int n_mom, long n_dofs, cudaStream_t s, long len = -1);
// the same two contractions for FP64 data in double-float arithmetic (df64.cuh)
cudaError_t launch_expand_source_df64(const double* T, const double* iso, const double* m2d,
                                      double* q, int n_dir, int n_mom, long n_dofs, cudaStream_t s,
                                      long len = -1);
cudaError_t launch_reduce_moments_df64(const double* psi, const double* d2m_t, double* phi,
                                       int n_dir, int n_mom, long n_dofs, cudaStream_t s, long len = -1);
// the same with T, iso, q (and psi) stored as double-float pairs (the
// double-float sweep's storage)
cudaError_t launch_expand_source_pairs(const df64* T, const df64* iso, const double* m2d, df64* q,
                                       int n_dir, int n_mom, long n_dofs, cudaStream_t s, long len = -1);
cudaError_t launch_reduce_moments_pairs(const df64* psi, const double* d2m_t, double* phi, int n_dir,
                                        int n_mom, long n_dofs, cudaStream_t s, long len = -1);
// Octant symmetry of a quadrature: the directions form classes of P = 2^dim
// members with the same |Omega|, member f having Omega_a < 0 exactly for the
// bits a of f; every moment m belongs to a parity group g whose M2D (and D2M)
// entries on member f are those of member 0 times -1 where bit f of sign[g]
// is set.  Built on the host (operator.cu) when the quadrature has it.
struct SymTables {
  int n_class = 0, P = 0, G = 0;
  int pattern = 0;                    // 2 / 3: the canonical 2-D / 3-D groups (compile-time kernels), 0: other
  const int* cls_dir = nullptr;       // [n_class][P] direction of member f
  const int* mom_group = nullptr;     // [n_mom] parity group
  const unsigned* sign = nullptr;     // [G] bit f set: negative on member f
  const double* m2d_rep = nullptr;    // [n_class][n_mom] M2D of member 0
  const double* d2m_rep = nullptr;    // [n_class][n_mom] D2M of member 0
};
// the double-float pair contractions through the symmetry: each class forms
// its products once per parity group (expansion) or its signed sums of psi
// once per group (reduction), about half the arithmetic of the direct form
// 2 or 3 when the groups and signs are the canonical ones of the harmonic
// moments of a 2-D (P = 4) or 3-D (P = 8) set, else 0
int sym_canonical_pattern(int P, int nm, int G, const int* mom_group, const unsigned* sign);
cudaError_t launch_expand_sym_pairs(const df64* T, const df64* iso, const SymTables& st, df64* q, int n_mom,
                                    long n_dofs, cudaStream_t s, long len = -1);
// with xc: writes xc - phi into phi's place (the Apply's combination, fused)
cudaError_t launch_reduce_sym_pairs(const df64* psi, const SymTables& st, double* phi, int n_mom, long n_dofs,
                                    cudaStream_t s, long len = -1, const double* xc = nullptr);
// The FP32 contractions on the tensor cores (contract_tc.cu): B operand
// images of M2D and D2M (three BF16 parts each, K-major core-matrix layout),
// built once per handle on the host.
struct TcTables {
  const uint8_t* m2d_img = nullptr;  // [3][npad directions][16 moments]
  const uint8_t* d2m_img = nullptr;  // [3][16 moment slots][kpad directions]
  int n_dir = 0, n_mom = 0, npad = 0, kpad = 0;
};
// FP64-accurate contractions of the double-float sweep on the tensor cores
// (contract_oz.cu): seven BF16 digits per value on power-of-two grids, digit
// products summed exactly per level in FP32 accumulators.  B operand images
// of M2D (digits per direction) and D2M (digits per moment and chunk of 48
// directions) with their exponents, built once per handle on the host.
struct OzHost {
  std::vector<uint8_t> m2d_img, d2m_img;  // [7][npad][16], [nch][7][16][48] (K-major BF16)
  std::vector<int> m2d_exp, d2m_exp;      // [npad], [nch][16]
  int n_dir = 0, n_mom = 0, npad = 0, nch = 0;
};
struct OzTables {
  const uint8_t* m2d_img = nullptr;
  const int* m2d_exp = nullptr;
  const uint8_t* d2m_img = nullptr;
  const int* d2m_exp = nullptr;
  int n_dir = 0, n_mom = 0, npad = 0, nch = 0;
};
bool oz_contractions_fit(int n_dir, int n_mom);
void oz_build_tables(const std::vector<double>& m2d, const std::vector<double>& d2m, int n_dir, int n_mom,
                     OzHost& h);
// q (pairs) = M2D T (+ iso) and phi (double) = D2M psi over the dofs [0, len)
// of the pointers (rows strided by n_dofs); a bounded wait that runs out sets
// bit 4 of *status
cudaError_t launch_expand_oz(const df64* T, const df64* iso, const OzTables& t, df64* q, long n_dofs, int* status,
                             long long limit_ns, cudaStream_t s, long len = -1);
cudaError_t launch_reduce_oz(const df64* psi, const OzTables& t, double* phi, long n_dofs, int* status,
                             long long limit_ns, cudaStream_t s, long len = -1, const double* xc = nullptr);
bool tc_contractions_fit(int n_dir, int n_mom);
void tc_build_images(const std::vector<double>& m2d, const std::vector<double>& d2m, int n_dir, int n_mom,
                     std::vector<uint8_t>& m2d_img, std::vector<uint8_t>& d2m_img, int& npad, int& kpad);
// q[d][e] = sum_m M2D[d][m] T[m][e] (+ iso[e]) and phi[m][e] = sum_d D2M[m][d]
// psi[d][e] for the dofs [0, len) of the pointers (rows n_dofs apart); a wait
// for the tensor cores that runs past limit_ns sets bit 4 of *status
cudaError_t launch_expand_tc(const float* T, const float* iso, const TcTables& t, float* q, long n_dofs, int* status,
                             long long limit_ns, cudaStream_t s, long len = -1);
cudaError_t launch_reduce_tc(const float* psi, const TcTables& t, float* phi, long n_dofs, int* status,
                             long long limit_ns, cudaStream_t s, long len = -1);
// phi[m][e] = sum_d D2M[m][d] psi[d][e]  -- direction -> moment reduction
template <typename real>
cudaError_t launch_reduce_moments(const real* psi, const real* d2m_t, real* phi, int n_dir,
                                  int n_mom, long n_dofs, cudaStream_t s, long len = -1);

// ------------------------------------------------------------ vector kernels
template <typename real>
cudaError_t launch_scatter_source(const double* x, const double* group_flux, real* src,
                                  const double* cell_mass, const double* sscale,
                                  const double* oscale, const int* material, int n_mat,
                                  int n_groups, int group, long n_cells, int n, int n_mom,
                                  long n_dofs, cudaStream_t s);
template <typename real>
cudaError_t launch_iso_source(real* iso, const double* qcell, const double* rowsum_mass,
                              const int* source_id, long n_cells, int n, cudaStream_t s);
template <typename real>
cudaError_t launch_combine(const double* x, const real* phi, double* y, long len, double sx,
                           double sp, cudaStream_t s);
template <typename real>
cudaError_t launch_combine_rows(const double* x, const real* phi, double* y, int rows, long len, long stride,
                                double sx, double sp, cudaStream_t s);
cudaError_t launch_permute(const double* in, double* out, const long* order, long n_cells,
                           int n, int n_vec, int to_internal, cudaStream_t s);
cudaError_t launch_axpby(double a, const double* x, double b, double* y, long len, cudaStream_t s);
// w += scale * sum_j coef[j] V[j] (coefficients on the device)
cudaError_t launch_multi_axpy(const double* const* V, int k, const double* coef, double scale,
                              double* w, long len, cudaStream_t s);
cudaError_t launch_bump_epoch(unsigned* epoch, cudaStream_t s);
cudaError_t launch_to_f32(const double* in, float* out, long n, cudaStream_t s);
cudaError_t launch_to_f32_pairs(const df64* in, float* out, long n, cudaStream_t s);
// q[d][c n + i] += inv_vdt sum_j M_ij psi[d][c n + j]  (implicit Euler's psi^n term)
template <typename real>
cudaError_t launch_angular_source(real* q, const float* psi, const double* cell_mass, double inv_vdt,
                                  int n, long n_cells, int n_dir, cudaStream_t s);
cudaError_t launch_scale_inv_norm(const double* nrm2, double* v, long len, cudaStream_t s);
constexpr int kDotGrid = 1216;  // blocks of the dot-product kernel (8 per SM: enough loads in flight)
// out[j] = xs[j] . y for j < k (k <= 32), FP64: per-block partials in chunks
// of 8 vectors into partial[k * kDotGrid], then one warp per output sums them
// in a fixed order (deterministic, no atomics)
cudaError_t launch_dots(const double* const* xs, const double* y, int k, long len, double* out,
                        double* partial, cudaStream_t s);

}  // namespace ouranos
namespace ouranos {
// Least squares of restarted GMRES on the host: the (m+1) x m Hessenberg
// matrix reduced by Givens rotations as columns arrive; g is the rotated
// right-hand side beta e_1, |g[k+1]| the residual estimate after k+1 columns.
struct Givens {
  int m;
  std::vector<double> H, cs, sn, g;
  explicit Givens(int m_) : m(m_), H((m_ + 1) * m_, 0.0), cs(m_), sn(m_), g(m_ + 1, 0.0) {}
  double& h(int i, int j) { return H[i * m + j]; }
  // column k of H holds h[0..k+1]; returns |g_{k+1}|
  double add_column(int k, const double* col) {
    for (int i = 0; i <= k + 1; ++i) h(i, k) = col[i];
    for (int j = 0; j < k; ++j) {
      const double a = h(j, k), b = h(j + 1, k);
      h(j, k) = cs[j] * a + sn[j] * b;
      h(j + 1, k) = -sn[j] * a + cs[j] * b;
    }
    const double a = h(k, k), b = h(k + 1, k);
    const double r = std::hypot(a, b);
    cs[k] = r > 0 ? a / r : 1.0;
    sn[k] = r > 0 ? b / r : 0.0;
    h(k, k) = r;
    h(k + 1, k) = 0.0;
    g[k + 1] = -sn[k] * g[k];
    g[k] = cs[k] * g[k];
    return std::fabs(g[k + 1]);
  }
  std::vector<double> solve(int k) {
    std::vector<double> y(k, 0.0);
    for (int i = k - 1; i >= 0; --i) {
      double s = g[i];
      for (int j = i + 1; j < k; ++j) s -= h(i, j) * y[j];
      y[i] = h(i, i) != 0.0 ? s / h(i, i) : 0.0;
    }
    return y;
  }
};
}  // namespace ouranos
struct ouranos_rt;
struct ouranos_cnn;
namespace ouranos {
// learned preconditioner glue (precond.cu)
int rt_pc_features(ouranos_rt* rt, const double* v, float* feat);
int rt_pc_correct(ouranos_rt* rt, const double* v, const float* y, double* z);
// diffusion synthetic acceleration (dsa.cu): out = v + f on the handle's stream
int rt_dsa_apply(ouranos_rt* rt, const double* v, double* out);
// the same with the CG started from a guess of f ([vertex] FP32, written by
// the caller into the buffer rt_dsa_guess_buffer returns)
int rt_dsa_guess_buffer(ouranos_rt* rt, float** guess, long* n_vertices);
int rt_dsa_apply_guess(ouranos_rt* rt, const double* v, double* out);
// learned preconditioner with the diffusion solve (precond.cu): the network's
// correction of v as the initial guess of the diffusion CG, out = v + f
int rt_pc_dsa_apply(ouranos_rt* rt, const double* v, double* out);
// the network's cell grid
void cnn_grid(const ouranos_cnn* net, int* nx, int* ny, int* nz);
// The network's forward of `features` into `out` in the order of stream s,
// without a host synchronisation.  The first call with a pair of buffers runs
// the launches on the network's own stream, fenced by events against s (this
// configures every kernel); the second records the same launches, the copy
// of the output and the copy of the status word into a CUDA graph; every
// call from then on launches that graph on s.  The status word reaches the
// host with the work of s: cnn_forward_status reads it once s is synchronised
// (OURANOS_ERR_TIMEOUT if a convolution's bounded wait ran out).
int cnn_forward_on(ouranos_cnn* net, const float* features, float* out, cudaStream_t s);
int cnn_forward_status(ouranos_cnn* net);
// drop the recorded graph (after its last launch has ended): the buffers it
// was recorded with may be freed
void cnn_forward_release(ouranos_cnn* net);
// Device-side pieces the solvers use (operator.cu).
int rt_apply_device(ouranos_rt* rt, const double* x, double* y);
// allocation-free Apply (noalloc.cu): resolve its scratch array on `device`,
// which must be current; once per device, called by ouranos_rt_create
int noalloc_setup(int device);
int rt_rhs_device(ouranos_rt* rt, const double* gf, double* rhs);
int rt_check_status(ouranos_rt* rt);
// batched Apply pieces (see operator.cu)
int rt_batch_prepare(ouranos_rt* rt, const double* x, SweepArgs<double>* a, int* fm, bool sources);
int rt_batch_prepare(ouranos_rt* rt, const double* x, SweepArgs<float>* a, int* fm, bool sources);
int rt_batch_finish(ouranos_rt* rt, const double* x, double* y, bool sources);
int rt_clear_status(ouranos_rt* rt);
// Scratch of the batched diffusion solve: the device problem table, block
// map, partials and barrier, and the page-locked staging of the table.
struct DsaBatchScratch {
  DevBuf dev;
  void* host = nullptr;
  size_t host_bytes = 0;
  ~DsaBatchScratch();
};
// out[i] = P_i v[i] for the problems rts[0..count) (device vectors, internal
// cell order) in one cooperative launch per mesh dimension on `stream`; a
// barrier wait that runs out sets bit 2 of *status.  Every problem must have
// the same CG step count.  One call per stream synchronisation (the staging
// block is reused).
int rt_dsa_apply_batch(ouranos_rt* const* rts, const double* const* v, double* const* out, int count,
                       cudaStream_t stream, int* status, DsaBatchScratch& sc, std::string& err);
int rt_stage_in(ouranos_rt* rt, const double* v, DevBuf& buf, int n_vec, const double** out);
int rt_stage_out(ouranos_rt* rt, const double* dv, double* user);
}  // namespace ouranos

// cell ranges of the host-vector Apply's overlapped copies
#define OURANOS_OVERLAP_CHUNKS 5

struct ouranos_rt {
  int device = 0;
  cudaStream_t stream = nullptr;      // stream in use
  cudaStream_t own_stream = nullptr;  // the handle's own stream
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // host-vector Apply: the copy stream and its chunk events (created on first use)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_chunk[2 * OURANOS_OVERLAP_CHUNKS + 2] = {};
  std::string err;
  // problem
  int dim = 2, p = 1, p1 = 2, n = 4, fd = 2;
  int nx[3] = {1, 1, 1};
  double h[3] = {1, 1, 1};
  long n_cells = 0, n_dofs = 0;
  int G = 1, group = 0, n_dir = 0, n_mom = 0, n_mat = 0, l_max = 0, n_src = 0;
  double ws = 1.0;
  std::vector<double> omega, m2d, d2m, sigma_t, sigma_s, source, inc_flux;
  std::vector<int> moment_l, most_normal, material_id, source_id;
  int bc[6] = {0, 0, 0, 0, 0, 0};
  std::vector<long> cell_order;
  ouranos::FETables fe;
  int precision = OURANOS_FP64;
  int fp64_contract = OURANOS_FP64_DF64_SWEEP;  // arithmetic of the FP64 path
  int fp32_contract = OURANOS_FP32_CONTRACT_CUDA_CORES;  // where the FP32 path's contractions run
  ouranos::TcTables tc;                                  // their tensor-core tables (tc.npad 0: none)
  ouranos::DevBuf d_tc_m2d, d_tc_d2m;
  ouranos::OzTables oz;                                  // exact-digit tensor-core tables (oz.npad 0: none)
  ouranos::DevBuf d_oz_m2d, d_oz_d2m, d_oz_m2d_exp, d_oz_d2m_exp;
  // schedule
  int wx = 0, wy = 1, kd = 0;          // 0 = not chosen yet
  int lpc = 1;                         // lanes per cell (2 only for cells of >= 9 dofs)
  int tiles_x = 0, tiles_y = 0, n_groups_dir = 0, n_tasks = 0;
  std::vector<int> dir_class_h;
  std::vector<double> class_abs_omega;  // [n_dir_class][3]
  int n_dir_class = 0;
  std::vector<double> sigma_class_value; // per sigma_t class
  std::vector<int> cell_class_h;
  long long wait_limit_ns = 2000000000LL;
  int wait_bias = 0;
  unsigned epoch = 0;                  // sweep counter, tags edge-buffer words
  double last_ms = 0.0;
  int last_kernels = 0;
  bool ainv_valid = false;
  bool scat_valid = false;             // src_* holds compute_scattering_source(x)
  // device: geometry / tables (both precisions where the sweep reads them)
  ouranos::DevBuf d_material, d_source_id, d_cell_class, d_cell_order;
  ouranos::DevBuf d_cell_mass, d_rowsum_mass, d_sscale, d_oscale, d_qcell;
  ouranos::DevBuf d_dir_class, d_abs64, d_abs32, d_m2d64, d_m2d32, d_d2m64, d_d2m32;
  ouranos::DevBuf d_ainv64, d_ainv32, d_face64, d_face32, d_bnd64, d_bnd32;
  ouranos::DevBuf d_absdf, d_m2ddf, d_ainvdf, d_facedf, d_bnddf;  // double-float sweep tables
  ouranos::DevBuf d_tasks, d_group_dirs, d_group_flip, d_progress, d_ctrl;
  ouranos::DevBuf d_edge_x, d_edge_y;
  // device: vectors
  ouranos::DevBuf d_src64, d_src32, d_phi64, d_phi32, d_iso64, d_iso32, d_q, d_psi;
  ouranos::DevBuf d_x, d_y, d_gf, d_tmp, d_scatx;  // staging; d_scatx: scattering-source argument
  // solver workspace
  ouranos::DevBuf d_krylov;
  // implicit Euler in time: 1/(v dt) added to sigma_t, inv_vdt M psi^n added to
  // the source of source sweeps; psi^n (FP32, [dir][dof]) kept on the device
  double inv_vdt = 0.0;
  ouranos::DevBuf d_psi_prev;
  // octant symmetry of the quadrature (empty: contractions take the direct form)
  ouranos::SymTables sym;
  ouranos::DevBuf d_sym_dir, d_sym_group, d_sym_sign, d_sym_m2d, d_sym_d2m;
  // learned preconditioner
  ouranos_cnn* cnn = nullptr;
  bool cnn_pending = false;  // a forward of cnn ran on the stream since the last status check
  int pc_group = -1;
  ouranos::DevBuf d_pc_prop, d_pc_work, d_pc_feat, d_pc_nodal, d_pc_vert;
  // diffusion synthetic acceleration: CG steps (0 = off), cell coefficients,
  // CG vectors and reductions; tables valid for (dsa_group, dsa_inv_vdt)
  int dsa_iters = 0, dsa_group = -1, dsa_grid = 0;
  double dsa_inv_vdt = -1.0;
  ouranos::DevBuf d_dsa_cell, d_dsa_coef, d_dsa_vec, d_dsa_red, d_dsa_fe;
};
