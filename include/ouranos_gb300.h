/*
 * ouranos_gb300 -- C-ABI of the GB300-native transport-sweep operator.
 *
 * The operator replaces the reference's
 *   class RadiativeTransfer<dim,tensor_dim> : public Epetra_Operator
 * (Rombur/ouranos src/RadiativeTransfer.hh:46-263) on the path the SI/GMRES
 * driver of src/ouranos.cc:43-209 calls.  Each entry point below names the
 * reference member it stands in for.  Conventions:
 *   - every function returns an int status: OURANOS_OK (0) or a negative
 *     OURANOS_ERR_* code; ouranos_rt_last_error() gives the message.  No C++
 *     exception crosses this boundary.
 *   - flux-moment vectors use the reference's Epetra layout [mom][dof]
 *     (src/RadiativeTransfer.cc:831,995): entry m*n_dofs + cell*n + i, where
 *     cell = i_x + n_x*(i_y + n_y*i_z) unless the descriptor supplies
 *     cell_order, and i is the lexicographic (x fastest) local Lagrange dof.
 *   - vector arguments may be host or device (cudaMalloc / managed) pointers;
 *     the operator detects which.  Host buffers are copied in and out inside
 *     the call.
 *   - one handle = one CUDA stream; calls on one handle are not thread-safe
 *     (the reference operator mutates `mutable` state inside const methods and
 *     is not reentrant either, src/RadiativeTransfer.hh:195-212).
 */
#ifndef OURANOS_GB300_H
#define OURANOS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OURANOS_OK 0
#define OURANOS_ERR_BAD_INPUT (-1)
#define OURANOS_ERR_CUDA (-2)
#define OURANOS_ERR_TIMEOUT (-3)
#define OURANOS_ERR_UNSUPPORTED (-4)
#define OURANOS_ERR_NO_DEVICE (-5)
#define OURANOS_ERR_NOT_CONVERGED (-6)

/* Boundary kinds, src/Parameters.hh:21.  REFLECTIVE is accepted and, as in the
 * reference (src/RadiativeTransfer.cc:958-975), treated as vacuum. */
#define OURANOS_BC_VACUUM 0
#define OURANOS_BC_ISOTROPIC 1
#define OURANOS_BC_MOST_NORMAL 2
#define OURANOS_BC_REFLECTIVE 3

/* Quadrature families: src/LS.hh, src/GLC.hh. */
#define OURANOS_QUAD_LS 0
#define OURANOS_QUAD_GLC 1

/* Harmonic conventions for the moment-to-discrete matrix (src/RTQuadrature.cc:97-198):
 * ORTHONORMAL: real spherical harmonics at polar angle arccos(Omega_z), sqrt(2)
 *   on m>0 (orthonormal set; default).
 * REFERENCE: the reference's literal boost call, polar-angle argument Omega_z,
 *   no sqrt(2) (src/RTQuadrature.cc:126-131). */
#define OURANOS_HARM_ORTHONORMAL 0
#define OURANOS_HARM_REFERENCE 1

/* Arithmetic of the sweep. */
#define OURANOS_FP64 0
#define OURANOS_FP32 1
/* How the FP64 path computes (double-float = pairs of FP32 numbers on the FP32
 * pipes, about 48 significant bits and the FP32 exponent range; GB300 issues
 * FP32 at 64x its FP64 rate):
 *   NATIVE     native FP64 everywhere;
 *   DF64       moment <-> direction contractions in double-float, sweep in FP64;
 *   DF64_SWEEP contractions and the cell solves of the sweep in double-float,
 *              sources and angular fluxes stored as pairs (the default);
 *   DF64_SWEEP_TC  the double-float sweep with its two contractions on the
 *              tensor cores: seven BF16 digits per value on power-of-two
 *              grids, digit products summed exactly per level (up to 192
 *              directions and 16 moments).
 * All four meet the 1e-12 parity bar against the FP64 oracle. */
#define OURANOS_FP64_NATIVE 0
#define OURANOS_FP64_DF64 1
#define OURANOS_FP64_DF64_SWEEP 2
#define OURANOS_FP64_DF64_SWEEP_TC 3
/* Where the FP32 path's moment <-> direction contractions run:
 *   CUDA_CORES FP32 multiply-adds on the CUDA cores;
 *   TENSOR     tcgen05 MMAs on the tensor cores, every FP32 operand split
 *              into three BF16 parts (products of part order <= 2 summed in
 *              FP32: FP32 accuracy); up to 256 directions and 16 moments. */
#define OURANOS_FP32_CONTRACT_CUDA_CORES 0
#define OURANOS_FP32_CONTRACT_TENSOR 1

/* Problem description: the data the reference spreads over Parameters,
 * Geometry, RTQuadrature and RTMaterialProperties (src/*.hh), restricted to a
 * uniform Cartesian mesh.  All arrays are host memory and are copied. */
typedef struct ouranos_problem_desc {
  int dim;                  /* 2 or 3 */
  int fe_order;             /* 1..5 (DG Q_p, equidistant nodes) */
  int n_cells[3];           /* cells per axis */
  double lower[3];          /* box corners */
  double upper[3];
  int n_groups;
  /* quadrature, as RTQuadrature::get_omega/get_M2D/get_D2M/get_l return it */
  int n_dir;
  int n_mom;
  const double* omega;      /* [n_dir][3] */
  const double* m2d;        /* [n_dir][n_mom] */
  const double* d2m;        /* [n_mom][n_dir] */
  const int* moment_l;      /* [n_mom] Legendre order of each moment */
  const int* most_normal;   /* [2*dim][n_dir] flags or NULL */
  double weight_sum;        /* Parameters::get_weight_sum */
  /* materials, RTMaterialProperties layout (src/RTMaterialProperties.hh:84-101) */
  int n_materials;
  int l_max;
  const double* sigma_t;    /* [mat][g] */
  const double* sigma_s;    /* [mat][g_from][g_to][l] */
  const int* material_id;   /* [cell] */
  const int* source_id;     /* [cell] or NULL */
  int n_sources;
  const double* source;     /* [src][g] or NULL (Parameters::get_src) */
  int bc_type[6];           /* per face x-,x+,y-,y+,z-,z+ */
  const double* inc_flux;   /* [face][g] or NULL (Parameters::get_inc_flux) */
  const long* cell_order;   /* optional: caller's index of each lexicographic cell
                               (e.g. deal.II's z-order); NULL = lexicographic */
} ouranos_problem_desc;

typedef struct ouranos_rt ouranos_rt;

/* ---------------------------------------------------------------- quadrature */
/* RTQuadrature::RTQuadrature sizes (src/RTQuadrature.cc:10-25); 3-D deploys 8
 * octants (the reference's deploy_octant fills 4, src/RTQuadrature.cc:61). */
int ouranos_quadrature_sizes(int sn, int l_max, int galerkin, int dim, int* n_dir, int* n_mom);
/* RTQuadrature::build_quadrature (src/RTQuadrature.cc:27-56) with LS::build_octant
 * (src/LS.cc:14-682, S2..S16) or GLC::build_octant (src/GLC.cc:14-58, Gauss-Legendre
 * nodes computed, any even order).  Any output pointer may be NULL. */
int ouranos_quadrature_build(int type, int sn, int l_max, int galerkin, double weight_sum,
                             int dim, int harmonics, double* omega, double* weight,
                             double* m2d, double* d2m, int* moment_l, int* most_normal);

/* ------------------------------------------------------------------ operator */
/* RadiativeTransfer constructor + setup() (src/RadiativeTransfer.cc:12-78):
 * builds the FE tables, the per-octant wavefront schedule and the device
 * arrays.  Selects CUDA device `device` (-1 = current). */
int ouranos_rt_create(const ouranos_problem_desc* desc, int device, ouranos_rt** out);
/* ~RadiativeTransfer (src/RadiativeTransfer.cc:38-47). */
int ouranos_rt_destroy(ouranos_rt* rt);
/* RadiativeTransfer::set_group (src/RadiativeTransfer.hh:230 area). */
int ouranos_rt_set_group(ouranos_rt* rt, int group);
/* Sweep arithmetic: OURANOS_FP64 (default, parity path) or OURANOS_FP32. No
 * reference counterpart (the reference is FP64 only). */
int ouranos_rt_set_precision(ouranos_rt* rt, int precision);
/* Select OURANOS_FP64_NATIVE, OURANOS_FP64_DF64, OURANOS_FP64_DF64_SWEEP or
 * OURANOS_FP64_DF64_SWEEP_TC (UNSUPPORTED beyond 192 directions or 16 moments)
 * for the FP64 path.  No reference counterpart. */
int ouranos_rt_set_fp64_contractions(ouranos_rt* rt, int mode);
/* Select OURANOS_FP32_CONTRACT_CUDA_CORES or OURANOS_FP32_CONTRACT_TENSOR for
 * the FP32 path (UNSUPPORTED beyond 256 directions or 16 moments).  No
 * reference counterpart. */
int ouranos_rt_set_fp32_contractions(ouranos_rt* rt, int mode);
/* Length of a flux-moment vector, n_mom * n_dofs: the size of the Epetra_Map
 * returned by OperatorDomainMap/OperatorRangeMap (src/RadiativeTransfer.hh:240-249). */
int ouranos_rt_vector_length(const ouranos_rt* rt, long* length);
/* Number of (cell, direction) tasks one sweep executes: the value
 * RadiativeTransfer::get_n_tasks_to_execute holds after initialize_scheduler. */
int ouranos_rt_n_tasks(const ouranos_rt* rt, long* n_tasks);
/* compute_scattering_source (src/RadiativeTransfer.cc:811-843): S_m = sigma_s,l(m) M x_m,
 * kept inside the handle for the next ouranos_rt_sweep. */
int ouranos_rt_scattering_source(ouranos_rt* rt, const double* x);
/* The driver's sweep loop `initialize_scheduler(); while (tasks) sweep(...)`
 * (src/ouranos.cc:74-84,150-158): flux_moments += D L^-1 (M2D S [+ q + other-group
 * scattering + boundary inflow when group_flux != NULL]).  group_flux is
 * [g][mom][dof] (the reference's group_flux vector of MPI vectors). */
int ouranos_rt_sweep(ouranos_rt* rt, double* flux_moments, const double* group_flux);
/* Epetra_Operator::Apply (src/RadiativeTransfer.cc:780-809): y = x - D L^-1 M2D S x.
 * x and y may be host or device pointers (y == x allowed).  With page-locked
 * host vectors the copies travel in cell ranges on a second stream,
 * overlapped with the kernels before and after the sweep; the result is
 * bit-identical to the device-pointer call. */
int ouranos_rt_apply(ouranos_rt* rt, const double* x, double* y);
/* Right-hand side of the Krylov form (src/ouranos.cc:149-158): rhs += D L^-1 (q +
 * other-group scattering + boundary inflow), with the in-group scattering source
 * taken as zero (its value before the first Apply). */
int ouranos_rt_sweep_rhs(ouranos_rt* rt, const double* group_flux, double* rhs);
/* Per-octant wavefront level of every task, [dir][cell] (cell in the
 * lexicographic numbering): the longest-path depth in the task graph that
 * compute_sweep_ordering builds (src/RadiativeTransfer.cc:80-232). */
int ouranos_rt_task_levels(const ouranos_rt* rt, int* levels);
/* The same levels without a handle (host integer work, no GPU needed):
 * n_cells[dim], omega[n_dir][3] -> levels[n_dir][cells]. */
int ouranos_wavefront_levels(int dim, const int* n_cells, int n_dir, const double* omega,
                             int* levels);
/* Run the handle's work on the caller's CUDA stream (a cudaStream_t; NULL
 * returns to the handle's own stream).  Calls still synchronise that stream
 * before returning. */
int ouranos_rt_set_stream(ouranos_rt* rt, void* stream);
/* Copy of the last error message. */
int ouranos_rt_last_error(const ouranos_rt* rt, char* buf, size_t len);
/* Device time (ms) of the last sweep kernel launch, measured with CUDA events
 * on the handle's stream; and the number of kernels the last call launched
 * (an Apply: scattering source, expansion, sweep, reduction and, unless the
 * reduction writes y = x - phi itself, the combination). */
int ouranos_rt_last_sweep_ms(const ouranos_rt* rt, double* ms, int* kernels);
/* Tiling of the sweep kernel: cells per warp along x (and y in 3-D) and
 * directions per warp, with cells_x * cells_y * dirs == 32 (one lane per cell),
 * or == 16 for cells of 9 or more dofs (2-D Q2+, 3-D Q2): two lanes share each
 * cell solve, or 1 x 1 x 1: one warp per cell (every order; the only tiling
 * of 2-D Q5 and 3-D Q3..Q5).  0s = the default (one direction per warp; 2-D
 * 32 x 1, 3-D 4 x 8; two lanes per cell and 16 cells where allowed: 2-D
 * 16 x 1, 3-D 4 x 4; one warp per cell for 2-D Q5 and 3-D Q3..Q5). */
int ouranos_rt_set_tiling(ouranos_rt* rt, int cells_x, int cells_y, int dirs_per_warp);
int ouranos_rt_get_tiling(const ouranos_rt* rt, int* cells_x, int* cells_y, int* dirs_per_warp);
/* Spin limit of the in-kernel dependency waits, in nanoseconds (default 2 s).
 * A wait that runs out sets an error status, every warp leaves, and the call
 * returns OURANOS_ERR_TIMEOUT with the context still usable. */
int ouranos_rt_set_wait_limit(ouranos_rt* rt, double ns);
/* Test hook: bias the dependency target the sweep waits for by `extra` steps
 * (0 = normal).  A positive value makes the first dependent wait unsatisfiable
 * (the sweep's edge words and the diffusion solve's grid barriers alike) so
 * the timeout path can be exercised without faulting the GPU. */
int ouranos_rt_debug_wait_bias(ouranos_rt* rt, int extra);

/* Apply, y = x - D L^-1 M2D S x, that allocates no device memory during the
 * call.  No counterpart in the reference.  For callers that cannot allocate
 * device memory when they apply the operator -- a solver framework that owns
 * the device memory pool and forbids allocations inside its operator
 * callbacks, or a driver that allows allocations only at set-up.  Every
 * scratch buffer of the Apply lives in one file-scope device array of
 * OURANOS_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * the process exits; problems needing more scratch are rejected with
 * OURANOS_ERR_BAD_INPUT.  x and y must be device pointers.  ouranos_rt_create
 * looks the array's address up on the handle's device (cudaGetSymbolAddress,
 * which under CUDA's lazy module loading is also what places the array
 * there), so the call itself only reads that address.  It runs the kernels
 * ouranos_rt_apply runs for the handle's precision and FP64 arithmetic, and
 * returns once its GPU work has finished.  All calls share the array, so
 * calls whose GPU work overlaps (two streams, threads or handles) race. */
#define OURANOS_NOALLOC_SCRATCH_BYTES (32u << 20)
int ouranos_rt_apply_noalloc(ouranos_rt* rt, const double* x, double* y);

/* ------------------------------------------------------------------- solvers */
/* Drivers of src/ouranos.cc:43-209, on device vectors.
 * OURANOS_SOLVER_SI: source iteration, relative-change test (src/ouranos.cc:72-95).
 * OURANOS_SOLVER_GMRES: restarted GMRES(restart), FP64 sweeps.
 * OURANOS_SOLVER_BICGSTAB: BiCGSTAB, FP64 sweeps (tests/RadiativeTransfer_test.cc:78).
 * OURANOS_SOLVER_FGMRES_MIXED: FGMRES(restart) whose Arnoldi operator applies use
 *   FP32 sweeps, with FP64 Gram-Schmidt, FP64 true residual at every restart. */
#define OURANOS_SOLVER_SI 0
#define OURANOS_SOLVER_GMRES 1
#define OURANOS_SOLVER_BICGSTAB 2
#define OURANOS_SOLVER_FGMRES_MIXED 3
/* FGMRES_MIXED with the learned right preconditioner installed by
 * ouranos_rt_set_preconditioner; falls back to the plain method for the rest of
 * the solve when a preconditioned restart cycle stagnates.  With
 * OURANOS_SOLVER_DSA the network's output is the initial guess of the
 * diffusion correction's CG (ouranos_rt_pc_dsa_apply), and the diffusion
 * correction from a zero guess is the fallback. */
#define OURANOS_SOLVER_FGMRES_LEARNED 4
/* OR into the solver: x holds the initial guess (not with BiCGSTAB) */
#define OURANOS_SOLVER_WARM_START 0x100
/* OR into SI, GMRES, FGMRES_MIXED or FGMRES_LEARNED: diffusion synthetic
 * acceleration (ouranos_rt_set_dsa) as the right preconditioner (GMRES becomes
 * FGMRES with FP64 sweeps), or as the acceleration step of SI */
#define OURANOS_SOLVER_DSA 0x200

typedef struct ouranos_solve_info {
  int iterations;           /* operator applications in the Krylov/SI loop */
  int restarts;
  double residual;          /* final ||b - (I-T)x|| / ||b|| in FP64 (SI: last relative change) */
  double seconds;           /* wall time of the solve */
  int converged;
} ouranos_solve_info;

/* Solve (I - T) phi = rhs for the current group (rhs from ouranos_rt_sweep_rhs
 * with group_flux), x is [mom][dof] (host or device).  hist (host, may be NULL)
 * receives max_it+1 relative residuals. */
int ouranos_solve(ouranos_rt* rt, int solver, int restart, int max_it, double tol,
                  const double* group_flux, double* x, double* hist, ouranos_solve_info* info);

/* Multigroup outer iteration (src/ouranos.cc:62-128 for SI, 141-207 for the
 * Krylov solvers): Gauss-Seidel over the groups -- each outer iteration
 * solves every group g in turn, (I - T_g) phi_g = rhs_g(phi of the other
 * groups), with `solver` (flags allowed; warm-started from the group's last
 * flux except with BiCGSTAB) to inner_tol within max_inner_it, until the
 * relative L2 change of all group fluxes falls below outer_tol (the
 * reference's sqrt(num/denom) test) or max_outer_it iterations have run.
 * group_flux: [n_groups][n_mom][n_dofs], host or device; in: initial fluxes,
 * out: the solution.  Leaves the handle on the last group. */
typedef struct ouranos_multigroup_info {
  int outer_iterations;
  int inner_iterations;     /* operator applications summed over all group solves */
  double change;            /* last relative change of the group fluxes */
  double seconds;
  int converged;
} ouranos_multigroup_info;
int ouranos_solve_multigroup(ouranos_rt* rt, int solver, int restart, int max_inner_it, double inner_tol,
                             int max_outer_it, double outer_tol, double* group_flux,
                             ouranos_multigroup_info* info);

/* ------------------------------------------------------- time dependence
 * Implicit Euler in time.  No counterpart in the reference operator (its
 * TimeDiscretization class, src/TimeDiscretization.cc:10-82, is never
 * called).  With inv_vdt = 1/(v dt) > 0 each step solves
 *   Omega.grad psi + (sigma_t + inv_vdt) psi = S phi + q/ws + inv_vdt psi^n
 * and keeps psi^n (FP32, [dir][dof]) on the device, starting from 0; 0
 * switches it off.  sigma_t in the description stays the physical one. */
int ouranos_rt_set_time_step(ouranos_rt* rt, double inv_vdt);
/* replace the fixed-source strengths ([n_sources][n_groups]), e.g. a pulse */
int ouranos_rt_set_source(ouranos_rt* rt, const double* source);
/* one step: phi in = initial guess (phi^n), out = phi^{n+1}; then psi^n
 * advances by one FP64 source sweep of phi^{n+1}, stored in FP32 (only after
 * convergence) */
int ouranos_rt_time_advance(ouranos_rt* rt, int solver, int restart, int max_it, double tol, double* phi,
                            ouranos_solve_info* info);
/* psi^n as doubles, [dir][dof] with lexicographic cells: checkpoint / resume */
int ouranos_rt_get_angular_flux(ouranos_rt* rt, double* psi);
int ouranos_rt_set_angular_flux(ouranos_rt* rt, const double* psi);

/* ------------------------------------------------------- many problems
 * No counterpart in the reference, which runs one problem per MPI job
 * (src/ouranos.cc:43-209).  A batch holds `count` independent problems
 * (descs is an array of count descriptions); its vectors are the problems'
 * [mom][dof] vectors one after another (ouranos_batch_layout gives the
 * offsets).  A batched Apply runs every problem's sweep in one persistent
 * launch per (dimension, FE order, fused-moment form) class and is captured
 * into a CUDA graph on its second use, replayed after (ouranos_batch_set_graphs
 * switches that off).  Pointers may be host or device; calls return after the
 * result is written.  One batch is not thread-safe, like a single handle. */
typedef struct ouranos_batch ouranos_batch;
int ouranos_batch_create(const ouranos_problem_desc* descs, int count, int device, ouranos_batch** out);
int ouranos_batch_destroy(ouranos_batch* b);
/* count, total vector length and offsets[count + 1] (each may be NULL) */
int ouranos_batch_layout(const ouranos_batch* b, int* count, long* total_length, long* offsets);
/* y = x - D L^-1 M2D S x for every problem, sweeps in `precision` */
int ouranos_batch_apply(ouranos_batch* b, int precision, const double* x, double* y);
/* rhs = D L^-1 (q + inflow) for every problem (FP64) */
int ouranos_batch_rhs(ouranos_batch* b, double* rhs);
/* restarted GMRES on every problem at once: inner = OURANOS_FP32 (FP32 Arnoldi
 * sweeps, FP64 restarts) or OURANOS_FP64; info[count]; NOT_CONVERGED if any
 * problem missed tol within max_it */
int ouranos_batch_solve(ouranos_batch* b, int inner, int restart, int max_it, double tol, double* x,
                        ouranos_solve_info* info);
/* time the warp tilings of each problem's sweep in `precision` (reps timed
 * runs each), keep the fastest; tiling (may be NULL) gets count x 3 ints */
int ouranos_batch_autotune(ouranos_batch* b, int precision, int reps, int* tiling);
int ouranos_batch_set_graphs(ouranos_batch* b, int enable);
/* diffusion synthetic acceleration on every problem (ouranos_rt_set_dsa);
 * ouranos_batch_solve uses it when OURANOS_SOLVER_DSA is OR'ed into `inner`
 * (FGMRES with each problem's diffusion correction as right preconditioner) */
int ouranos_batch_set_dsa(ouranos_batch* b, int cg_iterations);
/* z = P x for every member (concatenated layout, host or device pointers):
 * each member's diffusion correction, all members' CG solves in one
 * cooperative launch (the form OURANOS_SOLVER_DSA batch solves use). */
int ouranos_batch_dsa_apply(ouranos_batch* b, const double* x, double* z);
/* device time of the last batched sweep launches, graph launches so far */
int ouranos_batch_stats(const ouranos_batch* b, double* last_sweep_ms, int* graph_launches);
int ouranos_batch_last_error(const ouranos_batch* b, char* buf, size_t len);

/* ------------------------------------------------- learned preconditioner
 * No counterpart in the reference (its Krylov solves use an identity
 * preconditioner, src/ouranos.cc:160-171).  A 3-D convolutional network on the
 * cell grid of a 3-D DG Q1 mesh maps (the residual's normalised scalar-flux
 * nodal values, 8 per cell; log sigma_t / log 100; scattering ratio) to a
 * nodal scalar-flux correction -- a learned synthetic acceleration used as the
 * right preconditioner of FGMRES.  Grid sides must be multiples of 4. */
#define OURANOS_CNN_FEATURES 10 /* input channels per cell */
#define OURANOS_CNN_OUTPUTS 8   /* output channels per cell (Q1 nodes) */
typedef struct ouranos_cnn ouranos_cnn;
int ouranos_cnn_create(int nx, int ny, int nz, unsigned long long seed, ouranos_cnn** out);
int ouranos_cnn_destroy(ouranos_cnn* net);
int ouranos_cnn_n_params(const ouranos_cnn* net, long* n);
int ouranos_cnn_get_params(const ouranos_cnn* net, float* host);
int ouranos_cnn_set_params(ouranos_cnn* net, const float* host);
/* features: device [cells][OURANOS_CNN_FEATURES] FP32; out: device
 * [cells][OURANOS_CNN_OUTPUTS] FP32 */
int ouranos_cnn_forward(ouranos_cnn* net, const float* features, float* out);
/* MSE loss of forward(features) against target ([cells][OURANOS_CNN_OUTPUTS],
 * device), averaged over all entries; gradients of
 * all parameters to grads_host (may be NULL), no update */
int ouranos_cnn_gradients(ouranos_cnn* net, const float* features, const float* target,
                          float* grads_host, float* loss);
/* one Adam step (beta 0.9/0.999) on that loss */
int ouranos_cnn_train_step(ouranos_cnn* net, const float* features, const float* target, float lr,
                           float* loss);
int ouranos_cnn_last_error(const ouranos_cnn* net, char* buf, size_t len);
/* install (or, with NULL, remove) the network as the handle's preconditioner;
 * UNSUPPORTED unless the mesh is 3-D DG Q1, BAD_INPUT if the grids differ.
 * The learned applications run the network's forward in the order of the
 * handle's stream (a CUDA graph from the second call on), and a timeout of
 * one of its convolutions is reported by the handle's next synchronising
 * call, or by this call when it replaces or removes that network (TIMEOUT,
 * after the change).  The network must stay alive while it is installed. */
int ouranos_rt_set_preconditioner(ouranos_rt* rt, ouranos_cnn* net);
/* network features of a residual v ([mom][dof], device FP64) into features
 * (device [cells][OURANOS_CNN_FEATURES]); scale (host, may be NULL) gets the
 * normalisation s = RMS of v's scalar-moment values */
int ouranos_rt_pc_features(ouranos_rt* rt, const double* v, float* features, double* scale);
/* training target for the pair (v, e = A^-1 v): the scalar-moment nodal
 * values of (e - v) / (s g_c), g_c = 1/(1 - sigma_s0/sigma_t) of the cell
 * (device [cells][OURANOS_CNN_OUTPUTS]) */
int ouranos_rt_pc_target(ouranos_rt* rt, const double* v, const double* e, float* target);
/* z = v + s g_c y, y the network output on v's features (device vectors) */
int ouranos_rt_pc_apply(ouranos_rt* rt, const double* v, double* z);
/* z = P v of the diffusion acceleration (ouranos_rt_set_dsa) with its CG
 * started from the network's prediction of the correction f (vertex values
 * s K y averaged over the cells at each vertex, scaled to their
 * energy-norm-optimal multiple) instead of from zero (device vectors).  The
 * CG converges to the same f from any start: the network saves CG steps, it
 * cannot change what they converge to. */
int ouranos_rt_pc_dsa_apply(ouranos_rt* rt, const double* v, double* z);

/* ------------------------------------- diffusion synthetic acceleration
 * No counterpart in the reference (identity preconditioner, plain source
 * iteration: src/ouranos.cc:72-95,160-171).  For a DG Q_p mesh (2-D or 3-D):
 *   P v = v + f,  (-div D grad + sigma_a) f = sigma_s0 v_0,
 * f continuous Q1 on the mesh vertices (Marshak condition on vacuum and inflow
 * boundaries, zero current on reflective ones), D = 1/(3(sigma_t' - sigma_s1)),
 * sigma_a = sigma_t' - sigma_s0, sigma_t' = sigma_t + 1/(v dt); v_0 enters
 * through the mixed mass matrix of the vertex hat functions and the Q_p basis,
 * and f, interpolated at the Q_p nodes, is added to the scalar moment's nodal
 * values.  The diffusion system is solved by cg_iterations steps of
 * Jacobi-preconditioned CG (FP32, FP64 scalars); 0 switches the acceleration
 * off. */
int ouranos_rt_set_dsa(ouranos_rt* rt, int cg_iterations);
/* z = P v ([mom][dof], host or device; z may equal v) */
int ouranos_rt_dsa_apply(ouranos_rt* rt, const double* v, double* z);

#ifdef __cplusplus
}
#endif
#endif
