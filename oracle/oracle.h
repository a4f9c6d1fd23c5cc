/*
 * ORACLE -- test infrastructure only.
 *
 * A CPU restatement, in plain FP64 C++, of the Ouranos transport-sweep hot
 * path (Rombur/ouranos).  It exists to check the GB300 product against the
 * reference's algorithm; nothing in the product links, loads or calls it.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm use it.
 *
 * Parity anchoring: the reference cannot be compiled in this environment
 * (deal.II, Trilinos, p4est, boost and MPI are absent).  The restatement is
 * pinned instead against the reference's own test fixtures, extracted as
 * text into tests/golden/ by tests/golden/make_golden.py:
 *   - the 64-value golden scalar flux of tests/RadiativeTransfer_test.cc:84-152
 *   - every FE matrix entry of tests/FECell_test.cc:23-297
 *   - the quadrature facts of tests/RTQuadrature_test.cc:21-165
 *   - the LS / GLC tables of src/LS.cc:14-665 and src/GLC.cc:60-1285
 * Results on configurations those fixtures do not cover (Q2+, anisotropic
 * scattering, 3-D) are pinned only by this restatement plus analytic checks.
 */
#ifndef OURANOS_ORACLE_H
#define OURANOS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Boundary condition kinds, src/Parameters.hh:21 (VACUUM, MOST_NORMAL,
 * ISOTROPIC, REFLECTIVE -- reflective is parsed but never applied by the
 * reference, src/RadiativeTransfer.cc:958-975, so it behaves as vacuum). */
enum { ORC_BC_VACUUM = 0, ORC_BC_ISOTROPIC = 1, ORC_BC_MOST_NORMAL = 2, ORC_BC_REFLECTIVE = 3 };

/* Quadrature families, src/LS.hh and src/GLC.hh. */
enum { ORC_QUAD_LS = 0, ORC_QUAD_GLC = 1 };

/* Harmonics convention for M2D.
 * ORC_HARM_ORTHONORMAL: real spherical harmonics, polar angle arccos(Omega_z),
 *   sqrt(2) on m>0 so the set is orthonormal on the sphere (the default; this
 *   is what the reference's comment at src/RTQuadrature.cc:122-125 intends).
 * ORC_HARM_REFERENCE: the reference's literal evaluation,
 *   boost::math::spherical_harmonic_r/i(l, m, Omega_z, phi) -- the polar angle
 *   argument receives Omega_z itself (src/RTQuadrature.cc:126-131) and no
 *   sqrt(2) factor is applied. */
enum { ORC_HARM_ORTHONORMAL = 0, ORC_HARM_REFERENCE = 1 };

typedef struct {
  int dim;              /* 2 or 3 */
  int fe_order;         /* 1..5 */
  int n_cells[3];       /* cells per axis; cell index i + nx*(j + ny*k) */
  double lower[3];      /* domain box */
  double upper[3];
  int n_groups;
  int group;            /* current group, RadiativeTransfer::set_group */
  /* quadrature, as RTQuadrature exposes it */
  int n_dir;
  int n_mom;
  const double* omega;      /* [n_dir][3] */
  const double* m2d;        /* [n_dir][n_mom] */
  const double* d2m;        /* [n_mom][n_dir] */
  const int* moment_l;      /* [n_mom]   RTQuadrature::get_l */
  const int* most_normal;   /* [2*dim][n_dir] flags, may be NULL */
  double weight_sum;
  /* materials, RTMaterialProperties layout (src/RTMaterialProperties.hh:84-101) */
  int n_materials;
  int l_max;
  const double* sigma_t;    /* [mat][g] */
  const double* sigma_s;    /* [mat][g_from][g_to][l] */
  const int* material_id;   /* per cell */
  const int* source_id;     /* per cell, may be NULL (all 0) */
  int n_sources;
  const double* source;     /* [src][g], may be NULL */
  int bc_type[6];
  const double* inc_flux;   /* [face][g], may be NULL */
} orc_desc;

typedef struct orc_problem orc_problem;

/* Build the FE tables (RadiativeTransfer::setup, src/RadiativeTransfer.cc:50-78);
 * the task graph is built on its first use. Returns NULL on bad input. */
orc_problem* orc_create(const orc_desc* desc);
void orc_destroy(orc_problem* p);
void orc_set_group(orc_problem* p, int g);
/* The scheduler orc_apply, orc_solve and orc_advance_angular sweep with
 * (orc_sweep's argument; 0 by default). */
void orc_set_scheduler(orc_problem* p, int scheduler);
/* implicit Euler in time (an extension, not in the reference operator) */
void orc_set_time_step(orc_problem* p, double inv_vdt);
void orc_set_source(orc_problem* p, const double* source);   /* [n_sources][n_groups] */
void orc_advance_angular(orc_problem* p, const double* phi, int n_threads);
void orc_get_angular(const orc_problem* p, double* psi);     /* [dir][dof] */
void orc_set_angular(orc_problem* p, const double* psi);

long orc_n_dofs(const orc_problem* p);      /* cells * dofs per cell */
long orc_n_tasks(const orc_problem* p);     /* cells * directions */

/* compute_scattering_source, src/RadiativeTransfer.cc:811-843, with sigma_s
 * indexed by Legendre order l(m) (the reference indexes by moment number). */
void orc_scattering_source(orc_problem* p, const double* x);
/* Zero the scattering source (the state before any Apply). */
void orc_clear_scattering_source(orc_problem* p);

/* One full sweep: flux_moments += D L^-1 (M2D S [+ q + outer + inflow]).
 * group_flux != NULL selects the right-hand-side form (src/RadiativeTransfer.cc:914-925,
 * 958-975): [g][mom][dof].  scheduler: 0 = linear ready counters,
 * 1 = the reference's all-task scan (O(T^2)), 2 = no task graph: each
 * direction's cells in lexicographic upwind-first order (the same task
 * values, another order of the additions into the moments; for meshes whose
 * graph would not fit in memory).  n_threads > 1 splits the
 * directions over std::threads (each thread owns its directions' tasks). */
void orc_sweep(orc_problem* p, double* flux_moments, const double* group_flux,
               int scheduler, int n_threads);

/* Epetra_Operator::Apply, src/RadiativeTransfer.cc:780-809: y = x - D L^-1 M2D S x. */
void orc_apply(orc_problem* p, const double* x, double* y, int n_threads);

/* Order in which tasks ran in the last single-threaded sweep: [n_tasks] of
 * (dir * n_cells + cell). */
void orc_last_order(const orc_problem* p, long* order);
/* Longest-path depth of every task in the reference task DAG
 * (compute_sweep_ordering + build_*_tasks_maps): [dir][cell]. */
void orc_task_levels(orc_problem* p, int* levels);
/* Task ids as the reference assigns them (direction-major, breadth-first
 * from the upwind boundary): [dir][cell] -> id. */
void orc_task_ids(orc_problem* p, long* ids);

/* FE matrices of one cell (FECell, src/FECell.cc:10-78): mass [n][n],
 * grad [dim][n][n], downwind [2dim][n][n], upwind [2dim][n][n], normals [2dim][3]. */
void orc_fecell(const orc_problem* p, long cell, double* mass, double* grad,
                double* downwind, double* upwind, double* normals);

/* Krylov / SI drivers on the oracle operator (src/ouranos.cc:43-209).
 * rhs = RHS sweep; x0 = 0.  Return iterations, residual history in hist
 * (may be NULL, length >= max_it+1). kind: 0 SI, 1 GMRES(restart), 2 BiCGSTAB. */
int orc_solve(orc_problem* p, int kind, int restart, int max_it, double tol,
              const double* group_flux, double* x, double* hist, int n_threads);

/* Quadrature builder (RTQuadrature::build_quadrature, src/RTQuadrature.cc:27-56).
 * table_a/table_b: LS -> direction cosines [sn/2] and per-point octant weights
 * [sn(sn+2)/8]; GLC -> Gauss-Legendre nodes [sn/2] and weights [sn/2].
 * Outputs sized by orc_quadrature_sizes. Returns 0 on success. */
int orc_quadrature_sizes(int sn, int l_max, int galerkin, int dim, int* n_dir, int* n_mom);
int orc_quadrature_build(int type, int sn, int l_max, int galerkin, double weight_sum,
                         int dim, int harmonics, const double* table_a,
                         const double* table_b, double* omega, double* weight,
                         double* m2d, double* d2m, int* moment_l, int* most_normal);

#ifdef __cplusplus
}
#endif
#endif
