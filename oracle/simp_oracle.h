/* CPU oracle of the SIMP inner loop: a restatement of SparLab's algorithms in
 * plain C++ (no Eigen).  TEST INFRASTRUCTURE ONLY: tests, the smoke check and
 * the bench's CPU baseline use it as the checker; the product library never
 * links or calls it.
 *
 * Pinning: the restatement is checked against the reference's published
 * known-answer compliances (docs/results/solver_scaling.csv of the reference,
 * sparlab_bench model) and the identities its own tests assert
 * (tests/test_multigrid.cpp, tests/test_topopt.cpp).  Eigen's pivoted QR and
 * LDLT are re-derived from their published algorithms, so the tentative
 * prolongator's basis (signs, pivot order) is pinned only through identities. */
#ifndef SIMP_ORACLE_H
#define SIMP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  double strength_threshold;     /* 0.02 */
  int32_t max_levels;            /* 12 */
  int32_t coarse_size;           /* 1500 */
  int32_t smoother_degree;       /* 3 */
  double chebyshev_ratio;        /* 30 */
  double prolongator_damping;    /* 4/3 */
  int32_t lanczos_steps;         /* 12 */
  double coarse_pivot_tolerance; /* 1e-13 */
  int32_t reuse_aggregates;      /* 1 */
} orc_amg_options;

typedef struct {
  int32_t dim;                 /* 2 (Q4) or 3 (Hex8) */
  int32_t nx, ny, nz;          /* elements per axis (nz ignored in 2-D) */
  double lx, ly, lz;           /* extents; the grid starts at the origin */
  double young, poisson;       /* isotropic material */
  double thickness;            /* plane-stress thickness (2-D); 1 in 3-D */
  const uint8_t* fixed;        /* per DOF (node * dim + k): 1 = clamped */
  int32_t num_loads;           /* load cases */
  const double* loads;         /* num_loads x num_dofs, full-length vectors */
  const double* weights;       /* num_loads raw weights (normalised inside) */
  double filter_radius;        /* physical radius; <= 0 disables the filter */
  double volume_fraction;
  double initial_density;      /* < 0: use the volume fraction */
  double penalty, emin_ratio;  /* SIMP law */
  double move_limit, damping;  /* OC */
  double rtol;                 /* PCG relative tolerance */
  int32_t max_cg_iterations;   /* 0 -> 1000 */
  int32_t warm_start;
  orc_amg_options amg;
  /* Heaviside projection with beta continuation (ProjectionOptions,
   * include/sparlab/topopt/Projection.hpp:69-96); projection = 0 disables */
  int32_t projection;
  double eta, beta_start, beta_max, beta_factor;
  int32_t beta_interval, advance_on_convergence;
  double change_tolerance;     /* run_oc's design-change tolerance (beta advance) */
  /* Robust formulation (Projection.hpp:44-60): objective on the eroded design
   * (eta + delta), volume on the dilated one (eta - delta) against a target
   * rescaled every robust_volume_interval iterations to V* V_d / V_i. */
  int32_t robust;
  double robust_delta;
  int32_t robust_volume_interval;
} orc_problem_desc;

typedef struct orc_problem orc_problem;
typedef struct orc_solver orc_solver;

void orc_default_amg_options(orc_amg_options* o);
const char* orc_last_error(void);

/* Element stiffness of one box cell, 2 x 2 (x 2) Gauss, symmetrised. */
int orc_element_stiffness(int dim, double hx, double hy, double hz, double young,
                          double poisson, double thickness, double* ke);

/* Consistent mass of one box cell, 3 x 3 (x 3) Gauss, symmetrised. */
int orc_element_mass(int dim, double hx, double hy, double hz, double density,
                     double thickness, double* me);

/* ---- AMG-PCG on a caller's matrix (the LinearSolver boundary) ---- */
int orc_solver_create(const orc_amg_options* o, double rtol, int32_t max_iterations,
                      orc_solver** out);
void orc_solver_destroy(orc_solver* s);
int orc_solver_factorize(orc_solver* s, int32_t n, const int32_t* rowptr,
                         const int32_t* col, const double* val, int dim, int ndpn,
                         const double* coords, int32_t num_nodes, const int32_t* unknowns);
int orc_solver_solve(orc_solver* s, const double* b, const double* x0, double* x,
                     int32_t* iterations, double* relres);
int orc_solver_apply(orc_solver* s, const double* r, double* z);
int orc_solver_num_levels(orc_solver* s);
/* level l: rows, nnz, aggregates (nodes of l+1), lambda_max */
int orc_solver_level_info(orc_solver* s, int level, int64_t* info, double* lambda_max);
int orc_solver_level_matrix(orc_solver* s, int level, int32_t* rowptr, int32_t* col,
                            double* val);
int orc_solver_prolongator(orc_solver* s, int level, int tentative, int32_t* rowptr,
                           int32_t* col, double* val);
int orc_solver_prolongator_nnz(orc_solver* s, int level, int tentative, int64_t* nnz);
int orc_solver_aggregates(orc_solver* s, int level, int32_t* agg);
int orc_solver_num_nodes(orc_solver* s, int level, int32_t* num_nodes);
int orc_solver_nullspace(orc_solver* s, int level, int32_t* cols, double* b);
int orc_solver_stats(orc_solver* s, double* operator_complexity, double* coarse_pivot_ratio,
                     int32_t* reused);

/* Free-free stiffness of a structured problem for given element factors. */
int orc_problem_create(const orc_problem_desc* d, orc_problem** out);
void orc_problem_destroy(orc_problem* p);
int orc_problem_sizes(orc_problem* p, int64_t* sizes); /* ne, nn, ndof, nfree, nnz_ff */
int orc_problem_free_dofs(orc_problem* p, int32_t* free_dofs);
int orc_problem_coords(orc_problem* p, double* coords);
int orc_problem_kff(orc_problem* p, const double* scale, int32_t* rowptr, int32_t* col,
                    double* val);
int orc_problem_element_matrix(orc_problem* p, double* ke);
/* Free-free values (K_ff's pattern) of sum_e s_e E for a caller's element
 * matrix E (the mass matrix with M_e^0), and the sum of the full matrix. */
int orc_problem_assemble(orc_problem* p, const double* elem, const double* scale, double* val,
                         double* full_sum);
int orc_filter_forward(orc_problem* p, const double* x, double* y);
int orc_filter_adjoint(orc_problem* p, const double* v, double* g);
int orc_filter_row_sums(orc_problem* p, double* sums);

/* ComplianceObjective::evaluate with gradients.  out: compliance, volume,
 * volume fraction, linear iterations (as double).  Arrays may be NULL. */
int orc_evaluate(orc_problem* p, const double* x, double* out, double* rho_phys,
                 double* dc_dphys, double* dc_dx, double* dv_dx, double* strain_energy,
                 double* displacements /* num_loads x ndof */);
/* optimality_criteria_update: out = lambda, achieved volume, max change,
 * bisections, volume converged */
int orc_oc_update(orc_problem* p, const double* x, const double* dc_dx,
                  const double* dv_dx, double* xnew, double* out);
/* run_oc for `iterations` iterations (no early stop when change_tol <= 0;
 * with projection only the final beta stage may stop); history: per
 * iteration compliance, volume fraction, max change, lambda, linear
 * iterations, bisections, beta (0 without projection). */
int orc_run(orc_problem* p, int32_t iterations, double change_tol, double* x,
            double* history, int32_t* performed);
/* run_mma for `iterations` iterations (MMA with the volume constraint); history:
 * compliance, volume fraction, max change, lambda, linear iterations,
 * subproblem Newton iterations. */
int orc_run_mma(orc_problem* p, int32_t iterations, double* x, double* history,
                int32_t* performed);

/* MmaOptimizer(n, 1, 0, 1) on its own: n variables in [0, 1], one
 * constraint row.  Each update takes x, df0/dx, the constraint value and its
 * gradient row; out: lambda, y, z, max change, constraint row scale,
 * subproblem Newton iterations, MMA iteration count. */
typedef struct orc_mma orc_mma;
int orc_mma_create(int32_t n, orc_mma** out);
int orc_mma_update(orc_mma* h, const double* x, const double* df0, double fval, const double* dfdx,
                   double* x_out, double* out);
void orc_mma_destroy(orc_mma* h);

#ifdef __cplusplus
}
#endif
#endif
