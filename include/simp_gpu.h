/* simp_gpu.h - C ABI of the GB300 SIMP inner loop (libsimp_gb300.so).
 *
 * Two drop-in boundaries of SparLab:
 *
 *  1. The linear solver (sparlab::LinearSolver, include/sparlab/fem/
 *     LinearSolver.hpp:64-109 of the reference): set_layout, factorize (AMG
 *     setup, with aggregate reuse when the structure is unchanged, as
 *     src/fem/Multigrid.cpp:959-966) and solve/solve_from (PCG per load case).
 *     A caller that cannot change is served through this boundary alone.
 *
 *  2. The whole SIMP iteration (sparlab::ComplianceObjective::evaluate,
 *     include/sparlab/topopt/Sensitivity.hpp:66-107, plus
 *     optimality_criteria_update, include/sparlab/topopt/
 *     OptimalityCriteria.hpp:45-77, driven as TopologyOptimizer::run_oc,
 *     src/topopt/TopologyOptimizer.cpp:556-724): everything stays resident in
 *     device memory between calls.
 *
 * Conventions: plain C types, host pointers unless named *_device, column
 * indices int32, values FP64.  Every call returns a status code; on failure
 * simp_last_error() holds a message worded as the reference's exceptions
 * ("under-constrained", "did not converge", "not symmetric", ...).  A context
 * is not thread-safe: use one per host thread.
 */
#ifndef SIMP_GPU_H
#define SIMP_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  SIMP_BAD_INPUT / SIMP_BREAKDOWN / SIMP_UNDERCONSTRAINED /
 * SIMP_NONFINITE map to sparlab::SolverError, SIMP_MAXITER to
 * sparlab::ConvergenceError (src/fem/LinearSolver.cpp:268-280). */
#define SIMP_OK 0
#define SIMP_BAD_INPUT 1
#define SIMP_BREAKDOWN 2
#define SIMP_UNDERCONSTRAINED 3
#define SIMP_MAXITER 4
#define SIMP_NONFINITE 5
#define SIMP_CUDA_ERROR 6

/* FP64: every operator, vector and scalar in FP64.  MIXED: the V-cycle and
 * the reuse setups in FP32 (level 0 matrix-free on structured grids), the CG
 * operator in double-float arithmetic (K_ff as float pairs, ~2^-44 relative
 * to FP64); CG vectors and scalars, the true-residual restarts and the
 * coarsest dense inverse are FP64 in both. */
#define SIMP_PRECISION_FP64 0
#define SIMP_PRECISION_MIXED 1

/* Options: AmgOptions (include/sparlab/fem/Multigrid.hpp:75-103) plus the
 * iterative part of LinearSolverOptions (LinearSolver.hpp:36-61). */
typedef struct {
  double strength_threshold;     /* theta, 0.02 */
  int32_t max_levels;            /* 12 */
  int32_t coarse_size;           /* 1500 */
  int32_t smoother_degree;       /* Chebyshev degree, 3 */
  double chebyshev_ratio;        /* 30 */
  double prolongator_damping;    /* omega * lambda_max, 4/3 */
  int32_t lanczos_steps;         /* 12 */
  double coarse_pivot_tolerance; /* 1e-13 */
  int32_t reuse_aggregates;      /* 1 */
  double iterative_tolerance;    /* relative residual, 1e-12 */
  int32_t max_iterations;        /* 0 -> 1000 */
  int32_t precision;             /* SIMP_PRECISION_* */
  int32_t device;                /* CUDA device ordinal */
  int32_t cuda_graphs;           /* 1: each PCG iteration after the first is one CUDA graph
                                    launch (captured per workspace after every setup);
                                    0: the same kernels launched one by one */
  int32_t matrix_free_transfer;  /* MIXED on a 3-D structured grid: 1 applies level 0's
                                    restriction and prolongation in the V-cycle as
                                    P^T (I - w A D^-1) and (I - w D^-1 A) P^ with the
                                    matrix-free operator instead of reading the stored
                                    R and P; 0 reads them */
  int32_t matrix_free;           /* MIXED on a structured grid whose nodes are fully free
                                    or clamped: 0 level 0 assembled throughout (the FP32
                                    V-cycle on the assembled FP32 K_ff, the CG operator
                                    on its double-float values); 1 (default) level 0 of
                                    the FP32 V-cycle matrix-free (element-by-element
                                    from K_e^0 and the cell scales), the CG operator
                                    assembled double-float; 2 (3-D) also the CG operator
                                    matrix-free: FP32 element products inside CG, with
                                    the true residual of every restart taken by an FP64
                                    matrix-free product (iterative refinement) */
  int32_t tensor_cores;          /* 3-D matrix-free level 0 (matrix_free >= 1): 1 (default)
                                    the element products K_e^0 x_e of a layer of cells as
                                    TF32 tensor-core GEMMs, operands split hi + lo (3 x TF32,
                                    FP32 accumulation: about FP32 accuracy); 0 FP32 FMAs on
                                    the CUDA cores */
} simp_solver_options;

typedef struct {
  int32_t num_levels;
  int32_t reused_aggregates;
  double operator_complexity;
  double grid_complexity;
  double coarse_pivot_ratio;
  double setup_seconds;
  int64_t storage_nonzeros;
  int64_t level_rows[16];
  int64_t level_nnz[16];
  int64_t level_aggregates[16];
  double level_lambda[16];
} simp_amg_stats;

typedef struct simp_ctx simp_ctx;

void simp_default_options(simp_solver_options* opts);

/* ---- Boundary 1: LinearSolver ------------------------------------------ */
/* make_linear_solver(options) with type "gpu_amg_cg"
 * (src/fem/LinearSolver.cpp:424-443). */
int simp_ctx_create(const simp_solver_options* opts, simp_ctx** out);
void simp_ctx_destroy(simp_ctx* ctx);
/* Message of the last failed call on this context (thread-local when ctx is
 * NULL, for failures of create). */
const char* simp_last_error(const simp_ctx* ctx);

/* LinearSolver::set_layout(DofLayout) (LinearSolver.hpp:87, Multigrid.hpp:
 * 107-117): coordinates are dim x num_nodes (node-major), unknowns[i] is the
 * global DOF node * ndpn + k of unknown i, ascending.  Copied. */
int simp_set_layout(simp_ctx* ctx, int32_t dim, int32_t ndpn, const double* coords,
                    int32_t num_nodes, const int32_t* unknowns, int32_t n);

/* LinearSolver::factorize(const SparseMatrix&) (LinearSolver.hpp:71): the
 * symmetric K_ff as CSR (the reference's column-major storage read as rows).
 * Pattern and values are copied to the device; the aggregates of the last
 * setup are reused when n, nnz and the layout are unchanged. */
int simp_factorize(simp_ctx* ctx, int32_t n, const int32_t* rowptr, const int32_t* colidx,
                   const double* values);

/* The same factorization in steps: the pattern once (copied; n, nnz and the
 * layout are the reuse fingerprint, Multigrid.cpp:959-966), then per
 * iteration the values -- host FP64, or a device pointer of nnz FP64 values
 * that a GPU assembler wrote (read by simp_setup, after the caller's work on
 * the legacy default stream) -- and simp_setup. */
int simp_set_pattern(simp_ctx* ctx, int32_t n, const int32_t* rowptr, const int32_t* colidx);
int simp_set_values(simp_ctx* ctx, const double* values);
int simp_set_values_device(simp_ctx* ctx, const double* values_device);
int simp_setup(simp_ctx* ctx);

/* LinearSolver::solve / solve_from (LinearSolver.hpp:74-82) for nrhs
 * right-hand sides stored one after another (n doubles each).  X0 may be NULL
 * (zero guess).  iterations[k] and relres[k] (true relative residual) are
 * written per right-hand side when non-NULL. */
int simp_solve(simp_ctx* ctx, int32_t nrhs, const double* B, const double* X0, double* X,
               int32_t* iterations, double* relres);

/* AmgPreconditioner::apply (Multigrid.hpp:162): z = M^-1 r, one V-cycle. */
int simp_apply_preconditioner(simp_ctx* ctx, const double* r, double* z);

/* LinearSolver::amg_stats / last_iterations / storage_nonzeros. */
int simp_stats(simp_ctx* ctx, simp_amg_stats* stats);

/* Test access to the hierarchy (AmgPreconditioner, Multigrid.hpp:168-178):
 * node-to-aggregate map of level `level` (count = number of nodes), the level
 * operator A_l as CSR (call with NULL arrays for the sizes). */
int simp_level_aggregates(simp_ctx* ctx, int32_t level, int32_t* agg, int32_t* count);
int simp_level_matrix(simp_ctx* ctx, int32_t level, int32_t* rows, int64_t* nnz,
                      int32_t* rowptr, int32_t* colidx, double* values);
int simp_level_prolongator(simp_ctx* ctx, int32_t level, int32_t* rows, int32_t* cols,
                           int64_t* nnz, int32_t* rowptr, int32_t* colidx, double* values);

/* ---- Boundary 2: the whole SIMP iteration ------------------------------ */
typedef struct simp_problem simp_problem;

/* A structured Q4 / Hex8 problem: what FemModel, Assembler, DensityFilter,
 * DesignDomain and the SIMP/OC options of the reference hold for it. */
typedef struct {
  int32_t dim;                  /* 2 (Q4 plane stress) or 3 (Hex8) */
  int32_t nx, ny, nz;           /* cells per axis */
  double lx, ly, lz;            /* extents, grid at the origin */
  double thickness;             /* plane-stress thickness (2-D volumes); 1 in 3-D */
  const double* element_matrix; /* K_e^0 (8x8 or 24x24, row-major), from the
                                   caller's element (Assembler::element_stiffness) */
  const uint8_t* fixed;         /* per DOF: 1 = clamped (homogeneous) */
  int32_t num_loads;
  const double* loads;          /* num_loads x num_dofs */
  const double* weights;        /* raw load-case weights (normalised here) */
  double filter_radius;         /* physical; <= 0: no filter */
  double volume_fraction;
  double initial_density;       /* < 0: the volume fraction */
  double penalty, emin_ratio;   /* SimpOptions: penalty >= 1, emin_ratio in (0, 1) */
  double move_limit, damping;   /* OptimalityCriteriaOptions */
  int32_t warm_start;           /* 0: zero guess; 1: previous displacement
                                   (LinearSolverOptions::warm_start); 2: energy-
                                   optimal combination of the last 3 displacements;
                                   3: the same with the displacement surrogate's
                                   prediction as one more vector (first solve: the
                                   prediction's optimal multiple); needs
                                   simp_problem_set_surrogate, else as 2 */
  int32_t block_pcg;            /* several load cases: 0 solved one after another; 1 at the
                                   same time, each on its own workspace and stream from its
                                   own host thread; 2 advanced together, one CUDA graph
                                   launch running one PCG iteration of every load case
                                   still iterating (a conditional node per load case);
                                   all three compute the same values */
  int32_t optimizer;            /* simp_iterate's update: 0 OC, 1 MMA */
  /* Heaviside projection of the filtered density with beta continuation
   * (ProjectionOptions, include/sparlab/topopt/Projection.hpp:69-96,
   * BetaSchedule, src/topopt/TopologyOptimizer.cpp:17-46); 0 disables */
  int32_t projection;
  double eta, beta_start, beta_max, beta_factor;
  int32_t beta_interval, advance_on_convergence;
  double change_tolerance;      /* design-change tolerance of the beta advance */
  /* Robust formulation (Projection.hpp:44-60, run_oc at
   * src/topopt/TopologyOptimizer.cpp:567-651): the objective on the eroded
   * design (eta + robust_delta), the OC volume constraint on the dilated one
   * (eta - robust_delta) against a target moved to V* V_d / V_i every
   * robust_volume_interval iterations; needs the projection and OC. */
  int32_t robust;
  double robust_delta;
  int32_t robust_volume_interval;
  /* displacements of the history that warm starts 2 and 3 combine (1..3;
   * 0 takes 3); warm start 3 adds the surrogate's prediction to them */
  int32_t warm_history;
} simp_problem_desc;

/* ObjectiveEvaluation scalars (Sensitivity.hpp:66-107) and an OC step
 * (OptimalityCriteria.hpp:53-60). */
typedef struct {
  double compliance;
  double volume;
  double volume_fraction;
  int32_t linear_iterations;
  double relres_max;
} simp_evaluation;

typedef struct {
  double lambda;
  double achieved_volume;
  double max_change;
  int32_t bisections;
  int32_t volume_converged;
} simp_oc_step;

/* One history row (TopologyIteration, include/sparlab/topopt/
 * TopologyOptimizer.hpp): volume_converged is the OC step's bisection
 * convergence, or for MMA V/V* - 1 <= 1e-4 (the default constraint_tolerance). */
typedef struct {
  double compliance, volume_fraction, max_change, lambda, gray_level;
  int32_t linear_iterations, bisections;
  double seconds;
  int32_t volume_converged;
  int32_t final_stage;          /* 1: no projection, or its last beta stage (convergence may stop) */
  double beta;                  /* projection sharpness of the iteration (0: none) */
  /* robust runs: volume_fraction is the blueprint's; these are the eroded and
   * dilated designs' fractions and the dilated target's (0 otherwise) */
  double eroded_volume_fraction, dilated_volume_fraction, dilated_target_fraction;
} simp_iteration_record;

int simp_problem_create(const simp_problem_desc* desc, const simp_solver_options* opts,
                        simp_problem** out);
void simp_problem_destroy(simp_problem* p);
const char* simp_problem_last_error(const simp_problem* p);
/* ne, nn, ndof, nfree, nnz(K_ff) */
int simp_problem_sizes(simp_problem* p, int64_t* sizes);

/* Design vector on the device (host in / out). */
int simp_set_design(simp_problem* p, const double* x);
int simp_get_design(simp_problem* p, double* x);

/* ComplianceObjective::evaluate(x, true) at the resident design.  Output
 * arrays (host, may be NULL): physical density, dc/drho, dc/dx, dv/dx,
 * element strain energy (ne each), displacements (num_loads x ndof). */
int simp_evaluate(simp_problem* p, simp_evaluation* out, double* rho, double* dc_dphys,
                  double* dc_dx, double* dv_dx, double* strain_energy, double* displacements);

/* optimality_criteria_update with the resident gradients of the last
 * evaluate; the new design replaces the resident one when `apply` != 0. */
int simp_oc_update(simp_problem* p, int32_t apply, simp_oc_step* out, double* xnew);

/* MmaOptimizer::update (src/topopt/Mma.cpp:63-157) as run_mma drives it
 * (src/topopt/TopologyOptimizer.cpp:831-905): objective c / c_1, one
 * constraint V / V* - 1, with the resident gradients of the last evaluate.
 * out->lambda is the volume multiplier, out->bisections the subproblem's
 * Newton iterations; achieved_volume is not computed (0). */
int simp_mma_update(simp_problem* p, int32_t apply, simp_oc_step* out, double* xnew);

/* One run_oc (or run_mma, per desc->optimizer) iteration: evaluate + update +
 * clamp, device-resident. */
int simp_iterate(simp_problem* p, simp_iteration_record* rec);

/* One SIMP iteration (simp_iterate) of each of n independent problems, their
 * linear solves advanced together: every problem's filter, assembly and
 * AMG setup (host threads, one stream per problem), then the PCG of every
 * load case of every problem in lock step -- one CUDA graph launch runs one
 * iteration of each solve still iterating, each under a conditional node set
 * by its own convergence test -- then every problem's sensitivities and
 * update.  Each problem computes what simp_iterate computes alone, bit for
 * bit.  records: n entries.  The first failing problem's status is returned
 * (its message in simp_problem_last_error); the others still iterate. */
int simp_iterate_batch(simp_problem* const* problems, int32_t n, simp_iteration_record* records);

/* AMG statistics of the problem's solver. */
int simp_problem_stats(simp_problem* p, simp_amg_stats* stats);

/* Density filter of the problem (DensityFilter::to_physical / pull_back). */
int simp_filter_forward(simp_problem* p, const double* x, double* y);
int simp_filter_adjoint(simp_problem* p, const double* v, double* g);

/* Assembled K_ff of the problem at element factors `scale` (host), copied
 * out as CSR (NULL arrays: sizes only).  Test access to the assembly. */
int simp_problem_kff(simp_problem* p, const double* scale, int32_t* rowptr,
                     int32_t* colidx, double* values);

/* Element stiffness of a box cell (Quad4Element/Hex8Element::stiffness,
 * src/elements/Quad4.cpp:117-137, src/elements/Hex8.cpp:172-192), for callers
 * without an element library. */
int simp_element_stiffness(int32_t dim, double hx, double hy, double hz, double young,
                           double poisson, double thickness, double* ke);

/* y = K_ff x with the problem's current level-0 operator (as assembled by
 * the last evaluate), on device pointers of nfree doubles, on the library's
 * stream.  Exposed so a caller can time the dominant kernel in isolation. */
int simp_problem_apply_operator(simp_problem* p, const double* x_device, double* y_device);

/* y = K_ff x through the V-cycle's level-0 operator (MIXED: FP32, x rounded
 * to FP32 and y widened; matrix-free where enabled, on the tensor cores with
 * tensor_cores = 1; FP64: the CG operator), on device pointers of nfree
 * doubles, on the library's stream.  For checking and timing that operator
 * in isolation (AmgPreconditioner's level-0 spmv, src/fem/Multigrid.cpp:
 * 783-855, is the product it replaces). */
int simp_problem_apply_level0(simp_problem* p, const double* x_device, double* y_device);

/* Times `reps` launches of the level-0 CG operator (FP64 values in FP64 mode,
 * double-float hi + lo values in mixed mode) with CUDA events on the library's
 * stream: average milliseconds per launch and its algorithmic bytes (8 per
 * value, the index data the kernel reads, x read and y written once). */
int simp_problem_time_operator(simp_problem* p, int32_t reps, double* ms_per_launch,
                               double* bytes_per_launch);

/* No counterpart in the reference.  rho = clamp(H x, 0, 1) -- Heaviside-
 * projected at the problem's current beta and the objective's threshold when
 * the projection is on -- and the volume sum_e v_e rho_e: the physical density
 * and volume simp_evaluate reports for design x, on device pointers (x and rho:
 * num_elements doubles, volume: one double), launched on the library's stream.
 * It allocates no device memory: its partial sums live in a fixed 128 KiB
 * device array of the library, so a caller that must not call cudaMalloc at
 * that point (an optimiser evaluating many trial designs per iteration
 * without device synchronisation, an application running under its own
 * memory pool) can use it.  At most 67,108,864 elements (SIMP_BAD_INPUT
 * beyond).  The first call on a device sets the array up and should come
 * before any stream capture; a cudaDeviceReset after it is not supported.
 * Calls that overlap on the GPU share the array and race. */
int simp_filter_volume_noalloc(simp_problem* p, const double* x_device, double* rho_device,
                               double* volume_device);

/* RobustRecord (include/sparlab/topopt/TopologyOptimizer.hpp:153-166): the
 * current design projected at eta + delta (eroded), eta (blueprint) and
 * eta - delta (dilated) with the current beta, each evaluated (one solve per
 * load case): what TopologyOptimizer::finish records for a robust run and for
 * the erosion check of a projected one (src/topopt/TopologyOptimizer.cpp:
 * 344-415).  delta <= 0 takes the problem's robust_delta.  The densities
 * (host, num_elements, NULL to skip) are the eroded and dilated designs'.
 * The evaluations replace the problem's gradients, so an OC / MMA half-step
 * needs a new simp_evaluate first (simp_iterate always makes one). */
typedef struct simp_robust_record {
  double eta_eroded, eta_intermediate, eta_dilated;
  double compliance_eroded, compliance_intermediate, compliance_dilated;
  double volume_fraction_eroded, volume_fraction_intermediate, volume_fraction_dilated;
  double dilated_target_fraction;  /* robust runs: the last moved target; else 0 */
} simp_robust_record;

int simp_projection_variants(simp_problem* p, double delta, simp_robust_record* record,
                             double* eroded_density, double* dilated_density);

/* ---- Modal analysis (src/fem/ModalAnalysis.cpp) ---------------------- */

/* ModalAnalysisOptions (include/sparlab/fem/ModalAnalysis.hpp:37-65).  The
 * shifted systems K - sigma M are solved by the problem's AMG-PCG (its
 * tolerance, iteration cap and precision), so the shift must be <= 0.  The
 * reference's `seed` fills the start subspace only when it has more vectors
 * than the model has DOFs, which never happens on the iterative path, so it
 * has no field here. */
typedef struct simp_modal_options {
  int32_t num_modes;          /* lowest modes requested (6) */
  int32_t mass_type;          /* 0 consistent, 1 lumped (row sums) */
  int32_t max_iterations;     /* subspace iteration cap (200) */
  double tolerance;           /* relative eigenvalue change (1e-10) */
  double shift_factor;        /* sigma = shift_factor * min k_ii / m_ii (0; <= 0) */
  double rigid_body_ratio;    /* zero-eigenvalue screen (1e-10) */
  double residual_tolerance;  /* eigenpair residual bound (1e-6) */
  int32_t warm_start;         /* start each solve from x_c / (mu_c - sigma) (1) */
  double density;             /* material density, > 0 (1.0) */
  const double* element_mass; /* M_e^0 (ed x ed, row-major) or NULL: the cell's consistent mass */
  int32_t concurrent_solves;  /* subspace columns solved at the same time (4) */
} simp_modal_options;

/* ModalResult's scalars (include/sparlab/fem/ModalAnalysis.hpp:67-86). */
typedef struct simp_modal_info {
  int32_t num_modes;          /* modes returned (num_modes, or the free DOFs if fewer) */
  int32_t iterations;         /* subspace iterations (0 on the dense path) */
  int32_t subspace_size;
  int32_t converged;
  int64_t linear_iterations;  /* PCG iterations over every subspace solve */
  double final_change;
  double total_mass;          /* sum of the assembled mass / dim */
  int32_t num_warnings;       /* texts: simp_modal_warnings */
} simp_modal_info;

void simp_default_modal_options(simp_modal_options* o);

/* solve_modal (src/fem/ModalAnalysis.cpp:120-418) on the problem's grid and
 * supports: the lowest modes of K_ff phi = lambda M_ff phi, with K_ff and
 * M_ff assembled from the element factors stiffness_scale / mass_scale
 * (host, num_elements each; NULL: all ones).  Outputs (host, NULL to skip):
 * eigenvalues, frequencies_hz and residuals (num_modes each), mass_fraction
 * (num_modes; the kinetic-energy share of cells with mass factor < 0.3, zero
 * without mass_scale) and mode_shapes (num_modes x num_dofs, a mode per row,
 * M-orthonormal, zero on the supports; the memory layout of the reference's
 * num_dofs x num_modes column-major matrix).  Systems with at most 400 free
 * DOFs take the dense path.  The problem's own hierarchy, design and
 * displacements are left as they are.  SIMP_MAXITER when the subspace
 * iteration or a solve does not converge, SIMP_BREAKDOWN for a non-positive
 * pencil or a massless mode, SIMP_NONFINITE for a non-finite basis. */
int simp_modal(simp_problem* p, const simp_modal_options* options, const double* stiffness_scale,
               const double* mass_scale, double* eigenvalues, double* frequencies_hz,
               double* residuals, double* mass_fraction, double* mode_shapes,
               simp_modal_info* info);

/* Warning k of the last simp_modal (rigid-body modes, large residuals, fewer
 * modes than requested), or NULL. */
const char* simp_modal_warning(simp_problem* p, int32_t k);

/* ---- Linear buckling (src/fem/Buckling.cpp) ---------------------------- */

/* BucklingOptions (include/sparlab/fem/Buckling.hpp:91-109) and the material
 * constants of the prestress sigma = D B u (the problem holds only K_e^0). */
typedef struct simp_buckling_options {
  int32_t num_modes;          /* smallest positive load factors requested (4) */
  int32_t max_iterations;     /* subspace iteration cap (400) */
  double tolerance;           /* relative change of the requested load factors (1e-8) */
  double residual_tolerance;  /* eigenpair residual bound (1e-6) */
  double young;               /* Young's modulus of the material (required) */
  double poisson;             /* Poisson ratio (plane stress in 2-D) */
  int32_t transform;          /* 0 auto (plain, transformed once reversed-load modes
                                 crowd the subspace); 1 the spectral transformation
                                 from the start */
  int32_t concurrent_solves;  /* subspace columns solved at the same time (4) */
  double shift_hint;          /* positive: an estimate of the smallest load factor the
                                 transformation's shift search starts from (0) */
} simp_buckling_options;

/* BucklingResult's scalars (include/sparlab/fem/Buckling.hpp:111-140). */
typedef struct simp_buckling_info {
  int32_t num_modes;               /* positive load factors returned */
  int32_t iterations;              /* subspace iterations (0 on the dense path) */
  int32_t subspace_size;
  int32_t converged;
  int32_t no_positive_load_factor; /* the load case only stiffens the structure */
  int32_t subspace_cols;           /* columns written to `subspace` */
  int64_t linear_iterations;       /* PCG iterations, the static solve included */
  double final_change;
  int32_t num_warnings;            /* texts: simp_buckling_warning */
  int32_t transformed;             /* the spectral transformation was used */
  double sigma;                    /* its shift, a lower bound on lambda_1 */
  int32_t factorizations;          /* factorisations of K_ff + sigma K_G,ff */
} simp_buckling_info;

void simp_default_buckling_options(simp_buckling_options* o);

/* analyse_buckling (src/fem/Buckling.cpp:438-466) of load case `load_case`:
 * the static solution u of K_ff u = f, K_G(u) on the device, and the smallest
 * positive load factors lambda of (K_ff + lambda K_G,ff) phi = 0 by subspace
 * iteration X <- K^-1 (-K_G) X on the problem's AMG-PCG (its tolerance and
 * precision).  Host inputs, NULL for the defaults: stiffness_scale and
 * stress_scale (num_elements each; ones), solid_mask (num_elements bytes,
 * 1 = solid; all solid), start_subspace (nfree x start_cols, column-major:
 * the `subspace` of a previous analysis).  Outputs (host, NULL to skip):
 * load_factors, residuals and solid_energy_fraction (num_modes each),
 * mode_shapes (num_modes x num_dofs, phi^T K phi = 1, zero on the supports),
 * subspace (nfree x subspace_size, column-major).  Systems with at most 400
 * free DOFs take the dense path.  The spectral transformation
 * X <- (K - sigma G)^-1 K X (on request, or when reversed-load modes crowd
 * the subspace: mostly tensile stress states) places sigma by the inertia of
 * K - sigma G, which it factors densely on the device: systems above 16000
 * free DOFs that need it return SIMP_BAD_INPUT with a message saying so. */
int simp_buckling(simp_problem* p, const simp_buckling_options* options, int32_t load_case,
                  const double* stiffness_scale, const double* stress_scale,
                  const uint8_t* solid_mask, const double* start_subspace, int32_t start_cols,
                  double* load_factors, double* residuals, double* solid_energy_fraction,
                  double* mode_shapes, double* subspace, simp_buckling_info* info);

/* Warning k of the last simp_buckling, or NULL. */
const char* simp_buckling_warning(simp_problem* p, int32_t k);

/* Consistent mass of a box cell (Quad4Element/Hex8Element::consistent_mass,
 * src/elements/Quad4.cpp:139-173, src/elements/Hex8.cpp:194-214), 3-point
 * Gauss per direction. */
int simp_element_mass(int32_t dim, double hx, double hy, double hz, double density,
                      double thickness, double* me);

/* ---- Displacement surrogate (the learned PCG start, warm_start = 3) -----
 * No counterpart in the reference, whose solves start from the previous
 * displacement (src/topopt/Sensitivity.cpp:142, 169-176 with
 * src/fem/StaticAnalysis.cpp:134-143).  A 3-D convolutional encoder-decoder
 * on the nodal grid (4 levels, 16/32/64/64 channels, 3x3x3 kernels, BF16
 * weights and activations, FP32 accumulation on the tensor cores) maps the
 * physical (filtered) density and a load case to a displacement shape; its
 * prediction joins the energy-optimal PCG start, so the PCG converges to the
 * unchanged tolerance whatever the prediction's error.  3-D problems only. */
typedef struct simp_surrogate simp_surrogate;

/* Message of the last failed surrogate or layer call on this thread. */
const char* simp_surrogate_last_error(void);

/* A network with seeded He-uniform weights on `device`. */
int simp_surrogate_create(int32_t device, uint64_t seed, simp_surrogate** out);
void simp_surrogate_destroy(simp_surrogate* s);
/* FP32 parameters, layer by layer: weights [27][cout][cin] (tap t = 9 (dz+1)
 * + 3 (dy+1) + (dx+1)) then biases [cout]; in-order layers e0a e0b e1a e1b
 * e2a e2b e3a e3b d2 d1 d0 head. */
int simp_surrogate_num_params(simp_surrogate* s, int64_t* n);
int simp_surrogate_get_params(simp_surrogate* s, float* params);
int simp_surrogate_set_params(simp_surrogate* s, const float* params);
/* Adds (the problem's physical density and load case, its displacement of
 * the last evaluation) to the device-resident training set. */
int simp_surrogate_add_sample(simp_surrogate* s, simp_problem* p, int32_t load_case);
int simp_surrogate_num_samples(simp_surrogate* s, int32_t* n);
/* Adam on the samples (seeded shuffle), `batch` samples per step, learning
 * rate cosine-decayed from learning_rate to learning_rate / 20; the mean
 * loss of each epoch goes to epoch_losses (epochs values) when non-NULL. */
int simp_surrogate_train(simp_surrogate* s, int32_t epochs, double learning_rate, int32_t batch, uint64_t seed,
                         double* epoch_losses);
/* Predicted displacement shape of load case `load_case` at the problem's
 * current physical density: nfree doubles on the device. */
int simp_surrogate_predict(simp_surrogate* s, simp_problem* p, int32_t load_case, double* u_device);
/* The network on a caller's input: nx x ny x nz nodes, 16 BF16 channels per
 * node (channels-last, x fastest) -> 3 FP32 values per node (device). */
int simp_surrogate_forward(simp_surrogate* s, int32_t nx, int32_t ny, int32_t nz, const void* input_device,
                           float* output_device);
/* One training example on a caller's tensors: input as for
 * simp_surrogate_forward, target 3 BF16 values per node, mask one byte per
 * node (bit k: component k counts); loss = sum over counted components of
 * (prediction - target)^2 / count, and its parameter gradient (host, FP32,
 * simp_surrogate_num_params values, the layout of simp_surrogate_get_params). */
int simp_surrogate_loss_gradient(simp_surrogate* s, int32_t nx, int32_t ny, int32_t nz, const void* input_device,
                                  const void* target_device, const uint8_t* mask_device, int64_t count, double* loss,
                                  float* gradient);
/* Attaches the surrogate (not owned; NULL detaches) for warm_start 3. */
int simp_problem_set_surrogate(simp_problem* p, simp_surrogate* s);
/* Seconds the problem's solves spent in the surrogate's predictions. */
int simp_problem_learned_seconds(simp_problem* p, double* seconds);

/* Layers of the surrogate on device pointers (BF16 channels-last tensors,
 * x fastest).  simp_conv3d_bf16: out = act(sum_t W_t in[. + o_t] + bias) for
 * the 27 taps o_t of a 3x3x3 stencil with zero padding; `nseg` inputs
 * concatenated along channels (16, 32 or 64 each), weights [27][n][sum cseg]
 * BF16, n output columns (16..128, step 16) written to `nout` tensors
 * (columns split at out_c[0]; BF16, or FP32 where out_f32[k]).  flip != 0
 * negates the offsets (the data gradient, with transposed weights).
 * simp_conv3d_wgrad: gw[t][co][ci] += sum_v dy[v][co] in[v + o_t][ci],
 * gb[co] += sum_v dy[v][co] (FP32, device; dy has cdy channels). */
int simp_conv3d_bf16(int32_t nx, int32_t ny, int32_t nz, int32_t nseg, const void* const* in, const int32_t* cseg,
                     const void* weights, int32_t n, const float* bias, int32_t relu, int32_t flip, int32_t nout,
                     void* const* out, const int32_t* out_c, const int32_t* out_pitch, const int32_t* out_f32);
int simp_conv3d_wgrad(int32_t nx, int32_t ny, int32_t nz, int32_t nseg, const void* const* in, const int32_t* cseg,
                      const void* dy, int32_t cdy, int32_t cout, float* gw, float* gb);

/* Launch-shape autotuner (no counterpart in the reference).  Kernels with
 * several launch shapes that compute the same values bit for bit (the tile
 * shape of the matrix-free operator, the warps per block of the Galerkin row
 * products) are timed on the problem's own data the first time a shape key is
 * seen and the fastest shape is kept (environment SIMP_TUNE_CACHE: a file the
 * choices are read from and appended to).  simp_autotune_enable(0) keeps the
 * default shapes.  simp_autotune_report writes one line per key, "key chosen
 * ms_0 ms_1 ...", into buf (NUL-terminated, truncated to size) and the bytes
 * the full report needs into *needed. */
void simp_autotune_enable(int32_t on);
/* Pins the choice for a key (as it appears in the report). */
int simp_autotune_set(const char* key, int32_t variant);
int simp_autotune_report(char* buf, int64_t size, int64_t* needed);

/* Number of kernels this library has launched (for launch accounting). */
int64_t simp_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif
