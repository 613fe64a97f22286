// The whole SIMP iteration on the GPU for a structured Q4 / Hex8 problem:
// ComplianceObjective::evaluate (src/topopt/Sensitivity.cpp:110-237),
// optimality_criteria_update (src/topopt/OptimalityCriteria.cpp:40-149) and
// one iteration of TopologyOptimizer::run_oc (src/topopt/TopologyOptimizer.cpp:
// 608-705), with the design, densities, displacements and gradients resident
// in device memory.
#pragma once

#include "amg.h"
#include "common.h"

#include <memory>
#include <string>
#include <vector>

namespace simp {

constexpr int kHistory = 3;  // displacements kept per load case by warm starts 2 and 3
constexpr int kBasis = kHistory + 1;  // + the surrogate's prediction (warm start 3)

namespace sg {
class Surrogate;
}

struct ProblemDesc {
  int dim = 3;
  i32 nx = 0, ny = 0, nz = 1;
  double lx = 0, ly = 0, lz = 0;
  double thickness = 1.0;
  std::vector<double> ke;       // element matrix, row-major
  std::vector<uint8_t> fixed;   // per DOF
  int nloads = 0;
  std::vector<double> loads;    // nloads x ndof
  std::vector<double> weights;  // normalised
  double radius = 1.5, vf = 0.5, x0 = 0.5, penalty = 3.0, emin = 1e-9, move = 0.2, damping = 0.5;
  int warm = 1;  // 0 zero start, 1 previous displacement, 2 projection on the last warm_history,
                 // 3 projection on the last warm_history and the surrogate's prediction
  int warm_history = kHistory;
  int block_pcg = 0;  // load cases: 0 one after another, 1 concurrent threads, 2 one graph
  int optimizer = 0;  // 0 OC, 1 MMA
  // Heaviside projection (src/topopt/Projection.cpp) with beta continuation
  bool projection = false;
  double eta = 0.5, beta_start = 1.0, beta_max = 32.0, beta_factor = 2.0, change_tol = 1e-3;
  int beta_interval = 50;
  bool advance_on_convergence = true;
  // robust formulation (Projection.hpp:44-60): the objective on the eroded
  // design (eta + delta), the volume on the dilated one (eta - delta)
  bool robust = false;
  double robust_delta = 0.1;
  int robust_interval = 1;
  double eta_override = -1.0;  // > 0: the threshold of a one-off evaluation (projection_variants)
  double objective_eta() const { return eta_override > 0.0 ? eta_override : robust ? eta + robust_delta : eta; }
  double volume_eta() const { return robust ? eta - robust_delta : eta; }
};

struct Evaluation {
  double compliance = 0, volume = 0, volume_fraction = 0, relres_max = 0;
  int linear_iterations = 0;
  // robust runs: the blueprint's and the dilated design's volumes
  double volume_intermediate = 0, volume_dilated = 0;
};

struct OcStep {
  double lambda = 0, volume = 0, max_change = 0;
  int bisections = 0;
  bool converged = false;
};

class GpuProblem {
 public:
  GpuProblem(const ProblemDesc& d, const AmgOptions& o);
  ~GpuProblem();

  ProblemDesc d;
  GpuAmg amg;
  i64 ne = 0, nn = 0, ndof = 0;
  i32 nfree = 0;
  double hx = 0, hy = 0, hz = 0, elem_volume = 0, domain_volume = 0;

  void set_design(const double* h);
  void get_design(double* h);
  Evaluation evaluate();
  // evaluate() in phases, for solves advanced together across problems
  // (simp_iterate_batch): prepare (filter .. AMG setup), per load case its
  // start, a SolveTask, and after the solve its compliance and history, then
  // finish (sensitivities, pull-back, volumes) with the solves' results
  void evaluate_prepare();
  void start_load(int l, SolveWork& w);
  SolveTask load_task(int l, SolveWork& w);
  void end_load(int l, SolveWork& w);
  Evaluation evaluate_finish(const std::vector<GpuAmg::PcgResult>& res);
  void launch_sensitivities(cudaStream_t s);
  OcStep oc_update(bool apply, double* xnew_host);
  // MMA step with the gradients of the last evaluate (mma.cu); lambda is the
  // volume multiplier, `bisections` the subproblem's Newton iterations.
  OcStep mma_update(bool apply, double* xnew_host);
  void filter_forward(const double* x, double* y);   // device pointers
  void filter_adjoint(const double* v, double* g);   // device pointers
  // exact: rounded products and sums in element order (the structure-
  // defining first assembly); otherwise fused multiply-adds
  void assemble(const double* scale_device, bool exact);
  // FP64 sum_e s_e E over level 0's pattern for a device element matrix E
  // (K_e^0, or M_e^0 for the mass), with the same kernel and order; FP32
  // (hi) and interleaved double-float (hi, lo) copies when those are given
  void assemble_into(const double* elem, const double* scale_device, bool exact, double* v64, float* hi,
                     float2* pair, cudaStream_t stream);
  const std::vector<i32>& free_dofs() const { return free_dofs_; }

  // device state
  DBuf<double> x, xnew, rho, sf, df, dc_dphys, dc_dx, dv_dx, se, vols, tmp;
  DBuf<double> b, u;        // free load vectors / displacements, nloads x nfree
  DBuf<i32> dof_map;        // DOF -> free index or -1
  DBuf<double> ke_d, weights_d;
  DBuf<double> hw;          // filter weights, slot-major
  DBuf<i32> gnode;
  DBuf<uint8_t> cmask, ucomp;
  DBuf<uint32_t> nmask;     // per free node: free neighbours by offset
  DBuf<double> opart;
  DBuf<double> ovol;  // volumes of one speculative bisection pass
  DBuf<double> oc_g, oc_lo, oc_hi;  // OC candidate factors of the current update
  // matrix-free level-0 operator (mixed precision, fully free / clamped nodes)
  DBuf<float> ke32, sf32;
  DBuf<float> scale_hi, scale_lo;  // double-float split of the stiffness factors (mixed assembly)
  DBuf<i32> nindex;
  void* stencil_d = nullptr;
  std::vector<double> last_compliance;
  Evaluation last_evaluation;
  // MMA state: previous designs, asymptotes, subproblem vectors
  bool mma_ready = false;
  int mma_iteration = 0;
  double c_ref = 0.0;
  DBuf<double> m_x1, m_x2, m_low, m_upp, m_alfa, m_beta, m_p0, m_q0, m_p, m_q, m_x, m_xsi, m_eta, m_xo, m_xsio,
      m_etao, m_dx, m_dxsi, m_deta, m_delx, m_diagx, m_gg, mpart;
  void mma_reduce(int k, std::vector<double>& out);
  double mma_reduce_max(int which);
  // warm starts 2 and 3 (warmstart.cu): newest-first displacement history
  // per load (kBasis slots: the last one takes the surrogate's prediction)
  DBuf<double> hist, khist, hpart;
  std::vector<int> hist_count;
  sg::Surrogate* surrogate = nullptr;  // warm start 3 (not owned)
  double learned_seconds = 0.0;        // time in the surrogate's predictions
  // warm start 3: the predictions of the current evaluation (nloads x nfree),
  // enqueued on the network's stream right after the physical density so
  // they overlap the assembly and AMG setup; the events bracket them
  DBuf<double> predicted;
  cudaEvent_t pred_t0 = nullptr, pred_ready = nullptr;
  bool pred_pending = false;
  std::vector<double> load_absmax;     // largest load component per load case
  void projected_start(int l, double* ul, bool learned);
  void record_history(int l, const double* ul);
  // projection state: current beta, its stage, the stage's first iteration
  double beta = 0.0;
  int beta_stage = 0, beta_stage_start = 1, iteration = 0;
  DBuf<double> rhot, dproj;  // clamped filtered density and d rho_bar / d rho_tilde
  // robust runs: the dilated design's volume target (moved every
  // robust_interval iterations to V* V_d / V_i) and scratch
  double dilated_target = 0.0;
  DBuf<double> rtmp, dv_dilated;
  void update_robust_target();
  // RobustRecord (TopologyOptimizer.hpp:153-166) of the current design: its
  // compliance and volume fraction projected at eta + delta, eta and
  // eta - delta with the current beta (TopologyOptimizer.cpp:344-415); the
  // densities of the eroded and dilated designs when asked for (host).
  struct Variants {
    double eta[3], compliance[3], volume_fraction[3];
  };
  Variants projection_variants(double delta, double* eroded_density, double* dilated_density);
  bool beta_at_final() const;
  // BetaSchedule::advance after iteration `iteration` with its design change
  void advance_beta(double max_change);
  bool evaluated = false;
  int evaluations = 0;
  double gray = 0.0;

 private:
  bool structure_built_ = false;
  int stencil_count_ = 0;
  std::vector<i32> free_dofs_;
  void build();
};

int beta_stages(const ProblemDesc& d);
double beta_of_stage(const ProblemDesc& d, int k);

void element_stiffness(int dim, double hx, double hy, double hz, double young, double nu, double thick,
                       double* ke);
// Consistent mass of a box cell, 3-point Gauss per direction (modal.cu).
void element_mass(int dim, double hx, double hy, double hz, double density, double thick, double* me);

// Undamped free vibration of the structured model (modal.cu):
// ModalAnalysisOptions (include/sparlab/fem/ModalAnalysis.hpp:37-65).
struct ModalOptions {
  int num_modes = 6;
  int mass_type = 0;  // 0 consistent, 1 lumped (row sums)
  int max_iterations = 200;
  double tolerance = 1.0e-10, shift_factor = 0.0, rigid_body_ratio = 1.0e-10, residual_tolerance = 1.0e-6;
  bool warm_start = true;
  double density = 1.0;
  std::vector<double> element_mass;  // M_e^0 (row-major); empty: the cell's consistent mass
  int concurrent_solves = 4;
};

// ModalResult (include/sparlab/fem/ModalAnalysis.hpp:67-86)
struct ModalResult {
  std::vector<double> eigenvalues, residuals, mass_fraction;
  std::vector<double> shapes;  // modes x ndof (a mode per row), M-orthonormal, zero on supports
  double total_mass = 0.0, final_change = 0.0;
  int iterations = 0, subspace_size = 0;
  bool converged = false;
  i64 linear_iterations = 0;
  std::vector<std::string> warnings;
};

// solve_modal (src/fem/ModalAnalysis.cpp:120-418) with the problem's grid,
// supports and solver options; host element factors (null: ones).
ModalResult solve_modal(GpuProblem& p, const ModalOptions& o, const double* stiffness_scale,
                        const double* mass_scale, bool want_shapes);

// rho = clamp(H x, 0, 1) and sum_e v_e rho_e without allocating (noalloc.cu).
void filter_volume_noalloc(GpuProblem& p, const double* x, double* rho, double* volume);

// BucklingOptions (include/sparlab/fem/Buckling.hpp:91-109) with the
// material constants the prestress needs (the problem holds only K_e^0).
struct BucklingOptions {
  int num_modes = 4;
  int max_iterations = 400;
  double tolerance = 1.0e-8, residual_tolerance = 1.0e-6;
  double young = 0.0, poisson = 0.0;
  int transform = 0;  // 0 auto (plain iteration, transformed when crowded), 1 shift-invert from the start
  int concurrent_solves = 4;
  double shift_hint = 0.0;  // positive: an estimate of lambda_1 the shift search starts from
};

// BucklingResult (include/sparlab/fem/Buckling.hpp:111-140)
struct BucklingResult {
  std::vector<double> load_factors, residuals, solid_fraction;
  std::vector<double> shapes;    // modes x ndof, phi^T K phi = 1, zero on supports
  std::vector<double> subspace;  // free DOFs x subspace_cols, column-major
  int subspace_cols = 0;
  bool no_positive = false, converged = false;
  bool transformed = false;  // the spectral transformation was used
  double sigma = 0.0;        // its shift, below lambda_1
  int factorizations = 0;    // factorisations of K - sigma G
  int iterations = 0, subspace_size = 0;
  double final_change = 0.0;
  i64 linear_iterations = 0;
  std::vector<std::string> warnings;
};

// analyse_buckling (src/fem/Buckling.cpp:438-466) of load case `load_case`
// with optional element stiffness and stress factors, solid flags and a
// start subspace (free DOFs x start_cols, column-major), all on the host.
BucklingResult solve_buckling(GpuProblem& p, const BucklingOptions& o, int load_case, const double* stiffness_scale,
                              const double* stress_scale, const uint8_t* solid, const double* start,
                              int start_cols, bool want_shapes);

}  // namespace simp
