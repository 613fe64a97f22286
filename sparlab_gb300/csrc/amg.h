// Smoothed-aggregation AMG preconditioned CG on the GPU: the hierarchy of
// src/fem/Multigrid.cpp with every per-setup numeric product, the V-cycle and
// PCG on the device, and the once-per-structure aggregation, QR and symbolic
// patterns on the host.
//
// Precision: SIMP_PRECISION_FP64 runs everything in FP64 (the reference's
// arithmetic).  SIMP_PRECISION_MIXED keeps FP32 copies of every operator,
// prolongator and restriction and runs the V-cycle (smoother, residuals,
// transfers; level 0 matrix-free on structured grids), the Lanczos estimates
// and the reused-structure Galerkin products in FP32.  CG itself -- its
// operator, vectors, scalars and the true-residual restarts -- and the
// coarsest dense inverse stay FP64 in both modes, so both stop on the same
// FP64 residual test.
#pragma once

#include "common.h"
#include "structure.h"

#include <memory>
#include <string>
#include <vector>

namespace simp {

struct AmgOptions {
  double theta = 0.02;
  int max_levels = 12;
  i32 coarse_size = 1500;
  int degree = 3;
  double cheb_ratio = 30.0;
  double damping = 4.0 / 3.0;
  int lanczos_steps = 12;
  double pivot_tol = 1.0e-13;
  bool reuse = true;
  double rtol = 1.0e-12;
  int maxit = 1000;
  int precision = 0;  // 0 FP64, 1 mixed
  bool graphs = true; // PCG iterations after the first as one CUDA graph launch
  bool mf_transfer = true;  // level-0 R and P of the FP32 cycle applied matrix-free
  // mixed precision, structured grids: 0 level 0 assembled throughout; 1 the
  // FP32 V-cycle's level 0 matrix-free; 2 also the CG operator (FP32 element
  // products, FP64 matrix-free true residuals at the restarts)
  int matrix_free = 1;
  // the 3-D matrix-free level 0 on the tensor cores (3 x TF32 element GEMMs)
  int tensor_cores = 0;
};

struct DevPattern {
  DBuf<i32> ptr, nbr, off;
  void upload(const NodePattern& p, cudaStream_t s = 0);
  NodeView view() const { return {ptr.p, nbr.p, off.p}; }
};

struct DevCsr {
  i32 rows = 0, cols = 0;
  i64 nnz = 0;
  DBuf<i32> ptr, col;
  DBuf<double> v64;
  DBuf<float> v32;
  DBuf<float2> v2;    // level 0, mixed: (v32, v64 - v32) pairs, interleaved (the double-float CG operator)
};

// A node-chunked matrix as the operator kernels see it (see nbspmv.cuh).
struct NbOp {
  i32 nodes = 0;                // row nodes
  const i32* row_first = nullptr;
  NodeView pat{nullptr, nullptr, nullptr};
  const i32* rowptr = nullptr;
  const i32* col = nullptr;
  int block = 0;                // uniform column-node width (2, 3, 6): no column reads; or 0
  const i32* node_of = nullptr; // row -> row node
  i32 rows = 0;
  int lanes32 = 8, lanes64 = 4; // lanes per row of the FP32 / FP64 kernels
  // lanes per row of the double-float kernels (level 0): 4 -- each lane's
  // longer row chain and twice the rows per warp hide the gathers' latency
  // better than 8 lanes (0.700 against 0.779 ms per launch at 192x96x96)
  int lanes_df = 4;
};

// Shared-memory shape of a warp-per-row-node product (galerkin.cuh).
struct WarpRows {
  int acc = 0;    // max rows x row length of the output, per row node
  int slots = 0;  // max output slots per row node
  int inner = 0;  // max slots of an inner row
};

struct Level {
  i32 n = 0, nnodes = 0;
  std::vector<i32> first;
  DBuf<i32> d_first, d_node_of;
  NodePattern apat;
  DevPattern d_apat;
  DBuf<i32> d_self;
  DevCsr a;
  NbOp opA, opP, opR;
  DBuf<double> dinv64;
  DBuf<float> dinv32;
  DBuf<double> cheb64;  // Chebyshev coefficients for the kernels: [1 / theta, c1_0, c2_0, ..., 0, 0]
  DBuf<float> cheb32;
  double lambda = 0.0;
  std::vector<double> null;  // near-null space, n x m row-major (host)
  // transfer to the next level
  std::vector<i32> agg;
  i32 naggs = 0;
  DBuf<i32> d_agg, phat_ptr;
  DBuf<double> phat64;
  DBuf<float> phat32;
  // matrix-free transfers of level 0 (FP32 cycle, 3-D grid, 3 -> 6 unknowns
  // per node): the aggregates' member nodes (CSR, ascending) and the
  // prolongator damping w = damping / lambda in device memory
  bool mf_transfer = false;
  DBuf<i32> d_members_ptr, d_members;
  DBuf<float> omega32;
  NodePattern ppat, rpat, appat;
  WarpRows wr_p, wr_ap, wr_rap;
  DevPattern d_ppat, d_rpat, d_appat;
  DBuf<i32> d_r_to_p, d_sym_t;
  // per P slot: its contributors, the A slots of its row whose neighbour is
  // in its aggregate, as (block offset in the A row, first P-hat value)
  DBuf<i32> d_pc_ptr;
  DBuf<int2> d_pc;
  DevCsr p, r, ap;
  DBuf<double> raw64;
  DBuf<float> raw32;
  std::vector<double> c1, c2;
  double inv_theta = 0.0;
  DBuf<double> lz[5];  // Lanczos work vectors (FP64 setups)
  DBuf<float> lz32[5];  // (FP32 reuse setups)
  DBuf<double> lz_start;  // Lanczos start vector (depends on n only) and its norm
  double lz_norm = 0.0;
};

// Matrix-free level-0 operator of a structured grid (see mfree.cuh), used
// by the FP32 V-cycle and the mixed-precision CG operator when enabled.
struct MfOp {
  bool enabled = false;
  int dim = 3;
  i32 nx = 0, ny = 0, nz = 1, nnx = 0, nny = 0;
  const i32* gnode = nullptr;   // free node -> grid node
  const i32* nindex = nullptr;  // grid node -> free node or -1
  const float* ke = nullptr;    // K_e^0, FP32
  const float* scale = nullptr; // s_e, FP32
  float ke_host[24 * 24] = {};  // K_e^0, FP32 (kernel parameter of the tiled 3-D kernel)
  // variant of the tiled 3-D kernel per mode (0..8): shape
  // kMfTileShape[tile % 5], float4 halo if >= 5 (tuned per mode)
  int tile[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const double* scale64 = nullptr;  // s_e, FP64 (the matrix-free CG operator's true residuals)
  double ke64_host[24 * 24] = {};   // K_e^0, FP64
  bool tensor = false;     // 3-D: the tensor-core kernel (mfree_tc.cuh) instead of the tiled FMA kernel
  int tc_layers = 0;       // node layers per CTA of the tensor-core kernel (tuned; 0: all)
  int* status = nullptr;   // device word the tensor-core kernel sets when a wait runs out
};

// Work vectors of one solve: the cycle vectors of every level, the PCG
// vectors, reduction scratch and a stream.  Solves on different workspaces
// (the load cases of one problem) run concurrently from host threads; every
// solve computes exactly what it computes alone.
struct LevelWork {
  DBuf<double> x64, b64, r64, d64, e64;
  DBuf<float> x32, b32, r32, d32, e32;
};

struct SolveWork {
  cudaStream_t stream = 0;
  bool own_stream = false;
  std::vector<LevelWork> lv;
  DBuf<double> part, scal, pr, pz, pp, pq;
  DBuf<float2> xsplit;  // op0's input as (hi, lo) pairs (mixed mode)
  DBuf<float> p32;      // the CG direction in FP32 (matrix-free CG operator)
  // PCG iteration body (V-cycle, direction, operator, update) captured as a
  // CUDA graph on this workspace's buffers; valid for one hierarchy epoch
  DBuf<double> px;      // the iterate (the caller's x is copied in and out)
  // solves advanced together (solve_together): [0] iterating, [1] iterations
  // done, [2] budget; loopd[0] the stopping residual norm
  DBuf<int> loop;
  DBuf<double> loopd;
  cudaGraphExec_t body = nullptr;
  uint64_t body_epoch = 0;
  int64_t body_kernels = 0;
  SolveWork() = default;
  SolveWork(const SolveWork&) = delete;
  SolveWork& operator=(const SolveWork&) = delete;
  ~SolveWork();
};

struct AmgStats {
  int num_levels = 0;
  bool reused = false;
  double operator_complexity = 0, grid_complexity = 0, pivot_ratio = 0, setup_seconds = 0;
  i64 storage = 0;
};

class GpuAmg;

// drops cached solve_together graphs that hold this hierarchy
void together_forget(const GpuAmg* a);

// One linear solve of solve_together: the hierarchy, a workspace of it, the
// right-hand side and the guess / solution (device, level-0 length).
struct SolveTask {
  GpuAmg* amg = nullptr;
  SolveWork* w = nullptr;
  const double* b = nullptr;
  double* x = nullptr;
};

class GpuAmg {
 public:
  explicit GpuAmg(const AmgOptions& o);
  ~GpuAmg();

  AmgOptions opt;
  std::vector<std::unique_ptr<Level>> levels;
  AmgStats stats;
  cudaStream_t stream = 0;

  bool mixed() const { return opt.precision == 1; }
  // the CG operator is the FP32 matrix-free product (matrix_free = 2, 3-D)
  bool mf_cg() const { return mixed() && opt.matrix_free >= 2 && mf.enabled && mf.dim == 3; }
  // Set by an assembler that wrote level 0's FP32 values (hi in a.v32 and
  // (hi, lo) pairs in a.v2) itself; otherwise setup splits the FP64 values (mixed
  // mode).  In mixed mode the CG operator reads hi/lo only, so an assembler
  // may leave a.v64 stale after the structure-defining first setup.
  bool level0_fp32_fresh = false;
  MfOp mf;
  // Level 0: the caller fills levels[0]->a (device CSR with FP64 values, and
  // FP32 values in mixed mode), its node layout (first) and pattern (apat),
  // and the near-null space.
  Level& level0();
  // structure_changed: rebuild aggregates / patterns (first setup or a new
  // structure); otherwise reuse them when opt.reuse.
  void setup(bool structure_changed);
  bool ready() const { return ready_; }
  // level-0 FP32 hi/lo values from the FP64 ones (mixed mode)
  void refresh_level0_fp32();

  // Workspace k: 0 is the context's own (its stream); k > 0 are made on
  // demand with their own streams.  ensure() sizes one for the hierarchy.
  SolveWork& work(int k = 0);
  void ensure(SolveWork& w);

  // z = M^-1 r (FP64 device vectors of level-0 length).
  void apply(const double* r, double* z) { apply(work(0), r, z); }
  void apply(SolveWork& w, const double* r, double* z);
  struct PcgResult {
    int iterations = 0;
    double relres = 0.0;
    bool converged = false;
  };
  // PCG (src/fem/Multigrid.cpp:1152-1237); x holds the guess on entry.
  PcgResult solve(const double* b, double* x) { return solve(work(0), b, x); }
  PcgResult solve(SolveWork& w, const double* b, double* x);
  // The CG operator on FP64 vectors: y = A0 x (rhs null) or y = rhs - A0 x.
  // FP64 values in fp64 mode; double-float values in mixed mode.
  // split_ready: x's double-float split is already in w.xsplit (written by
  // the PCG direction update).
  void op0(SolveWork& w, const double* x, double* y, const double* rhs, bool split_ready = false);
  void spmv0(const double* x, double* y) { op0(work(0), x, y, nullptr); }
  // y = A x on FP64 vectors through the FP32 operator of the V-cycle's level
  // 0 (matrix-free where enabled), on the context's stream: an approximate
  // product for the start of a solve.  fp64 mode: the FP64 operator.
  void spmv0_fast(const double* x, double* y);
  // q = A p, the CG's own product: op0, or with mf_cg() the FP32 matrix-free
  // product of p's FP32 copy (p32_ready: already in w.p32)
  void cg_op(SolveWork& w, const double* p, double* q, bool p32_ready);
  // y = V x for caller's FP64 values V on level 0's pattern (a matrix of the
  // same structure: the stiffness or mass of a modal analysis)
  void apply_values0(SolveWork& w, const double* values, const double* x, double* y);
  // CUDA-event time of one op0 launch (ms) and its algorithmic bytes
  void time_operator(int reps, double* ms, double* bytes);
  // The PCG of solve() for several systems at once (load cases of one
  // problem on their own workspaces, or independent problems): the same
  // iterations, restarts and stopping tests per system, with every round's
  // iterations after the first advanced together -- one CUDA graph launch
  // runs one PCG iteration of each system still iterating, each under a
  // conditional node its own convergence test sets.  Results and iteration
  // counts equal solve()'s bit for bit.  Errors (breakdown, no convergence)
  // are thrown after every task has stopped, the first task's first.
  struct TaskResult {
    PcgResult r;
    int error_code = 0;
    std::string error;
  };
  static std::vector<TaskResult> solve_together(std::vector<SolveTask>& tasks);
  double dot(SolveWork& w, const double* a, const double* b, i64 n);

  DBuf<double> part, scal;  // reductions of setup and of callers on the context stream
  DBuf<int> dstatus;
  DBuf<int> mf_status;  // the tensor-core matrix-free kernel's wait status
  // throws when a tensor-core matrix-free launch on this stream reported a
  // wait that ran out (reads one word)
  void check_mf_status(cudaStream_t s);

 private:
  bool ready_ = false;
  i32 nc_ = 0;
  DBuf<double> lz_ab_;  // Lanczos coefficients of the level in setup, and its stop flag
  DBuf<double> dense_, swept_, piv_, panel_;  // A_c^-1 (full), the sweep's lower triangle, pivots, U/V/P
  SolveWork main_;
  std::vector<std::unique_ptr<SolveWork>> extra_;

  void numeric_level(size_t l);
  template <class T>
  void lanczos(size_t l, int m, double* ab);
  void build_transfer(size_t l);
  void galerkin(size_t l, bool fp32);
  void coarse_factorize();
  void make_ops(size_t l);
  void alloc32(DBuf<float>& v, i64 n, cudaStream_t s);
  template <class T> void coarse_solve(SolveWork& w, size_t l);
  template <class T> void smooth(SolveWork& w, size_t l, bool zero_guess);
  template <class T> void cycle(SolveWork& w, size_t l);
  double dot(const double* a, const double* b, i64 n) { return dot(work(0), a, b, n); }
  PcgResult pcg(SolveWork& w, const double* b, double* x, double target, int budget, bool restarts,
                double bnorm);
  // the iterations after the first: [V-cycle, beta, direction, operator,
  // alpha, update] -- launched one by one, or as w's captured graph
  void pcg_tail(SolveWork& w, float2* psplit);
  // op_done: q = A p is already in w.pq (a fused multi-RHS launch)
  void pcg_head(SolveWork& w, double* x, bool split_ready, bool op_done = false);
  // q = A0 p of several workspaces of this hierarchy (mixed precision, p's
  // split in each xsplit) as one fused multi-RHS kernel node of g after
  // deps; a workspace whose loop flag is clear is skipped
  cudaGraphNode_t add_op0_multi(cudaGraph_t g, const std::vector<SolveWork*>& ws,
                                const std::vector<cudaGraphNode_t>& deps);
  void pcg_body(SolveWork& w, double* x, float2* psplit);
  float2* psplit_of(SolveWork& w) { return mixed() && !mf_cg() ? w.xsplit.p : nullptr; }
  friend struct TogetherGraph;
  uint64_t epoch_ = 1;  // bumped by every setup: captured graphs are stale
  void compute_stats();
  void tune_level0();
  void tune_df();
  int df_unroll_ = 4;  // row steps in flight per lane of the double-float operator (tuned)
  void df_apply(const float2* xsplit, double* y, const double* rhs, cudaStream_t stream);
  void df_apply_unroll(const float2* xsplit, double* y, const double* rhs, cudaStream_t stream, int unroll);
};

}  // namespace simp
