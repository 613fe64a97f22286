// Smoothed-aggregation AMG preconditioned CG on the GPU: the hierarchy of
// src/fem/Multigrid.cpp with every per-setup numeric product, the V-cycle and
// PCG on the device, and the once-per-structure aggregation, QR and symbolic
// patterns on the host.
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
  int precision = 0;  // 0 FP64, 1 mixed (FP32 operator / smoother / transfers)
};

struct DevPattern {
  DBuf<i32> ptr, nbr, off;
  void upload(const NodePattern& p);
  NodeView view() const { return {ptr.p, nbr.p, off.p}; }
};

struct DevCsr {
  i32 rows = 0, cols = 0;
  i64 nnz = 0;
  DBuf<i32> ptr, col;
  DBuf<double> v64;
  DBuf<float> v32;
};

struct Level {
  i32 n = 0, nnodes = 0;
  std::vector<i32> first;
  DBuf<i32> d_first, d_node_of;
  NodePattern apat;
  DevPattern d_apat;
  DBuf<i32> d_self;
  DevCsr a;
  DBuf<double> dinv64;
  DBuf<float> dinv32;
  double lambda = 0.0;
  std::vector<double> null;  // near-null space, n x m row-major (host)
  // transfer to the next level
  std::vector<i32> agg;
  i32 naggs = 0;
  DBuf<i32> d_agg, phat_ptr;
  DBuf<double> phat64;
  DBuf<float> phat32;
  NodePattern ppat, rpat, appat;
  DevPattern d_ppat, d_rpat, d_appat;
  DBuf<i32> d_r_to_p, d_sym_t;
  DevCsr p, r, ap;
  DBuf<double> raw64;
  DBuf<float> raw32;
  // cycle workspace
  DBuf<double> x64, b64, r64, d64, e64;
  DBuf<float> x32, b32, r32, d32, e32;
  std::vector<double> c1, c2;
  double inv_theta = 0.0;
};

struct AmgStats {
  int num_levels = 0;
  bool reused = false;
  double operator_complexity = 0, grid_complexity = 0, pivot_ratio = 0, setup_seconds = 0;
  i64 storage = 0;
};

class GpuAmg {
 public:
  explicit GpuAmg(const AmgOptions& o);
  ~GpuAmg();

  AmgOptions opt;
  std::vector<std::unique_ptr<Level>> levels;
  AmgStats stats;
  cudaStream_t stream = 0;

  // Level 0: the caller fills levels[0]->a (device CSR, FP64 values), its
  // node layout (first) and pattern (apat), and the near-null space.
  Level& level0();
  // structure_changed: rebuild aggregates / patterns (first setup or a new
  // structure); otherwise reuse them when opt.reuse.
  void setup(bool structure_changed);
  bool ready() const { return ready_; }

  // z = M^-1 r (FP64 device vectors of level-0 length).
  void apply(const double* r, double* z);
  // PCG (src/fem/Multigrid.cpp:1152-1237); x holds the guess on entry.
  struct PcgResult {
    int iterations = 0;
    double relres = 0.0;
    bool converged = false;
  };
  PcgResult solve(const double* b, double* x);
  // y = A0 x
  void spmv0(const double* x, double* y);

  // scratch for reductions and PCG
  DBuf<double> part, scal;
  DBuf<double> pr, pz, pp, pq;
  DBuf<int> dstatus;

 private:
  bool ready_ = false;
  // coarse direct solve
  i32 nc_ = 0;
  DBuf<double> dense_, inv_t_, piv_, tmp_;
  std::vector<double> lanczos_start_;

  void numeric_level(size_t l);
  void build_transfer(size_t l);
  void galerkin(size_t l);
  void coarse_factorize();
  void coarse_solve(const Level& lv);
  void smooth(size_t l, bool zero_guess);
  void cycle(size_t l);
  double dot(const double* a, const double* b, i64 n);
  void compute_stats();
};

// y = A x for a level operator (selects lanes per row from the row length).
void csr_apply(const DevCsr& a, const double* x, double* y, cudaStream_t s);

}  // namespace simp
