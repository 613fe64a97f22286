// Projected initial guess for the per-load PCG (warm_start = 2 and 3).
//
// The reference warm-starts each solve from the previous iteration's
// displacement (StaticAnalysis::solve_load_vector with LinearSolverOptions::
// warm_start, src/fem/StaticAnalysis.cpp:134-143).  Mode 2 keeps the last
// kHistory displacements U = [u_1 .. u_k] of the load case and starts from
// the energy-optimal combination over their span under the NEW stiffness:
//
//   x0 = U c,  (U^T K U) c = U^T f,
//
// which is never worse in the energy norm than x0 = u_1 (c = e_1 lies in the
// search space).  Mode 3 adds the displacement surrogate's prediction for the
// current density as one more basis vector (after the history, so a
// prediction that adds nothing is the one dropped); on the first solve, with
// no history, the start is the prediction's energy-optimal multiple.  A
// non-finite or zero prediction drops out the same way, which leaves the
// history's start (or zero).  Nearly dependent vectors are dropped by a
// pivoted LDL^T of the Gram matrix.  The products K U use the V-cycle's FP32
// level-0 operator (FP64 in fp64 mode): the start need not be optimal to the
// last bit.  Cost: one such product per basis vector, one fused multi-dot pass
// and (mode 3) one network inference; the PCG itself is unchanged.
#include "kernels.cuh"
#include "problem.h"
#include "surrogate_net.h"

#include <chrono>
#include <cmath>

namespace simp {

namespace {

constexpr int kDots = kBasis * (kBasis + 1) / 2 + kBasis;

// partials of u_i . (K u_j) (i <= j) and u_i . f, per block
__global__ void __launch_bounds__(kRedThreads) k_history_dots(i64 n, int k, const double* __restrict__ u,
                                                              const double* __restrict__ ku,
                                                              const double* __restrict__ f,
                                                              double* __restrict__ part) {
  double acc[kDots];
#pragma unroll
  for (int q = 0; q < kDots; ++q) acc[q] = 0.0;
  for (i64 e = blockIdx.x * (i64)kRedThreads + threadIdx.x; e < n; e += (i64)gridDim.x * kRedThreads) {
    double ue[kBasis], ke[kBasis];
#pragma unroll
    for (int i = 0; i < kBasis; ++i) {
      ue[i] = i < k ? u[i * n + e] : 0.0;
      ke[i] = i < k ? ku[i * n + e] : 0.0;
    }
    const double fe = f[e];
    int q = 0;
#pragma unroll
    for (int i = 0; i < kBasis; ++i)
#pragma unroll
      for (int j = i; j < kBasis; ++j) acc[q++] += ue[i] * ke[j];
#pragma unroll
    for (int i = 0; i < kBasis; ++i) acc[q++] += ue[i] * fe;
  }
#pragma unroll
  for (int q = 0; q < kDots; ++q) {
    const double s = block_sum<kRedThreads>(acc[q]);
    if (threadIdx.x == 0) part[q * gridDim.x + blockIdx.x] = s;
  }
}

struct Coefs {
  double c[kBasis];
};

__global__ void k_history_combine(i64 n, int k, const double* __restrict__ u, Coefs c, double* __restrict__ x) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < n; e += (i64)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int i = 0; i < k; ++i) s += c.c[i] * u[i * n + e];
    x[e] = s;
  }
}

}  // namespace

void GpuProblem::projected_start(int l, double* ul, bool learned) {
  cudaStream_t s = amg.stream;
  int k = std::min(hist_count[l], d.warm_history);
  const i64 n = nfree;
  double* U = hist.p + static_cast<size_t>(l) * kBasis * n;
  if (learned) {  // the prediction takes the slot after the history
    double* slot = U + static_cast<size_t>(k) * n;
    if (pred_pending) {  // enqueued after the physical density (evaluate_prepare)
      SIMP_CUDA(cudaStreamWaitEvent(s, pred_ready, 0));
      SIMP_CUDA(cudaMemcpyAsync(slot, predicted.p + static_cast<size_t>(l) * n, sizeof(double) * n,
                                cudaMemcpyDeviceToDevice, s));
    } else {
      const auto t0 = std::chrono::steady_clock::now();
      surrogate->predict(*this, l, slot);
      learned_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    ++k;
  }
  if (k == 0) {
    SIMP_CUDA(cudaMemsetAsync(ul, 0, sizeof(double) * n, s));
    return;
  }
  const double* f = b.p + static_cast<size_t>(l) * n;
  // the Gram system only sets the start's coefficients: the FP32 operator of
  // the V-cycle is accurate enough for them (the PCG then converges to the
  // unchanged tolerance from whatever start)
  for (int i = 0; i < k; ++i) amg.spmv0_fast(U + i * n, khist.p + i * n);
  k_history_dots<<<kRedBlocks, kRedThreads, 0, s>>>(n, k, U, khist.p, f, hpart.p);
  SIMP_CHECK_LAUNCH();
  std::vector<double> hp(static_cast<size_t>(kDots) * kRedBlocks);
  SIMP_CUDA(cudaMemcpyAsync(hp.data(), hpart.p, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost, s));
  SIMP_CUDA(cudaStreamSynchronize(s));
  double dots[kDots];
  for (int q = 0; q < kDots; ++q) {
    double t = 0.0;
    for (int p = 0; p < kRedBlocks; ++p) t += hp[static_cast<size_t>(q) * kRedBlocks + p];
    dots[q] = t;
  }
  double G[kBasis][kBasis] = {}, g[kBasis] = {};
  int q = 0;
  for (int i = 0; i < kBasis; ++i)
    for (int j = i; j < kBasis; ++j) {
      G[i][j] = G[j][i] = dots[q];
      ++q;
    }
  for (int i = 0; i < kBasis; ++i) g[i] = dots[q++];
  // LDL^T in history order (newest first); a pivot below 1e-10 of its
  // diagonal marks a dependent vector, whose coefficient is zero
  double L[kBasis][kBasis] = {}, D[kBasis] = {};
  bool keep[kBasis] = {};
  for (int j = 0; j < k; ++j) {
    double dj = G[j][j];
    for (int p = 0; p < j; ++p)
      if (keep[p]) dj -= L[j][p] * L[j][p] * D[p];
    keep[j] = dj > 1.0e-10 * G[j][j] && G[j][j] > 0.0;
    D[j] = keep[j] ? dj : 0.0;
    for (int i = j + 1; i < k; ++i) {
      double v = G[i][j];
      for (int p = 0; p < j; ++p)
        if (keep[p]) v -= L[i][p] * L[j][p] * D[p];
      L[i][j] = keep[j] ? v / dj : 0.0;
    }
  }
  Coefs c{};
  double y[kBasis] = {};
  for (int i = 0; i < k; ++i) {
    double v = g[i];
    for (int p = 0; p < i; ++p) v -= L[i][p] * y[p];
    y[i] = keep[i] ? v : 0.0;
  }
  for (int i = k - 1; i >= 0; --i) {
    double v = keep[i] ? y[i] / D[i] : 0.0;
    for (int p = i + 1; p < k; ++p) v -= L[p][i] * c.c[p];
    c.c[i] = keep[i] ? v : 0.0;
  }
  bool finite = true;
  for (int i = 0; i < k; ++i) finite = finite && std::isfinite(c.c[i]);
  if (!finite) {  // keep the previous displacement (zero on a first solve)
    if (hist_count[l] == 0) SIMP_CUDA(cudaMemsetAsync(ul, 0, sizeof(double) * n, s));
    return;
  }
  k_history_combine<<<grid_for(n, 256, 8192), 256, 0, s>>>(n, k, U, c, ul);
  SIMP_CHECK_LAUNCH();
}

void GpuProblem::record_history(int l, const double* ul) {
  const i64 n = nfree;
  double* U = hist.p + static_cast<size_t>(l) * kBasis * n;
  // newest first: shift the older vectors down one slot
  const int k = std::min(hist_count[l] + 1, kHistory);
  for (int i = k - 1; i > 0; --i)
    SIMP_CUDA(cudaMemcpyAsync(U + i * n, U + (i - 1) * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, amg.stream));
  SIMP_CUDA(cudaMemcpyAsync(U, ul, sizeof(double) * n, cudaMemcpyDeviceToDevice, amg.stream));
  hist_count[l] = k;
}

}  // namespace simp
