// Shared pieces of the subspace iterations (modal and buckling analyses):
// tall-skinny Gram products and rotations of column-major n x q blocks on
// the device, dense symmetric pencils on the host, and the copy of the
// level-0 structure into a solver of its own.
#pragma once

#include "amg.h"
#include "kernels.cuh"
#include "problem.h"
#include "topopt.cuh"

#include <algorithm>
#include <cmath>
#include <exception>
#include <numeric>
#include <sstream>
#include <thread>
#include <vector>

namespace simp {
namespace {

constexpr int kGramRows = 32;     // rows of X staged per Gram tile
constexpr int kGramBlocks = 304;  // 2 x 152 SMs
constexpr int kMaxSubspace = 64;  // q <= 64: num_modes <= 32

GridView grid_of_desc(const ProblemDesc& d) {
  GridView g;
  g.dim = d.dim;
  g.nx = d.nx;
  g.ny = d.ny;
  g.nz = d.dim == 3 ? d.nz : 1;
  g.nnx = d.nx + 1;
  g.nny = d.ny + 1;
  g.nnz = d.dim == 3 ? d.nz + 1 : 1;
  return g;
}

// out[i] = the diagonal entry of row i
__global__ void k_diag_of(i32 n, const i32* __restrict__ node_of, const i32* __restrict__ first,
                          const i32* __restrict__ self_slot, NodeView a, const i32* __restrict__ rowptr,
                          const double* __restrict__ val, double* __restrict__ out) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const i32 I = node_of[i];
    out[i] = val[rowptr[i] + a.off[self_slot[I]] + (static_cast<i32>(i) - first[I])];
  }
}

__global__ void k_scaled(i64 n, const double* __restrict__ x, double a, double* __restrict__ y) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    y[i] = a * x[i];
}

// w = kx - lam mx
__global__ void k_pair_residual(i64 n, const double* __restrict__ kx, const double* __restrict__ mx, double lam,
                                double* __restrict__ w) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    w[i] = kx[i] - lam * mx[i];
}

// Partial Gram products C = A^T B of two n x q column-major matrices: each
// block stages kGramRows rows of both in shared memory and accumulates its
// share of the q x q entries over a fixed set of row tiles.
__global__ void __launch_bounds__(256) k_gram(i32 n, int q, const double* __restrict__ A,
                                              const double* __restrict__ B, double* __restrict__ partial) {
  extern __shared__ double gram_smem[];
  double* As = gram_smem;
  double* Bs = gram_smem + kGramRows * q;
  const int qq = q * q;
  const int per = (qq + blockDim.x - 1) / blockDim.x;
  double acc[kMaxSubspace * kMaxSubspace / 256];
  for (int s = 0; s < per; ++s) acc[s] = 0.0;
  for (i64 row0 = static_cast<i64>(blockIdx.x) * kGramRows; row0 < n;
       row0 += static_cast<i64>(gridDim.x) * kGramRows) {
    for (int t = threadIdx.x; t < kGramRows * q; t += blockDim.x) {
      const int c = t / kGramRows, r = t % kGramRows;
      const i64 row = row0 + r;
      As[r * q + c] = row < n ? A[static_cast<i64>(c) * n + row] : 0.0;
      Bs[r * q + c] = row < n ? B[static_cast<i64>(c) * n + row] : 0.0;
    }
    __syncthreads();
    for (int s = 0; s < per; ++s) {
      const int e = threadIdx.x + s * blockDim.x;
      if (e < qq) {
        const int i = e / q, j = e % q;
        double v = acc[s];
        for (int r = 0; r < kGramRows; ++r) v = fma(As[r * q + i], Bs[r * q + j], v);
        acc[s] = v;
      }
    }
    __syncthreads();
  }
  for (int s = 0; s < per; ++s) {
    const int e = threadIdx.x + s * blockDim.x;
    if (e < qq) partial[static_cast<i64>(blockIdx.x) * qq + e] = acc[s];
  }
}

__global__ void k_gram_finish(int qq, int blocks, const double* __restrict__ partial, double* __restrict__ out) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < qq; e += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < blocks; ++b) s += partial[static_cast<i64>(b) * qq + e];
    out[e] = s;
  }
}

// Y = X R for column-major n x q X and Y, R q x q row-major (R[k q + c])
__global__ void __launch_bounds__(256) k_rotate(i32 n, int q, const double* __restrict__ X,
                                                const double* __restrict__ R, double* __restrict__ Y) {
  extern __shared__ double rot_smem[];
  for (int t = threadIdx.x; t < q * q; t += blockDim.x) rot_smem[t] = R[t];
  __syncthreads();
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    double xr[kMaxSubspace];
    for (int k = 0; k < q; ++k) xr[k] = X[static_cast<i64>(k) * n + i];
    for (int c = 0; c < q; ++c) {
      double s = 0.0;
      for (int k = 0; k < q; ++k) s = fma(xr[k], rot_smem[k * q + c], s);
      Y[static_cast<i64>(c) * n + i] = s;
    }
  }
}

// full[g] = phi[free index of g], 0 on the supports
__global__ void k_expand_free(i64 ndof, const i32* __restrict__ dof_map, const double* __restrict__ phi,
                              double* __restrict__ full) {
  for (i64 g = blockIdx.x * (i64)blockDim.x + threadIdx.x; g < ndof; g += (i64)gridDim.x * blockDim.x) {
    const i32 f = dof_map[g];
    full[g] = f >= 0 ? phi[f] : 0.0;
  }
}

// per-block max |v|
__global__ void __launch_bounds__(kRedThreads) k_absmax(i64 n, const double* __restrict__ v,
                                                        double* __restrict__ part) {
  __shared__ double m[kRedThreads];
  double a = 0.0;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    a = fmax(a, fabs(v[i]));
  m[threadIdx.x] = a;
  __syncthreads();
  for (int s = kRedThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) m[threadIdx.x] = fmax(m[threadIdx.x], m[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = m[0];
}

// ---------------------------------------------------------------------------
// dense symmetric pencils on the host
// ---------------------------------------------------------------------------
using Mat = std::vector<double>;  // row-major n x n

// A = L L^T in place (lower triangle); false when A is not positive definite
bool cholesky(Mat& a, int n) {
  for (int j = 0; j < n; ++j) {
    double d = a[static_cast<size_t>(j) * n + j];
    for (int k = 0; k < j; ++k) d -= a[static_cast<size_t>(j) * n + k] * a[static_cast<size_t>(j) * n + k];
    if (!(d > 0.0) || !std::isfinite(d)) return false;
    const double l = std::sqrt(d);
    a[static_cast<size_t>(j) * n + j] = l;
    for (int i = j + 1; i < n; ++i) {
      double s = a[static_cast<size_t>(i) * n + j];
      for (int k = 0; k < j; ++k) s -= a[static_cast<size_t>(i) * n + k] * a[static_cast<size_t>(j) * n + k];
      a[static_cast<size_t>(i) * n + j] = s / l;
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) a[static_cast<size_t>(i) * n + j] = 0.0;
  return true;
}

// Eigenvalues w and orthonormal eigenvectors v (columns of row-major v) of a
// symmetric matrix by the cyclic Jacobi method (Golub & Van Loan, Matrix
// Computations, 4th ed., Algorithms 8.5.1-8.5.3).
void jacobi_eigen(Mat a, int n, std::vector<double>& w, Mat& v) {
  v.assign(static_cast<size_t>(n) * n, 0.0);
  for (int i = 0; i < n; ++i) v[static_cast<size_t>(i) * n + i] = 1.0;
  auto A = [&](int i, int j) -> double& { return a[static_cast<size_t>(i) * n + j]; };
  double fro = 0.0;
  for (double x : a) fro += x * x;
  fro = std::sqrt(fro);
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) off += A(i, j) * A(i, j);
    if (std::sqrt(2.0 * off) <= 1e-17 * fro || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A(p, q);
        if (apq == 0.0) continue;
        // symmetric Schur decomposition of the (p, q) 2 x 2 block
        const double tau = (A(q, q) - A(p, p)) / (2.0 * apq);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < n; ++k) {  // A <- A J
          const double akp = A(k, p), akq = A(k, q);
          A(k, p) = c * akp - s * akq;
          A(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // A <- J^T A
          const double apk = A(p, k), aqk = A(q, k);
          A(p, k) = c * apk - s * aqk;
          A(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {  // V <- V J
          double& vkp = v[static_cast<size_t>(k) * n + p];
          double& vkq = v[static_cast<size_t>(k) * n + q];
          const double x = vkp, y = vkq;
          vkp = c * x - s * y;
          vkq = s * x + c * y;
        }
      }
  }
  w.resize(n);
  for (int i = 0; i < n; ++i) w[i] = A(i, i);
}

// C = L^-1 S L^-T for lower-triangular L
Mat reduce_pencil(const Mat& l, const Mat& s, int n) {
  Mat w(s);  // W = L^-1 S (forward substitution on every column)
  for (int c = 0; c < n; ++c)
    for (int i = 0; i < n; ++i) {
      double x = w[static_cast<size_t>(i) * n + c];
      for (int k = 0; k < i; ++k) x -= l[static_cast<size_t>(i) * n + k] * w[static_cast<size_t>(k) * n + c];
      w[static_cast<size_t>(i) * n + c] = x / l[static_cast<size_t>(i) * n + i];
    }
  Mat c(static_cast<size_t>(n) * n);  // C = W L^-T = (L^-1 W^T)^T
  for (int r = 0; r < n; ++r)
    for (int i = 0; i < n; ++i) {
      double x = w[static_cast<size_t>(r) * n + i];
      for (int k = 0; k < i; ++k) x -= l[static_cast<size_t>(i) * n + k] * c[static_cast<size_t>(r) * n + k];
      c[static_cast<size_t>(r) * n + i] = x / l[static_cast<size_t>(i) * n + i];
    }
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) {
      const double m = 0.5 * (c[static_cast<size_t>(i) * n + j] + c[static_cast<size_t>(j) * n + i]);
      c[static_cast<size_t>(i) * n + j] = c[static_cast<size_t>(j) * n + i] = m;
    }
  return c;
}

// x = L^-T y (back substitution), column by column of the n x m matrix y
void back_substitute(const Mat& l, int n, const Mat& y, int m, Mat& x) {
  x.assign(static_cast<size_t>(n) * m, 0.0);
  for (int c = 0; c < m; ++c)
    for (int i = n - 1; i >= 0; --i) {
      double s = y[static_cast<size_t>(i) * m + c];
      for (int k = i + 1; k < n; ++k) s -= l[static_cast<size_t>(k) * n + i] * x[static_cast<size_t>(k) * m + c];
      x[static_cast<size_t>(i) * m + c] = s / l[static_cast<size_t>(i) * n + i];
    }
}

// The `count` lowest pairs of the symmetric pencil (K, M), ascending, vectors
// n x count row-major; through the reversed pencil M y = mu K y when M is
// only semi-definite (ModalAnalysis.cpp:27-48).  False when neither applies.
bool lowest_pencil_pairs(const Mat& k, const Mat& m, int n, int count, std::vector<double>& lam, Mat& vec) {
  Mat l(m);
  const bool forward = cholesky(l, n);
  if (!forward) {
    l = k;
    if (!cholesky(l, n)) return false;
  }
  std::vector<double> w;
  Mat y;
  jacobi_eigen(reduce_pencil(l, forward ? k : m, n), n, w, y);
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  if (forward)
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return w[a] < w[b]; });
  else
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return w[a] > w[b]; });
  Mat ys(static_cast<size_t>(n) * count);
  lam.assign(count, 0.0);
  for (int c = 0; c < count; ++c) {
    const int src = order[c];
    if (forward) {
      lam[c] = w[src];
    } else {
      if (!(w[src] > 0.0)) return false;
      lam[c] = 1.0 / w[src];
    }
    for (int i = 0; i < n; ++i) ys[static_cast<size_t>(i) * count + c] = y[static_cast<size_t>(i) * n + src];
  }
  back_substitute(l, n, ys, count, vec);
  return true;
}

void copy_level0(const Level& s, Level& t, cudaStream_t st) {
  t.n = s.n;
  t.nnodes = s.nnodes;
  t.first = s.first;
  t.apat = s.apat;
  t.null = s.null;
  copy_device(t.d_first, s.d_first, st);
  copy_device(t.d_node_of, s.d_node_of, st);
  copy_device(t.d_apat.ptr, s.d_apat.ptr, st);
  copy_device(t.d_apat.nbr, s.d_apat.nbr, st);
  copy_device(t.d_apat.off, s.d_apat.off, st);
  copy_device(t.d_self, s.d_self, st);
  t.a.rows = s.a.rows;
  t.a.cols = s.a.cols;
  t.a.nnz = s.a.nnz;
  copy_device(t.a.ptr, s.a.ptr, st);
  copy_device(t.a.col, s.a.col, st);
  t.a.v64.alloc(static_cast<size_t>(s.a.nnz));
}

// A z_c = y_c for the q columns of column-major n x q blocks y, z (z holds
// the initial guesses), the columns dealt round-robin to the workspaces, one
// host thread and stream each; every solve computes what it computes alone.
// Errors of any thread are rethrown after all have joined.
std::vector<GpuAmg::PcgResult> solve_columns(GpuAmg& amg, const std::vector<SolveWork*>& works, int q, i32 n,
                                             const double* y, double* z) {
  int dev = 0;
  SIMP_CUDA(cudaGetDevice(&dev));
  const int workers = static_cast<int>(works.size());
  std::vector<GpuAmg::PcgResult> pr(static_cast<size_t>(q));
  std::vector<std::exception_ptr> errs(static_cast<size_t>(workers));
  auto run = [&](int t) {
    try {
      SIMP_CUDA(cudaSetDevice(dev));
      for (int c = t; c < q; c += workers)
        pr[static_cast<size_t>(c)] =
            amg.solve(*works[static_cast<size_t>(t)], y + static_cast<size_t>(c) * n, z + static_cast<size_t>(c) * n);
      SIMP_CUDA(cudaStreamSynchronize(works[static_cast<size_t>(t)]->stream));
    } catch (...) {
      errs[static_cast<size_t>(t)] = std::current_exception();
    }
  };
  std::vector<std::thread> threads;
  for (int t = 1; t < workers; ++t) threads.emplace_back(run, t);
  run(0);
  for (auto& th : threads) th.join();
  for (auto& e : errs)
    if (e) std::rethrow_exception(e);
  return pr;
}

// Adds a solve's iterations to `total`; AmgCgSolver's ConvergenceError text
// when it did not converge (src/fem/LinearSolver.cpp:219-290)
void count_solve(const GpuAmg::PcgResult& r, double rtol, i64& total) {
  total += r.iterations;
  if (!r.converged) {
    std::ostringstream os;
    os << "AMG-CG(chebyshev) did not converge: " << r.iterations << " iterations left a relative residual of "
       << r.relres << " against a tolerance of " << rtol;
    throw Error(kMaxIter, os.str());
  }
}

// Workspaces 0 .. count-1 of `amg`, sized for its hierarchy.
std::vector<SolveWork*> workspaces(GpuAmg& amg, int count) {
  std::vector<SolveWork*> works;
  for (int t = 0; t < count; ++t) works.push_back(&amg.work(t));
  for (SolveWork* w : works) amg.ensure(*w);
  return works;
}

}  // namespace
}  // namespace simp
