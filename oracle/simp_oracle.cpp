// CPU oracle of SparLab's SIMP inner loop.
//
// TEST INFRASTRUCTURE, not product code: the tests, the smoke check and the
// bench's CPU-baseline leg call it as the checker of the CUDA path.  It is a
// restatement of the reference algorithms in plain C++ (the reference needs
// Eigen, which is not available), following, function by function:
//   structured mesh           src/mesh/StructuredMesh.cpp:157-247
//   element stiffness         src/elements/Hex8.cpp:44-101,172-192,
//                             src/elements/Quad4.cpp:43-90,117-137,
//                             src/material/IsotropicMaterial.cpp:34-65
//   pattern/scatter/reduce    src/fem/Assembler.cpp:85-214,410-455
//   density filter            src/topopt/DensityFilter.cpp:19-195
//   SIMP law                  src/topopt/SimpInterpolation.cpp:59-70
//   SA-AMG + PCG              src/fem/Multigrid.cpp (whole file)
//   AmgCgSolver               src/fem/LinearSolver.cpp:219-290
//   objective + gradients     src/topopt/Sensitivity.cpp:110-237
//   OC update                 src/topopt/OptimalityCriteria.cpp:14-149
//   OC loop                   src/topopt/TopologyOptimizer.cpp:556-724
// Eigen pieces are re-derived from their published algorithms: Householder
// QR with column pivoting and norm downdating (Businger-Golub; LAPACK xGEQPF,
// LAWN 176), LDL^T with diagonal pivoting, and the largest eigenvalue of a
// symmetric tridiagonal matrix by Sturm-sequence bisection.
//
// Parity pinning: the reference's published compliances
// (docs/results/solver_scaling.csv) and its test identities.  Parity with
// Eigen's exact QR signs/pivots is unpinned (identities only).

#include "simp_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

using Index = int32_t;
using Vec = std::vector<double>;

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
// Status codes shared in meaning with the product's C ABI.
enum { kOk = 0, kBadInput = 1, kBreakdown = 2, kUnderConstrained = 3, kMaxIter = 4,
       kNonFinite = 5 };

thread_local std::string g_error;

// ---------------------------------------------------------------------------
// CSR kernels (Multigrid.cpp:22-284)
// ---------------------------------------------------------------------------
constexpr Index kChunk = 4096;
constexpr Index kParallelRows = 16384;

struct Csr {
  Index rows = 0, cols = 0;
  std::vector<Index> ptr, col;
  Vec val;
  Index nnz() const { return ptr.empty() ? 0 : ptr.back(); }
};

struct View {
  Index rows = 0, cols = 0;
  const Index* ptr = nullptr;
  const Index* col = nullptr;
  const double* val = nullptr;
  Index nnz() const { return rows == 0 ? 0 : ptr[rows]; }
};

View view(const Csr& m) { return {m.rows, m.cols, m.ptr.data(), m.col.data(), m.val.data()}; }

double dot(const double* a, const double* b, Index n) {
  const Index chunks = (n + kChunk - 1) / kChunk;
  if (chunks <= 1) {
    double s = 0.0;
    for (Index i = 0; i < n; ++i) s += a[i] * b[i];
    return 0.0 + s;
  }
  Vec part(static_cast<size_t>(chunks), 0.0);
#pragma omp parallel for schedule(static) if (n >= kParallelRows)
  for (Index c = 0; c < chunks; ++c) {
    const Index lo = c * kChunk, hi = std::min(n, lo + kChunk);
    double s = 0.0;
    for (Index i = lo; i < hi; ++i) s += a[i] * b[i];
    part[static_cast<size_t>(c)] = s;
  }
  double t = 0.0;
  for (double p : part) t += p;
  return t;
}

void spmv(const View& a, const double* x, double* y) {
#pragma omp parallel for schedule(static) if (a.rows >= kParallelRows)
  for (Index i = 0; i < a.rows; ++i) {
    double s = 0.0;
    for (Index k = a.ptr[i]; k < a.ptr[i + 1]; ++k) s += a.val[k] * x[a.col[k]];
    y[i] = s;
  }
}

void residual(const View& a, const double* x, const double* b, double* r) {
#pragma omp parallel for schedule(static) if (a.rows >= kParallelRows)
  for (Index i = 0; i < a.rows; ++i) {
    double s = 0.0;
    for (Index k = a.ptr[i]; k < a.ptr[i + 1]; ++k) s += a.val[k] * x[a.col[k]];
    r[i] = b[i] - s;
  }
}

// Gustavson product: symbolic count, then numeric fill with columns sorted.
Csr multiply(const View& a, const View& b) {
  if (a.cols != b.rows) throw Error(kBadInput, "multigrid: inner dimensions of a product differ");
  Csr c;
  c.rows = a.rows;
  c.cols = b.cols;
  c.ptr.assign(static_cast<size_t>(a.rows) + 1, 0);
#pragma omp parallel if (a.rows >= kParallelRows)
  {
    std::vector<Index> mark(static_cast<size_t>(b.cols), -1);
#pragma omp for schedule(static)
    for (Index i = 0; i < a.rows; ++i) {
      Index cnt = 0;
      for (Index k = a.ptr[i]; k < a.ptr[i + 1]; ++k) {
        const Index j = a.col[k];
        for (Index kk = b.ptr[j]; kk < b.ptr[j + 1]; ++kk) {
          const Index cc = b.col[kk];
          if (mark[cc] != i) { mark[cc] = i; ++cnt; }
        }
      }
      c.ptr[static_cast<size_t>(i) + 1] = cnt;
    }
  }
  for (Index i = 0; i < a.rows; ++i) c.ptr[i + 1] += c.ptr[i];
  c.col.resize(static_cast<size_t>(c.nnz()));
  c.val.resize(static_cast<size_t>(c.nnz()));
#pragma omp parallel if (a.rows >= kParallelRows)
  {
    std::vector<Index> mark(static_cast<size_t>(b.cols), -1);
    Vec acc(static_cast<size_t>(b.cols), 0.0);
    std::vector<Index> cols;
#pragma omp for schedule(static)
    for (Index i = 0; i < a.rows; ++i) {
      cols.clear();
      for (Index k = a.ptr[i]; k < a.ptr[i + 1]; ++k) {
        const Index j = a.col[k];
        const double av = a.val[k];
        for (Index kk = b.ptr[j]; kk < b.ptr[j + 1]; ++kk) {
          const Index cc = b.col[kk];
          if (mark[cc] != i) {
            mark[cc] = i;
            acc[cc] = av * b.val[kk];
            cols.push_back(cc);
          } else {
            acc[cc] += av * b.val[kk];
          }
        }
      }
      std::sort(cols.begin(), cols.end());
      Index p = c.ptr[i];
      for (Index cc : cols) { c.col[p] = cc; c.val[p] = acc[cc]; ++p; }
    }
  }
  return c;
}

// C = A B into C's existing pattern, summed in the same order as multiply().
void multiply_numeric(const View& a, const View& b, Csr& c) {
#pragma omp parallel if (a.rows >= kParallelRows)
  {
    std::vector<Index> slot(static_cast<size_t>(b.cols), 0);
#pragma omp for schedule(static)
    for (Index i = 0; i < a.rows; ++i) {
      for (Index p = c.ptr[i]; p < c.ptr[i + 1]; ++p) { slot[c.col[p]] = p; c.val[p] = 0.0; }
      for (Index k = a.ptr[i]; k < a.ptr[i + 1]; ++k) {
        const Index j = a.col[k];
        const double av = a.val[k];
        for (Index kk = b.ptr[j]; kk < b.ptr[j + 1]; ++kk) c.val[slot[b.col[kk]]] += av * b.val[kk];
      }
    }
  }
}

Csr transpose(const View& a) {
  Csr t;
  t.rows = a.cols;
  t.cols = a.rows;
  t.ptr.assign(static_cast<size_t>(a.cols) + 1, 0);
  for (Index k = 0; k < a.nnz(); ++k) ++t.ptr[a.col[k] + 1];
  for (Index j = 0; j < a.cols; ++j) t.ptr[j + 1] += t.ptr[j];
  t.col.resize(static_cast<size_t>(a.nnz()));
  t.val.resize(static_cast<size_t>(a.nnz()));
  std::vector<Index> next(t.ptr.begin(), t.ptr.end() - 1);
  for (Index i = 0; i < a.rows; ++i)
    for (Index k = a.ptr[i]; k < a.ptr[i + 1]; ++k) {
      const Index p = next[a.col[k]]++;
      t.col[p] = i;
      t.val[p] = a.val[k];
    }
  return t;
}

Csr symmetrize(const Csr& a) {
  const Csr t = transpose(view(a));
  Csr s;
  s.rows = a.rows;
  s.cols = a.cols;
  s.ptr.assign(static_cast<size_t>(a.rows) + 1, 0);
  s.col.reserve(static_cast<size_t>(a.nnz()));
  s.val.reserve(static_cast<size_t>(a.nnz()));
  const Index big = std::numeric_limits<Index>::max();
  for (Index i = 0; i < a.rows; ++i) {
    Index p = a.ptr[i], q = t.ptr[i];
    const Index pe = a.ptr[i + 1], qe = t.ptr[i + 1];
    while (p < pe || q < qe) {
      const Index cp = p < pe ? a.col[p] : big;
      const Index cq = q < qe ? t.col[q] : big;
      if (cp == cq) {
        s.col.push_back(cp);
        s.val.push_back(0.5 * (a.val[p] + t.val[q]));
        ++p; ++q;
      } else if (cp < cq) {
        s.col.push_back(cp);
        s.val.push_back(0.5 * a.val[p]);
        ++p;
      } else {
        s.col.push_back(cq);
        s.val.push_back(0.5 * t.val[q]);
        ++q;
      }
    }
    s.ptr[i + 1] = static_cast<Index>(s.col.size());
  }
  return s;
}

// Largest eigenvalue of the symmetric tridiagonal matrix (diag a, off b) by
// Sturm-sequence bisection on the Gershgorin interval.
double tridiagonal_max_eigenvalue(const Vec& a, const Vec& b) {
  const size_t k = a.size();
  if (k == 1) return a[0];
  double lo = std::numeric_limits<double>::max(), hi = -lo;
  for (size_t i = 0; i < k; ++i) {
    double r = 0.0;
    if (i > 0) r += std::abs(b[i - 1]);
    if (i + 1 < k) r += std::abs(b[i]);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  // count of eigenvalues < x
  auto below = [&](double x) {
    int cnt = 0;
    double d = 1.0;
    for (size_t i = 0; i < k; ++i) {
      const double off = i > 0 ? b[i - 1] * b[i - 1] : 0.0;
      d = (a[i] - x) - (i > 0 ? off / d : 0.0);
      if (d == 0.0) d = -1e-300;
      if (d < 0.0) ++cnt;
    }
    return cnt;
  };
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (below(mid) == static_cast<int>(k)) hi = mid; else lo = mid;
  }
  return 0.5 * (lo + hi);
}

double lanczos_lambda_max(const View& a, const Vec& inv_diag, int steps) {
  const Index n = a.rows;
  if (n == 0) return 0.0;
  Vec s(static_cast<size_t>(n));
  for (Index i = 0; i < n; ++i) s[i] = std::sqrt(inv_diag[i]);
  Vec v(static_cast<size_t>(n)), vp(static_cast<size_t>(n), 0.0), w(static_cast<size_t>(n)),
      tmp(static_cast<size_t>(n));
  for (Index i = 0; i < n; ++i) v[i] = 1.0 + 0.5 * std::sin(1.7 * static_cast<double>(i) + 0.3);
  {
    const double nv = std::sqrt(dot(v.data(), v.data(), n));
    for (auto& e : v) e /= nv;
  }
  Vec alpha, beta;
  const int m = std::max(1, std::min<int>(steps, static_cast<int>(n)));
  for (int j = 0; j < m; ++j) {
    for (Index i = 0; i < n; ++i) tmp[i] = s[i] * v[i];
    spmv(a, tmp.data(), w.data());
    for (Index i = 0; i < n; ++i) w[i] *= s[i];
    if (j > 0) {
      const double bb = beta.back();
      for (Index i = 0; i < n; ++i) w[i] -= bb * vp[i];
    }
    const double aj = dot(w.data(), v.data(), n);
    alpha.push_back(aj);
    for (Index i = 0; i < n; ++i) w[i] -= aj * v[i];
    const double bj = std::sqrt(dot(w.data(), w.data(), n));
    if (j + 1 == m || !(bj > 1.0e-12 * std::abs(aj))) break;
    beta.push_back(bj);
    vp = v;
    for (Index i = 0; i < n; ++i) v[i] = w[i] / bj;
  }
  Vec off(beta.begin(), beta.begin() + static_cast<long>(alpha.size() - 1));
  return tridiagonal_max_eigenvalue(alpha, off);
}

// ---------------------------------------------------------------------------
// Dense helpers: pivoted Householder QR and pivoted LDL^T
// ---------------------------------------------------------------------------
// Column-major m x n matrix.
struct Dense {
  Index rows = 0, cols = 0;
  Vec a;
  Dense() = default;
  Dense(Index r, Index c) : rows(r), cols(c), a(static_cast<size_t>(r) * c, 0.0) {}
  double& operator()(Index i, Index j) { return a[static_cast<size_t>(j) * rows + i]; }
  double operator()(Index i, Index j) const { return a[static_cast<size_t>(j) * rows + i]; }
};

// Householder QR with column pivoting.  Returns the first `rank` columns of
// Q and R * P^T (rank x cols), with rank decided as the reference does
// (Multigrid.cpp:617-628): |R_ii| > 1e-10 |R_00|, at least 1.
void pivoted_qr(const Dense& block, Dense& q, Dense& r_out) {
  const Index m = block.rows, n = block.cols;
  Dense a = block;
  const Index size = std::min(m, n);
  Vec hcoef(static_cast<size_t>(size), 0.0);
  std::vector<Index> perm(static_cast<size_t>(n));
  std::iota(perm.begin(), perm.end(), 0);
  Vec norm_upd(static_cast<size_t>(n)), norm_dir(static_cast<size_t>(n));
  for (Index j = 0; j < n; ++j) {
    double s = 0.0;
    for (Index i = 0; i < m; ++i) s += a(i, j) * a(i, j);
    norm_upd[j] = norm_dir[j] = std::sqrt(s);
  }
  const double downdate_threshold = std::sqrt(std::numeric_limits<double>::epsilon());
  for (Index k = 0; k < size; ++k) {
    Index best = k;
    for (Index j = k + 1; j < n; ++j) if (norm_upd[j] > norm_upd[best]) best = j;
    if (best != k) {
      for (Index i = 0; i < m; ++i) std::swap(a(i, k), a(i, best));
      std::swap(norm_upd[k], norm_upd[best]);
      std::swap(norm_dir[k], norm_dir[best]);
      std::swap(perm[k], perm[best]);
    }
    // Householder vector of column k below the diagonal.
    const double c0 = a(k, k);
    double tail = 0.0;
    for (Index i = k + 1; i < m; ++i) tail += a(i, k) * a(i, k);
    double beta, tau;
    if (tail <= std::numeric_limits<double>::min()) {
      tau = 0.0;
      beta = c0;
      for (Index i = k + 1; i < m; ++i) a(i, k) = 0.0;
    } else {
      beta = std::sqrt(c0 * c0 + tail);
      if (c0 >= 0.0) beta = -beta;
      const double inv = 1.0 / (c0 - beta);
      for (Index i = k + 1; i < m; ++i) a(i, k) *= inv;
      tau = (beta - c0) / beta;
    }
    hcoef[k] = tau;
    a(k, k) = beta;
    // Apply H = I - tau v v^T (v = [1; a(k+1:, k)]) to the trailing columns.
    if (tau != 0.0) {
      for (Index j = k + 1; j < n; ++j) {
        double t = a(k, j);
        for (Index i = k + 1; i < m; ++i) t += a(i, k) * a(i, j);
        a(k, j) -= tau * t;
        for (Index i = k + 1; i < m; ++i) a(i, j) -= tau * a(i, k) * t;
      }
    }
    // Norm downdating (LAWN 176) with direct recomputation when inaccurate.
    for (Index j = k + 1; j < n; ++j) {
      if (norm_upd[j] != 0.0) {
        double t = std::abs(a(k, j)) / norm_upd[j];
        t = (1.0 + t) * (1.0 - t);
        if (t < 0.0) t = 0.0;
        const double ratio = norm_upd[j] / norm_dir[j];
        const double t2 = t * ratio * ratio;
        if (t2 <= downdate_threshold) {
          double s = 0.0;
          for (Index i = k + 1; i < m; ++i) s += a(i, j) * a(i, j);
          norm_dir[j] = std::sqrt(s);
          norm_upd[j] = norm_dir[j];
        } else {
          norm_upd[j] *= std::sqrt(t);
        }
      }
    }
  }
  const Index kmax = std::min(m, n);
  const double lead = kmax > 0 ? std::abs(a(0, 0)) : 0.0;
  Index rank = 0;
  for (Index i = 0; i < kmax; ++i) if (std::abs(a(i, i)) > 1.0e-10 * lead) ++rank;
  rank = std::max<Index>(rank, 1);
  // Q = H_0 H_1 ... H_{size-1} applied to the first `rank` identity columns.
  q = Dense(m, rank);
  for (Index j = 0; j < rank; ++j) q(j, j) = 1.0;
  for (Index k = size - 1; k >= 0; --k) {
    const double tau = hcoef[k];
    if (tau == 0.0) continue;
    for (Index j = 0; j < rank; ++j) {
      double t = q(k, j);
      for (Index i = k + 1; i < m; ++i) t += a(i, k) * q(i, j);
      q(k, j) -= tau * t;
      for (Index i = k + 1; i < m; ++i) q(i, j) -= tau * a(i, k) * t;
    }
  }
  r_out = Dense(rank, n);
  for (Index i = 0; i < rank; ++i)
    for (Index k = 0; k < n; ++k) {
      const double v = (k >= i && i < m) ? a(i, k) : 0.0;
      r_out(i, perm[k]) = v;
    }
}

// LDL^T with symmetric diagonal pivoting (largest remaining |diagonal|).
struct Ldlt {
  Index n = 0;
  Dense lu;                 // unit lower factor below the diagonal, D on it
  std::vector<Index> perm;  // row i of the pivoted matrix = original row perm[i]
  Vec d;
  bool ok = true;
  void compute(const Dense& a) {
    n = a.rows;
    lu = a;
    perm.resize(static_cast<size_t>(n));
    std::iota(perm.begin(), perm.end(), 0);
    d.assign(static_cast<size_t>(n), 0.0);
    ok = true;
    Vec w(static_cast<size_t>(n));
    // Only the lower triangle is referenced.
    for (Index k = 0; k < n; ++k) {
      Index piv = k;
      double big = std::abs(lu(k, k));
      for (Index i = k + 1; i < n; ++i)
        if (std::abs(lu(i, i)) > big) { big = std::abs(lu(i, i)); piv = i; }
      if (piv != k) {
        // symmetric interchange of k and piv in the lower triangle
        for (Index j = 0; j < k; ++j) std::swap(lu(k, j), lu(piv, j));
        std::swap(lu(k, k), lu(piv, piv));
        for (Index i = k + 1; i < piv; ++i) std::swap(lu(i, k), lu(piv, i));
        for (Index i = piv + 1; i < n; ++i) std::swap(lu(i, k), lu(i, piv));
        std::swap(perm[k], perm[piv]);
      }
      const double dk = lu(k, k);
      d[k] = dk;
      if (dk == 0.0 || !std::isfinite(dk)) { ok = false; continue; }
      for (Index i = k + 1; i < n; ++i) w[i] = lu(i, k);
      for (Index i = k + 1; i < n; ++i) lu(i, k) = w[i] / dk;
      for (Index j = k + 1; j < n; ++j) {
        const double wj = w[j];
        for (Index i = j; i < n; ++i) lu(i, j) -= lu(i, k) * wj;
      }
    }
  }
  void solve(const double* b, double* x) const {
    Vec y(static_cast<size_t>(n));
    for (Index i = 0; i < n; ++i) y[i] = b[perm[i]];
    for (Index i = 0; i < n; ++i) {
      double s = y[i];
      for (Index j = 0; j < i; ++j) s -= lu(i, j) * y[j];
      y[i] = s;
    }
    for (Index i = 0; i < n; ++i) y[i] /= d[i];
    for (Index i = n - 1; i >= 0; --i) {
      double s = y[i];
      for (Index j = i + 1; j < n; ++j) s -= lu(j, i) * y[j];
      y[i] = s;
    }
    for (Index i = 0; i < n; ++i) x[perm[i]] = y[i];
  }
};

// ---------------------------------------------------------------------------
// SA-AMG (Multigrid.cpp:334-1111)
// ---------------------------------------------------------------------------
struct AmgOptions {
  double theta = 0.02;
  int max_levels = 12;
  Index coarse_size = 1500;
  int degree = 3;
  double cheb_ratio = 30.0;
  double damping = 4.0 / 3.0;
  int lanczos_steps = 12;
  double pivot_tol = 1.0e-13;
  bool reuse = true;
};

struct Layout {
  int dim = 0, ndpn = 0;
  const double* coords = nullptr;  // dim x num_nodes
  Index num_nodes = 0;
  const Index* unknowns = nullptr;
  Index n = 0;
};

struct Level {
  Csr owned;
  View a;
  Vec inv_diag;
  double lambda = 0.0;
  Index num_nodes = 0;
  std::vector<Index> node_ptr;
  Dense nullspace;  // n x m
  std::vector<Index> aggregate;
  Csr p_tent, p, r, ap, raw;
  mutable Vec x, b, res, d;
};

struct Amg {
  AmgOptions opt;
  std::vector<Level> levels;
  Ldlt coarse;
  bool ready = false;
  Index fp_rows = -1, fp_nnz = -1;
  const Index* fp_unknowns = nullptr;
  Index fp_unknowns_n = -1;
  double op_complexity = 0.0, pivot_ratio = 0.0;
  bool reused = false;

  void finest_nodes(const Layout& lay) {
    Level& lvl = levels.front();
    lvl.node_ptr.clear();
    lvl.node_ptr.push_back(0);
    Index prev = -1;
    for (Index i = 0; i < lay.n; ++i) {
      const Index g = lay.unknowns[i];
      const Index node = g / lay.ndpn;
      if (node >= lay.num_nodes || g < 0) {
        std::ostringstream os;
        os << "multigrid: unknown " << i << " maps to DOF " << g << ", outside the model's "
           << lay.num_nodes << " nodes";
        throw Error(kBadInput, os.str());
      }
      if (i > 0 && g <= lay.unknowns[i - 1])
        throw Error(kBadInput, "multigrid: the DOF layout must list unknowns in ascending order");
      if (node != prev) {
        if (i > 0) lvl.node_ptr.push_back(i);
        prev = node;
      }
    }
    lvl.node_ptr.push_back(lay.n);
    lvl.num_nodes = static_cast<Index>(lvl.node_ptr.size()) - 1;
    double lo[3] = {1e308, 1e308, 1e308}, hi[3] = {-1e308, -1e308, -1e308};
    for (Index c = 0; c < lay.num_nodes; ++c)
      for (int d = 0; d < 3; ++d) {
        const double x = d < lay.dim ? lay.coords[static_cast<size_t>(c) * lay.dim + d] : 0.0;
        lo[d] = std::min(lo[d], x);
        hi[d] = std::max(hi[d], x);
      }
    double centre[3], scale = 0.0;
    for (int d = 0; d < 3; ++d) {
      centre[d] = 0.5 * (lo[d] + hi[d]);
      scale = std::max(scale, hi[d] - lo[d]);
    }
    scale = std::max(scale, 1.0e-300);
    const int m = lay.dim == 2 ? 3 : 6;
    lvl.nullspace = Dense(lay.n, m);
    for (Index i = 0; i < lay.n; ++i) {
      const Index g = lay.unknowns[i];
      const Index node = g / lay.ndpn;
      const int k = static_cast<int>(g % lay.ndpn);
      double r[3];
      for (int d = 0; d < 3; ++d) {
        const double x = d < lay.dim ? lay.coords[static_cast<size_t>(node) * lay.dim + d] : 0.0;
        r[d] = (x - centre[d]) / scale;
      }
      lvl.nullspace(i, k) = 1.0;
      if (lay.dim == 2) {
        lvl.nullspace(i, 2) = k == 0 ? -r[1] : r[0];
      } else {
        // rotations about x, y, z: u = e_axis x r
        const double rx[3] = {0.0, -r[2], r[1]};
        const double ry[3] = {r[2], 0.0, -r[0]};
        const double rz[3] = {-r[1], r[0], 0.0};
        lvl.nullspace(i, 3) = rx[k];
        lvl.nullspace(i, 4) = ry[k];
        lvl.nullspace(i, 5) = rz[k];
      }
    }
  }

  void aggregate_level(Level& lvl) const {
    const View& a = lvl.a;
    const Index nn = lvl.num_nodes;
    std::vector<Index> node_of(static_cast<size_t>(a.rows));
    for (Index node = 0; node < nn; ++node)
      for (Index i = lvl.node_ptr[node]; i < lvl.node_ptr[node + 1]; ++i) node_of[i] = node;
    Vec bdiag(static_cast<size_t>(nn), 0.0);
    for (Index node = 0; node < nn; ++node) {
      double s = 0.0;
      for (Index i = lvl.node_ptr[node]; i < lvl.node_ptr[node + 1]; ++i)
        for (Index k = a.ptr[i]; k < a.ptr[i + 1]; ++k)
          if (node_of[a.col[k]] == node) s += a.val[k] * a.val[k];
      bdiag[node] = std::sqrt(s);
    }
    std::vector<Index> sptr(static_cast<size_t>(nn) + 1, 0), strong;
    Vec sval;
    {
      std::vector<Index> mark(static_cast<size_t>(nn), -1), touched;
      Vec acc(static_cast<size_t>(nn), 0.0);
      for (Index node = 0; node < nn; ++node) {
        touched.clear();
        for (Index i = lvl.node_ptr[node]; i < lvl.node_ptr[node + 1]; ++i)
          for (Index k = a.ptr[i]; k < a.ptr[i + 1]; ++k) {
            const Index o = node_of[a.col[k]];
            if (o == node) continue;
            if (mark[o] != node) { mark[o] = node; acc[o] = 0.0; touched.push_back(o); }
            acc[o] += a.val[k] * a.val[k];
          }
        std::sort(touched.begin(), touched.end());
        const double di = bdiag[node];
        for (Index o : touched) {
          const double s = std::sqrt(acc[o]);
          const double ref = std::sqrt(di * bdiag[o]);
          if (s > 0.0 && s >= opt.theta * ref) {
            strong.push_back(o);
            sval.push_back(ref > 0.0 ? s / ref : 0.0);
          }
        }
        sptr[node + 1] = static_cast<Index>(strong.size());
      }
    }
    std::vector<Index>& agg = const_cast<Level&>(lvl).aggregate;
    agg.assign(static_cast<size_t>(nn), -1);
    Index count = 0;
    for (Index node = 0; node < nn; ++node) {
      if (agg[node] >= 0) continue;
      const Index b = sptr[node], e = sptr[node + 1];
      if (b == e) continue;
      bool free_nb = true;
      for (Index k = b; k < e; ++k) if (agg[strong[k]] >= 0) { free_nb = false; break; }
      if (!free_nb) continue;
      agg[node] = count;
      for (Index k = b; k < e; ++k) agg[strong[k]] = count;
      ++count;
    }
    const std::vector<Index> first = agg;
    for (Index node = 0; node < nn; ++node) {
      if (first[node] >= 0) continue;
      Index best = -1;
      double bv = -1.0;
      for (Index k = sptr[node]; k < sptr[node + 1]; ++k) {
        const Index t = first[strong[k]];
        if (t >= 0 && sval[k] > bv) { best = t; bv = sval[k]; }
      }
      if (best >= 0) agg[node] = best;
    }
    for (Index node = 0; node < nn; ++node) {
      if (agg[node] >= 0) continue;
      agg[node] = count;
      for (Index k = sptr[node]; k < sptr[node + 1]; ++k)
        if (agg[strong[k]] < 0) agg[strong[k]] = count;
      ++count;
    }
  }

  void tentative(Level& lvl, Level& next) const {
    const Index n = lvl.a.rows, nn = lvl.num_nodes;
    const Index m = lvl.nullspace.cols;
    const std::vector<Index>& agg = lvl.aggregate;
    const Index na = agg.empty() ? 0 : *std::max_element(agg.begin(), agg.end()) + 1;
    std::vector<Index> aptr(static_cast<size_t>(na) + 1, 0);
    for (Index node = 0; node < nn; ++node) ++aptr[agg[node] + 1];
    for (Index g = 0; g < na; ++g) aptr[g + 1] += aptr[g];
    std::vector<Index> anodes(static_cast<size_t>(nn));
    {
      std::vector<Index> fill(aptr.begin(), aptr.end() - 1);
      for (Index node = 0; node < nn; ++node) anodes[fill[agg[node]]++] = node;
    }
    std::vector<Dense> q(static_cast<size_t>(na)), r(static_cast<size_t>(na));
#pragma omp parallel for schedule(dynamic, 256) if (na >= 4096)
    for (Index g = 0; g < na; ++g) {
      Index rows = 0;
      for (Index k = aptr[g]; k < aptr[g + 1]; ++k) {
        const Index node = anodes[k];
        rows += lvl.node_ptr[node + 1] - lvl.node_ptr[node];
      }
      Dense block(rows, m);
      Index row = 0;
      for (Index k = aptr[g]; k < aptr[g + 1]; ++k) {
        const Index node = anodes[k];
        for (Index i = lvl.node_ptr[node]; i < lvl.node_ptr[node + 1]; ++i, ++row)
          for (Index j = 0; j < m; ++j) block(row, j) = lvl.nullspace(i, j);
      }
      pivoted_qr(block, q[g], r[g]);
    }
    next.node_ptr.assign(static_cast<size_t>(na) + 1, 0);
    for (Index g = 0; g < na; ++g) next.node_ptr[g + 1] = next.node_ptr[g] + q[g].cols;
    next.num_nodes = na;
    const Index nc = next.node_ptr.back();
    next.nullspace = Dense(nc, m);
    for (Index g = 0; g < na; ++g)
      for (Index i = 0; i < r[g].rows; ++i)
        for (Index j = 0; j < m; ++j) next.nullspace(next.node_ptr[g] + i, j) = r[g](i, j);
    Csr& pt = lvl.p_tent;
    pt.rows = n;
    pt.cols = nc;
    pt.ptr.assign(static_cast<size_t>(n) + 1, 0);
    std::vector<Index> agg_of(static_cast<size_t>(n)), local(static_cast<size_t>(n));
    for (Index g = 0; g < na; ++g) {
      Index loc = 0;
      for (Index k = aptr[g]; k < aptr[g + 1]; ++k) {
        const Index node = anodes[k];
        for (Index i = lvl.node_ptr[node]; i < lvl.node_ptr[node + 1]; ++i) {
          agg_of[i] = g;
          local[i] = loc++;
        }
      }
    }
    for (Index i = 0; i < n; ++i) pt.ptr[i + 1] = pt.ptr[i] + q[agg_of[i]].cols;
    pt.col.resize(static_cast<size_t>(pt.nnz()));
    pt.val.resize(static_cast<size_t>(pt.nnz()));
    for (Index i = 0; i < n; ++i) {
      const Index g = agg_of[i];
      Index p = pt.ptr[i];
      for (Index j = 0; j < q[g].cols; ++j, ++p) {
        pt.col[p] = next.node_ptr[g] + j;
        pt.val[p] = q[g](local[i], j);
      }
    }
  }

  void smooth_prolongator(Level& lvl, bool numeric_only) const {
    const double omega = opt.damping / lvl.lambda;
    Csr ap;
    if (numeric_only) {
      ap = std::move(lvl.p);
      multiply_numeric(lvl.a, view(lvl.p_tent), ap);
    } else {
      ap = multiply(lvl.a, view(lvl.p_tent));
    }
    const Csr& pt = lvl.p_tent;
#pragma omp parallel for schedule(static) if (ap.rows >= kParallelRows)
    for (Index i = 0; i < ap.rows; ++i) {
      const double sc = omega * lvl.inv_diag[i];
      for (Index k = ap.ptr[i]; k < ap.ptr[i + 1]; ++k) ap.val[k] *= -sc;
      for (Index kk = pt.ptr[i]; kk < pt.ptr[i + 1]; ++kk) {
        const Index c = pt.col[kk];
        const Index* b = ap.col.data() + ap.ptr[i];
        const Index* e = ap.col.data() + ap.ptr[i + 1];
        const Index* hit = std::lower_bound(b, e, c);
        ap.val[hit - ap.col.data()] += pt.val[kk];
      }
    }
    lvl.p = std::move(ap);
    if (numeric_only) {
      Csr& r = lvl.r;
      std::vector<Index> next(r.ptr.begin(), r.ptr.end() - 1);
      for (Index i = 0; i < lvl.p.rows; ++i)
        for (Index k = lvl.p.ptr[i]; k < lvl.p.ptr[i + 1]; ++k) r.val[next[lvl.p.col[k]]++] = lvl.p.val[k];
    } else {
      lvl.r = transpose(view(lvl.p));
    }
  }

  void numeric_level(size_t l) {
    Level& lvl = levels[l];
    const View& a = lvl.a;
    lvl.inv_diag.assign(static_cast<size_t>(a.rows), 0.0);
    for (Index i = 0; i < a.rows; ++i) {
      double d = 0.0;
      for (Index k = a.ptr[i]; k < a.ptr[i + 1]; ++k) if (a.col[k] == i) d += a.val[k];
      if (!(d > 0.0)) {
        std::ostringstream os;
        os << "multigrid level " << l << ": diagonal entry " << i << " is " << d
           << "; a stiffness matrix must have a positive diagonal";
        throw Error(kBreakdown, os.str());
      }
      lvl.inv_diag[i] = 1.0 / d;
    }
    lvl.lambda = lanczos_lambda_max(a, lvl.inv_diag, opt.lanczos_steps);
    if (!(lvl.lambda > 0.0) || !std::isfinite(lvl.lambda)) {
      std::ostringstream os;
      os << "multigrid level " << l << ": the spectral estimate of D^-1 A is " << lvl.lambda
         << "; the matrix is not positive definite";
      throw Error(kBreakdown, os.str());
    }
    lvl.x.assign(static_cast<size_t>(a.rows), 0.0);
    lvl.b.assign(static_cast<size_t>(a.rows), 0.0);
    lvl.res.assign(static_cast<size_t>(a.rows), 0.0);
    lvl.d.assign(static_cast<size_t>(a.rows), 0.0);
  }

  void coarse_factorize(const Level& lvl) {
    const Index n = lvl.a.rows;
    Dense dense(n, n);
    for (Index i = 0; i < n; ++i)
      for (Index k = lvl.a.ptr[i]; k < lvl.a.ptr[i + 1]; ++k) dense(i, lvl.a.col[k]) = lvl.a.val[k];
    coarse.compute(dense);
    double mx = 0.0, mn = std::numeric_limits<double>::max();
    for (double v : coarse.d) { mx = std::max(mx, std::abs(v)); mn = std::min(mn, v); }
    const double ratio = mx > 0.0 ? mn / mx : 0.0;
    pivot_ratio = ratio;
    if (!coarse.ok || !(ratio > opt.pivot_tol)) {
      std::ostringstream os;
      os << "multigrid: the coarsest operator (" << n << " unknowns) is singular or indefinite "
         << "(smallest / largest pivot " << ratio << "). A rigid-body mode survived to the "
         << "coarse level, so the model is under-constrained";
      throw Error(kUnderConstrained, os.str());
    }
  }

  void smooth(const Level& lvl, bool zero_guess) const {
    const View& a = lvl.a;
    const Index n = a.rows;
    Vec& x = lvl.x;
    const Vec& b = lvl.b;
    const double upper = 1.1 * lvl.lambda, lower = upper / opt.cheb_ratio;
    const double theta = 0.5 * (upper + lower), delta = 0.5 * (upper - lower);
    const double sigma = theta / delta;
    double rho = 1.0 / sigma;
    Vec& r = lvl.res;
    Vec& d = lvl.d;
    if (zero_guess) {
      std::fill(x.begin(), x.end(), 0.0);
      r = b;
    } else {
      residual(a, x.data(), b.data(), r.data());
    }
    const Vec& dinv = lvl.inv_diag;
#pragma omp parallel for schedule(static) if (n >= kParallelRows)
    for (Index i = 0; i < n; ++i) {
      d[i] = dinv[i] * r[i] / theta;
      x[i] += d[i];
    }
    for (int k = 1; k < opt.degree; ++k) {
#pragma omp parallel for schedule(static) if (n >= kParallelRows)
      for (Index i = 0; i < n; ++i) {
        double s = 0.0;
        for (Index kk = a.ptr[i]; kk < a.ptr[i + 1]; ++kk) s += a.val[kk] * d[a.col[kk]];
        r[i] -= s;
      }
      const double rho_new = 1.0 / (2.0 * sigma - rho);
      const double c1 = rho_new * rho, c2 = 2.0 * rho_new / delta;
#pragma omp parallel for schedule(static) if (n >= kParallelRows)
      for (Index i = 0; i < n; ++i) {
        d[i] = c1 * d[i] + c2 * dinv[i] * r[i];
        x[i] += d[i];
      }
      rho = rho_new;
    }
  }

  void cycle(size_t l) const {
    const Level& lvl = levels[l];
    if (l + 1 == levels.size()) {
      coarse.solve(lvl.b.data(), lvl.x.data());
      return;
    }
    smooth(lvl, true);
    residual(lvl.a, lvl.x.data(), lvl.b.data(), lvl.res.data());
    const Level& next = levels[l + 1];
    spmv(view(lvl.r), lvl.res.data(), next.b.data());
    cycle(l + 1);
    const Csr& p = lvl.p;
#pragma omp parallel for schedule(static) if (p.rows >= kParallelRows)
    for (Index i = 0; i < p.rows; ++i) {
      double s = 0.0;
      for (Index k = p.ptr[i]; k < p.ptr[i + 1]; ++k) s += p.val[k] * next.x[p.col[k]];
      lvl.x[i] += s;
    }
    smooth(lvl, false);
  }

  void apply(const double* r, double* z) const {
    const Level& f = levels.front();
    std::copy(r, r + f.a.rows, f.b.begin());
    cycle(0);
    std::copy(f.x.begin(), f.x.end(), z);
  }

  void setup(const View& a, const Layout& lay) {
    if (a.rows != a.cols || a.rows == 0)
      throw Error(kBadInput, "multigrid: the system matrix must be square and non-empty");
    if (lay.dim != 2 && lay.dim != 3)
      throw Error(kBadInput, "multigrid: the DOF layout must be two- or three-dimensional");
    if (lay.ndpn != lay.dim)
      throw Error(kBadInput, "multigrid: only translational DOF layouts are supported");
    if (lay.unknowns == nullptr || lay.n != a.rows) {
      std::ostringstream os;
      os << "multigrid: the DOF layout lists " << lay.n << " unknowns for a matrix of " << a.rows
         << " rows";
      throw Error(kBadInput, os.str());
    }
    const Index n = a.rows;
    const bool same = ready && fp_rows == n && fp_nnz == a.nnz() && fp_unknowns == lay.unknowns &&
                      fp_unknowns_n == lay.n;
    const bool reuse = opt.reuse && same;
    if (!same) {
      double mx = 0.0;
      for (Index k = 0; k < a.nnz(); ++k) mx = std::max(mx, std::abs(a.val[k]));
      for (Index i = 0; i < n; ++i)
        for (Index k = a.ptr[i]; k < a.ptr[i + 1]; ++k) {
          const Index j = a.col[k];
          const Index* b = a.col + a.ptr[j];
          const Index* e = a.col + a.ptr[j + 1];
          const Index* hit = std::lower_bound(b, e, i);
          const double other = (hit != e && *hit == i) ? a.val[hit - a.col] : 0.0;
          if (std::abs(other - a.val[k]) > 1.0e-10 * mx) {
            std::ostringstream os;
            os << "multigrid: the system matrix is not symmetric (entry (" << i << ", " << j
               << ") = " << a.val[k] << " but (" << j << ", " << i << ") = " << other << ")";
            throw Error(kBadInput, os.str());
          }
        }
    }
    for (Index k = 0; k < a.nnz(); ++k)
      if (!std::isfinite(a.val[k])) throw Error(kNonFinite, "multigrid: the system matrix has a non-finite entry");
    if (!reuse) {
      levels.clear();
      levels.reserve(static_cast<size_t>(opt.max_levels) + 1);
      levels.emplace_back();
      finest_nodes(lay);
    }
    levels.front().a = a;
    size_t l = 0;
    const size_t reused_levels = levels.size();
    while (true) {
      Level& lvl = levels[l];
      numeric_level(l);
      const bool last_reused = reuse && l + 1 == reused_levels;
      const bool stop = reuse ? last_reused
                              : (lvl.a.rows <= opt.coarse_size || static_cast<int>(l) + 1 >= opt.max_levels);
      if (stop) break;
      if (!reuse) {
        aggregate_level(lvl);
        Level next;
        tentative(lvl, next);
        const Index nc = next.node_ptr.back();
        if (nc >= static_cast<Index>(0.85 * static_cast<double>(lvl.a.rows)) || nc == 0) {
          lvl.aggregate.clear();
          lvl.p_tent = Csr();
          break;
        }
        levels.push_back(std::move(next));
      }
      Level& cur = levels[l];
      smooth_prolongator(cur, reuse);
      Level& co = levels[l + 1];
      if (reuse) {
        multiply_numeric(cur.a, view(cur.p), cur.ap);
        multiply_numeric(view(cur.r), view(cur.ap), cur.raw);
      } else {
        cur.ap = multiply(cur.a, view(cur.p));
        cur.raw = multiply(view(cur.r), view(cur.ap));
      }
      co.owned = symmetrize(cur.raw);
      co.a = view(co.owned);
      ++l;
    }
    levels.resize(l + 1);
    coarse_factorize(levels.back());
    fp_rows = n;
    fp_nnz = a.nnz();
    fp_unknowns = lay.unknowns;
    fp_unknowns_n = lay.n;
    ready = true;
    reused = reuse;
    double nz = 0.0;
    for (const Level& lv : levels) nz += lv.a.nnz();
    op_complexity = nz / static_cast<double>(levels.front().a.nnz());
  }
};

struct PcgResult {
  int iterations = 0;
  double relres = 0.0;
  bool converged = false;
};

PcgResult pcg(const View& a, const double* b, double* x, const Amg& m, double tol, int maxit) {
  const Index n = a.rows;
  PcgResult res;
  const double bnorm = std::sqrt(dot(b, b, n));
  if (bnorm == 0.0) {
    std::fill(x, x + n, 0.0);
    res.converged = true;
    return res;
  }
  const double target = tol * bnorm;
  Vec r(static_cast<size_t>(n)), z(static_cast<size_t>(n)), p(static_cast<size_t>(n)),
      q(static_cast<size_t>(n));
  int total = 0;
  bool rec_conv = false;
  double best = std::numeric_limits<double>::max();
  for (int restart = 0; restart < 3; ++restart) {
    residual(a, x, b, r.data());
    double rnorm = std::sqrt(dot(r.data(), r.data(), n));
    res.relres = rnorm / bnorm;
    if (rnorm <= target) { res.converged = true; break; }
    m.apply(r.data(), z.data());
    p = z;
    double rz = dot(r.data(), z.data(), n);
    bool conv = false;
    while (total < maxit) {
      spmv(a, p.data(), q.data());
      const double pq = dot(p.data(), q.data(), n);
      if (!(pq > 0.0) || !std::isfinite(pq)) {
        std::ostringstream os;
        os << "preconditioned CG broke down at iteration " << total + 1 << " (p^T A p = " << pq
           << "): the stiffness matrix or the multigrid preconditioner is not positive definite";
        throw Error(kBreakdown, os.str());
      }
      const double alpha = rz / pq;
#pragma omp parallel for schedule(static) if (n >= kParallelRows)
      for (Index i = 0; i < n; ++i) {
        x[i] += alpha * p[i];
        r[i] -= alpha * q[i];
      }
      ++total;
      rnorm = std::sqrt(dot(r.data(), r.data(), n));
      if (rnorm <= target) { conv = true; break; }
      m.apply(r.data(), z.data());
      const double rzn = dot(r.data(), z.data(), n);
      const double beta = rzn / rz;
      rz = rzn;
#pragma omp parallel for schedule(static) if (n >= kParallelRows)
      for (Index i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
    residual(a, x, b, r.data());
    res.relres = std::sqrt(dot(r.data(), r.data(), n)) / bnorm;
    if (res.relres <= tol) { res.converged = true; break; }
    if (!conv) break;
    rec_conv = true;
    if (!(res.relres < 0.5 * best)) break;
    best = res.relres;
  }
  if (!res.converged && rec_conv) res.converged = true;
  res.iterations = total;
  return res;
}

// ---------------------------------------------------------------------------
// Structured model: mesh, element matrix, pattern, scatter, reduction
// ---------------------------------------------------------------------------
void element_stiffness(int dim, double hx, double hy, double hz, double young, double nu,
                       double thick, double* ke) {
  const double g = 1.0 / std::sqrt(3.0);
  const double gp[2] = {-g, g};
  if (dim == 2) {
    const double xy[4][2] = {{0, 0}, {hx, 0}, {hx, hy}, {0, hy}};
    const double f = young / (1.0 - nu * nu);
    const double D[3][3] = {{f, f * nu, 0}, {f * nu, f, 0}, {0, 0, f * (1.0 - nu) / 2.0}};
    double k[8][8] = {};
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) {
        const double xi = gp[i], eta = gp[j];
        const double dn[4][2] = {{-0.25 * (1 - eta), -0.25 * (1 - xi)},
                                 {0.25 * (1 - eta), -0.25 * (1 + xi)},
                                 {0.25 * (1 + eta), 0.25 * (1 + xi)},
                                 {-0.25 * (1 + eta), 0.25 * (1 - xi)}};
        double J[2][2] = {};
        for (int a = 0; a < 4; ++a)
          for (int r = 0; r < 2; ++r)
            for (int c = 0; c < 2; ++c) J[r][c] += xy[a][r] * dn[a][c];
        const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const double Ji[2][2] = {{J[1][1] / det, -J[0][1] / det}, {-J[1][0] / det, J[0][0] / det}};
        double B[3][8] = {};
        for (int a = 0; a < 4; ++a) {
          const double dx = dn[a][0] * Ji[0][0] + dn[a][1] * Ji[1][0];
          const double dy = dn[a][0] * Ji[0][1] + dn[a][1] * Ji[1][1];
          B[0][2 * a] = dx;
          B[1][2 * a + 1] = dy;
          B[2][2 * a] = dy;
          B[2][2 * a + 1] = dx;
        }
        const double w = thick * det;
        for (int r = 0; r < 8; ++r)
          for (int c = 0; c < 8; ++c) {
            double s = 0.0;
            for (int p = 0; p < 3; ++p)
              for (int q = 0; q < 3; ++q) s += B[p][r] * D[p][q] * B[q][c];
            k[r][c] += w * s;
          }
      }
    for (int r = 0; r < 8; ++r)
      for (int c = 0; c < 8; ++c) ke[r * 8 + c] = 0.5 * (k[r][c] + k[c][r]);
    return;
  }
  static const double corner[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                      {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  double X[8][3];
  for (int a = 0; a < 8; ++a) {
    X[a][0] = corner[a][0] > 0 ? hx : 0.0;
    X[a][1] = corner[a][1] > 0 ? hy : 0.0;
    X[a][2] = corner[a][2] > 0 ? hz : 0.0;
  }
  const double lam = young * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const double G = young / (2.0 * (1.0 + nu));
  double D[6][6] = {};
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) D[i][j] = lam;
    D[i][i] = lam + 2.0 * G;
    D[3 + i][3 + i] = G;
  }
  std::vector<double> k(24 * 24, 0.0);
  for (int gk = 0; gk < 2; ++gk)
    for (int gj = 0; gj < 2; ++gj)
      for (int gi = 0; gi < 2; ++gi) {
        const double xi = gp[gi], eta = gp[gj], zeta = gp[gk];
        double dn[8][3];
        for (int a = 0; a < 8; ++a) {
          const double fx = 1 + xi * corner[a][0], fy = 1 + eta * corner[a][1], fz = 1 + zeta * corner[a][2];
          dn[a][0] = 0.125 * corner[a][0] * fy * fz;
          dn[a][1] = 0.125 * corner[a][1] * fx * fz;
          dn[a][2] = 0.125 * corner[a][2] * fx * fy;
        }
        double J[3][3] = {};
        for (int a = 0; a < 8; ++a)
          for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) J[r][c] += X[a][r] * dn[a][c];
        const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        double Ji[3][3];
        Ji[0][0] = c00 / det;
        Ji[1][0] = c01 / det;
        Ji[2][0] = c02 / det;
        Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
        Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
        Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
        Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
        Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
        Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
        double B[6][24] = {};
        for (int a = 0; a < 8; ++a) {
          double g3[3];
          for (int c = 0; c < 3; ++c) g3[c] = dn[a][0] * Ji[0][c] + dn[a][1] * Ji[1][c] + dn[a][2] * Ji[2][c];
          const int c = 3 * a;
          B[0][c] = g3[0];
          B[1][c + 1] = g3[1];
          B[2][c + 2] = g3[2];
          B[3][c] = g3[1];
          B[3][c + 1] = g3[0];
          B[4][c + 1] = g3[2];
          B[4][c + 2] = g3[1];
          B[5][c] = g3[2];
          B[5][c + 2] = g3[0];
        }
        double DB[6][24];
        for (int p = 0; p < 6; ++p)
          for (int c = 0; c < 24; ++c) {
            double s = 0.0;
            for (int q = 0; q < 6; ++q) s += D[p][q] * B[q][c];
            DB[p][c] = s;
          }
        for (int r = 0; r < 24; ++r)
          for (int c = 0; c < 24; ++c) {
            double s = 0.0;
            for (int p = 0; p < 6; ++p) s += B[p][r] * DB[p][c];
            k[static_cast<size_t>(r) * 24 + c] += det * s;
          }
      }
  for (int r = 0; r < 24; ++r)
    for (int c = 0; c < 24; ++c) ke[r * 24 + c] = 0.5 * (k[static_cast<size_t>(r) * 24 + c] + k[static_cast<size_t>(c) * 24 + r]);
}

// Consistent mass of one box cell, 3 x 3 (x 3) Gauss (IntegrationOptions::
// mass_points), symmetrised: Quad4Element::consistent_mass
// (src/elements/Quad4.cpp:139-173) and Hex8Element::consistent_mass
// (src/elements/Hex8.cpp:194-214), M_e = sum_g rho t det(J) w_g N^T N.
void element_mass(int dim, double hx, double hy, double hz, double density, double thick,
                  double* me) {
  const double a3 = std::sqrt(3.0 / 5.0);
  const double gx[3] = {-a3, 0.0, a3};
  const double gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
  if (dim == 2) {
    const double xy[4][2] = {{0, 0}, {hx, 0}, {hx, hy}, {0, hy}};
    double m[8][8] = {};
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) {
        const double xi = gx[i], eta = gx[j], w = gw[i] * gw[j];
        const double n[4] = {0.25 * (1 - xi) * (1 - eta), 0.25 * (1 + xi) * (1 - eta),
                             0.25 * (1 + xi) * (1 + eta), 0.25 * (1 - xi) * (1 + eta)};
        const double dn[4][2] = {{-0.25 * (1 - eta), -0.25 * (1 - xi)},
                                 {0.25 * (1 - eta), -0.25 * (1 + xi)},
                                 {0.25 * (1 + eta), 0.25 * (1 + xi)},
                                 {-0.25 * (1 + eta), 0.25 * (1 - xi)}};
        double J[2][2] = {};
        for (int a = 0; a < 4; ++a)
          for (int r = 0; r < 2; ++r)
            for (int c = 0; c < 2; ++c) J[r][c] += xy[a][r] * dn[a][c];
        const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const double f = density * thick * det * w;
        for (int a = 0; a < 4; ++a)
          for (int b = 0; b < 4; ++b)
            for (int k = 0; k < 2; ++k) m[2 * a + k][2 * b + k] += f * (n[a] * n[b]);
      }
    for (int r = 0; r < 8; ++r)
      for (int c = 0; c < 8; ++c) me[r * 8 + c] = 0.5 * (m[r][c] + m[c][r]);
    return;
  }
  static const double corner[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                      {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  double X[8][3];
  for (int a = 0; a < 8; ++a) {
    X[a][0] = corner[a][0] > 0 ? hx : 0.0;
    X[a][1] = corner[a][1] > 0 ? hy : 0.0;
    X[a][2] = corner[a][2] > 0 ? hz : 0.0;
  }
  std::vector<double> m(24 * 24, 0.0);
  for (int gk = 0; gk < 3; ++gk)
    for (int gj = 0; gj < 3; ++gj)
      for (int gi = 0; gi < 3; ++gi) {
        const double xi = gx[gi], eta = gx[gj], zeta = gx[gk], w = gw[gi] * gw[gj] * gw[gk];
        double n[8], dn[8][3];
        for (int a = 0; a < 8; ++a) {
          const double fx = 1 + xi * corner[a][0], fy = 1 + eta * corner[a][1], fz = 1 + zeta * corner[a][2];
          n[a] = 0.125 * fx * fy * fz;
          dn[a][0] = 0.125 * corner[a][0] * fy * fz;
          dn[a][1] = 0.125 * corner[a][1] * fx * fz;
          dn[a][2] = 0.125 * corner[a][2] * fx * fy;
        }
        double J[3][3] = {};
        for (int a = 0; a < 8; ++a)
          for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) J[r][c] += X[a][r] * dn[a][c];
        const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) +
                           J[0][1] * (J[1][2] * J[2][0] - J[1][0] * J[2][2]) +
                           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        const double f = density * det * w;
        for (int a = 0; a < 8; ++a)
          for (int b = 0; b < 8; ++b)
            for (int k = 0; k < 3; ++k) m[static_cast<size_t>(3 * a + k) * 24 + 3 * b + k] += f * (n[a] * n[b]);
      }
  for (int r = 0; r < 24; ++r)
    for (int c = 0; c < 24; ++c)
      me[r * 24 + c] = 0.5 * (m[static_cast<size_t>(r) * 24 + c] + m[static_cast<size_t>(c) * 24 + r]);
}

struct Problem {
  int dim = 2, npe = 4;
  Index nx = 0, ny = 0, nz = 1;
  double lx = 0, ly = 0, lz = 0;
  Index ne = 0, nn = 0, ndof = 0;
  Vec coords;                 // dim x nn
  std::vector<Index> conn;    // ne x npe
  Vec ke;                     // edofs x edofs, row-major (symmetric)
  int edofs = 0;
  std::vector<Index> free_dofs, reduced;  // reduced[d] = free index or -1
  // Assembler pattern (column-major full K) and free-free reduction map.
  std::vector<Index> outer, inner, block_offset;
  std::vector<Index> ff_ptr, ff_col;
  std::vector<int64_t> ff_src;
  // filter
  bool filter_on = false;
  double radius = 0.0;
  Csr h;       // row-normalised H, CSR sorted by column (the CSC of H^T)
  Csr ht;      // H^T as CSR (= H's CSC)
  Vec row_sums;
  Vec volumes;
  double domain_volume = 0.0;
  // optimisation data
  std::vector<Vec> loads;
  Vec weights;
  double vf = 0.5, x0 = 0.5, penalty = 3, emin = 1e-9, move = 0.2, damping = 0.5;
  double rtol = 1e-8;
  int maxit = 1000;
  bool warm = true;
  AmgOptions amg_opt;
  // Heaviside projection (src/topopt/Projection.cpp) and its beta schedule
  bool proj = false;
  double eta = 0.5, beta_start = 1.0, beta_max = 32.0, beta_factor = 2.0, change_tol = 1e-3;
  int beta_interval = 50;
  bool advance = true;
  double beta = 0.0;
  // robust formulation (Projection.hpp:44-60)
  bool robust = false;
  double robust_delta = 0.1;
  int robust_interval = 1;
  // the objective's projection threshold: the eroded design's in a robust run
  double objective_eta() const { return robust ? eta + robust_delta : eta; }
  std::unique_ptr<Amg> amg;
  std::vector<Vec> previous;
  Layout layout;
};

void build_mesh(Problem& p) {
  const Index nnx = p.nx + 1, nny = p.ny + 1;
  if (p.dim == 2) {
    p.nn = nnx * nny;
    p.ne = p.nx * p.ny;
    p.npe = 4;
    const double dx = p.lx / p.nx, dy = p.ly / p.ny;
    p.coords.resize(static_cast<size_t>(2) * p.nn);
    for (Index j = 0; j < nny; ++j)
      for (Index i = 0; i < nnx; ++i) {
        const Index n = j * nnx + i;
        p.coords[2 * n] = 0.0 + i * dx;
        p.coords[2 * n + 1] = 0.0 + j * dy;
      }
    p.conn.reserve(static_cast<size_t>(p.ne) * 4);
    for (Index j = 0; j < p.ny; ++j)
      for (Index i = 0; i < p.nx; ++i) {
        const Index n0 = j * nnx + i;
        p.conn.insert(p.conn.end(), {n0, n0 + 1, n0 + nnx + 1, n0 + nnx});
      }
  } else {
    const Index nnz = p.nz + 1;
    p.nn = nnx * nny * nnz;
    p.ne = p.nx * p.ny * p.nz;
    p.npe = 8;
    const double dx = p.lx / p.nx, dy = p.ly / p.ny, dz = p.lz / p.nz;
    p.coords.resize(static_cast<size_t>(3) * p.nn);
    for (Index k = 0; k < nnz; ++k)
      for (Index j = 0; j < nny; ++j)
        for (Index i = 0; i < nnx; ++i) {
          const size_t n = static_cast<size_t>(k) * nnx * nny + static_cast<size_t>(j) * nnx + i;
          p.coords[3 * n] = 0.0 + i * dx;
          p.coords[3 * n + 1] = 0.0 + j * dy;
          p.coords[3 * n + 2] = 0.0 + k * dz;
        }
    const Index layer = nnx * nny;
    p.conn.reserve(static_cast<size_t>(p.ne) * 8);
    for (Index k = 0; k < p.nz; ++k)
      for (Index j = 0; j < p.ny; ++j)
        for (Index i = 0; i < p.nx; ++i) {
          const Index n0 = k * layer + j * nnx + i;
          p.conn.insert(p.conn.end(), {n0, n0 + 1, n0 + nnx + 1, n0 + nnx, n0 + layer,
                                       n0 + layer + 1, n0 + layer + nnx + 1, n0 + layer + nnx});
        }
  }
  p.ndof = p.nn * p.dim;
}

void build_pattern(Problem& p) {
  const Index nn = p.nn, ne = p.ne;
  const int npe = p.npe, dim = p.dim;
  std::vector<Index> inc_ptr(static_cast<size_t>(nn) + 1, 0);
  for (Index e = 0; e < ne; ++e)
    for (int a = 0; a < npe; ++a) ++inc_ptr[p.conn[static_cast<size_t>(e) * npe + a] + 1];
  for (Index n = 0; n < nn; ++n) inc_ptr[n + 1] += inc_ptr[n];
  std::vector<Index> inc(static_cast<size_t>(inc_ptr.back()));
  {
    std::vector<Index> fill(inc_ptr.begin(), inc_ptr.end() - 1);
    for (Index e = 0; e < ne; ++e)
      for (int a = 0; a < npe; ++a) inc[fill[p.conn[static_cast<size_t>(e) * npe + a]]++] = e;
  }
  std::vector<Index> nbr_ptr(static_cast<size_t>(nn) + 1, 0), nbr;
  nbr.reserve(static_cast<size_t>(nn) * (dim == 3 ? 27 : 9));
  {
    std::vector<Index> mark(static_cast<size_t>(nn), -1), list;
    for (Index b = 0; b < nn; ++b) {
      list.clear();
      for (Index k = inc_ptr[b]; k < inc_ptr[b + 1]; ++k) {
        const Index* nodes = &p.conn[static_cast<size_t>(inc[k]) * npe];
        for (int a = 0; a < npe; ++a)
          if (mark[nodes[a]] != b) { mark[nodes[a]] = b; list.push_back(nodes[a]); }
      }
      std::sort(list.begin(), list.end());
      nbr.insert(nbr.end(), list.begin(), list.end());
      nbr_ptr[b + 1] = static_cast<Index>(nbr.size());
    }
  }
  const Index n = nn * dim;
  p.outer.assign(static_cast<size_t>(n) + 1, 0);
  for (Index b = 0; b < nn; ++b) {
    const Index deg = nbr_ptr[b + 1] - nbr_ptr[b];
    for (int kb = 0; kb < dim; ++kb) {
      const Index c = b * dim + kb;
      p.outer[c + 1] = p.outer[c] + deg * dim;
    }
  }
  p.inner.resize(static_cast<size_t>(p.outer.back()));
  for (Index b = 0; b < nn; ++b)
    for (int kb = 0; kb < dim; ++kb) {
      Index q = p.outer[b * dim + kb];
      for (Index k = nbr_ptr[b]; k < nbr_ptr[b + 1]; ++k)
        for (int ka = 0; ka < dim; ++ka) p.inner[q++] = nbr[k] * dim + ka;
    }
  p.block_offset.resize(static_cast<size_t>(ne) * npe * npe);
  for (Index e = 0; e < ne; ++e) {
    const Index* nodes = &p.conn[static_cast<size_t>(e) * npe];
    for (int b = 0; b < npe; ++b) {
      const Index* beg = nbr.data() + nbr_ptr[nodes[b]];
      const Index* end = nbr.data() + nbr_ptr[nodes[b] + 1];
      for (int a = 0; a < npe; ++a) {
        const Index* hit = std::lower_bound(beg, end, nodes[a]);
        p.block_offset[(static_cast<size_t>(e) * npe + a) * npe + b] = static_cast<Index>(hit - beg) * dim;
      }
    }
  }
  // free-free reduction map (Assembler.cpp:416-437)
  const Index nf = static_cast<Index>(p.free_dofs.size());
  p.ff_ptr.assign(static_cast<size_t>(nf) + 1, 0);
  p.ff_col.clear();
  p.ff_src.clear();
  for (Index rc = 0; rc < nf; ++rc) {
    const Index col = p.free_dofs[rc];
    for (Index k = p.outer[col]; k < p.outer[col + 1]; ++k) {
      const Index rr = p.reduced[p.inner[k]];
      if (rr < 0) continue;
      p.ff_col.push_back(rr);
      p.ff_src.push_back(k);
    }
    p.ff_ptr[rc + 1] = static_cast<Index>(p.ff_col.size());
  }
}

// Free-free values of sum_e s_e E (E = K_e^0, or M_e^0 for the mass) for
// element factors `scale` (Assembler.cpp:182-214, 260-275, 410-455).
void assemble_ff(const Problem& p, const double* elem, const double* scale, Vec& full, Vec& kff) {
  full.assign(p.inner.size(), 0.0);
  const int npe = p.npe, dim = p.dim, ed = p.edofs;
  for (Index e = 0; e < p.ne; ++e) {
    const double s = scale ? scale[e] : 1.0;
    const Index* nodes = &p.conn[static_cast<size_t>(e) * npe];
    const Index* off = &p.block_offset[static_cast<size_t>(e) * npe * npe];
    for (int b = 0; b < npe; ++b)
      for (int kb = 0; kb < dim; ++kb) {
        const int column = dim * b + kb;
        const Index base = p.outer[nodes[b] * dim + kb];
        for (int a = 0; a < npe; ++a) {
          double* t = full.data() + base + off[a * npe + b];
          for (int ka = 0; ka < dim; ++ka) t[ka] += s * elem[static_cast<size_t>(dim * a + ka) * ed + column];
        }
      }
  }
  kff.resize(p.ff_src.size());
  for (size_t k = 0; k < p.ff_src.size(); ++k) kff[k] = full[static_cast<size_t>(p.ff_src[k])];
}

void assemble_kff(const Problem& p, const double* scale, Vec& full, Vec& kff) {
  assemble_ff(p, p.ke.data(), scale, full, kff);
}

// Centroid hash of the reference's filter (DensityFilter.cpp:19-74): buckets of
// size `radius`, keyed by the same integer mixing, visited z, y, x.
struct CentroidHash {
  double cell;
  int dim;
  const Vec& c;  // dim x ne
  std::unordered_map<size_t, std::vector<Index>> buckets;
  CentroidHash(double cell_, int dim_, const Vec& cent, Index ne) : cell(cell_), dim(dim_), c(cent) {
    for (Index e = 0; e < ne; ++e) buckets[key(e)].push_back(e);
  }
  long idx(double v) const { return static_cast<long>(std::floor(v / cell)); }
  static size_t mix(long ix, long iy, long iz) {
    const size_t a = static_cast<size_t>(ix * 2654435761L);
    const size_t b = static_cast<size_t>(iy * 2246822519L);
    const size_t cc = static_cast<size_t>(iz * 3266489917L);
    const size_t ab = a ^ (b + 0x9e3779b97f4a7c15ULL + (a << 6) + (a >> 2));
    return ab ^ (cc + 0x9e3779b97f4a7c15ULL + (ab << 6) + (ab >> 2));
  }
  size_t key(Index e) const {
    return mix(idx(c[static_cast<size_t>(e) * dim]), idx(c[static_cast<size_t>(e) * dim + 1]),
               dim == 3 ? idx(c[static_cast<size_t>(e) * dim + 2]) : 0);
  }
  void neighbours(Index e, std::vector<Index>& out) const {
    out.clear();
    const long ix = idx(c[static_cast<size_t>(e) * dim]), iy = idx(c[static_cast<size_t>(e) * dim + 1]);
    const long iz = dim == 3 ? idx(c[static_cast<size_t>(e) * dim + 2]) : 0;
    const long zr = dim == 3 ? 1 : 0;
    for (long dz = -zr; dz <= zr; ++dz)
      for (long dy = -1; dy <= 1; ++dy)
        for (long dx = -1; dx <= 1; ++dx) {
          const auto it = buckets.find(mix(ix + dx, iy + dy, iz + dz));
          if (it == buckets.end()) continue;
          out.insert(out.end(), it->second.begin(), it->second.end());
        }
  }
};

void build_filter(Problem& p) {
  const int dim = p.dim;
  Vec cent(static_cast<size_t>(p.ne) * dim);
  for (Index e = 0; e < p.ne; ++e) {
    double s[3] = {0, 0, 0};
    for (int a = 0; a < p.npe; ++a)
      for (int d = 0; d < dim; ++d) s[d] += p.coords[static_cast<size_t>(p.conn[static_cast<size_t>(e) * p.npe + a]) * dim + d];
    for (int d = 0; d < dim; ++d) cent[static_cast<size_t>(e) * dim + d] = s[d] / p.npe;
  }
  CentroidHash hash(p.radius, dim, cent, p.ne);
  std::vector<Index> cand;
  // triplets (row e, col i, w) in visit order
  std::vector<Index> trow, tcol;
  Vec tw;
  p.row_sums.assign(static_cast<size_t>(p.ne), 0.0);
  for (Index e = 0; e < p.ne; ++e) {
    hash.neighbours(e, cand);
    double sum = 0.0;
    for (Index i : cand) {
      double d2 = 0.0;
      for (int d = 0; d < dim; ++d) {
        const double df = cent[static_cast<size_t>(e) * dim + d] - cent[static_cast<size_t>(i) * dim + d];
        d2 += df * df;
      }
      const double w = p.radius - std::sqrt(d2);
      if (w <= 0.0) continue;
      trow.push_back(e);
      tcol.push_back(i);
      tw.push_back(w);
      sum += w;
    }
    if (!(sum > 0.0)) throw Error(kBadInput, "filter row is empty");
    p.row_sums[e] = sum;
  }
  // H as CSR rows sorted by column (setFromTriplets sorts inner indices).
  const size_t nt = tw.size();
  Csr& h = p.h;
  h.rows = h.cols = p.ne;
  h.ptr.assign(static_cast<size_t>(p.ne) + 1, 0);
  for (size_t t = 0; t < nt; ++t) ++h.ptr[trow[t] + 1];
  for (Index e = 0; e < p.ne; ++e) h.ptr[e + 1] += h.ptr[e];
  h.col.resize(nt);
  h.val.resize(nt);
  {
    std::vector<Index> fill(h.ptr.begin(), h.ptr.end() - 1);
    for (size_t t = 0; t < nt; ++t) {
      const Index q = fill[trow[t]]++;
      h.col[q] = tcol[t];
      h.val[q] = tw[t] / p.row_sums[trow[t]];
    }
    for (Index e = 0; e < p.ne; ++e) {
      std::vector<std::pair<Index, double>> row;
      for (Index q = h.ptr[e]; q < h.ptr[e + 1]; ++q) row.emplace_back(h.col[q], h.val[q]);
      std::sort(row.begin(), row.end(), [](auto& a, auto& b) { return a.first < b.first; });
      for (Index q = h.ptr[e]; q < h.ptr[e + 1]; ++q) {
        h.col[q] = row[q - h.ptr[e]].first;
        h.val[q] = row[q - h.ptr[e]].second;
      }
    }
  }
  p.ht = transpose(view(h));
}

// y = H x summed as Eigen's column-major product does: ascending column j.
void filter_forward(const Problem& p, const double* x, double* y) {
  if (!p.filter_on) { std::copy(x, x + p.ne, y); return; }
  // Column-major accumulation (for j: for e in column j: y[e] += H(e,j) x_j)
  // gives each y[e] the sum over ascending j, which is a CSR row sweep.
  const Csr& h = p.h;
  for (Index e = 0; e < p.ne; ++e) {
    double s = 0.0;
    for (Index q = h.ptr[e]; q < h.ptr[e + 1]; ++q) s += h.val[q] * x[h.col[q]];
    y[e] = s;
  }
}

// g = H^T v: row j of H^T is column j of H, summed over ascending e.
void filter_adjoint(const Problem& p, const double* v, double* g) {
  if (!p.filter_on) { std::copy(v, v + p.ne, g); return; }
  const Csr& t = p.ht;
  for (Index j = 0; j < p.ne; ++j) {
    double s = 0.0;
    for (Index q = t.ptr[j]; q < t.ptr[j + 1]; ++q) s += t.val[q] * v[t.col[q]];
    g[j] = s;
  }
}

double simp_factor(double rho, double pen, double emin) {
  const double r = std::min(std::max(rho, 0.0), 1.0);
  return emin + (1.0 - emin) * std::pow(r, pen);
}
double simp_derivative(double rho, double pen, double emin) {
  const double r = std::min(std::max(rho, 0.0), 1.0);
  return pen * (1.0 - emin) * std::pow(r, pen - 1.0);
}

struct Evaluation {
  double compliance = 0.0, volume = 0.0, volume_fraction = 0.0;
  int linear_iterations = 0;
  Vec rho, rhot, dc_dphys, dc_dx, dv_dx, se;  // rhot: clamped filtered density
  std::vector<Vec> u;
};

// heaviside_project / heaviside_derivative (src/topopt/Projection.cpp:56-69)
double project(double r, double beta, double eta) {
  const double a = std::tanh(beta * eta);
  const double denom = a + std::tanh(beta * (1.0 - eta));
  return (a + std::tanh(beta * (r - eta))) / denom;
}

double project_derivative(double r, double beta, double eta) {
  const double denom = std::tanh(beta * eta) + std::tanh(beta * (1.0 - eta));
  const double t = std::tanh(beta * (r - eta));
  return beta * (1.0 - t * t) / denom;
}

// ProjectionOptions::num_stages / beta_of_stage (src/topopt/Projection.cpp:45-54)
int beta_stages(const Problem& p) {
  int stages = 1;
  double b = p.beta_start;
  while (b < p.beta_max && stages < 64) {
    b *= p.beta_factor;
    ++stages;
  }
  return stages;
}

double beta_of_stage(const Problem& p, int k) {
  double b = p.beta_start;
  for (int i = 0; i < k && b < p.beta_max; ++i) b *= p.beta_factor;
  return std::min(b, p.beta_max);
}

void evaluate(Problem& p, const double* x, Evaluation& out) {
  const Index ne = p.ne;
  for (Index e = 0; e < ne; ++e) if (!std::isfinite(x[e])) throw Error(kBadInput, "design vector contains NaN or Inf");
  out = Evaluation();
  out.rho.resize(static_cast<size_t>(ne));
  filter_forward(p, x, out.rho.data());
  for (auto& r : out.rho) r = std::min(std::max(r, 0.0), 1.0);
  // physical density: the projected filtered density (Sensitivity.cpp:69-73),
  // at the eroded threshold in a robust run
  Vec dproj;
  out.rhot = out.rho;
  if (p.proj) {
    dproj.resize(static_cast<size_t>(ne));
    const double eta = p.objective_eta();
    for (Index e = 0; e < ne; ++e) {
      dproj[e] = project_derivative(out.rho[e], p.beta, eta);
      out.rho[e] = project(out.rho[e], p.beta, eta);
    }
  }
  Vec sf(static_cast<size_t>(ne)), df(static_cast<size_t>(ne));
  for (Index e = 0; e < ne; ++e) {
    sf[e] = simp_factor(out.rho[e], p.penalty, p.emin);
    df[e] = simp_derivative(out.rho[e], p.penalty, p.emin);
  }
  Vec full, kff;
  assemble_kff(p, sf.data(), full, kff);
  full.clear();
  full.shrink_to_fit();
  if (!p.amg) {
    p.amg = std::make_unique<Amg>();
    p.amg->opt = p.amg_opt;
  }
  const Index nf = static_cast<Index>(p.free_dofs.size());
  View a{nf, nf, p.ff_ptr.data(), p.ff_col.data(), kff.data()};
  p.amg->setup(a, p.layout);
  p.previous.resize(p.loads.size());
  out.se.assign(static_cast<size_t>(ne), 0.0);
  out.dc_dphys.assign(static_cast<size_t>(ne), 0.0);
  const int ed = p.edofs, npe = p.npe, dim = p.dim;
  Vec ue(static_cast<size_t>(ed)), ku(static_cast<size_t>(ed));
  for (size_t l = 0; l < p.loads.size(); ++l) {
    const Vec& f = p.loads[l];
    Vec b(static_cast<size_t>(nf)), xf(static_cast<size_t>(nf), 0.0);
    for (Index i = 0; i < nf; ++i) b[i] = f[p.free_dofs[i]];
    Vec& prev = p.previous[l];
    if (p.warm && prev.size() == f.size())
      for (Index i = 0; i < nf; ++i) xf[i] = prev[p.free_dofs[i]];
    const PcgResult r = pcg(a, b.data(), xf.data(), *p.amg, p.rtol, p.maxit);
    if (!r.converged) {
      std::ostringstream os;
      os << "AMG-CG(chebyshev) did not converge: " << r.iterations
         << " iterations left a relative residual of " << r.relres << " against a tolerance of " << p.rtol;
      throw Error(kMaxIter, os.str());
    }
    out.linear_iterations += r.iterations;
    Vec u(static_cast<size_t>(p.ndof), 0.0);
    for (Index i = 0; i < nf; ++i) u[p.free_dofs[i]] = xf[i];
    if (p.warm) prev = u;
    double c = 0.0;
    for (Index d = 0; d < p.ndof; ++d) c += f[d] * u[d];
    out.compliance += p.weights[l] * c;
    for (Index e = 0; e < ne; ++e) {
      const Index* nodes = &p.conn[static_cast<size_t>(e) * npe];
      for (int a2 = 0; a2 < npe; ++a2)
        for (int k = 0; k < dim; ++k) ue[dim * a2 + k] = u[static_cast<size_t>(nodes[a2]) * dim + k];
      double quad = 0.0;
      for (int r2 = 0; r2 < ed; ++r2) {
        double s = 0.0;
        for (int c2 = 0; c2 < ed; ++c2) s += p.ke[static_cast<size_t>(r2) * ed + c2] * ue[c2];
        ku[r2] = s;
      }
      for (int r2 = 0; r2 < ed; ++r2) quad += ue[r2] * ku[r2];
      out.se[e] += p.weights[l] * 0.5 * sf[e] * quad;
      out.dc_dphys[e] -= p.weights[l] * df[e] * quad;
    }
    out.u.push_back(std::move(u));
  }
  double vol = 0.0;
  for (Index e = 0; e < ne; ++e) vol += out.rho[e] * p.volumes[e];
  out.volume = vol;
  out.volume_fraction = vol / p.domain_volume;
  out.dc_dx.resize(static_cast<size_t>(ne));
  out.dv_dx.resize(static_cast<size_t>(ne));
  if (p.proj) {  // chain_to_design (Sensitivity.cpp:100-108)
    Vec dc(static_cast<size_t>(ne)), dv(static_cast<size_t>(ne));
    for (Index e = 0; e < ne; ++e) {
      dc[e] = out.dc_dphys[e] * dproj[e];
      dv[e] = p.volumes[e] * dproj[e];
    }
    filter_adjoint(p, dc.data(), out.dc_dx.data());
    filter_adjoint(p, dv.data(), out.dv_dx.data());
  } else {
    filter_adjoint(p, out.dc_dphys.data(), out.dc_dx.data());
    filter_adjoint(p, p.volumes.data(), out.dv_dx.data());
  }
  if (!std::isfinite(out.compliance)) throw Error(kNonFinite, "the compliance objective evaluated to a non-finite value");
}

struct OcStep {
  Vec x;
  double lambda = 0.0, volume = 0.0, max_change = 0.0;
  int bisections = 0;
  bool converged = false;
};

void oc_candidate(const Problem& p, const double* x, const double* dc, const double* dv, double lam,
                  double* xn) {
  for (Index e = 0; e < p.ne; ++e) {
    const double lo = std::max(0.0, x[e] - p.move);
    const double hi = std::min(1.0, x[e] + p.move);
    const double den = lam * dv[e];
    double b = 0.0;
    if (den > 0.0) b = std::max(0.0, -dc[e] / den);
    const double t = x[e] * std::pow(b, p.damping);
    xn[e] = std::min(std::max(t, lo), hi);
  }
}

// Volume of the physical density of design xn, projected at threshold eta.
double design_volume(const Problem& p, const double* xn, Vec& tmp, double eta) {
  filter_forward(p, xn, tmp.data());
  double v = 0.0;
  for (Index e = 0; e < p.ne; ++e) {
    double r = std::min(std::max(tmp[e], 0.0), 1.0);
    if (p.proj) r = project(r, p.beta, eta);
    v += r * p.volumes[e];
  }
  return v;
}

// optimality_criteria_update (OptimalityCriteria.cpp:40-149): volume_target
// > 0 replaces the domain's target; step_toward takes the reachable corner
// when the move-limited box cannot bracket the target (the robust run's
// moved target) instead of failing.
OcStep oc_update(const Problem& p, const double* x, const double* dc, const double* dv,
                 double volume_target = 0.0, bool step_toward = false) {
  for (Index e = 0; e < p.ne; ++e)
    if (!std::isfinite(dc[e]) || !std::isfinite(dv[e])) throw Error(kNonFinite, "optimality criteria received a non-finite gradient");
  const double target = volume_target > 0.0 ? volume_target : p.vf * p.domain_volume;
  // the volume of a trial: the dilated design's in a robust run
  const double veta = p.robust ? p.eta - p.robust_delta : p.eta;
  Vec cand(static_cast<size_t>(p.ne)), tmp(static_cast<size_t>(p.ne));
  double lo = 1.0e-12, hi = 1.0e12;
  oc_candidate(p, x, dc, dv, lo, cand.data());
  double vlo = design_volume(p, cand.data(), tmp, veta);
  oc_candidate(p, x, dc, dv, hi, cand.data());
  double vhi = design_volume(p, cand.data(), tmp, veta);
  int widen = 0;
  while (vlo < target && widen < 60) {
    lo *= 1.0e-3;
    oc_candidate(p, x, dc, dv, lo, cand.data());
    vlo = design_volume(p, cand.data(), tmp, veta);
    ++widen;
  }
  while (vhi > target && widen < 120) {
    hi *= 1.0e3;
    oc_candidate(p, x, dc, dv, hi, cand.data());
    vhi = design_volume(p, cand.data(), tmp, veta);
    ++widen;
  }
  if ((vlo < target || vhi > target) && step_toward) {
    OcStep st;
    const bool too_light = vlo < target;
    st.lambda = too_light ? lo : hi;
    oc_candidate(p, x, dc, dv, st.lambda, cand.data());
    st.volume = too_light ? vlo : vhi;
    double mc = 0.0;
    for (Index e = 0; e < p.ne; ++e) mc = std::max(mc, std::abs(cand[e] - x[e]));
    st.max_change = mc;
    st.x = std::move(cand);
    return st;
  }
  if (vlo < target || vhi > target) {
    std::ostringstream os;
    os << "the optimality-criteria bisection cannot bracket the volume target " << target;
    throw Error(kMaxIter, os.str());
  }
  OcStep st;
  oc_candidate(p, x, dc, dv, lo, cand.data());
  double vol = vlo;
  for (int it = 0; it < 200; ++it) {
    const double mid = std::sqrt(lo * hi);
    oc_candidate(p, x, dc, dv, mid, cand.data());
    vol = design_volume(p, cand.data(), tmp, veta);
    st.bisections = it + 1;
    st.lambda = mid;
    if (std::abs(vol - target) <= 1.0e-10 * target) { st.converged = true; break; }
    if (vol > target) lo = mid; else hi = mid;
    if (hi / lo - 1.0 < 1.0e-15) {
      st.converged = std::abs(vol - target) <= 1.0e-6 * std::max(target, 1.0e-30);
      break;
    }
  }
  st.volume = vol;
  double mc = 0.0;
  for (Index e = 0; e < p.ne; ++e) mc = std::max(mc, std::abs(cand[e] - x[e]));
  st.max_change = mc;
  st.x = std::move(cand);
  return st;
}

// ---------------------------------------------------------------------------
// MMA (src/topopt/Mma.cpp:63-409), restated for one constraint row (the
// volume): the (lambda, z) Newton system of the subproblem is 2 x 2.
// ---------------------------------------------------------------------------
struct MmaState {
  int iteration = 0;
  Vec xold1, xold2, low, upp;
  double move = 0.2, asy_init = 0.5, asy_inc = 1.2, asy_dec = 0.7, albefa = 0.1, raa0 = 1.0e-5;
  double a0 = 1.0, c = 1000.0, d = 1.0, epsimin = 1.0e-7, scale_cap = 10.0;
  int max_inner = 500;
};

struct MmaResult {
  Vec x;
  double lam = 0.0, y = 0.0, z = 0.0, max_change = 0.0, row_scale = 1.0;
  int iterations = 0;
};

// xmin = 0, xmax = 1 for every variable (no passive regions)
MmaResult mma_update(MmaState& st, const Vec& x, const Vec& df0, double fval, const Vec& dfdx) {
  const size_t n = x.size();
  if (st.xold1.empty()) {
    st.xold1.assign(n, 0.0);
    st.xold2.assign(n, 0.0);
    st.low.assign(n, 0.0);
    st.upp.assign(n, 1.0);
  }
  ++st.iteration;
  const double xmami = 1.0;  // xmax - xmin
  Vec& low = st.low;
  Vec& upp = st.upp;
  if (st.iteration <= 2) {
    for (size_t j = 0; j < n; ++j) {
      low[j] = x[j] - st.asy_init * xmami;
      upp[j] = x[j] + st.asy_init * xmami;
    }
  } else {
    for (size_t j = 0; j < n; ++j) {
      const double zzz = (x[j] - st.xold1[j]) * (st.xold1[j] - st.xold2[j]);
      double f = 1.0;
      if (zzz > 0.0) f = st.asy_inc;
      if (zzz < 0.0) f = st.asy_dec;
      low[j] = x[j] - f * (st.xold1[j] - low[j]);
      upp[j] = x[j] + f * (upp[j] - st.xold1[j]);
      low[j] = std::min(std::max(low[j], x[j] - 10.0 * xmami), x[j] - 0.01 * xmami);
      upp[j] = std::min(std::max(upp[j], x[j] + 0.01 * xmami), x[j] + 10.0 * xmami);
    }
  }
  Vec alfa(n), beta(n), p0(n), q0(n), p(n), q(n);
  const double xmamiinv = 1.0 / std::max(xmami, 1.0e-5);
  // row scale of the constraint (Mma.cpp:141-149)
  double dmax = 0.0;
  for (size_t j = 0; j < n; ++j) dmax = std::max(dmax, std::abs(dfdx[j]));
  const double magnitude = std::max(std::abs(fval), dmax * st.move * xmami);
  const double row_scale = magnitude > st.scale_cap ? st.scale_cap / magnitude : 1.0;
  const double fs = row_scale * fval;
  double bsum = 0.0;
  for (size_t j = 0; j < n; ++j) {
    alfa[j] = std::max({low[j] + st.albefa * (x[j] - low[j]), x[j] - st.move * xmami, 0.0});
    beta[j] = std::min({upp[j] - st.albefa * (upp[j] - x[j]), x[j] + st.move * xmami, 1.0});
    const double ux1 = upp[j] - x[j], xl1 = x[j] - low[j];
    const double ux2 = ux1 * ux1, xl2 = xl1 * xl1;
    double pp0 = std::max(df0[j], 0.0), qq0 = std::max(-df0[j], 0.0);
    const double pq0 = 0.001 * (pp0 + qq0) + st.raa0 * xmamiinv;
    p0[j] = (pp0 + pq0) * ux2;
    q0[j] = (qq0 + pq0) * xl2;
    const double ds = row_scale * dfdx[j];
    double pp = std::max(ds, 0.0), qq = std::max(-ds, 0.0);
    const double pq = 0.001 * (pp + qq) + st.raa0 * xmamiinv;
    p[j] = (pp + pq) * ux2;
    q[j] = (qq + pq) * xl2;
    bsum += p[j] / ux1 + q[j] / xl1;
  }
  const double b = bsum - fs;
  // primal-dual subproblem (Mma.cpp:158-395)
  const double a = 0.0, c = st.c, d = st.d, a0 = st.a0;
  double epsi = 1.0;
  Vec xx(n), xsi(n), eta(n);
  for (size_t j = 0; j < n; ++j) {
    xx[j] = 0.5 * (alfa[j] + beta[j]);
    xsi[j] = std::max(1.0 / (xx[j] - alfa[j]), 1.0);
    eta[j] = std::max(1.0 / (beta[j] - xx[j]), 1.0);
  }
  double y = 1.0, z = 1.0, lam = 1.0, mu = std::max(0.5 * c, 1.0), zet = 1.0, s = 1.0;
  auto residual = [&](const Vec& xv, double yv, double zv, double lv, const Vec& xsiv, const Vec& etav,
                      double muv, double zetv, double sv, double& norm) {
    double sq = 0.0, mx = 0.0, gvec = 0.0;
    for (size_t j = 0; j < n; ++j) {
      const double ux1 = upp[j] - xv[j], xl1 = xv[j] - low[j];
      const double plam = p0[j] + p[j] * lv, qlam = q0[j] + q[j] * lv;
      gvec += p[j] / ux1 + q[j] / xl1;
      const double dpsidx = plam / (ux1 * ux1) - qlam / (xl1 * xl1);
      const double rex = dpsidx - xsiv[j] + etav[j];
      const double rexsi = xsiv[j] * (xv[j] - alfa[j]) - epsi;
      const double reeta = etav[j] * (beta[j] - xv[j]) - epsi;
      sq += rex * rex + rexsi * rexsi + reeta * reeta;
      mx = std::max({mx, std::abs(rex), std::abs(rexsi), std::abs(reeta)});
    }
    const double rey = c + d * yv - muv - lv;
    const double rez = a0 - zetv - a * lv;
    const double relam = gvec - a * zv - yv + sv - b;
    const double remu = muv * yv - epsi, rezet = zetv * zv - epsi, res = lv * sv - epsi;
    sq += rey * rey + rez * rez + relam * relam + remu * remu + rezet * rezet + res * res;
    mx = std::max({mx, std::abs(rey), std::abs(rez), std::abs(relam), std::abs(remu), std::abs(rezet),
                   std::abs(res)});
    norm = std::isfinite(sq) ? std::sqrt(sq) : std::numeric_limits<double>::infinity();
    return std::isfinite(sq) ? mx : std::numeric_limits<double>::infinity();
  };
  int total = 0;
  Vec dx(n), dxsi(n), deta(n), xo(n), xsio(n), etao(n);
  while (epsi > st.epsimin) {
    double cur_norm;
    double cur_max = residual(xx, y, z, lam, xsi, eta, mu, zet, s, cur_norm);
    int ittt = 0;
    while (cur_max > 0.9 * epsi && ittt < st.max_inner) {
      ++ittt;
      ++total;
      double sgd = 0.0, sgg = 0.0, gvec = 0.0;
      Vec delx(n), diagx(n), gg(n);
      for (size_t j = 0; j < n; ++j) {
        const double ux1 = upp[j] - xx[j], xl1 = xx[j] - low[j];
        const double ux2 = ux1 * ux1, xl2 = xl1 * xl1;
        const double plam = p0[j] + p[j] * lam, qlam = q0[j] + q[j] * lam;
        gvec += p[j] / ux1 + q[j] / xl1;
        gg[j] = p[j] / ux2 - q[j] / xl2;
        const double dpsidx = plam / ux2 - qlam / xl2;
        const double xa = xx[j] - alfa[j], bx = beta[j] - xx[j];
        delx[j] = dpsidx - epsi / xa + epsi / bx;
        diagx[j] = 2.0 * (plam / (ux2 * ux1) + qlam / (xl2 * xl1)) + xsi[j] / xa + eta[j] / bx;
        sgd += gg[j] * (delx[j] / diagx[j]);
        sgg += gg[j] * gg[j] / diagx[j];
      }
      const double dely = c + d * y - lam - epsi / y;
      const double delz = a0 - a * lam - epsi / z;
      const double dellam = gvec - a * z - y - b + epsi / lam;
      const double diagy = d + mu / y;
      const double diaglamyi = s / lam + 1.0 / diagy;
      const double blam = dellam + dely / diagy - sgd;
      // [alam a; a -zet/z] [dlam; dz] = [blam; delz]
      const double alam = diaglamyi + sgg;
      const double a11 = alam, a12 = a, a21 = a, a22 = -zet / z;
      const double det = a11 * a22 - a12 * a21;
      const double dlam = (blam * a22 - a12 * delz) / det;
      const double dz = (a11 * delz - a21 * blam) / det;
      for (size_t j = 0; j < n; ++j) dx[j] = -delx[j] / diagx[j] - (gg[j] * dlam) / diagx[j];
      const double dy = -dely / diagy + dlam / diagy;
      double stmxx = std::max({-1.01 * dy / y, -1.01 * dz / z, -1.01 * dlam / lam});
      for (size_t j = 0; j < n; ++j) {
        const double xa = xx[j] - alfa[j], bx = beta[j] - xx[j];
        dxsi[j] = -xsi[j] + epsi / xa - (xsi[j] * dx[j]) / xa;
        deta[j] = -eta[j] + epsi / bx + (eta[j] * dx[j]) / bx;
        stmxx = std::max({stmxx, -1.01 * dxsi[j] / xsi[j], -1.01 * deta[j] / eta[j], -1.01 * dx[j] / xa,
                          1.01 * dx[j] / bx});
      }
      const double dmu = -mu + epsi / y - (mu * dy) / y;
      const double dzet = -zet + epsi / z - zet * dz / z;
      const double dss = -s + epsi / lam - (s * dlam) / lam;
      stmxx = std::max({stmxx, -1.01 * dmu / mu, -1.01 * dzet / zet, -1.01 * dss / s});
      const double stminv = std::max(stmxx, 1.0);
      double steg = 1.0 / stminv;
      xo = xx;
      xsio = xsi;
      etao = eta;
      const double yo = y, zo = z, lamo = lam, muo = mu, zeto = zet, so = s;
      int itto = 0;
      double trial_norm = 2.0 * cur_norm, trial_max = cur_max;
      while (trial_norm > cur_norm && itto < 50) {
        ++itto;
        for (size_t j = 0; j < n; ++j) {
          xx[j] = xo[j] + steg * dx[j];
          xsi[j] = xsio[j] + steg * dxsi[j];
          eta[j] = etao[j] + steg * deta[j];
        }
        y = yo + steg * dy;
        z = zo + steg * dz;
        lam = lamo + steg * dlam;
        mu = muo + steg * dmu;
        zet = zeto + steg * dzet;
        s = so + steg * dss;
        trial_max = residual(xx, y, z, lam, xsi, eta, mu, zet, s, trial_norm);
        steg *= 0.5;
      }
      cur_norm = trial_norm;
      cur_max = trial_max;
    }
    if (ittt >= st.max_inner) throw Error(kMaxIter, "the MMA subproblem solver did not converge");
    epsi *= 0.1;
  }
  MmaResult r;
  r.x = xx;
  r.lam = lam * row_scale;
  r.y = y / row_scale;
  r.z = z;
  r.row_scale = row_scale;
  r.iterations = total;
  double mc = 0.0;
  for (size_t j = 0; j < n; ++j) mc = std::max(mc, std::abs(xx[j] - x[j]));
  r.max_change = mc;
  st.xold2 = st.xold1;
  st.xold1 = x;
  return r;
}

}  // namespace orc

using namespace orc;

struct orc_problem { Problem p; };
struct orc_solver {
  Amg amg;
  double rtol = 1e-12;
  int maxit = 1000;
  std::vector<Index> ptr, col, unknowns;
  Vec val, coords;
  Layout layout;
  View a;
};

namespace {
template <class F>
int guarded(F&& f) {
  try {
    f();
    return kOk;
  } catch (const Error& e) {
    g_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    g_error = e.what();
    return kBadInput;
  }
}
AmgOptions convert(const orc_amg_options* o) {
  AmgOptions a;
  if (!o) return a;
  a.theta = o->strength_threshold;
  a.max_levels = o->max_levels;
  a.coarse_size = o->coarse_size;
  a.degree = o->smoother_degree;
  a.cheb_ratio = o->chebyshev_ratio;
  a.damping = o->prolongator_damping;
  a.lanczos_steps = o->lanczos_steps;
  a.pivot_tol = o->coarse_pivot_tolerance;
  a.reuse = o->reuse_aggregates != 0;
  return a;
}
void copy_csr(const View& v, int32_t* ptr, int32_t* col, double* val) {
  if (ptr) std::copy(v.ptr, v.ptr + v.rows + 1, ptr);
  if (col) std::copy(v.col, v.col + v.nnz(), col);
  if (val) std::copy(v.val, v.val + v.nnz(), val);
}
}  // namespace

extern "C" {

const char* orc_last_error(void) { return g_error.c_str(); }

void orc_default_amg_options(orc_amg_options* o) {
  o->strength_threshold = 0.02;
  o->max_levels = 12;
  o->coarse_size = 1500;
  o->smoother_degree = 3;
  o->chebyshev_ratio = 30.0;
  o->prolongator_damping = 4.0 / 3.0;
  o->lanczos_steps = 12;
  o->coarse_pivot_tolerance = 1.0e-13;
  o->reuse_aggregates = 1;
}

int orc_element_stiffness(int dim, double hx, double hy, double hz, double young, double poisson,
                          double thickness, double* ke) {
  return guarded([&] { element_stiffness(dim, hx, hy, hz, young, poisson, thickness, ke); });
}

int orc_element_mass(int dim, double hx, double hy, double hz, double density, double thickness,
                     double* me) {
  return guarded([&] { element_mass(dim, hx, hy, hz, density, thickness, me); });
}

int orc_solver_create(const orc_amg_options* o, double rtol, int32_t maxit, orc_solver** out) {
  return guarded([&] {
    auto* s = new orc_solver();
    s->amg.opt = convert(o);
    s->rtol = rtol;
    s->maxit = maxit > 0 ? maxit : 1000;
    *out = s;
  });
}

void orc_solver_destroy(orc_solver* s) { delete s; }

int orc_solver_factorize(orc_solver* s, int32_t n, const int32_t* rowptr, const int32_t* col,
                         const double* val, int dim, int ndpn, const double* coords,
                         int32_t num_nodes, const int32_t* unknowns) {
  return guarded([&] {
    const Index nnz = rowptr[n];
    const bool same_layout = static_cast<Index>(s->unknowns.size()) == n &&
                             std::equal(unknowns, unknowns + n, s->unknowns.begin());
    s->ptr.assign(rowptr, rowptr + n + 1);
    s->col.assign(col, col + nnz);
    s->val.assign(val, val + nnz);
    if (!same_layout) s->unknowns.assign(unknowns, unknowns + n);
    s->coords.assign(coords, coords + static_cast<size_t>(num_nodes) * dim);
    s->layout = Layout{dim, ndpn, s->coords.data(), num_nodes, s->unknowns.data(), n};
    s->a = View{n, n, s->ptr.data(), s->col.data(), s->val.data()};
    s->amg.setup(s->a, s->layout);
  });
}

int orc_solver_solve(orc_solver* s, const double* b, const double* x0, double* x, int32_t* iters,
                     double* relres) {
  return guarded([&] {
    const Index n = s->a.rows;
    if (x0) std::copy(x0, x0 + n, x); else std::fill(x, x + n, 0.0);
    const PcgResult r = pcg(s->a, b, x, s->amg, s->rtol, s->maxit);
    if (iters) *iters = r.iterations;
    if (relres) *relres = r.relres;
    if (!r.converged) {
      std::ostringstream os;
      os << "AMG-CG(chebyshev) did not converge: " << r.iterations
         << " iterations left a relative residual of " << r.relres << " against a tolerance of " << s->rtol;
      throw Error(kMaxIter, os.str());
    }
  });
}

int orc_solver_apply(orc_solver* s, const double* r, double* z) {
  return guarded([&] { s->amg.apply(r, z); });
}

int orc_solver_num_levels(orc_solver* s) { return static_cast<int>(s->amg.levels.size()); }

int orc_solver_level_info(orc_solver* s, int level, int64_t* info, double* lam) {
  return guarded([&] {
    const Level& l = s->amg.levels.at(static_cast<size_t>(level));
    info[0] = l.a.rows;
    info[1] = l.a.nnz();
    info[2] = static_cast<size_t>(level) + 1 < s->amg.levels.size() ? s->amg.levels[level + 1].num_nodes : 0;
    if (lam) *lam = l.lambda;
  });
}

int orc_solver_level_matrix(orc_solver* s, int level, int32_t* ptr, int32_t* col, double* val) {
  return guarded([&] { copy_csr(s->amg.levels.at(static_cast<size_t>(level)).a, ptr, col, val); });
}

int orc_solver_prolongator_nnz(orc_solver* s, int level, int tent, int64_t* nnz) {
  return guarded([&] {
    const Level& l = s->amg.levels.at(static_cast<size_t>(level));
    const Csr& m = tent ? l.p_tent : l.p;
    nnz[0] = m.rows;
    nnz[1] = m.cols;
    nnz[2] = m.nnz();
  });
}

int orc_solver_prolongator(orc_solver* s, int level, int tent, int32_t* ptr, int32_t* col, double* val) {
  return guarded([&] {
    const Level& l = s->amg.levels.at(static_cast<size_t>(level));
    copy_csr(view(tent ? l.p_tent : l.p), ptr, col, val);
  });
}

int orc_solver_num_nodes(orc_solver* s, int level, int32_t* nn) {
  return guarded([&] { *nn = s->amg.levels.at(static_cast<size_t>(level)).num_nodes; });
}

int orc_solver_aggregates(orc_solver* s, int level, int32_t* agg) {
  return guarded([&] {
    const Level& l = s->amg.levels.at(static_cast<size_t>(level));
    std::copy(l.aggregate.begin(), l.aggregate.end(), agg);
  });
}

int orc_solver_nullspace(orc_solver* s, int level, int32_t* cols, double* b) {
  return guarded([&] {
    const Level& l = s->amg.levels.at(static_cast<size_t>(level));
    *cols = l.nullspace.cols;
    if (b)  // row-major rows x cols
      for (Index i = 0; i < l.nullspace.rows; ++i)
        for (Index j = 0; j < l.nullspace.cols; ++j) b[static_cast<size_t>(i) * l.nullspace.cols + j] = l.nullspace(i, j);
  });
}

int orc_solver_stats(orc_solver* s, double* oc, double* pr, int32_t* reused) {
  return guarded([&] {
    if (oc) *oc = s->amg.op_complexity;
    if (pr) *pr = s->amg.pivot_ratio;
    if (reused) *reused = s->amg.reused ? 1 : 0;
  });
}

int orc_problem_create(const orc_problem_desc* d, orc_problem** out) {
  return guarded([&] {
    if (d->dim != 2 && d->dim != 3) throw Error(kBadInput, "dim must be 2 or 3");
    auto holder = std::make_unique<orc_problem>();
    Problem& p = holder->p;
    p.dim = d->dim;
    p.nx = d->nx;
    p.ny = d->ny;
    p.nz = d->dim == 3 ? d->nz : 1;
    p.lx = d->lx;
    p.ly = d->ly;
    p.lz = d->lz;
    build_mesh(p);
    p.edofs = p.npe * p.dim;
    p.ke.resize(static_cast<size_t>(p.edofs) * p.edofs);
    const double hx = p.lx / p.nx, hy = p.ly / p.ny, hz = p.dim == 3 ? p.lz / p.nz : 0.0;
    element_stiffness(p.dim, hx, hy, hz, d->young, d->poisson, p.dim == 2 ? d->thickness : 1.0, p.ke.data());
    p.reduced.assign(static_cast<size_t>(p.ndof), -1);
    for (Index k = 0; k < p.ndof; ++k)
      if (!d->fixed[k]) { p.reduced[k] = static_cast<Index>(p.free_dofs.size()); p.free_dofs.push_back(k); }
    build_pattern(p);
    // element volumes (measure x thickness for 2-D)
    p.volumes.assign(static_cast<size_t>(p.ne), p.dim == 2 ? hx * hy * d->thickness : hx * hy * hz);
    p.domain_volume = 0.0;
    for (double v : p.volumes) p.domain_volume += v;
    p.filter_on = d->filter_radius > 0.0;
    p.radius = d->filter_radius;
    if (p.filter_on) build_filter(p);
    double wsum = 0.0;
    for (int l = 0; l < d->num_loads; ++l) wsum += d->weights[l];
    for (int l = 0; l < d->num_loads; ++l) {
      p.loads.emplace_back(d->loads + static_cast<size_t>(l) * p.ndof, d->loads + static_cast<size_t>(l + 1) * p.ndof);
      p.weights.push_back(d->weights[l] / wsum);
    }
    p.vf = d->volume_fraction;
    p.x0 = d->initial_density >= 0.0 ? d->initial_density : d->volume_fraction;
    p.penalty = d->penalty;
    p.emin = d->emin_ratio;
    p.move = d->move_limit;
    p.damping = d->damping;
    p.rtol = d->rtol;
    p.maxit = d->max_cg_iterations > 0 ? d->max_cg_iterations : 1000;
    p.warm = d->warm_start != 0;
    p.amg_opt = convert(&d->amg);
    p.proj = d->projection != 0;
    if (p.proj) {
      p.eta = d->eta;
      p.beta_start = d->beta_start;
      p.beta_max = d->beta_max;
      p.beta_factor = d->beta_factor;
      p.beta_interval = std::max(1, d->beta_interval);
      p.advance = d->advance_on_convergence != 0;
      p.change_tol = d->change_tolerance;
      p.beta = beta_of_stage(p, 0);
      p.robust = d->robust != 0;
      p.robust_delta = d->robust_delta;
      p.robust_interval = std::max(1, d->robust_volume_interval);
      if (p.robust && !(p.eta - p.robust_delta > 0.0 && p.eta + p.robust_delta < 1.0))
        throw Error(kBadInput, "projection.robust_delta must keep eta +- delta inside (0, 1)");
    }
    p.layout = Layout{p.dim, p.dim, p.coords.data(), p.nn, p.free_dofs.data(),
                      static_cast<Index>(p.free_dofs.size())};
    *out = holder.release();
  });
}

void orc_problem_destroy(orc_problem* p) { delete p; }

int orc_problem_sizes(orc_problem* h, int64_t* s) {
  const Problem& p = h->p;
  s[0] = p.ne;
  s[1] = p.nn;
  s[2] = p.ndof;
  s[3] = static_cast<int64_t>(p.free_dofs.size());
  s[4] = static_cast<int64_t>(p.ff_col.size());
  return kOk;
}

int orc_problem_free_dofs(orc_problem* h, int32_t* f) {
  std::copy(h->p.free_dofs.begin(), h->p.free_dofs.end(), f);
  return kOk;
}

int orc_problem_coords(orc_problem* h, double* c) {
  std::copy(h->p.coords.begin(), h->p.coords.end(), c);
  return kOk;
}

int orc_problem_element_matrix(orc_problem* h, double* ke) {
  std::copy(h->p.ke.begin(), h->p.ke.end(), ke);
  return kOk;
}

int orc_problem_kff(orc_problem* h, const double* scale, int32_t* ptr, int32_t* col, double* val) {
  return guarded([&] {
    const Problem& p = h->p;
    if (ptr) std::copy(p.ff_ptr.begin(), p.ff_ptr.end(), ptr);
    if (col) std::copy(p.ff_col.begin(), p.ff_col.end(), col);
    if (val) {
      Vec full, kff;
      assemble_kff(p, scale, full, kff);
      std::copy(kff.begin(), kff.end(), val);
    }
  });
}

int orc_problem_assemble(orc_problem* h, const double* elem, const double* scale, double* val,
                         double* full_sum) {
  return guarded([&] {
    Vec full, ff;
    assemble_ff(h->p, elem, scale, full, ff);
    std::copy(ff.begin(), ff.end(), val);
    if (full_sum) {
      // SparseMatrix::sum(): the stored values in storage order
      double t = 0.0;
      for (double v : full) t += v;
      *full_sum = t;
    }
  });
}

int orc_filter_forward(orc_problem* h, const double* x, double* y) {
  return guarded([&] { filter_forward(h->p, x, y); });
}
int orc_filter_adjoint(orc_problem* h, const double* v, double* g) {
  return guarded([&] { filter_adjoint(h->p, v, g); });
}
int orc_filter_row_sums(orc_problem* h, double* s) {
  std::copy(h->p.row_sums.begin(), h->p.row_sums.end(), s);
  return kOk;
}

int orc_evaluate(orc_problem* h, const double* x, double* out, double* rho, double* dcp, double* dcx,
                 double* dvx, double* se, double* disp) {
  return guarded([&] {
    Problem& p = h->p;
    Evaluation ev;
    evaluate(p, x, ev);
    out[0] = ev.compliance;
    out[1] = ev.volume;
    out[2] = ev.volume_fraction;
    out[3] = ev.linear_iterations;
    if (rho) std::copy(ev.rho.begin(), ev.rho.end(), rho);
    if (dcp) std::copy(ev.dc_dphys.begin(), ev.dc_dphys.end(), dcp);
    if (dcx) std::copy(ev.dc_dx.begin(), ev.dc_dx.end(), dcx);
    if (dvx) std::copy(ev.dv_dx.begin(), ev.dv_dx.end(), dvx);
    if (se) std::copy(ev.se.begin(), ev.se.end(), se);
    if (disp)
      for (size_t l = 0; l < ev.u.size(); ++l) std::copy(ev.u[l].begin(), ev.u[l].end(), disp + l * p.ndof);
  });
}

int orc_oc_update(orc_problem* h, const double* x, const double* dc, const double* dv, double* xn,
                  double* out) {
  return guarded([&] {
    const OcStep st = oc_update(h->p, x, dc, dv);
    std::copy(st.x.begin(), st.x.end(), xn);
    out[0] = st.lambda;
    out[1] = st.volume;
    out[2] = st.max_change;
    out[3] = st.bisections;
    out[4] = st.converged ? 1.0 : 0.0;
  });
}

// MmaOptimizer(n, 1, 0, 1) on its own (tests/test_mma.cpp:90-167 drive it
// with analytic functions): one update per call, the state kept between calls.
struct orc_mma {
  MmaState st;
  int32_t n = 0;
};

int orc_mma_create(int32_t n, orc_mma** out) {
  return guarded([&] {
    if (!out || n < 1) throw Error(kBadInput, "MMA needs at least one design variable");
    auto* h = new orc_mma();
    h->n = n;
    *out = h;
  });
}

void orc_mma_destroy(orc_mma* h) { delete h; }

int orc_mma_update(orc_mma* h, const double* x, const double* df0, double fval, const double* dfdx,
                   double* x_out, double* out) {
  return guarded([&] {
    const size_t n = static_cast<size_t>(h->n);
    const Vec xv(x, x + n), g0(df0, df0 + n), g1(dfdx, dfdx + n);
    const MmaResult r = mma_update(h->st, xv, g0, fval, g1);
    std::copy(r.x.begin(), r.x.end(), x_out);
    out[0] = r.lam;
    out[1] = r.y;
    out[2] = r.z;
    out[3] = r.max_change;
    out[4] = r.row_scale;
    out[5] = r.iterations;
    out[6] = h->st.iteration;
  });
}

// run_mma (src/topopt/TopologyOptimizer.cpp:730-905) for the compliance /
// volume problem: f0 = c / c_1, f1 = V / V* - 1.  history: compliance, volume
// fraction, max change, lambda, linear iterations, subproblem iterations.
int orc_run_mma(orc_problem* h, int32_t iterations, double* x, double* hist, int32_t* performed) {
  return guarded([&] {
    Problem& p = h->p;
    Vec xv(static_cast<size_t>(p.ne), p.x0);
    for (auto& v : xv) v = std::min(std::max(v, 0.0), 1.0);
    MmaState st;
    st.move = p.move;
    double c_ref = 0.0;
    const double target = p.vf * p.domain_volume;
    // beta continuation and the robust volume row (run_mma,
    // src/topopt/TopologyOptimizer.cpp:730-980)
    const int stages = p.proj ? beta_stages(p) : 1;
    int stage = 0, stage_start = 1;
    if (p.proj) p.beta = beta_of_stage(p, 0);
    const bool robust = p.proj && p.robust;
    double dilated_target = target;
    int it = 0;
    for (it = 1; it <= iterations; ++it) {
      Evaluation ev;
      evaluate(p, xv.data(), ev);
      if (it == 1) c_ref = ev.compliance;
      Vec df0(static_cast<size_t>(p.ne)), dfdx(static_cast<size_t>(p.ne));
      double vol_i = 0.0, vol_d = 0.0, fval = 0.0;
      if (robust) {
        const double eta_d = p.eta - p.robust_delta;
        Vec w(static_cast<size_t>(p.ne)), g(static_cast<size_t>(p.ne));
        for (Index e = 0; e < p.ne; ++e) {
          vol_d += project(ev.rhot[e], p.beta, eta_d) * p.volumes[e];
          vol_i += project(ev.rhot[e], p.beta, p.eta) * p.volumes[e];
          w[e] = p.volumes[e] * project_derivative(ev.rhot[e], p.beta, eta_d);
        }
        filter_adjoint(p, w.data(), g.data());
        if ((it - 1) % p.robust_interval == 0 && vol_i > 0.0) dilated_target = target * vol_d / vol_i;
        for (Index e = 0; e < p.ne; ++e) dfdx[e] = g[e] / dilated_target;
        fval = vol_d / dilated_target - 1.0;
      } else {
        for (Index e = 0; e < p.ne; ++e) dfdx[e] = ev.dv_dx[e] / target;
        fval = ev.volume / target - 1.0;
      }
      for (Index e = 0; e < p.ne; ++e) df0[e] = ev.dc_dx[e] / c_ref;
      const MmaResult r = mma_update(st, xv, df0, fval, dfdx);
      double* row = hist + static_cast<size_t>(it - 1) * 10;
      row[0] = ev.compliance;
      row[1] = robust ? vol_i / p.domain_volume : ev.volume_fraction;
      row[2] = r.max_change;
      row[3] = r.lam;
      row[4] = ev.linear_iterations;
      row[5] = r.iterations;
      row[6] = p.proj ? p.beta : 0.0;
      row[7] = robust ? ev.volume_fraction : 0.0;
      row[8] = robust ? vol_d / p.domain_volume : 0.0;
      row[9] = robust ? dilated_target / p.domain_volume : 0.0;
      xv = r.x;
      for (auto& v : xv) v = std::min(std::max(v, 0.0), 1.0);
      const bool at_final = !p.proj || stage + 1 >= stages;
      if (!at_final && (it - stage_start + 1 >= p.beta_interval || (p.advance && r.max_change <= p.change_tol))) {
        ++stage;
        stage_start = it + 1;
        p.beta = beta_of_stage(p, stage);
      }
    }
    *performed = std::min(it, iterations);
    std::copy(xv.begin(), xv.end(), x);
  });
}

int orc_run(orc_problem* h, int32_t iterations, double change_tol, double* x, double* hist,
            int32_t* performed) {
  return guarded([&] {
    Problem& p = h->p;
    Vec xv(static_cast<size_t>(p.ne), p.x0);
    for (auto& v : xv) v = std::min(std::max(v, 0.0), 1.0);
    // beta continuation (BetaSchedule, src/topopt/TopologyOptimizer.cpp:17-46)
    const int stages = p.proj ? beta_stages(p) : 1;
    int stage = 0, stage_start = 1;
    if (p.proj) p.beta = beta_of_stage(p, 0);
    int it = 0;
    const bool robust = p.proj && p.robust;
    double dilated_target = p.vf * p.domain_volume;
    for (it = 1; it <= iterations; ++it) {
      Evaluation ev;
      evaluate(p, xv.data(), ev);
      // robust volumes (TopologyOptimizer.cpp:61-80, 625-636): the dilated
      // design's volume and gradient, the blueprint's volume, the moved target
      double vol_i = 0.0, vol_d = 0.0;
      Vec dv_dilated;
      if (robust) {
        const double eta_d = p.eta - p.robust_delta;
        Vec w(static_cast<size_t>(p.ne));
        dv_dilated.resize(static_cast<size_t>(p.ne));
        for (Index e = 0; e < p.ne; ++e) {
          vol_d += project(ev.rhot[e], p.beta, eta_d) * p.volumes[e];
          vol_i += project(ev.rhot[e], p.beta, p.eta) * p.volumes[e];
          w[e] = p.volumes[e] * project_derivative(ev.rhot[e], p.beta, eta_d);
        }
        filter_adjoint(p, w.data(), dv_dilated.data());
        if ((it - 1) % p.robust_interval == 0 && vol_i > 0.0)
          dilated_target = p.vf * p.domain_volume * vol_d / vol_i;
      }
      const OcStep st = robust ? oc_update(p, xv.data(), ev.dc_dx.data(), dv_dilated.data(), dilated_target, true)
                               : oc_update(p, xv.data(), ev.dc_dx.data(), ev.dv_dx.data());
      double* row = hist + static_cast<size_t>(it - 1) * 10;
      row[0] = ev.compliance;
      row[1] = robust ? vol_i / p.domain_volume : ev.volume_fraction;
      row[2] = st.max_change;
      row[3] = st.lambda;
      row[4] = ev.linear_iterations;
      row[5] = st.bisections;
      row[6] = p.proj ? p.beta : 0.0;
      row[7] = robust ? ev.volume_fraction : 0.0;
      row[8] = robust ? vol_d / p.domain_volume : 0.0;
      row[9] = robust ? dilated_target / p.domain_volume : 0.0;
      xv = st.x;
      for (auto& v : xv) v = std::min(std::max(v, 0.0), 1.0);
      const bool at_final = !p.proj || stage + 1 >= stages;
      if (at_final && change_tol > 0.0 && st.max_change <= change_tol) break;
      if (!at_final && (it - stage_start + 1 >= p.beta_interval ||
                        (p.advance && st.max_change <= p.change_tol))) {
        ++stage;
        stage_start = it + 1;
        p.beta = beta_of_stage(p, stage);
      }
    }
    *performed = std::min(it, iterations);
    std::copy(xv.begin(), xv.end(), x);
  });
}

}  // extern "C"
