// GPU SA-AMG hierarchy, V-cycle and PCG (see amg.h).  Setup steps follow
// AmgPreconditioner::setup (src/fem/Multigrid.cpp:929-1111); the cycle
// follows Impl::cycle (:857-885) and Impl::smooth (:783-855); PCG follows
// pcg_solve (:1152-1237).
#include "amg.h"
#include "dense.cuh"
#include "kernels.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <sstream>

namespace simp {

std::atomic<int64_t> g_launches{0};

void DevPattern::upload(const NodePattern& p) {
  ptr.upload(p.ptr);
  nbr.upload(p.nbr);
  off.upload(p.off);
}

__global__ void k_expand_columns(i32 n, const i32* __restrict__ node_of, NodeView p,
                                 const i32* __restrict__ col_first, const i32* __restrict__ rowptr,
                                 i32* __restrict__ col) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const i32 I = node_of[i];
    i32 k = rowptr[i];
    for (i32 t = p.ptr[I]; t < p.ptr[I + 1]; ++t) {
      const i32 J = p.nbr[t];
      for (i32 c = col_first[J]; c < col_first[J + 1]; ++c) col[k++] = c;
    }
  }
}

namespace {

int lanes_for(const DevCsr& a) {
  const double avg = a.rows > 0 ? static_cast<double>(a.nnz) / a.rows : 1.0;
  if (avg <= 3) return 2;
  if (avg <= 10) return 4;
  if (avg <= 24) return 8;
  if (avg <= 64) return 16;
  return 32;
}

template <int VS, int MODE>
void launch_csr_vs(const DevCsr& a, const double* x, double* y, const double* b, cudaStream_t s) {
  const i64 threads = static_cast<i64>(a.rows) * VS;
  k_csr<VS, MODE, double, double><<<grid_for(threads, 256), 256, 0, s>>>(a.rows, a.ptr.p, a.col.p, a.v64.p, x, y, b);
  SIMP_CHECK_LAUNCH();
}

template <int MODE>
void launch_csr(const DevCsr& a, const double* x, double* y, const double* b, cudaStream_t s) {
  switch (lanes_for(a)) {
    case 2: launch_csr_vs<2, MODE>(a, x, y, b, s); break;
    case 4: launch_csr_vs<4, MODE>(a, x, y, b, s); break;
    case 8: launch_csr_vs<8, MODE>(a, x, y, b, s); break;
    case 16: launch_csr_vs<16, MODE>(a, x, y, b, s); break;
    default: launch_csr_vs<32, MODE>(a, x, y, b, s); break;
  }
}

template <int VS>
void launch_cheb_step_vs(const DevCsr& a, const double* d, const double* rin, double* r, double* dn,
                         double* x, const double* dinv, double c1, double c2, int add_d, cudaStream_t s) {
  const i64 threads = static_cast<i64>(a.rows) * VS;
  k_cheb_step<VS, double, double><<<grid_for(threads, 256), 256, 0, s>>>(
      a.rows, a.ptr.p, a.col.p, a.v64.p, d, rin, r, dn, x, dinv, c1, c2, add_d);
  SIMP_CHECK_LAUNCH();
}

void launch_cheb_step(const DevCsr& a, const double* d, const double* rin, double* r, double* dn,
                      double* x, const double* dinv, double c1, double c2, int add_d, cudaStream_t s) {
  switch (lanes_for(a)) {
    case 2: launch_cheb_step_vs<2>(a, d, rin, r, dn, x, dinv, c1, c2, add_d, s); break;
    case 4: launch_cheb_step_vs<4>(a, d, rin, r, dn, x, dinv, c1, c2, add_d, s); break;
    case 8: launch_cheb_step_vs<8>(a, d, rin, r, dn, x, dinv, c1, c2, add_d, s); break;
    case 16: launch_cheb_step_vs<16>(a, d, rin, r, dn, x, dinv, c1, c2, add_d, s); break;
    default: launch_cheb_step_vs<32>(a, d, rin, r, dn, x, dinv, c1, c2, add_d, s); break;
  }
}

template <int VS>
void launch_cheb_first_vs(const DevCsr& a, const double* x, const double* b, double* r, double* d,
                          const double* dinv, double inv_theta, cudaStream_t s) {
  const i64 threads = static_cast<i64>(a.rows) * VS;
  k_cheb_first<VS, double, double><<<grid_for(threads, 256), 256, 0, s>>>(
      a.rows, a.ptr.p, a.col.p, a.v64.p, x, b, r, d, dinv, inv_theta);
  SIMP_CHECK_LAUNCH();
}

void launch_cheb_first(const DevCsr& a, const double* x, const double* b, double* r, double* d,
                       const double* dinv, double inv_theta, cudaStream_t s) {
  switch (lanes_for(a)) {
    case 2: launch_cheb_first_vs<2>(a, x, b, r, d, dinv, inv_theta, s); break;
    case 4: launch_cheb_first_vs<4>(a, x, b, r, d, dinv, inv_theta, s); break;
    case 8: launch_cheb_first_vs<8>(a, x, b, r, d, dinv, inv_theta, s); break;
    case 16: launch_cheb_first_vs<16>(a, x, b, r, d, dinv, inv_theta, s); break;
    default: launch_cheb_first_vs<32>(a, x, b, r, d, dinv, inv_theta, s); break;
  }
}

template <int VS>
void launch_lanczos_vs(const DevCsr& a, const double* tmp, const double* s, const double* vp, double beta,
                       double* w, cudaStream_t st) {
  const i64 threads = static_cast<i64>(a.rows) * VS;
  k_lanczos_apply<VS, double><<<grid_for(threads, 256), 256, 0, st>>>(a.rows, a.ptr.p, a.col.p, a.v64.p,
                                                                      tmp, s, vp, beta, w);
  SIMP_CHECK_LAUNCH();
}

void launch_lanczos(const DevCsr& a, const double* tmp, const double* s, const double* vp, double beta,
                    double* w, cudaStream_t st) {
  switch (lanes_for(a)) {
    case 2: launch_lanczos_vs<2>(a, tmp, s, vp, beta, w, st); break;
    case 4: launch_lanczos_vs<4>(a, tmp, s, vp, beta, w, st); break;
    case 8: launch_lanczos_vs<8>(a, tmp, s, vp, beta, w, st); break;
    case 16: launch_lanczos_vs<16>(a, tmp, s, vp, beta, w, st); break;
    default: launch_lanczos_vs<32>(a, tmp, s, vp, beta, w, st); break;
  }
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

void csr_apply(const DevCsr& a, const double* x, double* y, cudaStream_t s) { launch_csr<0>(a, x, y, nullptr, s); }

GpuAmg::GpuAmg(const AmgOptions& o) : opt(o) {
  part.alloc(kRedBlocks);
  scal.alloc(16);
  dstatus.alloc(4);
}

GpuAmg::~GpuAmg() = default;

Level& GpuAmg::level0() {
  if (levels.empty()) levels.emplace_back(new Level());
  return *levels.front();
}

double GpuAmg::dot(const double* a, const double* b, i64 n) {
  k_dot_partial<double, double><<<kRedBlocks, kRedThreads, 0, stream>>>(a, b, n, part.p);
  SIMP_CHECK_LAUNCH();
  k_reduce_final<<<1, kRedThreads, 0, stream>>>(part.p, kRedBlocks, scal.p, 0);
  SIMP_CHECK_LAUNCH();
  double h = 0.0;
  SIMP_CUDA(cudaMemcpyAsync(&h, scal.p, sizeof(double), cudaMemcpyDeviceToHost, stream));
  SIMP_CUDA(cudaStreamSynchronize(stream));
  return h;
}

void GpuAmg::spmv0(const double* x, double* y) { launch_csr<0>(levels.front()->a, x, y, nullptr, stream); }

// inverse diagonal and lambda_max(D^-1 A) of one level (Multigrid.cpp:718-747)
void GpuAmg::numeric_level(size_t l) {
  Level& lv = *levels[l];
  const i32 n = lv.n;
  lv.dinv64.alloc(n);
  SIMP_CUDA(cudaMemsetAsync(dstatus.p, 0x7f, sizeof(int), stream));
  k_inv_diag<double><<<grid_for(n, 256), 256, 0, stream>>>(n, lv.d_node_of.p, lv.d_first.p, lv.d_self.p,
                                                           lv.d_apat.view(), lv.a.ptr.p, lv.a.v64.p,
                                                           lv.dinv64.p, dstatus.p);
  SIMP_CHECK_LAUNCH();
  int bad = 0;
  SIMP_CUDA(cudaMemcpyAsync(&bad, dstatus.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
  SIMP_CUDA(cudaStreamSynchronize(stream));
  if (bad != 0x7f7f7f7f) {
    std::ostringstream os;
    os << "multigrid level " << l << ": diagonal entry " << bad
       << " is not positive; a stiffness matrix must have a positive diagonal. The model has an "
          "unconnected degree of freedom or a non-positive stiffness";
    throw Error(kBreakdown, os.str());
  }
  // Lanczos on D^-1/2 A D^-1/2 with the reference's start vector.
  DBuf<double> v(n), vp(n), w(n), s(n), tmp(n);
  {
    std::vector<double> h(static_cast<size_t>(n));
    for (i32 i = 0; i < n; ++i) h[i] = 1.0 + 0.5 * std::sin(1.7 * static_cast<double>(i) + 0.3);
    v.upload(h, stream);
    const double nv = std::sqrt(dot(v.p, v.p, n));
    SIMP_CUDA(cudaMemcpyAsync(scal.p + 1, &nv, sizeof(double), cudaMemcpyHostToDevice, stream));
    k_lanczos_start<<<grid_for(n, 256), 256, 0, stream>>>(v.p, scal.p + 1, lv.dinv64.p, s.p, tmp.p, n);
    SIMP_CHECK_LAUNCH();
  }
  std::vector<double> alpha, beta;
  const int m = std::max(1, std::min<int>(opt.lanczos_steps, n));
  for (int j = 0; j < m; ++j) {
    launch_lanczos(lv.a, tmp.p, s.p, j > 0 ? vp.p : nullptr, j > 0 ? beta.back() : 0.0, w.p, stream);
    const double aj = dot(w.p, v.p, n);
    alpha.push_back(aj);
    SIMP_CUDA(cudaMemcpyAsync(scal.p + 2, &aj, sizeof(double), cudaMemcpyHostToDevice, stream));
    k_axpy_norm<<<kRedBlocks, kRedThreads, 0, stream>>>(w.p, v.p, scal.p + 2, n, part.p);
    SIMP_CHECK_LAUNCH();
    k_reduce_final<<<1, kRedThreads, 0, stream>>>(part.p, kRedBlocks, scal.p + 3, 1);
    SIMP_CHECK_LAUNCH();
    double bj = 0.0;
    SIMP_CUDA(cudaMemcpyAsync(&bj, scal.p + 3, sizeof(double), cudaMemcpyDeviceToHost, stream));
    SIMP_CUDA(cudaStreamSynchronize(stream));
    if (j + 1 == m || !(bj > 1.0e-12 * std::abs(aj))) break;
    beta.push_back(bj);
    k_lanczos_shift<<<grid_for(n, 256), 256, 0, stream>>>(v.p, vp.p, w.p, s.p, tmp.p, bj, n);
    SIMP_CHECK_LAUNCH();
  }
  std::vector<double> off(beta.begin(), beta.begin() + static_cast<long>(alpha.size() - 1));
  lv.lambda = tridiagonal_max_eigenvalue(alpha, off);
  if (!(lv.lambda > 0.0) || !std::isfinite(lv.lambda)) {
    std::ostringstream os;
    os << "multigrid level " << l << ": the spectral estimate of D^-1 A is " << lv.lambda
       << "; the matrix is not positive definite";
    throw Error(kBreakdown, os.str());
  }
  // Chebyshev coefficients on [lambda / ratio, 1.1 lambda] (Multigrid.cpp:812-853)
  const double upper = 1.1 * lv.lambda, lower = upper / opt.cheb_ratio;
  const double theta = 0.5 * (upper + lower), delta = 0.5 * (upper - lower);
  const double sigma = theta / delta;
  double rho = 1.0 / sigma;
  lv.inv_theta = 1.0 / theta;
  lv.c1.clear();
  lv.c2.clear();
  for (int k = 1; k < opt.degree; ++k) {
    const double rn = 1.0 / (2.0 * sigma - rho);
    lv.c1.push_back(rn * rho);
    lv.c2.push_back(2.0 * rn / delta);
    rho = rn;
  }
  lv.x64.alloc(n);
  lv.b64.alloc(n);
  lv.r64.alloc(n);
  lv.d64.alloc(n);
  lv.e64.alloc(n);
}

// Aggregates, tentative prolongator and symbolic patterns of level l -> l+1.
// Returns with levels[l+1] created, or leaves the hierarchy unchanged when
// coarsening stalls.
void GpuAmg::build_transfer(size_t l) {
  Level& lv = *levels[l];
  // strength of connection from the FP64 values (block sums of squares)
  DBuf<double> acc(static_cast<size_t>(lv.apat.slots()));
  k_block_sumsq<<<grid_for(lv.nnodes, 128), 128, 0, stream>>>(lv.nnodes, lv.d_first.p, lv.d_apat.view(),
                                                               lv.d_first.p, lv.a.ptr.p, lv.a.v64.p, acc.p);
  SIMP_CHECK_LAUNCH();
  const std::vector<double> hacc = acc.to_host(stream);
  const std::vector<i32> self = pattern_self_slots(lv.apat);
  std::vector<double> bdiag(static_cast<size_t>(lv.nnodes));
  for (i32 I = 0; I < lv.nnodes; ++I) bdiag[I] = self[I] >= 0 ? std::sqrt(hacc[self[I]]) : 0.0;
  lv.naggs = aggregate_nodes(lv.apat, hacc, bdiag, opt.theta, lv.agg);
  const int m = static_cast<int>(lv.null.size() / std::max<i32>(lv.n, 1));
  Tentative t = tentative_prolongator(lv.first, lv.agg, lv.naggs, lv.null, m);
  const i32 nc = t.next_first.back();
  if (nc >= static_cast<i32>(0.85 * static_cast<double>(lv.n)) || nc == 0) {
    lv.agg.clear();
    lv.naggs = 0;
    return;
  }
  std::unique_ptr<Level> nx(new Level());
  Level& nv = *nx;
  nv.first = std::move(t.next_first);
  nv.nnodes = lv.naggs;
  nv.n = nc;
  nv.null = std::move(t.next_null);
  nv.d_first.upload(nv.first, stream);
  nv.d_node_of.upload(node_of_unknowns(nv.first), stream);
  lv.d_agg.upload(lv.agg, stream);
  lv.phat_ptr.upload(t.phat_ptr, stream);
  lv.phat64.upload(t.phat, stream);
  // symbolic patterns
  lv.ppat = pattern_prolongator(lv.apat, lv.agg, lv.naggs);
  finish_offsets(lv.ppat, nv.first);
  std::vector<i32> r_to_p;
  lv.rpat = pattern_transpose(lv.ppat, &r_to_p);
  finish_offsets(lv.rpat, lv.first);
  lv.appat = pattern_product(lv.apat, lv.ppat);
  finish_offsets(lv.appat, nv.first);
  nv.apat = pattern_product(lv.rpat, lv.appat);
  finish_offsets(nv.apat, nv.first);
  const std::vector<i32> sym_t = pattern_transpose_slots(nv.apat);
  lv.d_ppat.upload(lv.ppat);
  lv.d_rpat.upload(lv.rpat);
  lv.d_appat.upload(lv.appat);
  nv.d_apat.upload(nv.apat);
  lv.d_r_to_p.upload(r_to_p, stream);
  lv.d_sym_t.upload(sym_t, stream);
  nv.d_self.upload(pattern_self_slots(nv.apat), stream);
  // scalar CSR structures
  auto make = [&](DevCsr& c, const NodePattern& pat, const std::vector<i32>& row_first,
                  const std::vector<i32>& col_first, const DBuf<i32>& row_node_of, const DevPattern& dpat,
                  const DBuf<i32>& d_col_first) {
    const std::vector<i32> ptr = scalar_rowptr(pat, row_first);
    c.rows = row_first.back();
    c.cols = col_first.back();
    c.nnz = ptr.back();
    c.ptr.upload(ptr, stream);
    c.col.alloc(static_cast<size_t>(c.nnz));
    k_expand_columns<<<grid_for(c.rows, 256), 256, 0, stream>>>(c.rows, row_node_of.p, dpat.view(),
                                                                d_col_first.p, c.ptr.p, c.col.p);
    SIMP_CHECK_LAUNCH();
    c.v64.alloc(static_cast<size_t>(c.nnz));
  };
  make(lv.p, lv.ppat, lv.first, nv.first, lv.d_node_of, lv.d_ppat, nv.d_first);
  make(lv.r, lv.rpat, nv.first, lv.first, nv.d_node_of, lv.d_rpat, lv.d_first);
  make(lv.ap, lv.appat, lv.first, nv.first, lv.d_node_of, lv.d_appat, nv.d_first);
  make(nv.a, nv.apat, nv.first, nv.first, nv.d_node_of, nv.d_apat, nv.d_first);
  lv.raw64.alloc(static_cast<size_t>(nv.a.nnz));
  levels.push_back(std::move(nx));
}

// Numeric P, R, AP, RAP and symmetrisation (Multigrid.cpp:671-716, 1047-1055).
void GpuAmg::galerkin(size_t l) {
  Level& lv = *levels[l];
  Level& nv = *levels[l + 1];
  const double omega = opt.damping / lv.lambda;
  {
    const i64 th = static_cast<i64>(lv.n) * 8;
    k_prolongator<8, double><<<grid_for(th, 256), 256, 0, stream>>>(
        lv.n, lv.d_node_of.p, lv.d_first.p, nv.d_first.p, lv.d_agg.p, lv.d_apat.view(), lv.a.ptr.p,
        lv.a.v64.p, lv.d_ppat.view(), lv.p.ptr.p, lv.p.v64.p, lv.phat_ptr.p, lv.phat64.p, lv.dinv64.p, omega);
    SIMP_CHECK_LAUNCH();
  }
  {
    const i64 th = static_cast<i64>(nv.n) * 32;
    k_restriction<32, double><<<grid_for(th, 256), 256, 0, stream>>>(
        nv.n, nv.d_node_of.p, nv.d_first.p, lv.d_first.p, lv.d_rpat.view(), lv.r.ptr.p, lv.r.v64.p,
        lv.d_r_to_p.p, lv.d_ppat.view(), lv.p.ptr.p, lv.p.v64.p);
    SIMP_CHECK_LAUNCH();
  }
  {
    const i64 th = static_cast<i64>(lv.n) * 32;
    k_product_ap<32, double><<<grid_for(th, 256), 256, 0, stream>>>(
        lv.n, lv.d_node_of.p, lv.d_first.p, nv.d_first.p, lv.d_apat.view(), lv.a.ptr.p, lv.a.v64.p,
        lv.d_ppat.view(), lv.p.ptr.p, lv.p.v64.p, lv.d_appat.view(), lv.ap.ptr.p, lv.ap.v64.p);
    SIMP_CHECK_LAUNCH();
  }
  {
    const i64 th = static_cast<i64>(nv.n) * 32;
    k_product_rap<32, double><<<grid_for(th, 256), 256, 0, stream>>>(
        nv.n, nv.d_node_of.p, nv.d_first.p, lv.d_first.p, lv.d_rpat.view(), lv.r.ptr.p, lv.r.v64.p,
        lv.d_appat.view(), lv.ap.ptr.p, lv.ap.v64.p, nv.d_apat.view(), nv.a.ptr.p, lv.raw64.p);
    SIMP_CHECK_LAUNCH();
  }
  k_symmetrize<double, double><<<grid_for(nv.n, 128), 128, 0, stream>>>(
      nv.n, nv.d_node_of.p, nv.d_first.p, nv.d_apat.view(), nv.a.ptr.p, lv.d_sym_t.p, lv.raw64.p, nv.a.v64.p,
      nullptr);
  SIMP_CHECK_LAUNCH();
}

// Dense FP64 Cholesky of the coarsest operator and W = L^-1.
void GpuAmg::coarse_factorize() {
  Level& lv = *levels.back();
  const i32 n = lv.n;
  if (n > 16000) {
    std::ostringstream os;
    os << "multigrid: the coarsest level has " << n
       << " unknowns, beyond the dense direct solve (16000); raise max_levels";
    throw Error(kBadInput, os.str());
  }
  nc_ = n;
  const size_t nn = static_cast<size_t>(n) * n;
  dense_.alloc(nn);
  inv_t_.alloc(nn);
  piv_.alloc(n);
  tmp_.alloc(n);
  SIMP_CUDA(cudaMemsetAsync(dense_.p, 0, nn * sizeof(double), stream));
  k_dense_from_csr<<<grid_for(n, 128), 128, 0, stream>>>(n, lv.a.ptr.p, lv.a.col.p, lv.a.v64.p, dense_.p);
  SIMP_CHECK_LAUNCH();
  SIMP_CUDA(cudaMemsetAsync(dstatus.p, 0, sizeof(int), stream));
  for (int k0 = 0; k0 < n; k0 += kNB) {
    const int kb = std::min(kNB, n - k0);
    k_potrf_diag<<<1, 256, 0, stream>>>(dense_.p, n, k0, kb, piv_.p, dstatus.p);
    SIMP_CHECK_LAUNCH();
    const int rest = n - k0 - kb;
    if (rest <= 0) break;
    k_trsm_panel<<<grid_for(rest, 128), 128, 0, stream>>>(dense_.p, n, k0, kb);
    SIMP_CHECK_LAUNCH();
    dim3 grid((rest + 31) / 32, (rest + 31) / 32);
    k_tile_update<<<grid, 256, 0, stream>>>(dense_.p, n, k0 + kb, k0 + kb, rest, rest, dense_.p, k0,
                                            dense_.p + k0, 1, n, kb, 1);
    SIMP_CHECK_LAUNCH();
  }
  int status = 0;
  SIMP_CUDA(cudaMemcpyAsync(&status, dstatus.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
  const std::vector<double> piv = piv_.to_host(stream);
  double mx = 0.0, mn = std::numeric_limits<double>::max();
  for (double v : piv) {
    mx = std::max(mx, std::abs(v));
    mn = std::min(mn, v);
  }
  const double ratio = mx > 0.0 ? mn / mx : 0.0;
  stats.pivot_ratio = ratio;
  if (status != 0 || !(ratio > opt.pivot_tol)) {
    std::ostringstream os;
    os << "multigrid: the coarsest operator (" << n << " unknowns) is singular or indefinite "
       << "(smallest / largest pivot " << ratio << "). A rigid-body mode survived to the coarse "
       << "level, so the model is under-constrained: too few supports, or a part connected to nothing";
    throw Error(kUnderConstrained, os.str());
  }
  // W = L^-1 into inv_t_ (row-major, lower), then keep W in inv_t_ and W^T in dense_
  k_identity<<<grid_for(static_cast<i64>(nn), 256), 256, 0, stream>>>(inv_t_.p, n);
  SIMP_CHECK_LAUNCH();
  for (int k0 = 0; k0 < n; k0 += kNB) {
    const int kb = std::min(kNB, n - k0);
    k_trsm_rows<<<grid_for(k0 + kb, 128), 128, 0, stream>>>(inv_t_.p, dense_.p, n, k0, kb);
    SIMP_CHECK_LAUNCH();
    const int rest = n - k0 - kb;
    if (rest <= 0) break;
    dim3 grid((k0 + kb + 31) / 32, (rest + 31) / 32);
    k_tile_update<<<grid, 256, 0, stream>>>(inv_t_.p, n, k0 + kb, 0, rest, k0 + kb, dense_.p, k0,
                                            inv_t_.p + static_cast<size_t>(k0) * n, n, 1, kb, 0);
    SIMP_CHECK_LAUNCH();
  }
  dim3 tg((n + 31) / 32, (n + 31) / 32), tb(32, 8);
  k_transpose<<<tg, tb, 0, stream>>>(inv_t_.p, dense_.p, n);
  SIMP_CHECK_LAUNCH();
}

// x = W^T (W b) at the coarsest level
void GpuAmg::coarse_solve(const Level& lv) {
  const int n = nc_;
  const i64 th = static_cast<i64>(n) * 32;
  k_gemv<double, double><<<grid_for(th, 256), 256, 0, stream>>>(inv_t_.p, n, lv.b64.p, tmp_.p, 1);
  SIMP_CHECK_LAUNCH();
  k_gemv<double, double><<<grid_for(th, 256), 256, 0, stream>>>(dense_.p, n, tmp_.p, lv.x64.p, 2);
  SIMP_CHECK_LAUNCH();
}

void GpuAmg::setup(bool structure_changed) {
  const auto t0 = std::chrono::steady_clock::now();
  const bool reuse = opt.reuse && !structure_changed && ready_;
  if (!reuse) {
    // drop the coarse levels of an earlier structure
    while (levels.size() > 1) levels.pop_back();
    Level& l0 = *levels.front();
    l0.agg.clear();
    l0.naggs = 0;
  }
  const size_t reused_levels = levels.size();
  size_t l = 0;
  while (true) {
    numeric_level(l);
    Level& lv = *levels[l];
    const bool stop = reuse ? (l + 1 == reused_levels)
                            : (lv.n <= opt.coarse_size || static_cast<int>(l) + 1 >= opt.max_levels);
    if (stop) break;
    if (!reuse) {
      build_transfer(l);
      if (levels.size() == l + 1) break;  // coarsening stalled
    }
    galerkin(l);
    ++l;
  }
  levels.resize(l + 1);
  coarse_factorize();
  // PCG workspace
  const i32 n0 = levels.front()->n;
  pr.alloc(n0);
  pz.alloc(n0);
  pp.alloc(n0);
  pq.alloc(n0);
  ready_ = true;
  stats.reused = reuse;
  compute_stats();
  SIMP_CUDA(cudaStreamSynchronize(stream));
  stats.setup_seconds = seconds_since(t0);
}

void GpuAmg::compute_stats() {
  stats.num_levels = static_cast<int>(levels.size());
  double nz = 0, rows = 0, stored = 0;
  for (size_t k = 0; k < levels.size(); ++k) {
    const Level& lv = *levels[k];
    nz += static_cast<double>(lv.a.nnz);
    rows += lv.n;
    if (k > 0) stored += static_cast<double>(lv.a.nnz);
    if (k + 1 < levels.size())
      stored += static_cast<double>(lv.p.nnz + lv.r.nnz + lv.ap.nnz + levels[k + 1]->a.nnz + lv.phat64.n);
  }
  stored += static_cast<double>(nc_) * nc_;
  stats.operator_complexity = nz / static_cast<double>(levels.front()->a.nnz);
  stats.grid_complexity = rows / static_cast<double>(levels.front()->n);
  stats.storage = static_cast<i64>(std::min(stored, 2.0e9));
}

// Chebyshev smoothing of x (Multigrid.cpp:783-855) on level l.
void GpuAmg::smooth(size_t l, bool zero_guess) {
  Level& lv = *levels[l];
  const i32 n = lv.n;
  double* d = lv.d64.p;
  double* e = lv.e64.p;
  if (zero_guess) {
    k_cheb_zero<double><<<grid_for(n, 256), 256, 0, stream>>>(n, lv.b64.p, lv.dinv64.p, d, lv.x64.p, lv.inv_theta);
    SIMP_CHECK_LAUNCH();
  } else {
    launch_cheb_first(lv.a, lv.x64.p, lv.b64.p, lv.r64.p, d, lv.dinv64.p, lv.inv_theta, stream);
  }
  for (int k = 1; k < opt.degree; ++k) {
    const double* rin = (k == 1 && zero_guess) ? lv.b64.p : lv.r64.p;
    const int add_d = (k == 1 && !zero_guess) ? 1 : 0;
    launch_cheb_step(lv.a, d, rin, lv.r64.p, e, lv.x64.p, lv.dinv64.p, lv.c1[k - 1], lv.c2[k - 1], add_d,
                     stream);
    std::swap(d, e);
  }
  if (opt.degree == 1 && !zero_guess) {
    // x += d (degree 1 from a guess)
    launch_cheb_step(lv.a, d, lv.r64.p, lv.r64.p, e, lv.x64.p, lv.dinv64.p, 0.0, 0.0, 1, stream);
  }
}

void GpuAmg::cycle(size_t l) {
  Level& lv = *levels[l];
  if (l + 1 == levels.size()) {
    coarse_solve(lv);
    return;
  }
  Level& nv = *levels[l + 1];
  smooth(l, true);
  launch_csr<1>(lv.a, lv.x64.p, lv.r64.p, lv.b64.p, stream);     // residual
  launch_csr<0>(lv.r, lv.r64.p, nv.b64.p, nullptr, stream);      // restrict
  cycle(l + 1);
  launch_csr<2>(lv.p, nv.x64.p, lv.x64.p, nullptr, stream);      // x += P x_c
  smooth(l, false);
}

void GpuAmg::apply(const double* r, double* z) {
  if (!ready_) throw Error(kBadInput, "multigrid: apply() called before setup()");
  Level& f = *levels.front();
  SIMP_CUDA(cudaMemcpyAsync(f.b64.p, r, sizeof(double) * f.n, cudaMemcpyDeviceToDevice, stream));
  cycle(0);
  SIMP_CUDA(cudaMemcpyAsync(z, f.x64.p, sizeof(double) * f.n, cudaMemcpyDeviceToDevice, stream));
}

GpuAmg::PcgResult GpuAmg::solve(const double* b, double* x) {
  if (!ready_) throw Error(kBadInput, "solve called before factorize");
  Level& f = *levels.front();
  const i32 n = f.n;
  PcgResult res;
  const double bnorm = std::sqrt(dot(b, b, n));
  if (bnorm == 0.0) {
    SIMP_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, stream));
    res.converged = true;
    return res;
  }
  const double target = opt.rtol * bnorm;
  PcgScalars* sc = reinterpret_cast<PcgScalars*>(scal.p + 8);
  static_assert(sizeof(PcgScalars) <= 8 * sizeof(double), "scalar block");
  int total = 0;
  bool rec_conv = false;
  double best = std::numeric_limits<double>::max();
  for (int restart = 0; restart < 3; ++restart) {
    launch_csr<1>(f.a, x, pr.p, b, stream);
    double rnorm = std::sqrt(dot(pr.p, pr.p, n));
    res.relres = rnorm / bnorm;
    if (rnorm <= target) { res.converged = true; break; }
    apply(pr.p, pz.p);
    SIMP_CUDA(cudaMemcpyAsync(pp.p, pz.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
    const double rz = dot(pr.p, pz.p, n);
    {
      PcgScalars h{};
      h.rz = rz;
      SIMP_CUDA(cudaMemcpyAsync(sc, &h, sizeof(h), cudaMemcpyHostToDevice, stream));
    }
    bool conv = false;
    while (total < opt.maxit) {
      launch_csr<0>(f.a, pp.p, pq.p, nullptr, stream);
      k_dot_partial<double, double><<<kRedBlocks, kRedThreads, 0, stream>>>(pp.p, pq.p, n, part.p);
      SIMP_CHECK_LAUNCH();
      k_pcg_alpha<<<1, kRedThreads, 0, stream>>>(part.p, kRedBlocks, sc);
      SIMP_CHECK_LAUNCH();
      k_pcg_update<<<kRedBlocks, kRedThreads, 0, stream>>>(x, pr.p, pp.p, pq.p, n, sc, part.p);
      SIMP_CHECK_LAUNCH();
      k_reduce_final<<<1, kRedThreads, 0, stream>>>(part.p, kRedBlocks, &sc->rr, 0);
      SIMP_CHECK_LAUNCH();
      PcgScalars h{};
      SIMP_CUDA(cudaMemcpyAsync(&h, sc, sizeof(h), cudaMemcpyDeviceToHost, stream));
      SIMP_CUDA(cudaStreamSynchronize(stream));
      if (h.status != 0) {
        std::ostringstream os;
        os << "preconditioned CG broke down at iteration " << total + 1 << " (p^T A p = " << h.pq
           << "): the stiffness matrix or the multigrid preconditioner is not positive definite. "
              "Check the supports, or use a direct solver to confirm";
        throw Error(kBreakdown, os.str());
      }
      ++total;
      rnorm = std::sqrt(h.rr);
      if (rnorm <= target) { conv = true; break; }
      apply(pr.p, pz.p);
      k_dot_partial<double, double><<<kRedBlocks, kRedThreads, 0, stream>>>(pr.p, pz.p, n, part.p);
      SIMP_CHECK_LAUNCH();
      k_pcg_beta<<<1, kRedThreads, 0, stream>>>(part.p, kRedBlocks, sc);
      SIMP_CHECK_LAUNCH();
      k_pcg_direction<<<grid_for(n, 256), 256, 0, stream>>>(pp.p, pz.p, n, sc);
      SIMP_CHECK_LAUNCH();
    }
    launch_csr<1>(f.a, x, pr.p, b, stream);
    res.relres = std::sqrt(dot(pr.p, pr.p, n)) / bnorm;
    if (res.relres <= opt.rtol) { res.converged = true; break; }
    if (!conv) break;
    rec_conv = true;
    if (!(res.relres < 0.5 * best)) break;
    best = res.relres;
  }
  if (!res.converged && rec_conv) res.converged = true;
  res.iterations = total;
  return res;
}

}  // namespace simp
