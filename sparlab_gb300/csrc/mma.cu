// MMA update on the GPU for the compliance / volume problem
// (src/topopt/Mma.cpp:63-409, driven as src/topopt/TopologyOptimizer.cpp:
// 730-905): f0 = c / c_1, one constraint f1 = V / V* - 1, bounds [0, 1].
//
// The design-sized vectors of the outer update and of the primal-dual
// subproblem live on the device; the handful of scalars (y, z, lambda, mu,
// zeta, s and the barrier) stay on the host, and each Newton step needs three
// fixed-shape reductions: the residual (sum of squares, largest entry and the
// constraint's separable term), the reduced (lambda, z) system, and the step
// length.
#include "kernels.cuh"
#include "problem.h"
#include "topopt.cuh"

#include <algorithm>
#include <cmath>
#include <sstream>

namespace simp {
namespace {

struct MmaCoef {
  const double* alfa;
  const double* beta;
  const double* low;
  const double* upp;
  const double* p0;
  const double* q0;
  const double* p;
  const double* q;
};

// Asymptotes (Mma.cpp:76-95).
__global__ void k_mma_asymptotes(i64 n, int iteration, const double* __restrict__ x, const double* __restrict__ x1,
                                 const double* __restrict__ x2, double* __restrict__ low, double* __restrict__ upp,
                                 double init, double inc, double dec) {
  for (i64 j = blockIdx.x * (i64)blockDim.x + threadIdx.x; j < n; j += (i64)gridDim.x * blockDim.x) {
    const double xj = x[j];
    if (iteration <= 2) {
      low[j] = xj - init;
      upp[j] = xj + init;
    } else {
      const double zzz = (xj - x1[j]) * (x1[j] - x2[j]);
      double f = 1.0;
      if (zzz > 0.0) f = inc;
      if (zzz < 0.0) f = dec;
      double l = xj - f * (x1[j] - low[j]);
      double u = xj + f * (upp[j] - x1[j]);
      l = fmin(fmax(l, xj - 10.0), xj - 0.01);
      u = fmin(fmax(u, xj + 0.01), xj + 10.0);
      low[j] = l;
      upp[j] = u;
    }
  }
}

// Bounds and approximation coefficients (Mma.cpp:97-151); partial sums of
// the constraint's sum_j p_j / (u_j - x_j) + q_j / (x_j - l_j).
__global__ void __launch_bounds__(kRedThreads) k_mma_coeffs(i64 n, const double* __restrict__ x,
                                                            const double* __restrict__ low,
                                                            const double* __restrict__ upp,
                                                            const double* __restrict__ dc, double dc_scale,
                                                            const double* __restrict__ dv, double dv_scale,
                                                            double move, double albefa, double raa0,
                                                            double* __restrict__ alfa, double* __restrict__ beta,
                                                            double* __restrict__ p0, double* __restrict__ q0,
                                                            double* __restrict__ p, double* __restrict__ q,
                                                            double* __restrict__ part) {
  double bs = 0.0;
  for (i64 j = blockIdx.x * (i64)kRedThreads + threadIdx.x; j < n; j += (i64)gridDim.x * kRedThreads) {
    const double xj = x[j], lj = low[j], uj = upp[j];
    alfa[j] = fmax(fmax(lj + albefa * (xj - lj), xj - move), 0.0);
    beta[j] = fmin(fmin(uj - albefa * (uj - xj), xj + move), 1.0);
    const double ux1 = uj - xj, xl1 = xj - lj;
    const double ux2 = ux1 * ux1, xl2 = xl1 * xl1;
    const double g0 = dc[j] * dc_scale;
    const double pp0 = fmax(g0, 0.0), qq0 = fmax(-g0, 0.0);
    const double pq0 = 0.001 * (pp0 + qq0) + raa0;
    p0[j] = (pp0 + pq0) * ux2;
    q0[j] = (qq0 + pq0) * xl2;
    const double g1 = dv[j] * dv_scale;
    const double pp = fmax(g1, 0.0), qq = fmax(-g1, 0.0);
    const double pq = 0.001 * (pp + qq) + raa0;
    const double pj = (pp + pq) * ux2, qj = (qq + pq) * xl2;
    p[j] = pj;
    q[j] = qj;
    bs += pj / ux1 + qj / xl1;
  }
  bs = block_sum<kRedThreads>(bs);
  if (threadIdx.x == 0) part[blockIdx.x] = bs;
}

__device__ __forceinline__ double block_max(double v) {
  __shared__ double wmax[kRedThreads / 32];
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = v;
  __syncthreads();
  double m = 0.0;
  if (threadIdx.x < 32) {
    m = threadIdx.x < kRedThreads / 32 ? wmax[threadIdx.x] : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  }
  __syncthreads();
  return m;
}

// Trial point (optional) and the design-sized part of the KKT residual
// (Mma.cpp:186-238): partials of sum of squares, largest |entry| and the
// constraint term sum_j p_j / (u_j - x_j) + q_j / (x_j - l_j).
__global__ void __launch_bounds__(kRedThreads) k_mma_residual(
    i64 n, MmaCoef c, double lam, double epsi, double steg, const double* __restrict__ xo,
    const double* __restrict__ xsio, const double* __restrict__ etao, const double* __restrict__ dx,
    const double* __restrict__ dxsi, const double* __restrict__ deta, double* __restrict__ x,
    double* __restrict__ xsi, double* __restrict__ eta, double* __restrict__ part) {
  double sq = 0.0, mx = 0.0, gv = 0.0;
  for (i64 j = blockIdx.x * (i64)kRedThreads + threadIdx.x; j < n; j += (i64)gridDim.x * kRedThreads) {
    double xj, sj, ej;
    if (xo) {
      xj = xo[j] + steg * dx[j];
      sj = xsio[j] + steg * dxsi[j];
      ej = etao[j] + steg * deta[j];
      x[j] = xj;
      xsi[j] = sj;
      eta[j] = ej;
    } else {
      xj = x[j];
      sj = xsi[j];
      ej = eta[j];
    }
    const double ux1 = c.upp[j] - xj, xl1 = xj - c.low[j];
    const double plam = c.p0[j] + c.p[j] * lam, qlam = c.q0[j] + c.q[j] * lam;
    gv += c.p[j] / ux1 + c.q[j] / xl1;
    const double rex = plam / (ux1 * ux1) - qlam / (xl1 * xl1) - sj + ej;
    const double rexsi = sj * (xj - c.alfa[j]) - epsi;
    const double reeta = ej * (c.beta[j] - xj) - epsi;
    sq += rex * rex + rexsi * rexsi + reeta * reeta;
    mx = fmax(mx, fmax(fabs(rex), fmax(fabs(rexsi), fabs(reeta))));
    if (!isfinite(rex) || !isfinite(rexsi) || !isfinite(reeta)) mx = INFINITY;
  }
  const double bsq = block_sum<kRedThreads>(sq);
  const double bgv = block_sum<kRedThreads>(gv);
  const double bmx = block_max(mx);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = bsq;
    part[gridDim.x + blockIdx.x] = bmx;
    part[2 * gridDim.x + blockIdx.x] = bgv;
  }
}

// Newton system pieces (Mma.cpp:246-282): delx, diagx, gg per variable and
// partials of sum gg delx / diagx, sum gg^2 / diagx and the constraint term.
__global__ void __launch_bounds__(kRedThreads) k_mma_newton(i64 n, MmaCoef c, double lam, double epsi,
                                                            const double* __restrict__ x,
                                                            const double* __restrict__ xsi,
                                                            const double* __restrict__ eta,
                                                            double* __restrict__ delx, double* __restrict__ diagx,
                                                            double* __restrict__ gg, double* __restrict__ part) {
  double sgd = 0.0, sgg = 0.0, gv = 0.0;
  for (i64 j = blockIdx.x * (i64)kRedThreads + threadIdx.x; j < n; j += (i64)gridDim.x * kRedThreads) {
    const double xj = x[j];
    const double ux1 = c.upp[j] - xj, xl1 = xj - c.low[j];
    const double ux2 = ux1 * ux1, xl2 = xl1 * xl1;
    const double plam = c.p0[j] + c.p[j] * lam, qlam = c.q0[j] + c.q[j] * lam;
    gv += c.p[j] / ux1 + c.q[j] / xl1;
    const double g = c.p[j] / ux2 - c.q[j] / xl2;
    const double xa = xj - c.alfa[j], bx = c.beta[j] - xj;
    const double dl = plam / ux2 - qlam / xl2 - epsi / xa + epsi / bx;
    const double dg = 2.0 * (plam / (ux2 * ux1) + qlam / (xl2 * xl1)) + xsi[j] / xa + eta[j] / bx;
    delx[j] = dl;
    diagx[j] = dg;
    gg[j] = g;
    sgd += g * (dl / dg);
    sgg += g * g / dg;
  }
  const double a = block_sum<kRedThreads>(sgd);
  const double b = block_sum<kRedThreads>(sgg);
  const double d = block_sum<kRedThreads>(gv);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = a;
    part[gridDim.x + blockIdx.x] = b;
    part[2 * gridDim.x + blockIdx.x] = d;
  }
}

// Directions of x, xsi, eta and the partial maxima of the step-length ratios
// (Mma.cpp:312-332).
__global__ void __launch_bounds__(kRedThreads) k_mma_direction(i64 n, MmaCoef c, double dlam, double epsi,
                                                               const double* __restrict__ x,
                                                               const double* __restrict__ xsi,
                                                               const double* __restrict__ eta,
                                                               const double* __restrict__ delx,
                                                               const double* __restrict__ diagx,
                                                               const double* __restrict__ gg,
                                                               double* __restrict__ dx, double* __restrict__ dxsi,
                                                               double* __restrict__ deta, double* __restrict__ part) {
  double st = -INFINITY;
  for (i64 j = blockIdx.x * (i64)kRedThreads + threadIdx.x; j < n; j += (i64)gridDim.x * kRedThreads) {
    const double xj = x[j];
    const double d = -delx[j] / diagx[j] - (gg[j] * dlam) / diagx[j];
    const double xa = xj - c.alfa[j], bx = c.beta[j] - xj;
    const double ds = -xsi[j] + epsi / xa - (xsi[j] * d) / xa;
    const double de = -eta[j] + epsi / bx + (eta[j] * d) / bx;
    dx[j] = d;
    dxsi[j] = ds;
    deta[j] = de;
    st = fmax(st, fmax(fmax(-1.01 * ds / xsi[j], -1.01 * de / eta[j]), fmax(-1.01 * d / xa, 1.01 * d / bx)));
  }
  const double m = block_max(st);
  if (threadIdx.x == 0) part[blockIdx.x] = m;
}

__global__ void k_mma_start(i64 n, const double* __restrict__ alfa, const double* __restrict__ beta,
                            double* __restrict__ x, double* __restrict__ xsi, double* __restrict__ eta) {
  for (i64 j = blockIdx.x * (i64)blockDim.x + threadIdx.x; j < n; j += (i64)gridDim.x * blockDim.x) {
    const double xj = 0.5 * (alfa[j] + beta[j]);
    x[j] = xj;
    xsi[j] = fmax(1.0 / (xj - alfa[j]), 1.0);
    eta[j] = fmax(1.0 / (beta[j] - xj), 1.0);
  }
}

__global__ void __launch_bounds__(kRedThreads) k_max_abs(i64 n, const double* __restrict__ v, double* __restrict__ part) {
  double m = 0.0;
  for (i64 j = blockIdx.x * (i64)kRedThreads + threadIdx.x; j < n; j += (i64)gridDim.x * kRedThreads)
    m = fmax(m, fabs(v[j]));
  m = block_max(m);
  if (threadIdx.x == 0) part[blockIdx.x] = m;
}

}  // namespace

void GpuProblem::mma_reduce(int k, std::vector<double>& out) {
  std::vector<double> h(static_cast<size_t>(k) * kRedBlocks);
  SIMP_CUDA(cudaMemcpyAsync(h.data(), mpart.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, amg.stream));
  SIMP_CUDA(cudaStreamSynchronize(amg.stream));
  out.assign(k, 0.0);
  for (int q = 0; q < k; ++q) {
    double s = 0.0;
    for (int b = 0; b < kRedBlocks; ++b) s += h[static_cast<size_t>(q) * kRedBlocks + b];
    out[q] = s;
  }
}

double GpuProblem::mma_reduce_max(int which) {
  std::vector<double> h(kRedBlocks);
  SIMP_CUDA(cudaMemcpyAsync(h.data(), mpart.p + static_cast<size_t>(which) * kRedBlocks, sizeof(double) * kRedBlocks,
                            cudaMemcpyDeviceToHost, amg.stream));
  SIMP_CUDA(cudaStreamSynchronize(amg.stream));
  double m = -INFINITY;
  for (double v : h) m = std::max(m, v);
  return m;
}

OcStep GpuProblem::mma_update(bool apply, double* xnew_host) {
  if (!evaluated) throw Error(kBadInput, "mma_update needs gradients: call evaluate first");
  cudaStream_t s = amg.stream;
  const size_t nn = static_cast<size_t>(ne);
  if (!mma_ready) {
    for (DBuf<double>* b : {&m_x1, &m_x2, &m_low, &m_upp, &m_alfa, &m_beta, &m_p0, &m_q0, &m_p, &m_q, &m_x, &m_xsi,
                            &m_eta, &m_xo, &m_xsio, &m_etao, &m_dx, &m_dxsi, &m_deta, &m_delx, &m_diagx, &m_gg})
      b->alloc(nn);
    mpart.alloc(3 * kRedBlocks);
    m_x1.zero(s);
    m_x2.zero(s);
    mma_iteration = 0;
    mma_ready = true;
  }
  ++mma_iteration;
  if (mma_iteration == 1) c_ref = last_evaluation.compliance;
  if (!(c_ref > 0.0)) throw Error(kBadInput, "the initial compliance is not positive; MMA cannot scale it");
  // the volume row: the dilated design against the moved target in a robust
  // run (TopologyOptimizer.cpp:823-836)
  if (d.robust && dilated_target <= 0.0) dilated_target = d.vf * domain_volume;
  const double target = d.robust ? dilated_target : d.vf * domain_volume;
  const double fval = (d.robust ? last_evaluation.volume_dilated : last_evaluation.volume) / target - 1.0;
  const double* dv = d.robust ? dv_dilated.p : dv_dx.p;
  const double move = d.move, albefa = 0.1, raa0 = 1.0e-5, a0 = 1.0, cc = 1000.0, dd = 1.0, epsimin = 1.0e-7;
  const int grid = kRedBlocks;
  k_mma_asymptotes<<<grid_for(ne, 256), 256, 0, s>>>(ne, mma_iteration, x.p, m_x1.p, m_x2.p, m_low.p, m_upp.p, 0.5,
                                                     1.2, 0.7);
  SIMP_CHECK_LAUNCH();
  // constraint row scale (Mma.cpp:138-149)
  k_max_abs<<<grid, kRedThreads, 0, s>>>(ne, dv, mpart.p);
  SIMP_CHECK_LAUNCH();
  const double dmax = mma_reduce_max(0) / target;
  const double magnitude = std::max(std::abs(fval), dmax * move);
  const double row_scale = magnitude > 10.0 ? 10.0 / magnitude : 1.0;
  k_mma_coeffs<<<grid, kRedThreads, 0, s>>>(ne, x.p, m_low.p, m_upp.p, dc_dx.p, 1.0 / c_ref, dv,
                                            row_scale / target, move, albefa, raa0, m_alfa.p, m_beta.p, m_p0.p, m_q0.p,
                                            m_p.p, m_q.p, mpart.p);
  SIMP_CHECK_LAUNCH();
  std::vector<double> red;
  mma_reduce(1, red);
  const double b = red[0] - row_scale * fval;
  MmaCoef co{m_alfa.p, m_beta.p, m_low.p, m_upp.p, m_p0.p, m_q0.p, m_p.p, m_q.p};
  // primal-dual interior point (Mma.cpp:158-395), one constraint
  double epsi = 1.0;
  k_mma_start<<<grid_for(ne, 256), 256, 0, s>>>(ne, m_alfa.p, m_beta.p, m_x.p, m_xsi.p, m_eta.p);
  SIMP_CHECK_LAUNCH();
  double y = 1.0, z = 1.0, lam = 1.0, mu = std::max(0.5 * cc, 1.0), zet = 1.0, sl = 1.0;
  auto residual = [&](const double* xo, double steg, double yv, double zv, double lv, double muv, double zetv,
                      double sv, double& norm) {
    k_mma_residual<<<grid, kRedThreads, 0, s>>>(ne, co, lv, epsi, steg, xo, xo ? m_xsio.p : nullptr,
                                                xo ? m_etao.p : nullptr, m_dx.p, m_dxsi.p, m_deta.p, m_x.p, m_xsi.p,
                                                m_eta.p, mpart.p);
    SIMP_CHECK_LAUNCH();
    std::vector<double> h(3 * static_cast<size_t>(kRedBlocks));
    SIMP_CUDA(cudaMemcpyAsync(h.data(), mpart.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s));
    SIMP_CUDA(cudaStreamSynchronize(s));
    double sq = 0.0, mx = 0.0, gv = 0.0;
    for (int k = 0; k < kRedBlocks; ++k) {
      sq += h[k];
      mx = std::max(mx, h[kRedBlocks + k]);
      gv += h[2 * kRedBlocks + k];
    }
    const double rey = cc + dd * yv - muv - lv;
    const double rez = a0 - zetv;
    const double relam = gv - yv + sv - b;
    const double remu = muv * yv - epsi, rezet = zetv * zv - epsi, res = lv * sv - epsi;
    sq += rey * rey + rez * rez + relam * relam + remu * remu + rezet * rezet + res * res;
    mx = std::max({mx, std::abs(rey), std::abs(rez), std::abs(relam), std::abs(remu), std::abs(rezet), std::abs(res)});
    if (!std::isfinite(sq)) {
      norm = INFINITY;
      return static_cast<double>(INFINITY);
    }
    norm = std::sqrt(sq);
    return mx;
  };
  int total = 0;
  while (epsi > epsimin) {
    double cur_norm;
    double cur_max = residual(nullptr, 0.0, y, z, lam, mu, zet, sl, cur_norm);
    int ittt = 0;
    while (cur_max > 0.9 * epsi && ittt < 500) {
      ++ittt;
      ++total;
      k_mma_newton<<<grid, kRedThreads, 0, s>>>(ne, co, lam, epsi, m_x.p, m_xsi.p, m_eta.p, m_delx.p, m_diagx.p,
                                                m_gg.p, mpart.p);
      SIMP_CHECK_LAUNCH();
      mma_reduce(3, red);
      const double sgd = red[0], sgg = red[1], gv = red[2];
      const double dely = cc + dd * y - lam - epsi / y;
      const double delz = a0 - epsi / z;
      const double dellam = gv - y - b + epsi / lam;
      const double diagy = dd + mu / y;
      const double diaglamyi = sl / lam + 1.0 / diagy;
      const double blam = dellam + dely / diagy - sgd;
      const double a11 = diaglamyi + sgg, a22 = -zet / z;
      const double det = a11 * a22;
      const double dlam = (blam * a22) / det;
      const double dz = (a11 * delz) / det;
      const double dy = -dely / diagy + dlam / diagy;
      k_mma_direction<<<grid, kRedThreads, 0, s>>>(ne, co, dlam, epsi, m_x.p, m_xsi.p, m_eta.p, m_delx.p, m_diagx.p,
                                                   m_gg.p, m_dx.p, m_dxsi.p, m_deta.p, mpart.p);
      SIMP_CHECK_LAUNCH();
      double stmxx = mma_reduce_max(0);
      const double dmu = -mu + epsi / y - (mu * dy) / y;
      const double dzet = -zet + epsi / z - zet * dz / z;
      const double dss = -sl + epsi / lam - (sl * dlam) / lam;
      stmxx = std::max({stmxx, -1.01 * dy / y, -1.01 * dz / z, -1.01 * dlam / lam, -1.01 * dmu / mu,
                        -1.01 * dzet / zet, -1.01 * dss / sl});
      double steg = 1.0 / std::max(stmxx, 1.0);
      SIMP_CUDA(cudaMemcpyAsync(m_xo.p, m_x.p, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s));
      SIMP_CUDA(cudaMemcpyAsync(m_xsio.p, m_xsi.p, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s));
      SIMP_CUDA(cudaMemcpyAsync(m_etao.p, m_eta.p, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s));
      const double yo = y, zo = z, lamo = lam, muo = mu, zeto = zet, so = sl;
      int itto = 0;
      double trial_norm = 2.0 * cur_norm, trial_max = cur_max;
      while (trial_norm > cur_norm && itto < 50) {
        ++itto;
        y = yo + steg * dy;
        z = zo + steg * dz;
        lam = lamo + steg * dlam;
        mu = muo + steg * dmu;
        zet = zeto + steg * dzet;
        sl = so + steg * dss;
        trial_max = residual(m_xo.p, steg, y, z, lam, mu, zet, sl, trial_norm);
        steg *= 0.5;
      }
      cur_norm = trial_norm;
      cur_max = trial_max;
    }
    if (ittt >= 500) {
      std::ostringstream os;
      os << "the MMA subproblem solver did not converge (final residual " << cur_max << " at barrier " << epsi
         << ")";
      throw Error(kMaxIter, os.str());
    }
    epsi *= 0.1;
  }
  OcStep st;
  st.lambda = lam * row_scale;
  st.bisections = total;
  st.converged = true;
  st.volume = 0.0;
  // max |x' - x| and the grey level of the evaluated density
  k_change_gray<<<kRedBlocks, kRedThreads, 0, s>>>(ne, m_x.p, x.p, rho.p, opart.p, opart.p + kRedBlocks);
  SIMP_CHECK_LAUNCH();
  std::vector<double> hp(2 * kRedBlocks);
  SIMP_CUDA(cudaMemcpyAsync(hp.data(), opart.p, sizeof(double) * 2 * kRedBlocks, cudaMemcpyDeviceToHost, s));
  SIMP_CUDA(cudaStreamSynchronize(s));
  double mc = 0.0, gs = 0.0;
  for (int k = 0; k < kRedBlocks; ++k) {
    mc = std::max(mc, hp[k]);
    gs += hp[kRedBlocks + k];
  }
  st.max_change = mc;
  gray = 4.0 * gs / static_cast<double>(ne);
  if (xnew_host) {
    m_x.download(xnew_host, nn, s);
    SIMP_CUDA(cudaStreamSynchronize(s));
  }
  // history of the asymptote rule: x_old2 <- x_old1 <- x
  std::swap(m_x2, m_x1);
  SIMP_CUDA(cudaMemcpyAsync(m_x1.p, x.p, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s));
  if (apply) {
    SIMP_CUDA(cudaMemcpyAsync(x.p, m_x.p, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s));
    k_clamp01<<<grid_for(ne, 256), 256, 0, s>>>(ne, x.p);
    SIMP_CHECK_LAUNCH();
  }
  return st;
}

}  // namespace simp
