// Undamped free vibration of the structured model on the GPU: SparLab's
// solve_modal (src/fem/ModalAnalysis.cpp:120-418), Bathe's subspace
// iteration with shift-invert, on an AMG-PCG hierarchy of its own.
//
// Device work per subspace iteration: Y = M X (q products with the mass on
// K_ff's pattern, or a diagonal for lumped mass); q AMG-PCG solves
// A Xbar = Y (A = K - sigma M, each column warm-started from
// x_c / (mu_c - sigma)), run concurrently on separate workspaces and
// streams; K Xbar and M Xbar; the projected q x q pencil as two tall-skinny
// Gram products with a fixed-order reduction; the rotation X = Xbar R; the
// eigenpair residuals of the requested modes.  Host work: the dense q x q
// generalised eigenproblem (Cholesky of the projected mass, cyclic Jacobi
// on the reduced symmetric matrix) and the convergence test.
#include "subspace.cuh"

#include <algorithm>
#include <cmath>
#include <exception>
#include <limits>
#include <numeric>
#include <sstream>
#include <thread>

namespace simp {

namespace {

// val[diag of row i] += add[i] * c
__global__ void k_add_diag(i32 n, const i32* __restrict__ node_of, const i32* __restrict__ first,
                           const i32* __restrict__ self_slot, NodeView a, const i32* __restrict__ rowptr,
                           double* __restrict__ val, const double* __restrict__ add, double c) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const i32 I = node_of[i];
    val[rowptr[i] + a.off[self_slot[I]] + (static_cast<i32>(i) - first[I])] += c * add[i];
  }
}

// Row-sum lumped mass of free DOF i: sum over its cells in ascending order
// of s_e * (row sum of M_e^0), cells with s_e = 0 left out
// (src/fem/Assembler.cpp:290-343).
__global__ void k_lumped_diag(i32 n, GridView g, const i32* __restrict__ node_of, const i32* __restrict__ gnode,
                              const uint8_t* __restrict__ ucomp, const double* __restrict__ rows,
                              const double* __restrict__ scale, double* __restrict__ out) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const i64 gn = gnode[node_of[i]];
    const int k = ucomp[i];
    const i32 ix = static_cast<i32>(gn % g.nnx), iy = static_cast<i32>((gn / g.nnx) % g.nny),
              iz = static_cast<i32>(gn / (static_cast<i64>(g.nnx) * g.nny));
    double acc = 0.0;
    for (i32 cz = max(iz - 1, 0); cz <= min(iz, g.nz - 1); ++cz)
      for (i32 cy = max(iy - 1, 0); cy <= min(iy, g.ny - 1); ++cy)
        for (i32 cx = max(ix - 1, 0); cx <= min(ix, g.nx - 1); ++cx) {
          const i64 c = (static_cast<i64>(cz) * g.ny + cy) * g.nx + cx;
          const double s = scale[c];
          if (s == 0.0) continue;
          const int a = corner_of(ix - cx, iy - cy, g.dim == 3 ? iz - cz : 0);
          acc = xadd(acc, xmul(s, rows[g.dim * a + k]));
        }
    out[i] = acc;
  }
}

__global__ void k_diag_mul(i64 n, const double* __restrict__ d, const double* __restrict__ x,
                           double* __restrict__ y) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    y[i] = d[i] * x[i];
}

// y = x + a z
__global__ void k_add_scaled(i64 n, const double* __restrict__ x, const double* __restrict__ z, double a,
                             double* __restrict__ y) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    y[i] = x[i] + a * z[i];
}

// Kinetic energy s_e pe^T M_e pe per cell, summed per block: total and the
// part in cells with s_e < 0.3 (ModalAnalysis.cpp:388-410)
__global__ void __launch_bounds__(kRedThreads) k_mode_energy(GridView g, i64 ne, const double* __restrict__ full,
                                                             const double* __restrict__ me,
                                                             const double* __restrict__ scale,
                                                             double* __restrict__ part) {
  const int npe = g.dim == 3 ? 8 : 4, ed = npe * g.dim;
  double tot = 0.0, low = 0.0;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < ne; e += (i64)gridDim.x * blockDim.x) {
    const i64 ex = e % g.nx, ey = (e / g.nx) % g.ny, ez = e / (static_cast<i64>(g.nx) * g.ny);
    const i64 n0 = (ez * g.nny + ey) * g.nnx + ex;
    const i64 lay = static_cast<i64>(g.nnx) * g.nny;
    const i64 base[4] = {n0, n0 + 1, n0 + g.nnx + 1, n0 + g.nnx};
    double pe[24];
    for (int a = 0; a < npe; ++a) {
      const i64 nd = base[a & 3] + (a >= 4 ? lay : 0);
      for (int k = 0; k < g.dim; ++k) pe[g.dim * a + k] = full[nd * g.dim + k];
    }
    double qf = 0.0;
    for (int r = 0; r < ed; ++r) {
      double row = 0.0;
      for (int c = 0; c < ed; ++c) row += me[r * ed + c] * pe[c];
      qf += pe[r] * row;
    }
    const double s = scale[e];
    const double ke = s * qf;
    tot += ke;
    if (s < 0.3) low += ke;
  }
  tot = block_sum<kRedThreads>(tot);
  low = block_sum<kRedThreads>(low);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = tot;
    part[2 * blockIdx.x + 1] = low;
  }
}

}  // namespace

// Consistent mass of one box cell (Quad4Element::consistent_mass,
// src/elements/Quad4.cpp:139-173; Hex8Element::consistent_mass,
// src/elements/Hex8.cpp:194-214): M_e = sum over the 3 x 3 (x 3) Gauss
// points of rho t det(J) w N^T N, symmetrised.
void element_mass(int dim, double hx, double hy, double hz, double density, double thick, double* me) {
  const double a3 = std::sqrt(3.0 / 5.0);
  const double gx[3] = {-a3, 0.0, a3};
  const double gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
  static const double corner[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                      {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  const int npe = dim == 3 ? 8 : 4, ed = npe * dim;
  std::vector<double> m(static_cast<size_t>(ed) * ed, 0.0);
  const int gz_count = dim == 3 ? 3 : 1;
  for (int gk = 0; gk < gz_count; ++gk)
    for (int gj = 0; gj < 3; ++gj)
      for (int gi = 0; gi < 3; ++gi) {
        const double xi = gx[gi], eta = gx[gj], zeta = dim == 3 ? gx[gk] : 0.0;
        const double w = dim == 3 ? gw[gi] * gw[gj] * gw[gk] : gw[gi] * gw[gj];
        double n[8], det;
        if (dim == 2) {
          n[0] = 0.25 * (1 - xi) * (1 - eta);
          n[1] = 0.25 * (1 + xi) * (1 - eta);
          n[2] = 0.25 * (1 + xi) * (1 + eta);
          n[3] = 0.25 * (1 - xi) * (1 + eta);
          const double dn[4][2] = {{-0.25 * (1 - eta), -0.25 * (1 - xi)},
                                   {0.25 * (1 - eta), -0.25 * (1 + xi)},
                                   {0.25 * (1 + eta), 0.25 * (1 + xi)},
                                   {-0.25 * (1 + eta), 0.25 * (1 - xi)}};
          const double xy[4][2] = {{0, 0}, {hx, 0}, {hx, hy}, {0, hy}};
          double J[2][2] = {};
          for (int a = 0; a < 4; ++a)
            for (int r = 0; r < 2; ++r)
              for (int c = 0; c < 2; ++c) J[r][c] += xy[a][r] * dn[a][c];
          det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        } else {
          double dn[8][3];
          for (int a = 0; a < 8; ++a) {
            const double fx = 1 + xi * corner[a][0], fy = 1 + eta * corner[a][1], fz = 1 + zeta * corner[a][2];
            n[a] = 0.125 * fx * fy * fz;
            dn[a][0] = 0.125 * corner[a][0] * fy * fz;
            dn[a][1] = 0.125 * corner[a][1] * fx * fz;
            dn[a][2] = 0.125 * corner[a][2] * fx * fy;
          }
          const double h[3] = {hx, hy, hz};
          double J[3][3] = {};
          for (int a = 0; a < 8; ++a)
            for (int r = 0; r < 3; ++r)
              for (int c = 0; c < 3; ++c) J[r][c] += (corner[a][r] > 0 ? h[r] : 0.0) * dn[a][c];
          det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) +
                J[0][1] * (J[1][2] * J[2][0] - J[1][0] * J[2][2]) +
                J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        }
        const double f = (dim == 2 ? density * thick * det : density * det) * w;
        for (int a = 0; a < npe; ++a)
          for (int b = 0; b < npe; ++b)
            for (int k = 0; k < dim; ++k)
              m[static_cast<size_t>(dim * a + k) * ed + dim * b + k] += f * (n[a] * n[b]);
      }
  for (int r = 0; r < ed; ++r)
    for (int c = 0; c < ed; ++c)
      me[r * ed + c] = 0.5 * (m[static_cast<size_t>(r) * ed + c] + m[static_cast<size_t>(c) * ed + r]);
}

ModalResult solve_modal(GpuProblem& p, const ModalOptions& o, const double* kscale_h, const double* mscale_h,
                        bool want_shapes) {
  if (o.num_modes < 1) throw Error(kBadInput, "modal analysis requires num_modes >= 1");
  if (!(o.density > 0.0))
    throw Error(kBadInput,
                "mass assembly requires a positive density; set the material density to run a modal analysis");
  if (o.mass_type != 0 && o.mass_type != 1) throw Error(kBadInput, "unknown mass type");
  if (o.max_iterations < 1) throw Error(kBadInput, "modal analysis needs max_iterations >= 1");
  const ProblemDesc& d = p.d;
  const int dim = d.dim, ed = dim == 3 ? 24 : 8;
  const i32 n = p.nfree;
  const i64 ne = p.ne;
  const GridView g = grid_of_desc(d);
  ModalResult res;

  std::vector<double> me = o.element_mass;
  if (me.empty()) {
    me.resize(static_cast<size_t>(ed) * ed);
    element_mass(dim, p.hx, p.hy, p.hz, o.density, dim == 2 ? d.thickness : 1.0, me.data());
  }
  if (static_cast<int>(me.size()) != ed * ed) throw Error(kBadInput, "element mass matrix has the wrong size");
  for (int r = 0; r < ed; ++r)
    for (int c = 0; c < ed; ++c)
      if (me[r * ed + c] != me[c * ed + r]) throw Error(kBadInput, "the element mass matrix is not symmetric");

  // the modal solver's own hierarchy over the problem's level-0 structure
  // (the optimisation's hierarchy and its aggregates stay as they are)
  GpuAmg amg(p.amg.opt);
  const cudaStream_t s = amg.stream;
  Level& src = *p.amg.levels.front();
  copy_level0(src, amg.level0(), s);
  Level& l0 = *amg.levels.front();
  const i64 nnz = l0.a.nnz;

  std::vector<double> ones(static_cast<size_t>(ne), 1.0);
  DBuf<double> ks, ms, me_d;
  ks.upload(kscale_h ? kscale_h : ones.data(), static_cast<size_t>(ne), s);
  ms.upload(mscale_h ? mscale_h : ones.data(), static_cast<size_t>(ne), s);
  me_d.upload(me, s);
  // K_ff (the shifted system's values are a separate array when sigma != 0)
  DBuf<double> kval(static_cast<size_t>(nnz)), mval, mdiag;
  p.assemble_into(p.ke_d.p, ks.p, true, kval.p, nullptr, nullptr, s);
  const bool lumped = o.mass_type == 1;
  if (!lumped) {
    mval.alloc(static_cast<size_t>(nnz));
    p.assemble_into(me_d.p, ms.p, true, mval.p, nullptr, nullptr, s);
  } else {
    std::vector<double> rows(static_cast<size_t>(ed));
    for (int r = 0; r < ed; ++r) {
      double t = 0.0;
      for (int c = 0; c < ed; ++c) t += me[r * ed + c];
      rows[r] = t;
    }
    DBuf<double> rows_d;
    rows_d.upload(rows, s);
    mdiag.alloc(static_cast<size_t>(n));
    k_lumped_diag<<<grid_for(n, 256), 256, 0, s>>>(n, g, l0.d_node_of.p, p.gnode.p, p.ucomp.p, rows_d.p, ms.p,
                                                   mdiag.p);
    SIMP_CHECK_LAUNCH();
    SIMP_CUDA(cudaStreamSynchronize(s));
  }
  // sum(M) / dim: every translation carries the mass once
  {
    double msum = 0.0;
    for (int r = 0; r < ed; ++r) {
      double t = 0.0;
      for (int c = 0; c < ed; ++c) t += me[r * ed + c];
      msum += t;
    }
    double total = 0.0;
    for (i64 e = 0; e < ne; ++e) total += (mscale_h ? mscale_h[e] : 1.0) * msum;
    res.total_mass = total / dim;
  }

  const int m_req = std::min<int>(o.num_modes, n);
  if (m_req < o.num_modes) {
    std::ostringstream os;
    os << "requested " << o.num_modes << " modes but the model has only " << n << " free DOFs; returning "
       << m_req;
    res.warnings.push_back(os.str());
  }
  const int q = std::min<int>(n, std::max(2 * m_req, m_req + 8));
  if (q > kMaxSubspace) throw Error(kBadInput, "modal analysis supports at most 32 modes (a 64-vector subspace)");
  res.subspace_size = q;

  SolveWork& w0 = amg.work(0);
  auto apply_k = [&](SolveWork& w, const double* x, double* y) { amg.apply_values0(w, kval.p, x, y); };
  auto apply_m = [&](SolveWork& w, const double* x, double* y) {
    if (lumped) {
      k_diag_mul<<<grid_for(n, 256, 4096), 256, 0, w.stream>>>(n, mdiag.p, x, y);
      SIMP_CHECK_LAUNCH();
    } else {
      amg.apply_values0(w, mval.p, x, y);
    }
  };
  auto diag_of = [&](const double* val, double* out) {
    k_diag_of<<<grid_for(n, 256), 256, 0, s>>>(n, l0.d_node_of.p, l0.d_first.p, l0.d_self.p, l0.d_apat.view(),
                                               l0.a.ptr.p, val, out);
    SIMP_CHECK_LAUNCH();
  };
  // level-0 operator shapes (lanes, column decode) come from a setup; the
  // dense path and the mass products need them as well
  SIMP_CUDA(cudaMemcpyAsync(l0.a.v64.p, kval.p, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, s));

  DBuf<double> X(static_cast<size_t>(n) * q), Xb(static_cast<size_t>(n) * q), Y(static_cast<size_t>(n) * q),
      Z(static_cast<size_t>(n) * q);
  std::vector<double> lam;
  DBuf<double> part(static_cast<size_t>(kGramBlocks) * q * q), gram(static_cast<size_t>(q) * q),
      rot(static_cast<size_t>(q) * q), tmp(static_cast<size_t>(n)), tmp2(static_cast<size_t>(n));

  bool dense = q >= n || n <= 400;
  if (dense) {
    // small system: a dense generalised eigensolve, normalised and checked
    // on the host
    std::vector<i32> ptr = l0.a.ptr.to_host(s), col = l0.a.col.to_host(s);
    std::vector<double> kv = kval.to_host(s), mv = lumped ? mdiag.to_host(s) : mval.to_host(s);
    Mat kd(static_cast<size_t>(n) * n, 0.0), md(static_cast<size_t>(n) * n, 0.0);
    for (i32 r = 0; r < n; ++r) {
      for (i32 k = ptr[r]; k < ptr[r + 1]; ++k) {
        kd[static_cast<size_t>(r) * n + col[k]] = kv[k];
        if (!lumped) md[static_cast<size_t>(r) * n + col[k]] = mv[k];
      }
      if (lumped) md[static_cast<size_t>(r) * n + r] = mv[r];
    }
    Mat vec;
    if (!lowest_pencil_pairs(kd, md, n, m_req, lam, vec))
      throw Error(kBreakdown,
                  "dense generalised eigensolve failed: the mass matrix is not positive definite and the stiffness "
                  "matrix is not either, or fewer DOFs than the modes requested carry mass (check material.density "
                  "and the mass interpolation floor)");
    res.converged = true;
    res.residuals.assign(static_cast<size_t>(m_req), 0.0);
    std::vector<double> colmajor(static_cast<size_t>(n) * q, 0.0), mx(static_cast<size_t>(n)),
        kx(static_cast<size_t>(n));
    for (int c = 0; c < m_req; ++c) {
      double* phi = colmajor.data() + static_cast<size_t>(c) * n;
      for (i32 i = 0; i < n; ++i) phi[i] = vec[static_cast<size_t>(i) * m_req + c];
      auto products = [&]() {
        for (i32 r = 0; r < n; ++r) {
          double a = 0.0, b = 0.0;
          for (i32 k = 0; k < n; ++k) {
            a += md[static_cast<size_t>(r) * n + k] * phi[k];
            b += kd[static_cast<size_t>(r) * n + k] * phi[k];
          }
          mx[r] = a;
          kx[r] = b;
        }
      };
      products();
      double mm = 0.0;
      for (i32 i = 0; i < n; ++i) mm += phi[i] * mx[i];
      const double mn = std::sqrt(std::max(mm, 0.0));
      if (!(mn > 0.0))
        throw Error(kBreakdown,
                    "a computed mode shape has zero modal mass; the mass matrix is singular on the free DOFs");
      for (i32 i = 0; i < n; ++i) phi[i] /= mn;
      products();
      double rr = 0.0, ref = 0.0;
      for (i32 i = 0; i < n; ++i) {
        const double r = kx[i] - lam[c] * mx[i];
        rr += r * r;
        ref += (lam[c] * mx[i]) * (lam[c] * mx[i]);
      }
      res.residuals[c] = std::sqrt(rr) / std::max(std::sqrt(ref), 1.0e-300);
    }
    X.upload(colmajor, s);
  } else {
    // shift: sigma = shift_factor * min k_ii / m_ii over massive DOFs
    std::vector<double> kd_h(static_cast<size_t>(n)), md_h(static_cast<size_t>(n));
    diag_of(kval.p, tmp.p);
    tmp.download(kd_h.data(), static_cast<size_t>(n), s);
    if (lumped) {
      mdiag.download(md_h.data(), static_cast<size_t>(n), s);
    } else {
      diag_of(mval.p, tmp2.p);
      tmp2.download(md_h.data(), static_cast<size_t>(n), s);
    }
    SIMP_CUDA(cudaStreamSynchronize(s));
    double sigma = 0.0;
    if (o.shift_factor != 0.0) {
      double min_ratio = std::numeric_limits<double>::max();
      for (i32 i = 0; i < n; ++i)
        if (md_h[i] > 0.0) min_ratio = std::min(min_ratio, kd_h[i] / md_h[i]);
      if (min_ratio < std::numeric_limits<double>::max()) sigma = o.shift_factor * min_ratio;
    }
    if (sigma > 0.0) {
      std::ostringstream os;
      os << "modal analysis: shift sigma = " << sigma
         << " > 0 can make K - sigma M indefinite, which CG cannot solve, and this library has no sparse "
            "factorisation; use shift_factor <= 0";
      throw Error(kBadInput, os.str());
    }
    if (sigma != 0.0) {  // A = K - sigma M
      if (lumped) {
        k_add_diag<<<grid_for(n, 256), 256, 0, s>>>(n, l0.d_node_of.p, l0.d_first.p, l0.d_self.p, l0.d_apat.view(),
                                                    l0.a.ptr.p, l0.a.v64.p, mdiag.p, -sigma);
      } else {
        k_add_scaled<<<grid_for(nnz, 256), 256, 0, s>>>(nnz, kval.p, mval.p, -sigma, l0.a.v64.p);
      }
      SIMP_CHECK_LAUNCH();
    }
    // mixed precision on a fully-free-or-clamped grid: the V-cycle's level-0
    // operator is the matrix-free K (FP32), as in the optimisation's solver;
    // only without a shift, where A = K
    DBuf<float> ks32;
    if (p.amg.mf.enabled && sigma == 0.0) {
      ks32.alloc(static_cast<size_t>(ne));
      k_convert<double, float><<<grid_for(ne, 256), 256, 0, s>>>(ks.p, ks32.p, ne);
      SIMP_CHECK_LAUNCH();
      amg.mf = p.amg.mf;
      amg.mf.scale = ks32.p;
    }
    amg.setup(true);
    const std::vector<SolveWork*> works = workspaces(amg, std::max(1, std::min(q, o.concurrent_solves)));

    // Bathe's start: the mass diagonal, then unit vectors at the DOFs of
    // largest m_ii / k_ii in stable order (ModalAnalysis.cpp:55-88)
    {
      std::vector<double> x0(static_cast<size_t>(n) * q, 0.0);
      std::copy(md_h.begin(), md_h.end(), x0.begin());
      std::vector<double> ratio(static_cast<size_t>(n));
      for (i32 i = 0; i < n; ++i) ratio[i] = kd_h[i] > 0.0 ? md_h[i] / kd_h[i] : 0.0;
      std::vector<i32> order(static_cast<size_t>(n));
      std::iota(order.begin(), order.end(), 0);
      std::partial_sort(order.begin(), order.begin() + (q - 1), order.end(), [&](i32 a, i32 b) {
        if (ratio[a] != ratio[b]) return ratio[a] > ratio[b];
        return a < b;
      });
      for (int c = 1; c < q; ++c) x0[static_cast<size_t>(c) * n + order[c - 1]] = 1.0;
      X.upload(x0, s);
    }
    std::vector<double> prev(static_cast<size_t>(m_req), std::numeric_limits<double>::max()), mu_prev;
    const size_t gram_smem = 2 * kGramRows * q * sizeof(double);
    auto gram_of = [&](const double* A, const double* B, Mat& out) {
      k_gram<<<kGramBlocks, 256, gram_smem, s>>>(n, q, A, B, part.p);
      SIMP_CHECK_LAUNCH();
      k_gram_finish<<<grid_for(q * q, 256), 256, 0, s>>>(q * q, kGramBlocks, part.p, gram.p);
      SIMP_CHECK_LAUNCH();
      out.resize(static_cast<size_t>(q) * q);
      gram.download(out.data(), out.size(), s);
      SIMP_CUDA(cudaStreamSynchronize(s));
    };
    for (int it = 1; it <= o.max_iterations; ++it) {
      for (int c = 0; c < q; ++c) apply_m(w0, X.p + static_cast<size_t>(c) * n, Y.p + static_cast<size_t>(c) * n);
      // initial guesses: the last Ritz pair gives x_c / (mu_c - sigma)
      const bool warm = o.warm_start && static_cast<int>(mu_prev.size()) == q;
      for (int c = 0; c < q; ++c) {
        double* xb = Xb.p + static_cast<size_t>(c) * n;
        if (warm && mu_prev[c] - sigma > 0.0) {
          k_scaled<<<grid_for(n, 256, 4096), 256, 0, s>>>(n, X.p + static_cast<size_t>(c) * n,
                                                          1.0 / (mu_prev[c] - sigma), xb);
          SIMP_CHECK_LAUNCH();
        } else {
          SIMP_CUDA(cudaMemsetAsync(xb, 0, sizeof(double) * n, s));
        }
      }
      SIMP_CUDA(cudaStreamSynchronize(s));
      for (const GpuAmg::PcgResult& r : solve_columns(amg, works, q, n, Y.p, Xb.p))
        count_solve(r, amg.opt.rtol, res.linear_iterations);
      // projected pencil: Xbar^T K Xbar and Xbar^T M Xbar
      for (int c = 0; c < q; ++c) apply_k(w0, Xb.p + static_cast<size_t>(c) * n, Y.p + static_cast<size_t>(c) * n);
      for (int c = 0; c < q; ++c) apply_m(w0, Xb.p + static_cast<size_t>(c) * n, Z.p + static_cast<size_t>(c) * n);
      Mat kr, mr;
      gram_of(Xb.p, Y.p, kr);
      gram_of(Xb.p, Z.p, mr);
      bool finite = true;
      for (size_t k = 0; k < kr.size(); ++k) finite = finite && std::isfinite(kr[k]) && std::isfinite(mr[k]);
      if (!finite)
        throw Error(kNonFinite,
                    "subspace iteration produced a non-finite basis; the shifted matrix K - sigma M is singular. "
                    "Reduce modal.shift_factor");
      for (int i = 0; i < q; ++i)
        for (int j = i + 1; j < q; ++j) {
          const double a = 0.5 * (kr[static_cast<size_t>(i) * q + j] + kr[static_cast<size_t>(j) * q + i]);
          const double b = 0.5 * (mr[static_cast<size_t>(i) * q + j] + mr[static_cast<size_t>(j) * q + i]);
          kr[static_cast<size_t>(i) * q + j] = kr[static_cast<size_t>(j) * q + i] = a;
          mr[static_cast<size_t>(i) * q + j] = mr[static_cast<size_t>(j) * q + i] = b;
        }
      std::vector<double> mu;
      Mat ritz;
      if (!lowest_pencil_pairs(kr, mr, q, q, mu, ritz)) {
        std::ostringstream os;
        os << "the projected " << q << " x " << q
           << " eigenproblem became numerically singular at subspace iteration " << it
           << "; the trial vectors lost independence. Reduce modal.num_modes or tighten modal.tolerance";
        throw Error(kBreakdown, os.str());
      }
      rot.upload(ritz, s);
      k_rotate<<<grid_for(n, 256), 256, sizeof(double) * q * q, s>>>(n, q, Xb.p, rot.p, X.p);
      SIMP_CHECK_LAUNCH();
      mu_prev = mu;
      double change = 0.0;
      for (int i = 0; i < m_req; ++i) {
        const double denom = std::max(std::fabs(mu[i]), 1.0e-300);
        change = std::max(change, std::fabs(mu[i] - prev[i]) / denom);
      }
      for (int i = 0; i < m_req; ++i) prev[i] = mu[i];
      res.iterations = it;
      res.final_change = change;
      // the eigenpair residual is part of the stopping rule
      double max_res = 0.0;
      for (int i = 0; i < m_req; ++i) {
        const double* xi = X.p + static_cast<size_t>(i) * n;
        apply_m(w0, xi, tmp.p);
        apply_k(w0, xi, tmp2.p);
        k_pair_residual<<<grid_for(n, 256, 4096), 256, 0, s>>>(n, tmp2.p, tmp.p, mu[i], tmp2.p);
        SIMP_CHECK_LAUNCH();
        const double rn = std::sqrt(amg.dot(w0, tmp2.p, tmp2.p, n));
        const double ref = std::max(std::fabs(mu[i]) * std::sqrt(amg.dot(w0, tmp.p, tmp.p, n)), 1.0e-300);
        max_res = std::max(max_res, rn / ref);
      }
      if (change < o.tolerance && max_res < o.residual_tolerance) {
        res.converged = true;
        break;
      }
    }
    if (!res.converged) {
      std::ostringstream os;
      os << "subspace iteration did not converge in " << o.max_iterations
         << " iterations; the relative eigenvalue change stalled at " << res.final_change
         << " against a tolerance of " << o.tolerance
         << " (the stopping rule also requires every eigenpair residual below " << o.residual_tolerance
         << "). Increase modal.max_iterations, loosen modal.tolerance or modal.residual_tolerance, or request "
            "fewer modes";
      throw Error(kMaxIter, os.str());
    }
    lam = prev;
  }

  // phi^T M phi = 1 exactly
  for (int i = 0; i < m_req && !dense; ++i) {
    double* xi = X.p + static_cast<size_t>(i) * n;
    apply_m(w0, xi, tmp.p);
    const double mn = std::sqrt(std::max(amg.dot(w0, xi, tmp.p, n), 0.0));
    if (!(mn > 0.0))
      throw Error(kBreakdown,
                  "a computed mode shape has zero modal mass; the mass matrix is singular on the free DOFs");
    k_scaled<<<grid_for(n, 256, 4096), 256, 0, s>>>(n, xi, 1.0 / mn, xi);
    SIMP_CHECK_LAUNCH();
  }
  // validity screening against the stiffness / mass scale
  auto absmax = [&](const double* v, i64 len) {
    k_absmax<<<kRedBlocks, kRedThreads, 0, s>>>(len, v, part.p);
    SIMP_CHECK_LAUNCH();
    std::vector<double> h(kRedBlocks);
    part.download(h.data(), kRedBlocks, s);
    SIMP_CUDA(cudaStreamSynchronize(s));
    return *std::max_element(h.begin(), h.end());
  };
  if (part.n < static_cast<size_t>(kRedBlocks) * 2) part.alloc(static_cast<size_t>(kRedBlocks) * 2);
  const double kscale_norm = nnz > 0 ? absmax(kval.p, nnz) : 0.0;
  const double mscale_norm = lumped ? (n > 0 ? absmax(mdiag.p, n) : 1.0) : (nnz > 0 ? absmax(mval.p, nnz) : 1.0);
  const double lambda_scale = mscale_norm > 0.0 ? kscale_norm / mscale_norm : 1.0;
  res.eigenvalues = lam;
  if (!dense) res.residuals.assign(static_cast<size_t>(m_req), 0.0);
  for (int i = 0; i < m_req; ++i) {
    const double l = lam[i];
    if (!std::isfinite(l)) {
      std::ostringstream os;
      os << "eigenvalue " << i << " is not finite; the eigenproblem is ill-posed";
      throw Error(kNonFinite, os.str());
    }
    if (l < -o.rigid_body_ratio * lambda_scale) {
      std::ostringstream os;
      os << "eigenvalue " << i << " is negative (" << l
         << " 1/s^2). K_ff is not positive definite, which is physically impossible for a properly constrained "
            "linear-elastic model: check the boundary conditions and the SIMP stiffness floor";
      throw Error(kBreakdown, os.str());
    }
    if (l < o.rigid_body_ratio * lambda_scale) {
      std::ostringstream os;
      os << "eigenvalue " << i << " is " << l << " 1/s^2, indistinguishable from zero at this stiffness/mass scale ("
         << lambda_scale << "): the model retains a rigid-body or mechanism mode. Add constraints.";
      res.warnings.push_back(os.str());
    }
    if (!dense) {
      const double* xi = X.p + static_cast<size_t>(i) * n;
      apply_m(w0, xi, tmp.p);
      apply_k(w0, xi, tmp2.p);
      k_pair_residual<<<grid_for(n, 256, 4096), 256, 0, s>>>(n, tmp2.p, tmp.p, l, tmp2.p);
      SIMP_CHECK_LAUNCH();
      const double rn = std::sqrt(amg.dot(w0, tmp2.p, tmp2.p, n));
      const double ref = std::max(std::fabs(l) * std::sqrt(amg.dot(w0, tmp.p, tmp.p, n)), 1.0e-300);
      res.residuals[i] = rn / ref;
    }
    if (res.residuals[i] > o.residual_tolerance) {
      std::ostringstream os;
      os << "mode " << i << " has an eigenpair residual of " << res.residuals[i] << ", above the tolerance "
         << o.residual_tolerance;
      res.warnings.push_back(os.str());
    }
  }
  // mode shapes on every DOF (zero on the supports) and the share of their
  // kinetic energy in low-density cells
  res.mass_fraction.assign(static_cast<size_t>(m_req), 0.0);
  const bool fractions = mscale_h != nullptr;
  if (want_shapes || fractions) {
    DBuf<double> full(static_cast<size_t>(p.ndof));
    if (want_shapes) res.shapes.assign(static_cast<size_t>(m_req) * p.ndof, 0.0);
    std::vector<double> h(static_cast<size_t>(kRedBlocks) * 2);
    for (int i = 0; i < m_req; ++i) {
      k_expand_free<<<grid_for(p.ndof, 256), 256, 0, s>>>(p.ndof, p.dof_map.p, X.p + static_cast<size_t>(i) * n,
                                                          full.p);
      SIMP_CHECK_LAUNCH();
      if (want_shapes) full.download(res.shapes.data() + static_cast<size_t>(i) * p.ndof, static_cast<size_t>(p.ndof), s);
      if (fractions) {
        k_mode_energy<<<kRedBlocks, kRedThreads, 0, s>>>(g, ne, full.p, me_d.p, ms.p, part.p);
        SIMP_CHECK_LAUNCH();
        part.download(h.data(), h.size(), s);
        SIMP_CUDA(cudaStreamSynchronize(s));
        double tot = 0.0, low = 0.0;
        for (int b = 0; b < kRedBlocks; ++b) {
          tot += h[2 * b];
          low += h[2 * b + 1];
        }
        res.mass_fraction[i] = tot > 0.0 ? low / tot : 0.0;
      }
    }
    SIMP_CUDA(cudaStreamSynchronize(s));
  }
  return res;
}

}  // namespace simp
