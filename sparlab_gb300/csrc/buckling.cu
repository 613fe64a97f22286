// Linear buckling of the structured model on the GPU: SparLab's
// analyse_buckling / solve_buckling (src/fem/Buckling.cpp:100-466).
//
// The static displacement u of one load case comes from an AMG-PCG
// hierarchy of the analysis's own; K_G(u) is assembled on the device into
// K_ff's pattern (k_assemble_geometric); mu = 1 / lambda of the definite
// pencil (G, K), G = -K_G, is found by subspace iteration X <- K^-1 G X:
// the q solves of an iteration run concurrently on separate workspaces and
// streams, the basis is made orthonormal through two passes of its Gram
// matrix (eigen-decomposition on the host, directions below 1e-10 of the
// largest singular value dropped), the projected pencil is two tall-skinny
// Gram products, and the dense q x q problem is solved on the host.
//
// When reversed-load modes crowd the subspace (or on request), the iteration
// switches to the buckling spectral transformation X <- (K - sigma G)^-1 K X
// with sigma placed below lambda_1 by the inertia of K - sigma G
// (src/fem/Buckling.cpp:184-245, 318-347).  The reference reads the inertia
// off a sparse LDL^T; here K - sigma G is formed densely on the device and
// inverted by the blocked symmetric sweep of the coarse solve with signed
// pivots, which are the D of its natural-order LDL^T (the same negative
// count by Sylvester's law), and the shifted solves are one dense product
// per iteration.  Systems above kShiftDenseLimit free DOFs (beyond a dense
// factorisation) end with SIMP_BAD_INPUT and a message saying so.
#include "dense.cuh"
#include "subspace.cuh"

#include <algorithm>
#include <cmath>
#include <exception>
#include <limits>
#include <memory>
#include <numeric>
#include <sstream>
#include <thread>

namespace simp {

namespace {

constexpr double kZeroFraction = 1.0e-10;  // |mu| below this share of the largest is zero
constexpr i32 kDenseLimit = 400;
constexpr i32 kShiftDenseLimit = 16000;  // dense K - sigma G: 2 x 2 GB at the limit
constexpr uint64_t kStartSeed = 20240917u;

// The project's SplitMix64 stream (the same numbers as problems.SplitMix64).
struct SplitMix64 {
  uint64_t state;
  explicit SplitMix64(uint64_t seed) : state(seed * 0xD1B54A32D192ED03ull) {}
  double uniform(double lo, double hi) {
    state += 0x9E3779B97F4A7C15ull;
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const double u = static_cast<double>(z >> 11) * (1.0 / 9007199254740992.0);
    return lo + (hi - lo) * u;
  }
};

// Symmetric geometric stiffness of a node pair, one value per pair (the
// element matrix is the scalar block times the identity on the components,
// src/elements/Element.cpp:77-100): sum over the shared cells c of
// s_c sum_k C[aI][aJ][k] u_c[k], with C the symmetrised block per unit cell
// displacement (the stress of the cell's 2 x 2 (x 2) points is linear in
// u_c).  Written into every free-component entry of the pair's block.
__global__ void k_assemble_geometric(GridView g, i32 nodes, const i32* __restrict__ first,
                                     const i32* __restrict__ gnode, const uint8_t* __restrict__ cmask, NodeView a,
                                     const i32* __restrict__ rowptr, const double* __restrict__ C,
                                     const double* __restrict__ u_full, const double* __restrict__ scale,
                                     double* __restrict__ val) {
  extern __shared__ double cs[];
  const int npe = g.dim == 3 ? 8 : 4, ed = npe * g.dim;
  for (int t = threadIdx.x; t < npe * npe * ed; t += blockDim.x) cs[t] = C[t];
  __syncthreads();
  const i64 lay = static_cast<i64>(g.nnx) * g.nny;
  for (i64 I = blockIdx.x * (i64)blockDim.x + threadIdx.x; I < nodes; I += (i64)gridDim.x * blockDim.x) {
    const i64 gi = gnode[I];
    const i32 ix = static_cast<i32>(gi % g.nnx), iy = static_cast<i32>((gi / g.nnx) % g.nny),
              iz = static_cast<i32>(gi / lay);
    const int maskI = cmask[I];
    const i32 r0 = first[I];
    for (i32 t = a.ptr[I]; t < a.ptr[I + 1]; ++t) {
      const i32 J = a.nbr[t];
      const i64 gj = gnode[J];
      const i32 jx = static_cast<i32>(gj % g.nnx), jy = static_cast<i32>((gj / g.nnx) % g.nny),
                jz = static_cast<i32>(gj / lay);
      const int maskJ = cmask[J];
      double v = 0.0;
      const i32 z0 = max(max(iz, jz) - 1, 0), z1 = min(min(iz, jz), g.nz - 1);
      const i32 y0 = max(max(iy, jy) - 1, 0), y1 = min(min(iy, jy), g.ny - 1);
      const i32 x0 = max(max(ix, jx) - 1, 0), x1 = min(min(ix, jx), g.nx - 1);
      for (i32 cz = z0; cz <= z1; ++cz)
        for (i32 cy = y0; cy <= y1; ++cy)
          for (i32 cx = x0; cx <= x1; ++cx) {
            const i64 c = (static_cast<i64>(cz) * g.ny + cy) * g.nx + cx;
            const double s = scale[c];
            if (s == 0.0) continue;
            const int aI = corner_of(ix - cx, iy - cy, g.dim == 3 ? iz - cz : 0);
            const int aJ = corner_of(jx - cx, jy - cy, g.dim == 3 ? jz - cz : 0);
            const double* crow = cs + (aI * npe + aJ) * ed;
            const i64 n0 = (static_cast<i64>(cz) * g.nny + cy) * g.nnx + cx;
            const i64 base[4] = {n0, n0 + 1, n0 + g.nnx + 1, n0 + g.nnx};
            double acc = 0.0;
            for (int b = 0; b < npe; ++b) {
              const i64 nd = base[b & 3] + (b >= 4 ? lay : 0);
              for (int k = 0; k < g.dim; ++k) acc += crow[g.dim * b + k] * u_full[nd * g.dim + k];
            }
            v += s * acc;
          }
      int qa = 0;
      for (int ka = 0; ka < g.dim; ++ka) {
        if (!(maskI & (1 << ka))) continue;
        const i32 rb = rowptr[r0 + qa] + a.off[t];
        int qb = 0;
        for (int kb = 0; kb < g.dim; ++kb) {
          if (!(maskJ & (1 << kb))) continue;
          val[rb + qb] = ka == kb ? v : 0.0;
          ++qb;
        }
        ++qa;
      }
    }
  }
}

// Strain energy s_e pe^T K_e pe per cell, summed per block: total and the
// part in cells flagged solid (Buckling.cpp:420-436)
__global__ void __launch_bounds__(kRedThreads) k_solid_energy(GridView g, i64 ne, const double* __restrict__ full,
                                                              const double* __restrict__ ke,
                                                              const double* __restrict__ scale,
                                                              const uint8_t* __restrict__ solid,
                                                              double* __restrict__ part) {
  const int npe = g.dim == 3 ? 8 : 4, ed = npe * g.dim;
  double tot = 0.0, sol = 0.0;
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
      for (int c = 0; c < ed; ++c) row += ke[r * ed + c] * pe[c];
      qf += pe[r] * row;
    }
    const double en = scale[e] * qf;
    tot += en;
    if (solid[e]) sol += en;
  }
  tot = block_sum<kRedThreads>(tot);
  sol = block_sum<kRedThreads>(sol);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = tot;
    part[2 * blockIdx.x + 1] = sol;
  }
}

// C[a][b][k]: the symmetrised scalar block of a unit cell displacement e_k,
// sum_g t w det(J) G_g^T S(D B_g e_k) G_g (box cell, 2-point Gauss)
std::vector<double> geometric_tensor(int dim, double hx, double hy, double hz, double young, double nu, double t) {
  const int npe = dim == 3 ? 8 : 4, ed = npe * dim, nv = dim == 3 ? 6 : 3;
  std::vector<double> D(static_cast<size_t>(nv) * nv, 0.0);
  if (dim == 2) {
    const double f = young / (1.0 - nu * nu);
    D[0] = f;
    D[1] = f * nu;
    D[3] = f * nu;
    D[4] = f;
    D[8] = f * (1.0 - nu) / 2.0;
  } else {
    const double lam = young * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), G = young / (2.0 * (1.0 + nu));
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) D[i * 6 + j] = lam;
      D[i * 6 + i] = lam + 2.0 * G;
      D[(3 + i) * 6 + 3 + i] = G;
    }
  }
  static const double corner[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                      {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  const double gq = 1.0 / std::sqrt(3.0);
  const double h[3] = {hx, hy, hz};
  const double wdet = dim == 3 ? 0.125 * hx * hy * hz : 0.25 * hx * hy;
  const double tt = dim == 2 ? t : 1.0;
  std::vector<double> C(static_cast<size_t>(npe) * npe * ed, 0.0);
  const int ngp = dim == 3 ? 8 : 4;
  for (int gp = 0; gp < ngp; ++gp) {
    const double nat[3] = {(gp & 1) ? gq : -gq, (gp & 2) ? gq : -gq, (gp & 4) ? gq : -gq};
    double grad[8][3] = {};
    for (int a = 0; a < npe; ++a)
      for (int c = 0; c < dim; ++c) {
        double v = (dim == 3 ? 0.125 : 0.25) * corner[a][c];
        for (int o = 0; o < dim; ++o)
          if (o != c) v *= 1.0 + nat[o] * corner[a][o];
        grad[a][c] = v * (2.0 / h[c]);
      }
    // B (nv x ed): voigt (xx, yy, xy) or (xx, yy, zz, xy, yz, zx)
    std::vector<double> B(static_cast<size_t>(nv) * ed, 0.0);
    for (int a = 0; a < npe; ++a) {
      if (dim == 2) {
        B[0 * ed + 2 * a] = grad[a][0];
        B[1 * ed + 2 * a + 1] = grad[a][1];
        B[2 * ed + 2 * a] = grad[a][1];
        B[2 * ed + 2 * a + 1] = grad[a][0];
      } else {
        B[0 * ed + 3 * a] = grad[a][0];
        B[1 * ed + 3 * a + 1] = grad[a][1];
        B[2 * ed + 3 * a + 2] = grad[a][2];
        B[3 * ed + 3 * a] = grad[a][1];
        B[3 * ed + 3 * a + 1] = grad[a][0];
        B[4 * ed + 3 * a + 1] = grad[a][2];
        B[4 * ed + 3 * a + 2] = grad[a][1];
        B[5 * ed + 3 * a] = grad[a][2];
        B[5 * ed + 3 * a + 2] = grad[a][0];
      }
    }
    for (int k = 0; k < ed; ++k) {
      double sv[6] = {};
      for (int r = 0; r < nv; ++r)
        for (int c = 0; c < nv; ++c) sv[r] += D[r * nv + c] * B[c * ed + k];
      double S[3][3];
      if (dim == 2) {
        S[0][0] = sv[0];
        S[0][1] = S[1][0] = sv[2];
        S[1][1] = sv[1];
      } else {
        S[0][0] = sv[0];
        S[1][1] = sv[1];
        S[2][2] = sv[2];
        S[0][1] = S[1][0] = sv[3];
        S[1][2] = S[2][1] = sv[4];
        S[0][2] = S[2][0] = sv[5];
      }
      for (int a = 0; a < npe; ++a)
        for (int b = 0; b < npe; ++b) {
          double v = 0.0;
          for (int i = 0; i < dim; ++i)
            for (int j = 0; j < dim; ++j) v += grad[a][i] * S[i][j] * grad[b][j];
          C[(static_cast<size_t>(a) * npe + b) * ed + k] += tt * wdet * v;
        }
    }
  }
  std::vector<double> Cs(C.size());
  for (int a = 0; a < npe; ++a)
    for (int b = 0; b < npe; ++b)
      for (int k = 0; k < ed; ++k)
        Cs[(static_cast<size_t>(a) * npe + b) * ed + k] =
            0.5 * (C[(static_cast<size_t>(a) * npe + b) * ed + k] + C[(static_cast<size_t>(b) * npe + a) * ed + k]);
  return Cs;
}

// (K - sigma G)^-1 for the spectral transformation: factor(s) forms K - s G
// from the CSR values on the device, sweeps it into its inverse and returns
// the number of negative pivots (the number of load factors in (0, s) when
// K is positive definite), or -1 when a pivot is zero or not finite;
// apply() multiplies the last inverse into q columns.
struct ShiftedInverse {
  i32 n = 0;
  DBuf<double> swept, inv, panel, piv;
  DBuf<int> status;
  cudaStream_t s = nullptr;

  ShiftedInverse(i32 n_, cudaStream_t stream) : n(n_), s(stream) {
    if (n > kShiftDenseLimit) {
      std::ostringstream os;
      os << "buckling: the spectral transformation factors K - sigma K_G densely, up to " << kShiftDenseLimit
         << " free DOFs; this system has " << n << " (a sparse LDL^T is not provided): request more modes, or "
         << "run this load case on the reference's CPU path";
      throw Error(kBadInput, os.str());
    }
    const size_t nn = static_cast<size_t>(n) * n;
    swept.alloc(nn);
    inv.alloc(nn);
    panel.alloc(2 * static_cast<size_t>(n) * kNB + kNB * kNB);
    piv.alloc(static_cast<size_t>(n));
    status.alloc(1);
  }

  int factor(const Level& l0, const double* kval, const double* gval, double sig) {
    const size_t nn = static_cast<size_t>(n) * n;
    double* pu = panel.p;
    double* pv = pu + static_cast<size_t>(n) * kNB;
    double* pp = pv + static_cast<size_t>(n) * kNB;
    SIMP_CUDA(cudaMemsetAsync(swept.p, 0, nn * sizeof(double), s));
    SIMP_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), s));
    k_dense_shifted<<<grid_for(n, 128), 128, 0, s>>>(n, l0.a.ptr.p, l0.a.col.p, kval, gval, sig, swept.p);
    SIMP_CHECK_LAUNCH();
    const int nt = (n + kNB - 1) / kNB;
    const dim3 tiles(nt, nt);
    for (int k0 = 0; k0 < n; k0 += kNB) {
      const int kb = std::min(kNB, n - k0);
      k_sweep_pivot<true><<<(n + kSweepRows - 1) / kSweepRows, 256, 0, s>>>(swept.p, n, k0, kb, pu, pv, pp,
                                                                            piv.p, status.p);
      SIMP_CHECK_LAUNCH();
      k_sweep_update<<<tiles, 256, 0, s>>>(swept.p, n, k0, kb, pu, pv, pp);
      SIMP_CHECK_LAUNCH();
    }
    k_sweep_finish<<<tiles, 256, 0, s>>>(swept.p, inv.p, n);
    SIMP_CHECK_LAUNCH();
    int bad = 0;
    SIMP_CUDA(cudaMemcpyAsync(&bad, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    const std::vector<double> d = piv.to_host(s);
    if (bad != 0) return -1;
    int negative = 0;
    for (double v : d) {
      if (!(v != 0.0) || !std::isfinite(v)) return -1;
      negative += v < 0.0 ? 1 : 0;
    }
    return negative;
  }

  void apply(const double* y, double* z, int q) {
    const dim3 grid((n + kNB - 1) / kNB, (q + kNB - 1) / kNB);
    k_dense_gemm_cols<<<grid, 256, 0, s>>>(inv.p, n, q, y, z);
    SIMP_CHECK_LAUNCH();
  }
};

// An orthonormalising transform T (q x r, row-major) of the columns whose
// Gram matrix is w: T = V_r Lambda_r^-1/2 over the eigenpairs above
// (1e-10)^2 of the largest eigenvalue.
int orthonormaliser(const Mat& w, int q, Mat& T) {
  std::vector<double> ev;
  Mat V;
  jacobi_eigen(w, q, ev, V);
  std::vector<int> order(q);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ev[a] > ev[b]; });
  const double top = ev[order[0]];
  int r = 0;
  while (r < q && top > 0.0 && ev[order[r]] > 1.0e-20 * top) ++r;
  T.assign(static_cast<size_t>(q) * std::max(r, 1), 0.0);
  for (int c = 0; c < r; ++c) {
    const double f = 1.0 / std::sqrt(ev[order[c]]);
    for (int i = 0; i < q; ++i) T[static_cast<size_t>(i) * r + c] = V[static_cast<size_t>(i) * q + order[c]] * f;
  }
  return r;
}

}  // namespace

BucklingResult solve_buckling(GpuProblem& p, const BucklingOptions& o, int load_case, const double* kscale_h,
                              const double* sscale_h, const uint8_t* solid_h, const double* start_h, int start_cols,
                              bool want_shapes) {
  if (o.num_modes < 1) throw Error(kBadInput, "buckling.num_modes must be at least 1");
  if (!(o.tolerance > 0.0)) throw Error(kBadInput, "buckling.tolerance must be positive");
  if (!(o.residual_tolerance > 0.0)) throw Error(kBadInput, "buckling.residual_tolerance must be positive");
  if (o.max_iterations < 1) throw Error(kBadInput, "buckling.max_iterations must be at least 1");
  if (load_case < 0 || load_case >= p.d.nloads)
    throw Error(kBadInput, "buckling analysis asked for a load case the model does not have");
  if (!(o.young > 0.0) || !(o.poisson > -1.0 && o.poisson < 0.5))
    throw Error(kBadInput, "buckling needs the material's Young's modulus and Poisson ratio");
  if (o.transform != 0 && o.transform != 1)
    throw Error(kBadInput, "buckling.transform must be 0 (auto) or 1 (shift-invert)");
  const ProblemDesc& d = p.d;
  const int dim = d.dim;
  const i32 n = p.nfree;
  const i64 ne = p.ne;
  const GridView g = grid_of_desc(d);
  BucklingResult res;

  GpuAmg amg(p.amg.opt);
  const cudaStream_t s = amg.stream;
  Level& src = *p.amg.levels.front();
  copy_level0(src, amg.level0(), s);
  Level& l0 = *amg.levels.front();
  const i64 nnz = l0.a.nnz;
  std::vector<double> ones(static_cast<size_t>(ne), 1.0);
  DBuf<double> ks, ss;
  ks.upload(kscale_h ? kscale_h : ones.data(), static_cast<size_t>(ne), s);
  ss.upload(sscale_h ? sscale_h : ones.data(), static_cast<size_t>(ne), s);
  // K_ff (level 0 of the analysis's own hierarchy) and its AMG setup
  p.assemble_into(p.ke_d.p, ks.p, true, l0.a.v64.p, nullptr, nullptr, s);
  const double* kval = l0.a.v64.p;
  DBuf<float> ks32;
  if (p.amg.mf.enabled) {
    ks32.alloc(static_cast<size_t>(ne));
    k_convert<double, float><<<grid_for(ne, 256), 256, 0, s>>>(ks.p, ks32.p, ne);
    SIMP_CHECK_LAUNCH();
    amg.mf = p.amg.mf;
    amg.mf.scale = ks32.p;
  }
  amg.setup(true);
  SolveWork& w0 = amg.work(0);

  // the static solution of the load case
  DBuf<double> u(static_cast<size_t>(n)), ufull(static_cast<size_t>(p.ndof));
  SIMP_CUDA(cudaMemsetAsync(u.p, 0, sizeof(double) * n, s));
  count_solve(amg.solve(w0, p.b.p + static_cast<size_t>(load_case) * n, u.p), amg.opt.rtol, res.linear_iterations);
  k_expand_free<<<grid_for(p.ndof, 256), 256, 0, s>>>(p.ndof, p.dof_map.p, u.p, ufull.p);
  SIMP_CHECK_LAUNCH();
  // G = -K_G(u) on K_ff's pattern
  DBuf<double> gval(static_cast<size_t>(nnz)), cten;
  {
    const double hz = dim == 3 ? p.hz : 0.0;
    std::vector<double> C = geometric_tensor(dim, p.hx, p.hy, hz, o.young, o.poisson, d.thickness);
    for (double& c : C) c = -c;
    cten.upload(C, s);
    const size_t smem = sizeof(double) * C.size();
    raise_dynamic_smem(reinterpret_cast<const void*>(k_assemble_geometric), smem);
    k_assemble_geometric<<<grid_for(l0.nnodes, 128), 128, smem, s>>>(g, l0.nnodes, l0.d_first.p, p.gnode.p,
                                                                    p.cmask.p, l0.d_apat.view(), l0.a.ptr.p,
                                                                    cten.p, ufull.p, ss.p, gval.p);
    SIMP_CHECK_LAUNCH();
  }
  DBuf<double> part(static_cast<size_t>(kRedBlocks) * 2);
  auto absmax = [&](const double* v, i64 len) {
    k_absmax<<<kRedBlocks, kRedThreads, 0, s>>>(len, v, part.p);
    SIMP_CHECK_LAUNCH();
    std::vector<double> h(kRedBlocks);
    part.download(h.data(), kRedBlocks, s);
    SIMP_CUDA(cudaStreamSynchronize(s));
    return *std::max_element(h.begin(), h.end());
  };
  const double g_norm = nnz > 0 ? absmax(gval.p, nnz) : 0.0;

  const int m_req = std::min<int>(o.num_modes, n);
  const int q = std::min<int>(n, std::max(2 * m_req, m_req + 8));
  if (q > kMaxSubspace) throw Error(kBadInput, "buckling analysis supports at most 32 modes (a 64-vector subspace)");
  res.subspace_size = q;
  auto apply_k = [&](SolveWork& w, const double* x, double* y) { amg.apply_values0(w, kval, x, y); };
  auto apply_g = [&](SolveWork& w, const double* x, double* y) { amg.apply_values0(w, gval.p, x, y); };

  std::vector<double> mu_top;       // descending
  DBuf<double> X(static_cast<size_t>(n) * q), Z(static_cast<size_t>(n) * q), B(static_cast<size_t>(n) * q),
      Y(static_cast<size_t>(n) * q), gram(static_cast<size_t>(q) * q), rot(static_cast<size_t>(q) * q),
      gpart(static_cast<size_t>(kGramBlocks) * q * q), tmp(static_cast<size_t>(n)), tmp2(static_cast<size_t>(n));
  int top_cols = 0;  // columns of X holding the top Ritz vectors (descending mu)
  const bool dense = n <= kDenseLimit || q >= n;
  if (!(g_norm > 0.0)) {
    // no stress at all: nothing can buckle
    res.converged = true;
    res.no_positive = true;
  } else if (dense) {
    std::vector<i32> ptr = l0.a.ptr.to_host(s), col = l0.a.col.to_host(s);
    std::vector<double> kv = l0.a.v64.to_host(s), gv = gval.to_host(s);
    Mat kd(static_cast<size_t>(n) * n, 0.0), gd(static_cast<size_t>(n) * n, 0.0);
    for (i32 r = 0; r < n; ++r)
      for (i32 k = ptr[r]; k < ptr[r + 1]; ++k) {
        kd[static_cast<size_t>(r) * n + col[k]] = kv[k];
        gd[static_cast<size_t>(r) * n + col[k]] = gv[k];
      }
    Mat l(kd);
    if (!cholesky(l, n))
      throw Error(kBreakdown,
                  "the dense buckling eigensolve failed; K_ff is not positive definite. Check the boundary conditions");
    std::vector<double> w;
    Mat y;
    jacobi_eigen(reduce_pencil(l, gd, n), n, w, y);
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return w[a] > w[b]; });
    Mat ys(static_cast<size_t>(n) * m_req), vec;
    mu_top.resize(m_req);
    for (int c = 0; c < m_req; ++c) {
      mu_top[c] = w[order[c]];
      for (i32 i = 0; i < n; ++i) ys[static_cast<size_t>(i) * m_req + c] = y[static_cast<size_t>(i) * n + order[c]];
    }
    back_substitute(l, n, ys, m_req, vec);
    std::vector<double> colmajor(static_cast<size_t>(n) * q, 0.0);
    for (int c = 0; c < m_req; ++c)
      for (i32 i = 0; i < n; ++i) colmajor[static_cast<size_t>(c) * n + i] = vec[static_cast<size_t>(i) * m_req + c];
    X.upload(colmajor, s);
    top_cols = m_req;
    res.converged = true;
  } else {
    const std::vector<SolveWork*> works = workspaces(amg, std::max(1, std::min(q, o.concurrent_solves)));
    // start: the caller's subspace (all but two columns at most), the rest
    // seeded uniform [-1, 1) columns
    SplitMix64 rng(kStartSeed);
    auto random_columns = [&](int from) {
      if (from >= q) return;
      std::vector<double> h(static_cast<size_t>(n) * (q - from));
      for (double& v : h) v = rng.uniform(-1.0, 1.0);
      SIMP_CUDA(cudaMemcpyAsync(X.p + static_cast<size_t>(from) * n, h.data(), sizeof(double) * h.size(),
                                cudaMemcpyHostToDevice, s));
      SIMP_CUDA(cudaStreamSynchronize(s));
    };
    int col0 = 0;
    if (start_h && start_cols > 0) {
      col0 = std::min(start_cols, q - 2);
      SIMP_CUDA(cudaMemcpyAsync(X.p, start_h, sizeof(double) * n * col0, cudaMemcpyHostToDevice, s));
    }
    random_columns(col0);
    const size_t gram_smem = 2 * kGramRows * q * sizeof(double);
    auto gram_of = [&](int cols, const double* A, const double* Bm, Mat& out) {
      k_gram<<<kGramBlocks, 256, gram_smem, s>>>(n, cols, A, Bm, gpart.p);
      SIMP_CHECK_LAUNCH();
      k_gram_finish<<<grid_for(cols * cols, 256), 256, 0, s>>>(cols * cols, kGramBlocks, gpart.p, gram.p);
      SIMP_CHECK_LAUNCH();
      out.resize(static_cast<size_t>(cols) * cols);
      gram.download(out.data(), out.size(), s);
      SIMP_CUDA(cudaStreamSynchronize(s));
    };
    auto rotate = [&](int cols_in, const double* in, const Mat& R, int cols_out, double* out) {
      // out (n x cols_out) = in (n x cols_in) R (cols_in x cols_out): k_rotate
      // takes a square R, so pad R to cols_in x cols_in
      Mat sq(static_cast<size_t>(cols_in) * cols_in, 0.0);
      for (int i = 0; i < cols_in; ++i)
        for (int c = 0; c < cols_out; ++c) sq[static_cast<size_t>(i) * cols_in + c] = R[static_cast<size_t>(i) * cols_out + c];
      SIMP_CUDA(cudaMemcpyAsync(rot.p, sq.data(), sizeof(double) * sq.size(), cudaMemcpyHostToDevice, s));
      k_rotate<<<grid_for(n, 256), 256, sizeof(double) * cols_in * cols_in, s>>>(n, cols_in, in, rot.p, Y.p);
      SIMP_CHECK_LAUNCH();
      SIMP_CUDA(cudaMemcpyAsync(out, Y.p, sizeof(double) * n * cols_out, cudaMemcpyDeviceToDevice, s));
    };
    // the spectral transformation's shift (src/fem/Buckling.cpp:184-245):
    // inertia(s) factors K - s G; choose_sigma places sigma below the
    // smallest positive load factor, from a guess (lowered by halving until
    // no load factor lies below it) or, without one, growing from 1 by
    // factors of 8; false when no positive load factor lies below 1e15
    std::unique_ptr<ShiftedInverse> shifted;
    bool refined = false;
    auto inertia = [&](double sg) {
      if (!shifted) shifted.reset(new ShiftedInverse(n, s));
      ++res.factorizations;
      return shifted->factor(l0, kval, gval.p, sg);
    };
    auto choose_sigma = [&](double guess) -> bool {
      double sg = guess > 0.0 ? guess : 1.0;
      int negative = inertia(sg);
      if (negative != 0) {
        for (int halvings = 1; negative != 0; ++halvings) {
          if (halvings > 120)
            throw Error(kBreakdown,
                        "the buckling shift search found no shift below the smallest load factor; K_ff is not "
                        "positive definite");
          sg *= 0.5;
          negative = inertia(sg);
        }
      } else if (!(guess > 0.0)) {
        double clean = sg;
        for (;;) {
          if (sg > 1.0e15) return false;
          const double next = 8.0 * sg;
          if (inertia(next) != 0) break;
          sg = next;
          clean = sg;
        }
        sg = clean;
        if (inertia(sg) != 0) throw Error(kBreakdown, "inconsistent inertia in the buckling shift search");
      }
      res.sigma = sg;
      res.transformed = true;
      return true;
    };
    if (o.transform == 1 && !choose_sigma(o.shift_hint > 0.0 ? 0.8 * o.shift_hint : 0.0)) {
      res.no_positive = true;
      res.converged = true;
    }
    std::vector<double> previous(static_cast<size_t>(m_req), std::numeric_limits<double>::quiet_NaN());
    std::vector<double> mu_desc;
    int r = 0;
    for (int it = 1; it <= o.max_iterations && !res.no_positive; ++it) {
      if (res.transformed) {
        // Z = (K - sigma G)^-1 K X
        for (int c = 0; c < q; ++c)
          apply_k(w0, X.p + static_cast<size_t>(c) * n, Y.p + static_cast<size_t>(c) * n);
        shifted->apply(Y.p, Z.p, q);
      } else {
        // Z = K^-1 G X
        for (int c = 0; c < q; ++c)
          apply_g(w0, X.p + static_cast<size_t>(c) * n, Y.p + static_cast<size_t>(c) * n);
        SIMP_CUDA(cudaMemsetAsync(Z.p, 0, sizeof(double) * n * q, s));
        SIMP_CUDA(cudaStreamSynchronize(s));
        for (const GpuAmg::PcgResult& x : solve_columns(amg, works, q, n, Y.p, Z.p))
          count_solve(x, amg.opt.rtol, res.linear_iterations);
      }
      // orthonormal basis B of Z, two passes through the Gram matrix
      Mat wz, T;
      gram_of(q, Z.p, Z.p, wz);
      for (double v : wz)
        if (!std::isfinite(v))
          throw Error(kNonFinite,
                      "buckling subspace iteration produced a non-finite basis; the stiffness matrix is singular or "
                      "severely ill-conditioned");
      r = orthonormaliser(wz, q, T);
      if (r < m_req) {
        std::ostringstream os;
        os << "the buckling subspace collapsed to " << r << " independent vectors, fewer than the " << m_req
           << " requested modes: the stress state loads fewer independent deformation patterns than that. Request "
              "fewer modes";
        throw Error(kBreakdown, os.str());
      }
      rotate(q, Z.p, T, r, B.p);
      Mat wb, T2;
      gram_of(r, B.p, B.p, wb);
      const int r2 = orthonormaliser(wb, r, T2);
      if (r2 < r) {
        Mat t2(static_cast<size_t>(r) * r, 0.0);
        for (int i = 0; i < r; ++i)
          for (int c = 0; c < r2; ++c) t2[static_cast<size_t>(i) * r + c] = T2[static_cast<size_t>(i) * r2 + c];
        T2.swap(t2);
        r = r2;
      }
      rotate(r, B.p, T2, r, B.p);
      // projected pencil (B^T G B, B^T K B)
      for (int c = 0; c < r; ++c) {
        apply_g(w0, B.p + static_cast<size_t>(c) * n, Y.p + static_cast<size_t>(c) * n);
        apply_k(w0, B.p + static_cast<size_t>(c) * n, Z.p + static_cast<size_t>(c) * n);
      }
      Mat gr, kr;
      gram_of(r, B.p, Y.p, gr);
      gram_of(r, B.p, Z.p, kr);
      for (int i = 0; i < r; ++i)
        for (int j = i + 1; j < r; ++j) {
          const double a = 0.5 * (gr[static_cast<size_t>(i) * r + j] + gr[static_cast<size_t>(j) * r + i]);
          const double b = 0.5 * (kr[static_cast<size_t>(i) * r + j] + kr[static_cast<size_t>(j) * r + i]);
          gr[static_cast<size_t>(i) * r + j] = gr[static_cast<size_t>(j) * r + i] = a;
          kr[static_cast<size_t>(i) * r + j] = kr[static_cast<size_t>(j) * r + i] = b;
        }
      Mat l(kr);
      if (!cholesky(l, r)) {
        std::ostringstream os;
        os << "the projected " << r << " x " << r << " buckling eigenproblem failed at subspace iteration " << it
           << "; K_ff is not positive definite on the subspace. Check the boundary conditions";
        throw Error(kBreakdown, os.str());
      }
      std::vector<double> w;
      Mat y;
      jacobi_eigen(reduce_pencil(l, gr, r), r, w, y);
      std::vector<int> order(r);
      std::iota(order.begin(), order.end(), 0);
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return w[a] > w[b]; });
      Mat ys(static_cast<size_t>(r) * r), vec;
      mu_desc.assign(static_cast<size_t>(r), 0.0);
      for (int c = 0; c < r; ++c) {
        mu_desc[c] = w[order[c]];
        for (int i = 0; i < r; ++i) ys[static_cast<size_t>(i) * r + c] = y[static_cast<size_t>(i) * r + order[c]];
      }
      back_substitute(l, r, ys, r, vec);
      rotate(r, B.p, vec, r, X.p);  // ritz vectors, K-normalised, descending mu
      random_columns(r);
      double scale = 0.0;
      for (double m : mu_desc) scale = std::max(scale, std::fabs(m));
      const double zero = kZeroFraction * scale;
      const double mu_m = mu_desc[m_req - 1] > zero ? mu_desc[m_req - 1] : 0.0;
      double change = 0.0, residual = 0.0;
      for (int i = 0; i < m_req; ++i) {
        const double m = mu_desc[i];
        const double denom = m > zero ? m : scale;
        const double delta = std::isnan(previous[i]) ? std::numeric_limits<double>::infinity()
                                                     : std::fabs(m - previous[i]) / denom;
        change = std::max(change, delta);
        if (m > zero) {
          const double* xi = X.p + static_cast<size_t>(i) * n;
          apply_k(w0, xi, tmp.p);
          apply_g(w0, xi, tmp2.p);
          k_pair_residual<<<grid_for(n, 256, 4096), 256, 0, s>>>(n, tmp2.p, tmp.p, m, tmp2.p);
          SIMP_CHECK_LAUNCH();
          const double rn = std::sqrt(amg.dot(w0, tmp2.p, tmp2.p, n));
          const double kn = std::sqrt(amg.dot(w0, tmp.p, tmp.p, n));
          residual = std::max(residual, rn / std::max(m * kn, 1.0e-300));
        }
      }
      for (int i = 0; i < m_req; ++i) previous[i] = mu_desc[i];
      res.iterations = it;
      res.final_change = change;
      if (change < o.tolerance && residual < o.residual_tolerance) {
        res.converged = true;
        break;
      }
      if (!res.transformed && o.transform == 0) {
        // reversed-load modes larger than the m-th wanted one take the
        // slots the wanted ones converge in: once more of them than the
        // spare slots appear, switch to the transformation
        int competing = 0;
        for (int j = 0; j < r; ++j) competing += mu_desc[j] < -mu_m ? 1 : 0;
        if (competing + m_req > q - 2) {
          const double estimate = mu_desc[0] > zero ? 0.8 / mu_desc[0] : 0.0;
          if (!choose_sigma(o.shift_hint > 0.0 ? 0.8 * o.shift_hint : estimate)) {
            res.no_positive = true;
            res.converged = true;
            break;
          }
          previous.assign(static_cast<size_t>(m_req), std::numeric_limits<double>::quiet_NaN());
        }
      } else if (res.transformed && !refined && mu_desc[0] > zero && change < 1.0e-3 &&
                 res.sigma < 0.5 / mu_desc[0]) {
        // a shift from the coarse search can sit far below lambda_1, where
        // the transformation separates the modes poorly: raise it to 0.8 of
        // the settled estimate
        refined = true;
        if (!choose_sigma(0.8 / mu_desc[0]))
          throw Error(kBreakdown, "the refined buckling shift found no load factor");
      }
    }
    if (!res.converged) {
      std::ostringstream os;
      os << "buckling subspace iteration did not converge in " << o.max_iterations
         << " iterations: the relative change of the requested load factors stalled at " << res.final_change
         << " against a tolerance of " << o.tolerance << " (every eigenpair residual must also fall below "
         << o.residual_tolerance
         << "). Increase buckling.max_iterations, request fewer modes, or loosen buckling.tolerance";
      throw Error(kMaxIter, os.str());
    }
    if (!res.no_positive) {
      mu_top.assign(mu_desc.begin(), mu_desc.begin() + m_req);
      top_cols = r;
    }
  }
  // the converged subspace (free DOFs, column-major), a warm start for the
  // next analysis
  if (top_cols > 0) {
    res.subspace.resize(static_cast<size_t>(n) * top_cols);
    X.download(res.subspace.data(), res.subspace.size(), s);
    SIMP_CUDA(cudaStreamSynchronize(s));
    res.subspace_cols = top_cols;
  }
  // the positive eigenvalues: the smallest positive load factors
  std::vector<int> keep;
  if (!mu_top.empty()) {
    double mx = 0.0;
    for (double m : mu_top) mx = std::max(mx, std::fabs(m));
    for (int i = 0; i < static_cast<int>(mu_top.size()); ++i)
      if (mu_top[i] > kZeroFraction * mx) keep.push_back(i);
  }
  const int found = static_cast<int>(keep.size());
  DBuf<double> full(static_cast<size_t>(p.ndof));
  DBuf<uint8_t> solid_d;
  if (solid_h) solid_d.upload(solid_h, static_cast<size_t>(ne), s);
  std::vector<double> h(static_cast<size_t>(kRedBlocks) * 2);
  if (want_shapes) res.shapes.assign(static_cast<size_t>(found) * p.ndof, 0.0);
  for (int j = 0; j < found; ++j) {
    const int i = keep[j];
    double* phi = X.p + static_cast<size_t>(i) * n;
    apply_k(w0, phi, tmp.p);
    const double kn = std::sqrt(std::max(amg.dot(w0, phi, tmp.p, n), 0.0));
    if (!(kn > 0.0)) throw Error(kBreakdown, "a buckling mode has zero strain energy");
    k_scaled<<<grid_for(n, 256, 4096), 256, 0, s>>>(n, phi, 1.0 / kn, phi);
    SIMP_CHECK_LAUNCH();
    const double lambda = 1.0 / mu_top[i];
    res.load_factors.push_back(lambda);
    apply_k(w0, phi, tmp.p);
    apply_g(w0, phi, tmp2.p);
    k_pair_residual<<<grid_for(n, 256, 4096), 256, 0, s>>>(n, tmp.p, tmp2.p, lambda, tmp2.p);
    SIMP_CHECK_LAUNCH();
    const double rn = std::sqrt(amg.dot(w0, tmp2.p, tmp2.p, n));
    const double kphi = std::sqrt(amg.dot(w0, tmp.p, tmp.p, n));
    res.residuals.push_back(rn / std::max(kphi, 1.0e-300));
    if (res.residuals.back() > o.residual_tolerance) {
      std::ostringstream os;
      os << "buckling mode " << j + 1 << " has an eigenpair residual of " << res.residuals.back()
         << ", above the tolerance " << o.residual_tolerance;
      res.warnings.push_back(os.str());
    }
    k_expand_free<<<grid_for(p.ndof, 256), 256, 0, s>>>(p.ndof, p.dof_map.p, phi, full.p);
    SIMP_CHECK_LAUNCH();
    if (want_shapes) full.download(res.shapes.data() + static_cast<size_t>(j) * p.ndof, static_cast<size_t>(p.ndof), s);
    double frac = 1.0;
    if (solid_h) {
      k_solid_energy<<<kRedBlocks, kRedThreads, 0, s>>>(g, ne, full.p, p.ke_d.p, ks.p, solid_d.p, part.p);
      SIMP_CHECK_LAUNCH();
      part.download(h.data(), h.size(), s);
      SIMP_CUDA(cudaStreamSynchronize(s));
      double tot = 0.0, sol = 0.0;
      for (int b = 0; b < kRedBlocks; ++b) {
        tot += h[2 * b];
        sol += h[2 * b + 1];
      }
      frac = tot > 0.0 ? sol / tot : 0.0;
    }
    res.solid_fraction.push_back(frac);
  }
  SIMP_CUDA(cudaStreamSynchronize(s));
  if (found == 0) {
    res.no_positive = true;
  } else if (found < m_req) {
    std::ostringstream os;
    os << "only " << found << " of the " << m_req
       << " requested modes have a positive load factor; the others belong to the reversed load";
    res.warnings.push_back(os.str());
  }
  return res;
}

}  // namespace simp
