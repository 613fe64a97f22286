// GPU SIMP iteration on a structured grid (see problem.h).
#include "kernels.cuh"
#include "problem.h"
#include "surrogate_net.h"
#include "topopt.cuh"

#include <algorithm>
#include <array>
#include <cmath>
#include <exception>
#include <sstream>
#include <thread>

namespace simp {

namespace {

GridView grid_of(const ProblemDesc& d) {
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

}  // namespace

// Element stiffness of a box cell by 2-point Gauss quadrature, symmetrised
// (src/elements/Hex8.cpp:172-192, src/elements/Quad4.cpp:117-137; constitutive
// matrices of src/material/IsotropicMaterial.cpp:34-65).
void element_stiffness(int dim, double hx, double hy, double hz, double young, double nu, double thick,
                       double* ke) {
  const double g = 1.0 / std::sqrt(3.0);
  const double gp[2] = {-g, g};
  if (dim == 2) {
    const double f = young / (1.0 - nu * nu);
    const double D[3][3] = {{f, f * nu, 0}, {f * nu, f, 0}, {0, 0, f * (1.0 - nu) / 2.0}};
    double k[8][8] = {};
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) {
        const double xi = gp[i], eta = gp[j];
        // natural gradients of the four shape functions
        const double dn[4][2] = {{-0.25 * (1 - eta), -0.25 * (1 - xi)},
                                 {0.25 * (1 - eta), -0.25 * (1 + xi)},
                                 {0.25 * (1 + eta), 0.25 * (1 + xi)},
                                 {-0.25 * (1 + eta), 0.25 * (1 - xi)}};
        const double X[4][2] = {{0, 0}, {hx, 0}, {hx, hy}, {0, hy}};
        double J[2][2] = {};
        for (int a = 0; a < 4; ++a)
          for (int r = 0; r < 2; ++r)
            for (int c = 0; c < 2; ++c) J[r][c] += X[a][r] * dn[a][c];
        const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const double Ji[2][2] = {{J[1][1] / det, -J[0][1] / det}, {-J[1][0] / det, J[0][0] / det}};
        double B[3][8] = {};
        for (int a = 0; a < 4; ++a) {
          const double gx = dn[a][0] * Ji[0][0] + dn[a][1] * Ji[1][0];
          const double gy = dn[a][0] * Ji[0][1] + dn[a][1] * Ji[1][1];
          B[0][2 * a] = gx;
          B[1][2 * a + 1] = gy;
          B[2][2 * a] = gy;
          B[2][2 * a + 1] = gx;
        }
        for (int r = 0; r < 8; ++r)
          for (int c = 0; c < 8; ++c) {
            double s = 0.0;
            for (int p = 0; p < 3; ++p)
              for (int q = 0; q < 3; ++q) s += B[p][r] * D[p][q] * B[q][c];
            k[r][c] += thick * det * s;
          }
      }
    for (int r = 0; r < 8; ++r)
      for (int c = 0; c < 8; ++c) ke[r * 8 + c] = 0.5 * (k[r][c] + k[c][r]);
    return;
  }
  static const double corner[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                      {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
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
        const double nat[3] = {gp[gi], gp[gj], gp[gk]};
        // box cell: J = diag(h/2), so dN/dx = dN/dxi * 2/h
        const double h[3] = {hx, hy, hz};
        double B[6][24] = {};
        for (int a = 0; a < 8; ++a) {
          double gr[3];
          for (int c = 0; c < 3; ++c) {
            double v = 0.125 * corner[a][c];
            for (int o = 0; o < 3; ++o)
              if (o != c) v *= 1.0 + nat[o] * corner[a][o];
            gr[c] = v * (2.0 / h[c]);
          }
          const int c3 = 3 * a;
          B[0][c3] = gr[0];
          B[1][c3 + 1] = gr[1];
          B[2][c3 + 2] = gr[2];
          B[3][c3] = gr[1];
          B[3][c3 + 1] = gr[0];
          B[4][c3 + 1] = gr[2];
          B[4][c3 + 2] = gr[1];
          B[5][c3] = gr[2];
          B[5][c3 + 2] = gr[0];
        }
        const double det = 0.125 * hx * hy * hz;
        for (int r = 0; r < 24; ++r)
          for (int c = 0; c < 24; ++c) {
            double s = 0.0;
            for (int p = 0; p < 6; ++p) {
              double db = 0.0;
              for (int q = 0; q < 6; ++q) db += D[p][q] * B[q][c];
              s += B[p][r] * db;
            }
            k[static_cast<size_t>(r) * 24 + c] += det * s;
          }
      }
  for (int r = 0; r < 24; ++r)
    for (int c = 0; c < 24; ++c)
      ke[r * 24 + c] = 0.5 * (k[static_cast<size_t>(r) * 24 + c] + k[static_cast<size_t>(c) * 24 + r]);
}

GpuProblem::GpuProblem(const ProblemDesc& desc, const AmgOptions& o) : d(desc), amg(o) {
  if (d.dim != 2 && d.dim != 3) throw Error(kBadInput, "the grid must be two- or three-dimensional");
  if (d.nx < 1 || d.ny < 1 || (d.dim == 3 && d.nz < 1)) throw Error(kBadInput, "the grid needs at least one cell per axis");
  if (d.dim == 2) d.nz = 1;
  build();
}

GpuProblem::~GpuProblem() {
  if (stencil_d) cudaFree(stencil_d);
  if (pred_t0) cudaEventDestroy(pred_t0);
  if (pred_ready) cudaEventDestroy(pred_ready);
}

void GpuProblem::build() {
  const GridView g = grid_of(d);
  const int dim = d.dim;
  ne = static_cast<i64>(d.nx) * d.ny * d.nz;
  nn = static_cast<i64>(g.nnx) * g.nny * g.nnz;
  ndof = nn * dim;
  hx = d.lx / d.nx;
  hy = d.ly / d.ny;
  hz = dim == 3 ? d.lz / d.nz : 0.0;
  if (static_cast<i64>(d.fixed.size()) != ndof) throw Error(kBadInput, "fixed mask has the wrong length");
  if (static_cast<i64>(d.loads.size()) != ndof * d.nloads) throw Error(kBadInput, "load vectors have the wrong length");
  if (d.nloads < 1) throw Error(kBadInput, "at least one load case is needed");
  const int ed = dim == 3 ? 24 : 8;
  if (static_cast<int>(d.ke.size()) != ed * ed) throw Error(kBadInput, "element matrix has the wrong size");
  for (int r = 0; r < ed; ++r)
    for (int c = 0; c < ed; ++c)
      if (d.ke[r * ed + c] != d.ke[c * ed + r])
        throw Error(kBadInput, "the element matrix is not symmetric");
  // element measure x volume factor (src/fem/FemModel.cpp:236-240, 422-429)
  elem_volume = dim == 3 ? hx * hy * hz : hx * hy * d.thickness;
  // free DOFs, ascending (src/fem/DofManager.cpp:58-71)
  std::vector<i32> map(static_cast<size_t>(ndof), -1);
  free_dofs_.clear();
  for (i64 k = 0; k < ndof; ++k)
    if (!d.fixed[k]) {
      map[k] = static_cast<i32>(free_dofs_.size());
      free_dofs_.push_back(static_cast<i32>(k));
    }
  nfree = static_cast<i32>(free_dofs_.size());
  if (nfree == 0) throw Error(kBadInput, "every degree of freedom is constrained");
  // free nodes and their components
  std::vector<i32> node_index(static_cast<size_t>(nn), -1), gnode_h, first(1, 0), ucomp_h;
  std::vector<uint8_t> cmask_h;
  for (i64 nd = 0; nd < nn; ++nd) {
    uint8_t m = 0;
    for (int k = 0; k < dim; ++k)
      if (!d.fixed[nd * dim + k]) m |= static_cast<uint8_t>(1 << k);
    if (!m) continue;
    node_index[nd] = static_cast<i32>(gnode_h.size());
    gnode_h.push_back(static_cast<i32>(nd));
    cmask_h.push_back(m);
    for (int k = 0; k < dim; ++k)
      if (m & (1 << k)) ucomp_h.push_back(k);
    first.push_back(static_cast<i32>(ucomp_h.size()));
  }
  const i32 nfn = static_cast<i32>(gnode_h.size());
  // level-0 node pattern: free grid neighbours sharing a cell, ascending
  NodePattern pat;
  pat.rows = pat.cols = nfn;
  pat.ptr.assign(static_cast<size_t>(nfn) + 1, 0);
  pat.nbr.reserve(static_cast<size_t>(nfn) * (dim == 3 ? 27 : 9));
  std::vector<uint32_t> nmask_h(static_cast<size_t>(nfn), 0u);
  for (i32 I = 0; I < nfn; ++I) {
    const i64 gi = gnode_h[I];
    const i32 ix = static_cast<i32>(gi % g.nnx), iy = static_cast<i32>((gi / g.nnx) % g.nny),
              iz = static_cast<i32>(gi / (static_cast<i64>(g.nnx) * g.nny));
    for (int dz = (dim == 3 ? -1 : 0); dz <= (dim == 3 ? 1 : 0); ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const i32 jx = ix + dx, jy = iy + dy, jz = iz + dz;
          if (jx < 0 || jx >= g.nnx || jy < 0 || jy >= g.nny || jz < 0 || jz >= g.nnz) continue;
          const i64 gj = (static_cast<i64>(jz) * g.nny + jy) * g.nnx + jx;
          if (node_index[gj] >= 0) {
            pat.nbr.push_back(node_index[gj]);
            const int o = (dim == 3 ? (dz + 1) * 9 : 0) + (dy + 1) * 3 + (dx + 1);
            nmask_h[I] |= 1u << o;
          }
        }
    pat.ptr[I + 1] = static_cast<i32>(pat.nbr.size());
  }
  nmask.upload(nmask_h);
  finish_offsets(pat, first);
  // AMG level 0
  Level& l0 = amg.level0();
  l0.n = nfree;
  l0.nnodes = nfn;
  l0.first = first;
  l0.apat = pat;
  l0.d_first.upload(first);
  l0.d_node_of.upload(node_of_unknowns(first));
  l0.d_apat.upload(pat);
  l0.d_self.upload(pattern_self_slots(pat));
  {
    const std::vector<i32> ptr = scalar_rowptr(pat, first);
    l0.a.rows = l0.a.cols = nfree;
    l0.a.nnz = ptr.back();
    l0.a.ptr.upload(ptr);
    l0.a.col.alloc(static_cast<size_t>(l0.a.nnz));
    k_expand_columns<<<grid_for(nfree, 256), 256>>>(nfree, l0.d_node_of.p, l0.d_apat.view(), l0.d_first.p,
                                                    l0.a.ptr.p, l0.a.col.p);
    SIMP_CHECK_LAUNCH();
    l0.a.v64.alloc(static_cast<size_t>(l0.a.nnz));
  }
  {
    // coordinates of the nodes (x0 + i * dx as the mesh generator forms them)
    std::vector<double> coords(static_cast<size_t>(nn) * dim);
    for (i64 nd = 0; nd < nn; ++nd) {
      const i64 i = nd % g.nnx, j = (nd / g.nnx) % g.nny, k = nd / (static_cast<i64>(g.nnx) * g.nny);
      coords[nd * dim] = 0.0 + static_cast<double>(i) * hx;
      coords[nd * dim + 1] = 0.0 + static_cast<double>(j) * hy;
      if (dim == 3) coords[nd * dim + 2] = 0.0 + static_cast<double>(k) * hz;
    }
    l0.null = rigid_body_modes(dim, dim, coords, static_cast<i32>(nn), free_dofs_);
  }
  gnode.upload(gnode_h);
  cmask.upload(cmask_h);
  // matrix-free level-0 operator where every node is fully free or clamped
  {
    const uint8_t full = static_cast<uint8_t>((1 << dim) - 1);
    bool all_or_nothing = true;
    for (uint8_t m : cmask_h) all_or_nothing = all_or_nothing && m == full;
    if (amg.mixed() && all_or_nothing && amg.opt.matrix_free >= 1) {
      std::vector<float> k32(d.ke.begin(), d.ke.end());
      ke32.upload(k32);
      sf32.alloc(static_cast<size_t>(ne));
      nindex.upload(node_index);
      MfOp& mf = amg.mf;
      mf.enabled = true;
      mf.dim = dim;
      mf.nx = d.nx;
      mf.ny = d.ny;
      mf.nz = d.nz;
      mf.nnx = g.nnx;
      mf.nny = g.nny;
      mf.gnode = gnode.p;
      mf.nindex = nindex.p;
      mf.ke = ke32.p;
      std::copy(k32.begin(), k32.end(), mf.ke_host);
      std::copy(d.ke.begin(), d.ke.end(), mf.ke64_host);
      mf.scale = sf32.p;
    }
  }
  std::vector<uint8_t> uc(ucomp_h.begin(), ucomp_h.end());
  ucomp.upload(uc);
  dof_map.upload(map);
  ke_d.upload(d.ke);
  // device design state
  const size_t ne_s = static_cast<size_t>(ne);
  x.alloc(ne_s);
  xnew.alloc(ne_s);
  rho.alloc(ne_s);
  sf.alloc(ne_s);
  amg.mf.scale64 = sf.p;  // the FP64 SIMP factors (matrix-free CG operator)
  df.alloc(ne_s);
  dc_dphys.alloc(ne_s);
  dc_dx.alloc(ne_s);
  dv_dx.alloc(ne_s);
  se.alloc(ne_s);
  tmp.alloc(ne_s);
  opart.alloc(static_cast<size_t>(std::max(2, kOcSpec)) * kRedBlocks);
  ovol.alloc(kOcSpec);
  // loads restricted to the free DOFs
  std::vector<double> bh(static_cast<size_t>(nfree) * d.nloads);
  for (int l = 0; l < d.nloads; ++l)
    for (i32 i = 0; i < nfree; ++i) bh[static_cast<size_t>(l) * nfree + i] = d.loads[l * ndof + free_dofs_[i]];
  b.upload(bh);
  u.alloc(static_cast<size_t>(nfree) * d.nloads);
  if (d.warm >= 2) {
    hist.alloc(static_cast<size_t>(nfree) * d.nloads * kBasis);
    khist.alloc(static_cast<size_t>(nfree) * kBasis);
    hpart.alloc(static_cast<size_t>(kRedBlocks) * (kBasis * (kBasis + 1) / 2 + kBasis));
    hist_count.assign(static_cast<size_t>(d.nloads), 0);
  }
  u.zero();
  weights_d.upload(d.weights);
  // element volumes (uniform cells)
  std::vector<double> vh(ne_s, elem_volume);
  vols.upload(vh);
  domain_volume = 0.0;
  for (double v : vh) domain_volume += v;
  // density filter: stencil offsets within the radius, weights w / row sum
  // with the row sums accumulated in the reference's hash-bucket order
  // (src/topopt/DensityFilter.cpp:36-51, 125-136).
  Stencil st{};
  std::vector<std::array<int, 3>> offs;
  const bool filter_on = d.radius > 0.0;
  if (filter_on) {
    const int rx = static_cast<int>(std::ceil(d.radius / hx)) + 1;
    const int ry = static_cast<int>(std::ceil(d.radius / hy)) + 1;
    const int rz = dim == 3 ? static_cast<int>(std::ceil(d.radius / hz)) + 1 : 0;
    for (int dz = -rz; dz <= rz; ++dz)
      for (int dy = -ry; dy <= ry; ++dy)
        for (int dx = -rx; dx <= rx; ++dx) {
          const double dd = std::sqrt((dx * hx) * (dx * hx) + (dy * hy) * (dy * hy) + (dz * hz) * (dz * hz));
          if (dd < d.radius * (1.0 + 1e-12)) offs.push_back({dx, dy, dz});
        }
    if (offs.size() > 128) throw Error(kBadInput, "filter radius spans more than 128 cells");
  } else {
    offs.push_back({0, 0, 0});
  }
  st.count = static_cast<int>(offs.size());
  for (int k = 0; k < st.count; ++k) {
    st.dx[k] = offs[k][0];
    st.dy[k] = offs[k][1];
    st.dz[k] = offs[k][2];
  }
  stencil_count_ = st.count;
  SIMP_CUDA(cudaMalloc(&stencil_d, sizeof(Stencil)));
  SIMP_CUDA(cudaMemcpy(stencil_d, &st, sizeof(Stencil), cudaMemcpyHostToDevice));
  std::vector<double> w(static_cast<size_t>(st.count) * ne_s, 0.0);
  if (!filter_on) {
    std::fill(w.begin(), w.end(), 1.0);
  } else {
    const int npe = dim == 3 ? 8 : 4;
    // centroid of a cell as the reference forms it: corner coordinates summed
    // in corner order, divided by the corner count
    auto centroid = [&](i64 e, double* c) {
      const i64 ix = e % d.nx, iy = (e / d.nx) % d.ny, iz = e / (static_cast<i64>(d.nx) * d.ny);
      const double xs[2] = {0.0 + ix * hx, 0.0 + (ix + 1) * hx};
      const double ys[2] = {0.0 + iy * hy, 0.0 + (iy + 1) * hy};
      const double zs[2] = {0.0 + iz * hz, 0.0 + (iz + 1) * hz};
      static const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1},
                       cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
      double s[3] = {0, 0, 0};
      for (int a = 0; a < npe; ++a) {
        s[0] += xs[cx[a]];
        s[1] += ys[cy[a]];
        if (dim == 3) s[2] += zs[cz[a]];
      }
      for (int k = 0; k < dim; ++k) c[k] = s[k] / npe;
    };
    const double r = d.radius;
    std::vector<double> rowsum(ne_s);
#pragma omp parallel
    {
      struct Cand {
        long bz, by, bx;
        i64 e;
        int slot;
        double w;
      };
      std::vector<Cand> cands;
#pragma omp for schedule(static)
      for (i64 e = 0; e < ne; ++e) {
        double ce[3] = {0, 0, 0};
        centroid(e, ce);
        const i64 ex = e % d.nx, ey = (e / d.nx) % d.ny, ez = e / (static_cast<i64>(d.nx) * d.ny);
        cands.clear();
        for (int k = 0; k < st.count; ++k) {
          const i64 qx = ex + st.dx[k], qy = ey + st.dy[k], qz = ez + st.dz[k];
          if (qx < 0 || qx >= d.nx || qy < 0 || qy >= d.ny || qz < 0 || qz >= d.nz) continue;
          const i64 q = (qz * d.ny + qy) * d.nx + qx;
          double cq[3] = {0, 0, 0};
          centroid(q, cq);
          double d2 = 0.0;
          for (int k2 = 0; k2 < dim; ++k2) {
            const double df2 = ce[k2] - cq[k2];
            d2 += df2 * df2;
          }
          const double wv = r - std::sqrt(d2);
          if (wv <= 0.0) continue;
          Cand c;
          c.bx = static_cast<long>(std::floor(cq[0] / r));
          c.by = static_cast<long>(std::floor(cq[1] / r));
          c.bz = dim == 3 ? static_cast<long>(std::floor(cq[2] / r)) : 0;
          c.e = q;
          c.slot = k;
          c.w = wv;
          cands.push_back(c);
        }
        std::sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& b) {
          if (a.bz != b.bz) return a.bz < b.bz;
          if (a.by != b.by) return a.by < b.by;
          if (a.bx != b.bx) return a.bx < b.bx;
          return a.e < b.e;
        });
        double sum = 0.0;
        for (const Cand& c : cands) sum += c.w;
        rowsum[e] = sum;
        for (const Cand& c : cands) w[static_cast<size_t>(c.slot) * ne_s + e] = c.w / sum;
      }
    }
  }
  hw.upload(w);
  // dv/dx = H^T v does not depend on the design (without projection)
  filter_adjoint(vols.p, dv_dx.p);
  if (d.projection) {
    rhot.alloc(ne_s);
    dproj.alloc(ne_s);
    beta = beta_of_stage(d, 0);
  }
  // initial design
  std::vector<double> x0(ne_s, std::min(std::max(d.x0, 0.0), 1.0));
  x.upload(x0);
  SIMP_CUDA(cudaDeviceSynchronize());
}

void GpuProblem::filter_forward(const double* xin, double* y) {
  k_filter_forward<<<grid_for(ne, kRedThreads), kRedThreads, 0, amg.stream>>>(
      grid_of(d), static_cast<const Stencil*>(stencil_d), hw.p, ne, xin, y, 0, nullptr, nullptr);
  SIMP_CHECK_LAUNCH();
}

void GpuProblem::filter_adjoint(const double* v, double* gout) {
  k_filter_adjoint<<<grid_for(ne, 256), 256, 0, amg.stream>>>(grid_of(d), static_cast<const Stencil*>(stencil_d),
                                                              hw.p, ne, v, gout);
  SIMP_CHECK_LAUNCH();
}

void GpuProblem::set_design(const double* h) { x.upload(h, static_cast<size_t>(ne), amg.stream); }

void GpuProblem::get_design(double* h) {
  x.download(h, static_cast<size_t>(ne), amg.stream);
  SIMP_CUDA(cudaStreamSynchronize(amg.stream));
}

void GpuProblem::assemble_into(const double* elem, const double* scale, bool exact, double* v64, float* hi,
                               float2* pair, cudaStream_t stream) {
  Level& l0 = *amg.levels.front();
  if (l0.nnodes == 0) return;
  const unsigned blocks = static_cast<unsigned>((l0.nnodes + kAsmTile - 1) / kAsmTile);
  const size_t smem = assemble_smem(d.dim);
  auto kernel = exact ? k_assemble_tiles<true, false> : k_assemble_tiles<false, false>;
  raise_dynamic_smem(reinterpret_cast<const void*>(kernel), smem);
  kernel<<<blocks, assemble_threads(d.dim), smem, stream>>>(grid_of(d), l0.nnodes, l0.d_first.p, gnode.p, cmask.p,
                                                            nmask.p, l0.d_apat.view(), l0.a.ptr.p, elem, scale,
                                                            nullptr, nullptr, v64, hi, pair);
  SIMP_CHECK_LAUNCH();
}

void GpuProblem::assemble(const double* scale, bool exact) {
  Level& l0 = *amg.levels.front();
  if (l0.nnodes == 0) return;
  const GridView g = grid_of(d);
  const unsigned blocks = static_cast<unsigned>((l0.nnodes + kAsmTile - 1) / kAsmTile);
  const size_t smem = assemble_smem(d.dim);
  const int threads = assemble_threads(d.dim);
  auto launch = [&](auto kernel, const float* sh, const float* sl, double* v64, float* hi, float2* pair) {
    raise_dynamic_smem(reinterpret_cast<const void*>(kernel), smem);
    kernel<<<blocks, threads, smem, amg.stream>>>(g, l0.nnodes, l0.d_first.p, gnode.p, cmask.p, nmask.p,
                                                  l0.d_apat.view(), l0.a.ptr.p, ke_d.p, scale, sh, sl, v64, hi,
                                                  pair);
    SIMP_CHECK_LAUNCH();
  };
  if (!amg.mixed()) {
    if (exact) launch(k_assemble_tiles<true, false>, nullptr, nullptr, l0.a.v64.p, nullptr, nullptr);
    else launch(k_assemble_tiles<false, false>, nullptr, nullptr, l0.a.v64.p, nullptr, nullptr);
    return;
  }
  // mixed: the double-float split (hi = the FP32 values of the preconditioner,
  // hi + lo = the CG operator); FP64 values only for the structure-defining
  // exact assembly
  l0.a.v32.alloc(static_cast<size_t>(l0.a.nnz));
  l0.a.v2.alloc(static_cast<size_t>(l0.a.nnz));
  if (exact) {
    launch(k_assemble_tiles<true, false>, nullptr, nullptr, l0.a.v64.p, l0.a.v32.p, l0.a.v2.p);
  } else if (!amg.opt.reuse) {
    // every setup rebuilds the hierarchy from FP64 values
    launch(k_assemble_tiles<false, false>, nullptr, nullptr, l0.a.v64.p, l0.a.v32.p, l0.a.v2.p);
  } else {
    scale_hi.alloc(static_cast<size_t>(ne));
    scale_lo.alloc(static_cast<size_t>(ne));
    k_split_values<<<grid_for(ne, 256, 8192), 256, 0, amg.stream>>>(ne, scale, scale_hi.p, scale_lo.p);
    SIMP_CHECK_LAUNCH();
    launch(k_assemble_tiles<false, true>, scale_hi.p, scale_lo.p, nullptr, l0.a.v32.p, l0.a.v2.p);
  }
  amg.level0_fp32_fresh = true;
}

// Element energies and compliance sensitivities of the current displacements
// (k_sensitivities with the upper triangle of K'_e^0 as its parameter).
void GpuProblem::launch_sensitivities(cudaStream_t s) {
  auto upper = [&](auto& ku, int ed) {
    int idx = 0;
    for (int r = 0; r < ed; ++r)
      for (int c = r; c < ed; ++c)
        ku.k[idx++] = c == r ? d.ke[static_cast<size_t>(r) * ed + r]
                             : d.ke[static_cast<size_t>(r) * ed + c] + d.ke[static_cast<size_t>(c) * ed + r];
  };
  if (d.dim == 3) {
    KeUpper<24> ku;
    upper(ku, 24);
    k_sensitivities<3><<<grid_for(ne, 128), 128, 0, s>>>(grid_of(d), ne, d.nloads, u.p, nfree, dof_map.p, ku,
                                                         weights_d.p, sf.p, df.p, dc_dphys.p, se.p);
  } else {
    KeUpper<8> ku;
    upper(ku, 8);
    k_sensitivities<2><<<grid_for(ne, 128), 128, 0, s>>>(grid_of(d), ne, d.nloads, u.p, nfree, dof_map.p, ku,
                                                         weights_d.p, sf.p, df.p, dc_dphys.p, se.p);
  }
  SIMP_CHECK_LAUNCH();
}

// Filter, projection, SIMP law, assembly and AMG setup of an evaluation
// (Sensitivity.cpp:121-139): everything before the load cases' solves.
void GpuProblem::evaluate_prepare() {
  cudaStream_t s = amg.stream;
  k_filter_forward<<<grid_for(ne, kRedThreads), kRedThreads, 0, s>>>(
      grid_of(d), static_cast<const Stencil*>(stencil_d), hw.p, ne, x.p, d.projection ? rhot.p : rho.p, 1,
      nullptr, nullptr);
  SIMP_CHECK_LAUNCH();
  if (d.projection) {  // the physical density is the projected one (Sensitivity.cpp:69-73)
    k_project<<<grid_for(ne, 256), 256, 0, s>>>(ne, rhot.p, beta, d.objective_eta(), rho.p, dproj.p);
    SIMP_CHECK_LAUNCH();
  }
  k_simp<<<grid_for(ne, 256), 256, 0, s>>>(ne, rho.p, d.penalty, d.emin, sf.p, df.p);
  SIMP_CHECK_LAUNCH();
  if (amg.mf.enabled) {
    k_convert<double, float><<<grid_for(ne, 256), 256, 0, s>>>(sf.p, sf32.p, ne);
    SIMP_CHECK_LAUNCH();
  }
  if (d.warm == 3 && surrogate) {
    // the learned starts depend on the physical density only: the network
    // runs on its own stream while this one assembles and sets up the AMG
    if (!pred_t0) {
      SIMP_CUDA(cudaEventCreate(&pred_t0));
      SIMP_CUDA(cudaEventCreate(&pred_ready));
    }
    predicted.alloc(static_cast<size_t>(nfree) * d.nloads);
    SIMP_CUDA(cudaEventRecord(pred_t0, s));
    for (int l = 0; l < d.nloads; ++l)
      surrogate->predict_async(*this, l, predicted.p + static_cast<size_t>(l) * nfree, pred_ready);
    pred_pending = true;
  }
  // the structure-defining first assembly is bit-exact (the aggregates come
  // from its values); later ones use fused multiply-adds
  assemble(sf.p, !structure_built_);
  amg.setup(!structure_built_);
  structure_built_ = true;
  last_compliance.assign(static_cast<size_t>(d.nloads), 0.0);
}

// The start of load case l's solve: zero, the previous displacement (in
// place), or the projected / learned start.
void GpuProblem::start_load(int l, SolveWork& w) {
  double* ul = u.p + static_cast<size_t>(l) * nfree;
  const bool learned = d.warm == 3 && surrogate != nullptr;
  if (learned) projected_start(l, ul, true);  // also the first solve: the prediction alone
  else if (d.warm == 0 || evaluations == 0) SIMP_CUDA(cudaMemsetAsync(ul, 0, sizeof(double) * nfree, w.stream));
  else if (d.warm >= 2 && hist_count[l] > 0) projected_start(l, ul, false);
}

// After load case l's solve: c_l = f^T u (u vanishes on the supports) and
// the displacement history.
void GpuProblem::end_load(int l, SolveWork& w) {
  double* ul = u.p + static_cast<size_t>(l) * nfree;
  const double* bl = b.p + static_cast<size_t>(l) * nfree;
  last_compliance[static_cast<size_t>(l)] = amg.dot(w, bl, ul, nfree);
  if (d.warm >= 2) record_history(l, ul);
}

SolveTask GpuProblem::load_task(int l, SolveWork& w) {
  SolveTask t;
  t.amg = &amg;
  t.w = &w;
  t.b = b.p + static_cast<size_t>(l) * nfree;
  t.x = u.p + static_cast<size_t>(l) * nfree;
  return t;
}

Evaluation GpuProblem::evaluate() {
  evaluate_prepare();
  cudaStream_t s = amg.stream;
  // one PCG per load case, warm-started from the previous displacement; with
  // several load cases, block_pcg 1 runs the solves at the same time, each on
  // its own workspace and stream from its own host thread, and block_pcg 2
  // advances them together in one CUDA graph (solve_together); both compute
  // what the solves compute one after another
  std::vector<GpuAmg::PcgResult> res(static_cast<size_t>(d.nloads));
  auto solve_load = [&](int l, SolveWork& w) {
    start_load(l, w);
    res[static_cast<size_t>(l)] = amg.solve(w, b.p + static_cast<size_t>(l) * nfree, u.p + static_cast<size_t>(l) * nfree);
    end_load(l, w);
  };
  const bool together = d.block_pcg == 1 && d.nloads > 1 && d.warm < 2;
  if (d.block_pcg == 2 && d.nloads > 1) {
    std::vector<SolveTask> tasks;
    for (int l = 0; l < d.nloads; ++l) {
      SolveWork& w = amg.work(l);
      amg.ensure(w);
      start_load(l, w);
      tasks.push_back(load_task(l, w));
    }
    SIMP_CUDA(cudaStreamSynchronize(s));
    const std::vector<GpuAmg::TaskResult> tr = GpuAmg::solve_together(tasks);
    for (int l = 0; l < d.nloads; ++l)
      if (tr[static_cast<size_t>(l)].error_code) throw Error(tr[static_cast<size_t>(l)].error_code, tr[static_cast<size_t>(l)].error);
    for (int l = 0; l < d.nloads; ++l) {
      res[static_cast<size_t>(l)] = tr[static_cast<size_t>(l)].r;
      end_load(l, amg.work(l));
    }
  } else if (together) {
    SIMP_CUDA(cudaStreamSynchronize(s));  // assembly and setup are done before the solves start
    int dev = 0;
    SIMP_CUDA(cudaGetDevice(&dev));
    std::vector<SolveWork*> works;
    for (int l = 0; l < d.nloads; ++l) works.push_back(&amg.work(l));
    for (SolveWork* w : works) amg.ensure(*w);
    std::vector<std::exception_ptr> errs(static_cast<size_t>(d.nloads));
    std::vector<std::thread> threads;
    for (int l = 1; l < d.nloads; ++l)
      threads.emplace_back([&, l] {
        try {
          SIMP_CUDA(cudaSetDevice(dev));
          solve_load(l, *works[static_cast<size_t>(l)]);
        } catch (...) {
          errs[static_cast<size_t>(l)] = std::current_exception();
        }
      });
    try {
      solve_load(0, *works[0]);
    } catch (...) {
      errs[0] = std::current_exception();
    }
    for (auto& t : threads) t.join();
    for (auto& e : errs)
      if (e) std::rethrow_exception(e);
  } else {
    for (int l = 0; l < d.nloads; ++l) solve_load(l, amg.work(0));
  }
  return evaluate_finish(res);
}

// Compliance, sensitivities, filter pull-back and volumes of an evaluation
// whose solves returned `res` (Sensitivity.cpp:177-237).
Evaluation GpuProblem::evaluate_finish(const std::vector<GpuAmg::PcgResult>& res) {
  cudaStream_t s = amg.stream;
  Evaluation ev;
  if (pred_pending) {  // the solves waited for the predictions: both events have completed
    SIMP_CUDA(cudaEventSynchronize(pred_ready));
    float ms = 0.0f;
    SIMP_CUDA(cudaEventElapsedTime(&ms, pred_t0, pred_ready));
    learned_seconds += 1e-3 * ms;
    pred_pending = false;
  }
  for (int l = 0; l < d.nloads; ++l) {
    const GpuAmg::PcgResult& r = res[static_cast<size_t>(l)];
    if (!r.converged) {
      std::ostringstream os;
      os << "AMG-CG(chebyshev) did not converge: " << r.iterations
         << " iterations left a relative residual of " << r.relres << " against a tolerance of "
         << amg.opt.rtol;
      throw Error(kMaxIter, os.str());
    }
    ev.linear_iterations += r.iterations;
    ev.relres_max = std::max(ev.relres_max, r.relres);
    ev.compliance += d.weights[l] * last_compliance[static_cast<size_t>(l)];
  }
  ++evaluations;
  // element energies and sensitivities
  launch_sensitivities(s);
  if (d.projection) {  // chain_to_design (Sensitivity.cpp:100-108)
    k_mul<<<grid_for(ne, 256), 256, 0, s>>>(ne, dc_dphys.p, dproj.p, tmp.p);
    SIMP_CHECK_LAUNCH();
    filter_adjoint(tmp.p, dc_dx.p);
    k_mul<<<grid_for(ne, 256), 256, 0, s>>>(ne, vols.p, dproj.p, tmp.p);
    SIMP_CHECK_LAUNCH();
    filter_adjoint(tmp.p, dv_dx.p);
  } else {
    filter_adjoint(dc_dphys.p, dc_dx.p);
  }
  // volume of the physical density
  k_dot_partial<double, double><<<kRedBlocks, kRedThreads, 0, s>>>(rho.p, vols.p, ne, amg.part.p);
  SIMP_CHECK_LAUNCH();
  k_reduce_final<<<1, kRedThreads, 0, s>>>(amg.part.p, kRedBlocks, amg.scal.p + 4, 0);
  SIMP_CHECK_LAUNCH();
  SIMP_CUDA(cudaMemcpyAsync(&ev.volume, amg.scal.p + 4, sizeof(double), cudaMemcpyDeviceToHost, s));
  SIMP_CUDA(cudaStreamSynchronize(s));
  ev.volume_fraction = ev.volume / domain_volume;
  if (d.robust && d.eta_override <= 0.0) {
    // robust_volumes (TopologyOptimizer.cpp:61-80): the blueprint's volume,
    // and the dilated design's volume and gradient, which the OC update
    // constrains
    rtmp.alloc(static_cast<size_t>(ne));
    k_project<<<grid_for(ne, 256), 256, 0, s>>>(ne, rhot.p, beta, d.eta, tmp.p, nullptr);
    SIMP_CHECK_LAUNCH();
    ev.volume_intermediate = amg.dot(amg.work(0), tmp.p, vols.p, ne);
    k_project<<<grid_for(ne, 256), 256, 0, s>>>(ne, rhot.p, beta, d.volume_eta(), tmp.p, rtmp.p);
    SIMP_CHECK_LAUNCH();
    ev.volume_dilated = amg.dot(amg.work(0), tmp.p, vols.p, ne);
    k_mul<<<grid_for(ne, 256), 256, 0, s>>>(ne, vols.p, rtmp.p, tmp.p);
    SIMP_CHECK_LAUNCH();
    dv_dilated.alloc(static_cast<size_t>(ne));
    filter_adjoint(tmp.p, dv_dilated.p);
  }
  if (!std::isfinite(ev.compliance)) throw Error(kNonFinite, "the compliance objective evaluated to a non-finite value");
  evaluated = true;
  last_evaluation = ev;
  return ev;
}

// optimality_criteria_update with the filtered candidate volume per trial
// (src/topopt/OptimalityCriteria.cpp:40-149).
// ProjectionOptions::num_stages / beta_of_stage (src/topopt/Projection.cpp:45-54)
int beta_stages(const ProblemDesc& d) {
  int stages = 1;
  double b = d.beta_start;
  while (b < d.beta_max && stages < 64) {
    b *= d.beta_factor;
    ++stages;
  }
  return stages;
}

double beta_of_stage(const ProblemDesc& d, int k) {
  double b = d.beta_start;
  for (int i = 0; i < k && b < d.beta_max; ++i) b *= d.beta_factor;
  return std::min(b, d.beta_max);
}

bool GpuProblem::beta_at_final() const { return !d.projection || beta_stage + 1 >= beta_stages(d); }

// BetaSchedule::advance (src/topopt/TopologyOptimizer.cpp:29-40)
void GpuProblem::advance_beta(double max_change) {
  if (beta_at_final()) return;
  if (iteration - beta_stage_start + 1 >= d.beta_interval ||
      (d.advance_on_convergence && max_change <= d.change_tol)) {
    ++beta_stage;
    beta_stage_start = iteration + 1;
    beta = beta_of_stage(d, beta_stage);
  }
}

GpuProblem::Variants GpuProblem::projection_variants(double delta, double* eroded_density, double* dilated_density) {
  if (!d.projection) throw Error(kBadInput, "the eroded and dilated variants need the projection");
  if (!(delta > 0.0 && d.eta - delta > 0.0 && d.eta + delta < 1.0))
    throw Error(kBadInput, "projection.robust_delta must keep eta - delta and eta + delta inside (0, 1)");
  Variants v;
  const double etas[3] = {d.eta + delta, d.eta, d.eta - delta};
  double* out[3] = {eroded_density, nullptr, dilated_density};
  for (int k = 0; k < 3; ++k) {
    d.eta_override = etas[k];
    Evaluation ev;
    try {
      ev = evaluate();
    } catch (...) {
      d.eta_override = -1.0;
      throw;
    }
    d.eta_override = -1.0;
    v.eta[k] = etas[k];
    v.compliance[k] = ev.compliance;
    v.volume_fraction[k] = ev.volume_fraction;
    if (out[k]) {
      rho.download(out[k], static_cast<size_t>(ne), amg.stream);
      SIMP_CUDA(cudaStreamSynchronize(amg.stream));
    }
  }
  // the gradients of these evaluations are not the loop's: the next update
  // needs a fresh evaluate
  evaluated = false;
  return v;
}

// The dilated target of a robust run, moved to V* V_d / V_i every
// robust_interval iterations (TopologyOptimizer.cpp:625-631).
void GpuProblem::update_robust_target() {
  if (!d.robust) return;
  if (dilated_target <= 0.0) dilated_target = d.vf * domain_volume;
  const Evaluation& ev = last_evaluation;
  if ((iteration - 1) % std::max(1, d.robust_interval) == 0 && ev.volume_intermediate > 0.0)
    dilated_target = d.vf * domain_volume * ev.volume_dilated / ev.volume_intermediate;
}

OcStep GpuProblem::oc_update(bool apply, double* xnew_host) {
  if (!evaluated) throw Error(kBadInput, "oc_update needs gradients: call evaluate first");
  cudaStream_t s = amg.stream;
  // a robust run constrains the dilated design's volume against the moved
  // target, and steps toward a target the move limit cannot reach
  if (d.robust && dilated_target <= 0.0) dilated_target = d.vf * domain_volume;
  const double target = d.robust ? dilated_target : d.vf * domain_volume;
  double* part = opart.p;
  // per-update factors of the candidate; a trial is one fused pass
  oc_g.alloc(static_cast<size_t>(ne));
  oc_lo.alloc(static_cast<size_t>(ne));
  oc_hi.alloc(static_cast<size_t>(ne));
  k_oc_prepare<<<grid_for(ne, 256), 256, 0, s>>>(ne, x.p, dc_dx.p, d.robust ? dv_dilated.p : dv_dx.p, d.move,
                                                d.damping, oc_g.p, oc_lo.p, oc_hi.p);
  SIMP_CHECK_LAUNCH();
  auto factor = [&](double lam) { return d.damping == 0.5 ? 1.0 / std::sqrt(lam) : std::pow(lam, -d.damping); };
  auto volume_of = [&](double lam) {
    if (d.projection) {
      // the projected volume is not linear in the design: candidate, then a
      // filter + projection pass (volume_of_design of run_oc)
      k_oc_apply<<<grid_for(ne, 256), 256, 0, s>>>(ne, oc_g.p, oc_lo.p, oc_hi.p, factor(lam), xnew.p);
      SIMP_CHECK_LAUNCH();
      k_filter_volume_projected<<<kRedBlocks, kRedThreads, 0, s>>>(
          grid_of(d), static_cast<const Stencil*>(stencil_d), hw.p, ne, xnew.p, vols.p, beta, d.volume_eta(), part);
    } else {
      k_oc_volume<<<kRedBlocks, kRedThreads, 0, s>>>(ne, oc_g.p, oc_lo.p, oc_hi.p, dv_dx.p, factor(lam), part);
    }
    SIMP_CHECK_LAUNCH();
    k_reduce_final<<<1, kRedThreads, 0, s>>>(part, kRedBlocks, amg.scal.p + 5, 0);
    SIMP_CHECK_LAUNCH();
    double v = 0.0;
    SIMP_CUDA(cudaMemcpyAsync(&v, amg.scal.p + 5, sizeof(double), cudaMemcpyDeviceToHost, s));
    SIMP_CUDA(cudaStreamSynchronize(s));
    return v;
  };
  double lo = 1.0e-12, hi = 1.0e12;
  double vlo = volume_of(lo), vhi = volume_of(hi);
  int widen = 0;
  while (vlo < target && widen < 60) {
    lo *= 1.0e-3;
    vlo = volume_of(lo);
    ++widen;
  }
  while (vhi > target && widen < 120) {
    hi *= 1.0e3;
    vhi = volume_of(hi);
    ++widen;
  }
  OcStep st;
  bool corner = false;
  if ((vlo < target || vhi > target) && d.robust) {
    // the most-material corner when even it is too light, else the least
    corner = true;
    const bool too_light = vlo < target;
    st.lambda = too_light ? lo : hi;
    st.volume = too_light ? vlo : vhi;
    st.converged = false;
  } else if (vlo < target || vhi > target) {
    std::ostringstream os;
    os << "the optimality-criteria bisection cannot bracket the volume target " << target
       << " m^3: the move-limited box yields volumes in [" << vhi << ", " << vlo << "] m^3";
    throw Error(kMaxIter, os.str());
  }
  double vol = corner ? st.volume : vlo;
  // The bisection of optimality_criteria_update, evaluated speculatively:
  // one pass computes the volumes of the bracket's midpoint and of the
  // midpoints either outcome leads to (a depth-3 tree of 7 multipliers), and
  // the host walks the tree with the sequential rules, so the multipliers,
  // volumes and stopping point are the one-by-one loop's.  It saves host
  // round trips where they dominate; on large grids, where a pass's 7 FP64
  // candidates cost more than the round trips, the depth is 1 (one midpoint
  // per pass, the plain loop).
  const int depth = (d.projection || ne > (1 << 20)) ? 1 : 3;
  int it = 0;
  bool done = corner;
  while (!done && it < 200) {
    double tl[kOcSpec], th[kOcSpec], mids[kOcSpec], vols[kOcSpec];
    const int nodes = (1 << depth) - 1;
    tl[0] = lo;
    th[0] = hi;
    for (int k = 0; k < nodes; ++k) {
      mids[k] = std::sqrt(tl[k] * th[k]);
      if (2 * k + 2 < nodes) {
        tl[2 * k + 1] = mids[k];  // vol > target: lo = mid
        th[2 * k + 1] = th[k];
        tl[2 * k + 2] = tl[k];    // else: hi = mid
        th[2 * k + 2] = mids[k];
      }
    }
    if (nodes == 1) {
      vols[0] = volume_of(mids[0]);
    } else {
      OcFactors f{};
      for (int k = 0; k < nodes; ++k) f.t[k] = factor(mids[k]);
      k_oc_volume_multi<kOcSpec><<<kRedBlocks, kRedThreads, 0, s>>>(ne, oc_g.p, oc_lo.p, oc_hi.p, dv_dx.p, f,
                                                                    part);
      SIMP_CHECK_LAUNCH();
      k_reduce_rows<<<nodes, kRedThreads, 0, s>>>(part, kRedBlocks, ovol.p);
      SIMP_CHECK_LAUNCH();
      SIMP_CUDA(cudaMemcpyAsync(vols, ovol.p, sizeof(double) * nodes, cudaMemcpyDeviceToHost, s));
      SIMP_CUDA(cudaStreamSynchronize(s));
    }
    for (int k = 0; k < nodes && !done;) {
      const double mid = mids[k];
      vol = vols[k];
      st.bisections = ++it;
      st.lambda = mid;
      if (std::abs(vol - target) <= 1.0e-10 * target) {
        st.converged = true;
        done = true;
        break;
      }
      if (vol > target) lo = mid; else hi = mid;
      if (hi / lo - 1.0 < 1.0e-15) {
        st.converged = std::abs(vol - target) <= 1.0e-6 * std::max(target, 1.0e-30);
        done = true;
        break;
      }
      if (it >= 200) break;
      k = vol > target ? 2 * k + 1 : 2 * k + 2;
      if (k >= nodes) break;
    }
  }
  // the design of the final multiplier (the lower bracket end when no
  // bisection ran)
  k_oc_apply<<<grid_for(ne, 256), 256, 0, s>>>(ne, oc_g.p, oc_lo.p, oc_hi.p,
                                              factor(corner ? st.lambda : (st.bisections == 0 ? lo : st.lambda)),
                                              xnew.p);
  SIMP_CHECK_LAUNCH();
  st.volume = vol;
  // max |x' - x| and the grey level of the evaluated density
  k_change_gray<<<kRedBlocks, kRedThreads, 0, s>>>(ne, xnew.p, x.p, rho.p, part, part + kRedBlocks);
  SIMP_CHECK_LAUNCH();
  std::vector<double> hp(2 * kRedBlocks);
  SIMP_CUDA(cudaMemcpyAsync(hp.data(), part, sizeof(double) * 2 * kRedBlocks, cudaMemcpyDeviceToHost, s));
  SIMP_CUDA(cudaStreamSynchronize(s));
  double mc = 0.0, gs = 0.0;
  for (int k = 0; k < kRedBlocks; ++k) {
    mc = std::max(mc, hp[k]);
    gs += hp[kRedBlocks + k];
  }
  st.max_change = mc;
  gray = 4.0 * gs / static_cast<double>(ne);
  if (xnew_host) {
    xnew.download(xnew_host, static_cast<size_t>(ne), s);
    SIMP_CUDA(cudaStreamSynchronize(s));
  }
  if (apply) {
    std::swap(x, xnew);
    k_clamp01<<<grid_for(ne, 256), 256, 0, s>>>(ne, x.p);
    SIMP_CHECK_LAUNCH();
  }
  return st;
}

}  // namespace simp
