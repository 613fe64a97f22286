// Device kernels of the SIMP iteration on a structured Q4 / Hex8 grid:
// value assembly of K_ff, the density filter as a stencil, the SIMP law,
// element strain energies / compliance sensitivities, and the OC candidate
// with its filtered volume.
#pragma once

#include "kernels.cuh"

namespace simp {
namespace {

struct GridView {
  int dim;            // 2 or 3
  i32 nx, ny, nz;     // cells (nz = 1 in 2-D)
  i32 nnx, nny, nnz;  // nodes per axis
};

// VTK corner index of the node at offset (dx, dy, dz) in {0,1}^3 of its cell
// (src/mesh/StructuredMesh.cpp:221-236).
__device__ __forceinline__ int corner_of(int dx, int dy, int dz) { return 4 * dz + (dy ? 3 - dx : dx); }

// K_ff values into the free-free pattern, row-owner gather: entry
// (row (I, ka), column (J, kb)) = sum over the cells shared by I and J, in
// ascending cell order, of s_e * K_e^0(J kb, I ka).  EXACT: rounded products
// and sums in the order of the reference's scatter (src/fem/Assembler.cpp:
// 182-214), so the FP64 values equal a sequential assembly bit for bit;
// otherwise fused multiply-adds.
//
// One block per tile of 32 consecutive free nodes; lane i of every warp owns
// node I0 + i, and warp g walks the neighbour offsets of group g (27 offsets
// in 3-D, 9 in 2-D).  An offset's work is the number of cells the two nodes
// share (8 for the centre, 4 for a face, 2 for an edge, 1 for a corner in
// 3-D), so the groups hold equal totals -- 3-D: the centre; two faces (three
// groups); four edges (three groups); the eight corners; 2-D: the centre
// and the corners; the four edges -- and no warp waits on another at the
// block's staging barrier.  A warp's lanes walk the same cells with the
// same corner indices (uniform trip counts, K_e^0 read as a shared-memory
// broadcast).  Each (node, offset) 3 x 3 block is computed by one thread in
// ascending cell order, whatever the grouping.  The block goes to a shared
// staging copy of the tile's rows, which are one contiguous range of the
// CSR values; the block then writes that range with coalesced stores.
// nmask[I] has bit o set when the neighbour at offset o is a free node; its
// slot is the rank of o among the set bits (the node pattern lists
// neighbours in ascending order = ascending offset order).
constexpr int kAsmTile = 32;
constexpr int kAsmGroups3 = 8, kAsmGroups2 = 2;  // warps per block
__device__ constexpr int kAsmOff3[27] = {13, 4, 10, 12, 14, 16, 22, 1, 3, 5, 7, 9, 11, 15,
                                         17, 19, 21, 23, 25, 0, 2, 6, 8, 18, 20, 24, 26};
__device__ constexpr int kAsmStart3[kAsmGroups3 + 1] = {0, 1, 3, 5, 7, 11, 15, 19, 27};
__device__ constexpr int kAsmOff2[9] = {4, 0, 2, 6, 8, 1, 3, 5, 7};
__device__ constexpr int kAsmStart2[kAsmGroups2 + 1] = {0, 5, 9};
inline int assemble_threads(int dim) { return (dim == 3 ? kAsmGroups3 : kAsmGroups2) * kAsmTile; }

inline size_t assemble_smem(int dim) {
  const int ed = dim == 3 ? 24 : 8, rowvals = dim == 3 ? 3 * 81 : 2 * 18;
  return sizeof(double) * (static_cast<size_t>(ed) * ed + static_cast<size_t>(kAsmTile) * rowvals);
}

// Outputs: val64 (FP64 values), hi (FP32) and pair (the double-float split
// (hi, lo), interleaved), each optional.  DF: the sums themselves run in double-float arithmetic on
// the FP32 pipes from the split scales (sh, sl) and the split element matrix
// (the mixed-precision reuse assemblies, which write hi/lo only); otherwise
// in FP64 (EXACT: rounded products and sums; else fused multiply-adds).
template <bool EXACT, bool DF>
__global__ void __launch_bounds__(kAsmGroups3 * kAsmTile) k_assemble_tiles(
    GridView g, i32 nodes, const i32* __restrict__ first, const i32* __restrict__ gnode,
    const uint8_t* __restrict__ cmask, const uint32_t* __restrict__ nmask, NodeView a,
    const i32* __restrict__ rowptr, const double* __restrict__ ke, const double* __restrict__ scale,
    const float* __restrict__ scale_hi, const float* __restrict__ scale_lo, double* __restrict__ val64,
    float* __restrict__ hi, float2* __restrict__ pair) {
  extern __shared__ double smem_asm[];
  const int ed = g.dim == 3 ? 24 : 8;
  double* ks = smem_asm;
  double* stage = smem_asm + ed * ed;
  float2* ks2 = reinterpret_cast<float2*>(ks);
  float2* stage2 = reinterpret_cast<float2*>(stage);
  for (int e = threadIdx.x; e < ed * ed; e += blockDim.x) {
    if constexpr (DF) {
      float h, l;
      df_split(ke[e], h, l);
      ks2[e] = make_float2(h, l);
    } else {
      ks[e] = ke[e];
    }
  }
  const i32 I0 = blockIdx.x * kAsmTile;
  const i32 I1 = min(I0 + kAsmTile, nodes);
  const i32 base = rowptr[first[I0]], end = rowptr[first[I1]];
  __syncthreads();
  const int grp = threadIdx.x >> 5;
  const i32 I = I0 + (threadIdx.x & 31);
  const uint32_t mk = I < I1 ? nmask[I] : 0u;
  const int q0 = g.dim == 3 ? kAsmStart3[grp] : kAsmStart2[grp];
  const int q1 = g.dim == 3 ? kAsmStart3[grp + 1] : kAsmStart2[grp + 1];
  for (int q = q0; q < q1; ++q) {
    const int o = g.dim == 3 ? kAsmOff3[q] : kAsmOff2[q];
    if (!(mk & (1u << o))) continue;
    const int odx = o % 3 - 1, ody = (o / 3) % 3 - 1, odz = g.dim == 3 ? o / 9 - 1 : 0;
    const i32 t = a.ptr[I] + __popc(mk & ((1u << o) - 1u));
    const i32 gi = gnode[I];
    const i32 ix = gi % g.nnx, iy = (gi / g.nnx) % g.nny, iz = gi / (g.nnx * g.nny);
    const i32 jx = ix + odx, jy = iy + ody, jz = iz + odz;
    const i32 J = a.nbr[t];
    const int maskI = cmask[I], maskJ = cmask[J];
    double acc[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    float ah[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
    float al[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
    const i32 z0 = max(max(iz, jz) - 1, 0), z1 = min(min(iz, jz), g.nz - 1);
    const i32 y0 = max(max(iy, jy) - 1, 0), y1 = min(min(iy, jy), g.ny - 1);
    const i32 x0 = max(max(ix, jx) - 1, 0), x1 = min(min(ix, jx), g.nx - 1);
    for (i32 cz = z0; cz <= z1; ++cz)
      for (i32 cy = y0; cy <= y1; ++cy)
        for (i32 cx = x0; cx <= x1; ++cx) {
          const i64 c = (static_cast<i64>(cz) * g.ny + cy) * g.nx + cx;
          const int aI = corner_of(ix - cx, iy - cy, g.dim == 3 ? iz - cz : 0);
          const int aJ = corner_of(jx - cx, jy - cy, g.dim == 3 ? jz - cz : 0);
          if constexpr (DF) {
            const float sh = scale_hi[c], sl = scale_lo[c];
#pragma unroll
            for (int ka = 0; ka < 3; ++ka)
#pragma unroll
              for (int kb = 0; kb < 3; ++kb)
                if (ka < g.dim && kb < g.dim) {
                  const float2 k = ks2[(g.dim * aJ + kb) * ed + g.dim * aI + ka];
                  df_fma(sh, sl, k.x, k.y, ah[ka][kb], al[ka][kb]);
                }
          } else {
            const double s = scale[c];
#pragma unroll
            for (int ka = 0; ka < 3; ++ka)
#pragma unroll
              for (int kb = 0; kb < 3; ++kb)
                if (ka < g.dim && kb < g.dim) {
                  const double k = ks[(g.dim * aJ + kb) * ed + g.dim * aI + ka];
                  acc[ka][kb] = EXACT ? xadd(acc[ka][kb], xmul(s, k)) : fma(s, k, acc[ka][kb]);
                }
          }
        }
    const i32 r0 = first[I];
    int qa = 0;
#pragma unroll
    for (int ka = 0; ka < 3; ++ka) {
      if (ka >= g.dim || !(maskI & (1 << ka))) continue;
      const i32 rb = rowptr[r0 + qa] + a.off[t] - base;
      int qb = 0;
#pragma unroll
      for (int kb = 0; kb < 3; ++kb) {
        if (kb >= g.dim || !(maskJ & (1 << kb))) continue;
        if constexpr (DF) {
          float s, e;  // renormalised pair
          two_sum(ah[ka][kb], al[ka][kb], s, e);
          stage2[rb + qb] = make_float2(s, e);
        } else {
          stage[rb + qb] = acc[ka][kb];
        }
        ++qb;
      }
      ++qa;
    }
  }
  __syncthreads();
  for (i32 k = threadIdx.x; k < end - base; k += blockDim.x) {
    if constexpr (DF) {
      const float2 v = stage2[k];
      hi[base + k] = v.x;
      pair[base + k] = v;
    } else {
      const double v = stage[k];
      if (val64) val64[base + k] = v;
      if (pair) {
        float h, l;
        df_split(v, h, l);
        hi[base + k] = h;
        pair[base + k] = make_float2(h, l);
      } else if (hi) {
        hi[base + k] = __double2float_rn(v);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// density filter as a stencil: H(e, e + o_s) = w[s][e] (w / row sum, FP64)
// ---------------------------------------------------------------------------
struct Stencil {
  int count;
  int dx[128], dy[128], dz[128];  // offsets, ascending linear order
};

__device__ __forceinline__ bool in_grid(const GridView& g, i32 x, i32 y, i32 z) {
  return x >= 0 && x < g.nx && y >= 0 && y < g.ny && z >= 0 && z < g.nz;
}

// y = H x (ascending neighbour order, as Eigen's column-major product sums);
// clamp01 != 0 also clamps the result to [0, 1]; vol != NULL accumulates
// sum_e v_e y_e into per-block partials.
__global__ void __launch_bounds__(kRedThreads) k_filter_forward(GridView g, const Stencil* __restrict__ st,
                                                                const double* __restrict__ w, i64 ne,
                                                                const double* __restrict__ x,
                                                                double* __restrict__ y, int clamp01,
                                                                const double* __restrict__ volumes,
                                                                double* __restrict__ part) {
  double vs = 0.0;
  for (i64 e = blockIdx.x * (i64)kRedThreads + threadIdx.x; e < ne; e += (i64)gridDim.x * kRedThreads) {
    const i32 ex = static_cast<i32>(e % g.nx), ey = static_cast<i32>((e / g.nx) % g.ny),
              ez = static_cast<i32>(e / ((i64)g.nx * g.ny));
    double s = 0.0;
    for (int k = 0; k < st->count; ++k) {
      const i32 qx = ex + st->dx[k], qy = ey + st->dy[k], qz = ez + st->dz[k];
      if (!in_grid(g, qx, qy, qz)) continue;
      const i64 q = (static_cast<i64>(qz) * g.ny + qy) * g.nx + qx;
      s = xadd(s, xmul(w[k * ne + e], x[q]));
    }
    if (clamp01) s = fmin(fmax(s, 0.0), 1.0);
    if (y) y[e] = s;
    if (part) vs += s * volumes[e];
  }
  if (part) {
    vs = block_sum<kRedThreads>(vs);
    if (threadIdx.x == 0) part[blockIdx.x] = vs;
  }
}

// g = H^T v: column j of H summed over ascending rows e = j - o_s.
__global__ void k_filter_adjoint(GridView g, const Stencil* __restrict__ st, const double* __restrict__ w,
                                 i64 ne, const double* __restrict__ v, double* __restrict__ out) {
  for (i64 j = blockIdx.x * (i64)blockDim.x + threadIdx.x; j < ne; j += (i64)gridDim.x * blockDim.x) {
    const i32 jx = static_cast<i32>(j % g.nx), jy = static_cast<i32>((j / g.nx) % g.ny),
              jz = static_cast<i32>(j / ((i64)g.nx * g.ny));
    double s = 0.0;
    for (int k = st->count - 1; k >= 0; --k) {
      const i32 ex = jx - st->dx[k], ey = jy - st->dy[k], ez = jz - st->dz[k];
      if (!in_grid(g, ex, ey, ez)) continue;
      const i64 e = (static_cast<i64>(ez) * g.ny + ey) * g.nx + ex;
      s = xadd(s, xmul(w[k * ne + e], v[e]));
    }
    out[j] = s;
  }
}

// Correctly rounded r^3 (double-double product): the FP64 SIMP law with the
// penalty 3 of every configuration gives the same factors as a correctly
// rounded pow.
__device__ __forceinline__ double cube_rn(double r) {
  const double h = r * r;
  const double l = fma(r, r, -h);            // r^2 = h + l exactly
  const double p = h * r;
  const double pe = fma(h, r, -p);           // h r = p + pe exactly
  return p + fma(l, r, pe);
}

__device__ __forceinline__ double simp_pow(double r, double p) {
  if (p == 3.0) return cube_rn(r);
  return pow(r, p);
}

// rho -> stiffness factor and its derivative (src/topopt/SimpInterpolation.cpp:59-70)
__global__ void k_simp(i64 ne, const double* __restrict__ rho, double pen, double emin,
                       double* __restrict__ sf, double* __restrict__ df) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < ne; e += (i64)gridDim.x * blockDim.x) {
    const double r = fmin(fmax(rho[e], 0.0), 1.0);
    sf[e] = xadd(emin, xmul(1.0 - emin, simp_pow(r, pen)));
    df[e] = xmul(xmul(pen, 1.0 - emin), pen == 3.0 ? xmul(r, r) : pow(r, pen - 1.0));
  }
}

// Element energies u_e^T K_e^0 u_e for every load case (src/topopt/
// Sensitivity.cpp:182-189): dc/drho_e -= w_l dE_e q, SE_e += w_l / 2 E_e q.
// The quadratic form runs over the upper triangle, q = sum_r u_r sum_{c>=r}
// K'_rc u_c with K'_rr = K_rr and K'_rc = K_rc + K_cr (the same value in exact
// arithmetic, 300 instead of 576 FP64 multiply-adds per Hex8 element and load
// case on GB300's FP64 pipe).  K' is a kernel parameter indexed by
// compile-time constants, so its entries are constant-bank operands.
template <int ED>
struct KeUpper {
  double k[ED * (ED + 1) / 2];  // row-major upper triangle of K'
};

template <int DIM>
__global__ void __launch_bounds__(128) k_sensitivities(GridView g, i64 ne, int nloads,
                                                       const double* __restrict__ u, i64 ldu,
                                                       const i32* __restrict__ dof_map,
                                                       const __grid_constant__ KeUpper<4 * DIM * (DIM - 1)> ku,
                                                       const double* __restrict__ weights,
                                                       const double* __restrict__ sf,
                                                       const double* __restrict__ df,
                                                       double* __restrict__ dc, double* __restrict__ se) {
  constexpr int NPE = DIM == 3 ? 8 : 4, ED = NPE * DIM;
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < ne; e += (i64)gridDim.x * blockDim.x) {
    const i32 ex = static_cast<i32>(e % g.nx), ey = static_cast<i32>((e / g.nx) % g.ny),
              ez = static_cast<i32>(e / ((i64)g.nx * g.ny));
    const i64 n0 = (static_cast<i64>(ez) * g.nny + ey) * g.nnx + ex;
    const i64 layer = static_cast<i64>(g.nnx) * g.nny;
    i64 nodes[NPE];
    nodes[0] = n0;
    nodes[1] = n0 + 1;
    nodes[2] = n0 + g.nnx + 1;
    nodes[3] = n0 + g.nnx;
    if constexpr (DIM == 3) {
#pragma unroll
      for (int a = 0; a < 4; ++a) nodes[4 + a] = nodes[a] + layer;
    }
    i32 f[ED];
#pragma unroll
    for (int a = 0; a < NPE; ++a)
#pragma unroll
      for (int k = 0; k < DIM; ++k) f[DIM * a + k] = dof_map[nodes[a] * DIM + k];
    double dcs = 0.0, ses = 0.0;
    for (int l = 0; l < nloads; ++l) {
      double ue[ED];
#pragma unroll
      for (int q = 0; q < ED; ++q) ue[q] = f[q] >= 0 ? u[l * ldu + f[q]] : 0.0;
      double quad = 0.0;
      int idx = 0;
#pragma unroll
      for (int r = 0; r < ED; ++r) {
        double kr = 0.0;
#pragma unroll
        for (int c = r; c < ED; ++c) kr = fma(ku.k[idx++], ue[c], kr);
        quad = fma(ue[r], kr, quad);
      }
      ses += weights[l] * 0.5 * sf[e] * quad;
      dcs -= weights[l] * df[e] * quad;
    }
    dc[e] = dcs;
    se[e] = ses;
  }
}

// Heaviside projection of the clamped filtered density and its derivative
// (heaviside_project / heaviside_derivative, src/topopt/Projection.cpp:56-69).
__device__ __forceinline__ double project_one(double r, double beta, double eta, double& deriv) {
  const double a = tanh(beta * eta);
  const double denom = a + tanh(beta * (1.0 - eta));
  const double t = tanh(beta * (r - eta));
  deriv = beta * (1.0 - t * t) / denom;
  return (a + t) / denom;
}

__global__ void k_project(i64 ne, const double* __restrict__ rt, double beta, double eta, double* __restrict__ rho,
                          double* __restrict__ dproj) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < ne; e += (i64)gridDim.x * blockDim.x) {
    double dp;
    rho[e] = project_one(rt[e], beta, eta, dp);
    if (dproj) dproj[e] = dp;
  }
}

__global__ void k_mul(i64 ne, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < ne; e += (i64)gridDim.x * blockDim.x)
    out[e] = a[e] * b[e];
}

// Projected filtered volume of a candidate design: block partials of
// sum_e v_e rho_bar(clamp((H x)_e)) (the OC trial volume with projection on).
__global__ void __launch_bounds__(kRedThreads) k_filter_volume_projected(GridView g, const Stencil* __restrict__ st,
                                                                         const double* __restrict__ w, i64 ne,
                                                                         const double* __restrict__ x,
                                                                         const double* __restrict__ volumes,
                                                                         double beta, double eta,
                                                                         double* __restrict__ part) {
  double vs = 0.0;
  for (i64 e = blockIdx.x * (i64)kRedThreads + threadIdx.x; e < ne; e += (i64)gridDim.x * kRedThreads) {
    const i32 ex = static_cast<i32>(e % g.nx), ey = static_cast<i32>((e / g.nx) % g.ny),
              ez = static_cast<i32>(e / ((i64)g.nx * g.ny));
    double s = 0.0;
    for (int k = 0; k < st->count; ++k) {
      const i32 qx = ex + st->dx[k], qy = ey + st->dy[k], qz = ez + st->dz[k];
      if (!in_grid(g, qx, qy, qz)) continue;
      const i64 q = (static_cast<i64>(qz) * g.ny + qy) * g.nx + qx;
      s = xadd(s, xmul(w[k * ne + e], x[q]));
    }
    s = fmin(fmax(s, 0.0), 1.0);
    double dp;
    vs += project_one(s, beta, eta, dp) * volumes[e];
  }
  vs = block_sum<kRedThreads>(vs);
  if (threadIdx.x == 0) part[blockIdx.x] = vs;
}

// Per OC update (src/topopt/OptimalityCriteria.cpp:14-38 restated for a
// multiplier search on the GPU): g_e = x_e max(0, -dc_e / dv_e)^eta (0 where
// dv_e <= 0) and the move-limited box [lo_e, hi_e], so that the candidate of
// multiplier lam is clamp(g_e lam^-eta, lo_e, hi_e) -- the reference's
// x (-dc / (lam dv))^eta with the quotient and the power taken once per
// update instead of once per bisection trial (GB300's FP64 division and
// square root are long instruction sequences on its 1/64-rate FP64 pipe).
__global__ void k_oc_prepare(i64 ne, const double* __restrict__ x, const double* __restrict__ dc,
                             const double* __restrict__ dv, double move, double eta, double* __restrict__ g,
                             double* __restrict__ lo, double* __restrict__ hi) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < ne; e += (i64)gridDim.x * blockDim.x) {
    const double xe = x[e];
    lo[e] = fmax(0.0, xe - move);
    hi[e] = fmin(1.0, xe + move);
    double q = 0.0;
    if (dv[e] > 0.0) q = fmax(0.0, -dc[e] / dv[e]);
    g[e] = xe * (eta == 0.5 ? sqrt(q) : pow(q, eta));
  }
}

// Filtered volume of the candidate of multiplier lam (t = lam^-eta): the
// volume sum_e v_e (H x')_e equals c^T x' with c = H^T v (dv_dx), so a trial
// needs no filter pass.  Block partials of sum_e c_e clamp(g_e t, lo_e, hi_e).
__global__ void __launch_bounds__(kRedThreads) k_oc_volume(i64 ne, const double* __restrict__ g,
                                                           const double* __restrict__ lo,
                                                           const double* __restrict__ hi,
                                                           const double* __restrict__ c, double t,
                                                           double* __restrict__ part) {
  double s = 0.0;
  for (i64 e = blockIdx.x * (i64)kRedThreads + threadIdx.x; e < ne; e += (i64)gridDim.x * kRedThreads)
    s += c[e] * fmin(fmax(g[e] * t, lo[e]), hi[e]);
  s = block_sum<kRedThreads>(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// The same block partials for K multipliers in one pass over the element
// arrays (part[k * gridDim.x + block] for t[k]); each multiplier's sum is
// formed exactly as k_oc_volume forms it.
constexpr int kOcSpec = 7;  // multipliers of one speculative bisection pass
struct OcFactors {
  double t[kOcSpec];
};

template <int K>
__global__ void __launch_bounds__(kRedThreads) k_oc_volume_multi(i64 ne, const double* __restrict__ g,
                                                                 const double* __restrict__ lo,
                                                                 const double* __restrict__ hi,
                                                                 const double* __restrict__ c, OcFactors f,
                                                                 double* __restrict__ part) {
  double s[K];
#pragma unroll
  for (int k = 0; k < K; ++k) s[k] = 0.0;
  for (i64 e = blockIdx.x * (i64)kRedThreads + threadIdx.x; e < ne; e += (i64)gridDim.x * kRedThreads) {
    const double ge = g[e], le = lo[e], he = hi[e], ce = c[e];
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] += ce * fmin(fmax(ge * f.t[k], le), he);
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const double v = block_sum<kRedThreads>(s[k]);
    if (threadIdx.x == 0) part[k * gridDim.x + blockIdx.x] = v;
  }
}

// out[k] = sum of part[k * m .. k * m + m), one block per k, each summed as
// k_reduce_final sums (no square root)
__global__ void __launch_bounds__(kRedThreads) k_reduce_rows(const double* __restrict__ part, int m,
                                                             double* __restrict__ out) {
  const double* pk = part + static_cast<i64>(blockIdx.x) * m;
  double s = 0.0;
  for (int i = threadIdx.x; i < m; i += kRedThreads) s += pk[i];
  s = block_sum<kRedThreads>(s);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

__global__ void k_oc_apply(i64 ne, const double* __restrict__ g, const double* __restrict__ lo,
                           const double* __restrict__ hi, double t, double* __restrict__ xn) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < ne; e += (i64)gridDim.x * blockDim.x)
    xn[e] = fmin(fmax(g[e] * t, lo[e]), hi[e]);
}

// max |a - b| and sum rho (1 - rho) partials
__global__ void __launch_bounds__(kRedThreads) k_change_gray(i64 ne, const double* __restrict__ a,
                                                             const double* __restrict__ b,
                                                             const double* __restrict__ rho,
                                                             double* __restrict__ part_max,
                                                             double* __restrict__ part_gray) {
  double m = 0.0, gsum = 0.0;
  for (i64 e = blockIdx.x * (i64)kRedThreads + threadIdx.x; e < ne; e += (i64)gridDim.x * kRedThreads) {
    m = fmax(m, fabs(a[e] - b[e]));
    if (rho) gsum += rho[e] * (1.0 - rho[e]);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ double wm[kRedThreads / 32];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
  gsum = block_sum<kRedThreads>(gsum);
  if (threadIdx.x == 0) {
    double mm = 0.0;
    for (int k = 0; k < kRedThreads / 32; ++k) mm = fmax(mm, wm[k]);
    part_max[blockIdx.x] = mm;
    if (part_gray) part_gray[blockIdx.x] = gsum;
  }
}

__global__ void k_clamp01(i64 ne, double* __restrict__ x) {
  for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < ne; e += (i64)gridDim.x * blockDim.x)
    x[e] = fmin(fmax(x[e], 0.0), 1.0);
}

}  // namespace
}  // namespace simp
