// Matrix-free level-0 operator of a structured Q4 / Hex8 grid (FP32).
//
// y_I = sum over the cells e around node I of s_e sum_J K_e^0(I, J) x_J, with
// one thread per free node gathering its (at most 8) cells: every output is
// written once, no atomics, and the result does not depend on the launch
// shape.  The 8 (4) cells around a node are visited in a fixed order, so all
// threads of a warp read the same K_e^0 rows at the same time (a broadcast
// from shared memory).  Used where every node is either fully free or fully
// clamped (the free DOFs of node I are 3I', 3I'+1, 3I'+2 for its free index
// I'); the assembled operator is used otherwise.
#pragma once

#include "kernels.cuh"

namespace simp {
namespace {

struct MfView {
  int dim;             // 2 or 3
  i32 nx, ny, nz;      // cells (nz = 1 in 2-D)
  i32 nnx, nny;        // nodes per axis in x, y
  const i32* gnode;    // free node -> grid node
  const i32* nindex;   // grid node -> free node or -1
  const float* ke;     // K_e^0 (ed x ed, row-major)
  const float* scale;  // s_e
};

// Per-node product (A x)_I for the free node I; out[k], k < dim.
template <class TX>
__device__ __forceinline__ void mf_node_apply(const MfView& m, const float* __restrict__ ks, i32 I,
                                              const TX* __restrict__ x, float (&out)[3]) {
  const int dim = m.dim;
  const int ed = dim == 3 ? 24 : 8;
  out[0] = out[1] = out[2] = 0.0f;
  const i32 g = m.gnode[I];
  const i32 ix = g % m.nnx, iy = (g / m.nnx) % m.nny, iz = g / (m.nnx * m.nny);
  const int zlo = dim == 3 ? -1 : 0;
  for (int dz = zlo; dz <= 0; ++dz)
    for (int dy = -1; dy <= 0; ++dy)
      for (int dx = -1; dx <= 0; ++dx) {
        const i32 cx = ix + dx, cy = iy + dy, cz = iz + dz;
        if (cx < 0 || cx >= m.nx || cy < 0 || cy >= m.ny || cz < 0 || cz >= m.nz) continue;
        const float s = m.scale[(static_cast<i64>(cz) * m.ny + cy) * m.nx + cx];
        // corner index of node I in cell c: offsets (-dx, -dy, -dz)
        const int ox = -dx, oy = -dy, oz = -dz;
        const int aI = 4 * oz + (oy ? 3 - ox : ox);
        float acc[3] = {0.0f, 0.0f, 0.0f};
        const int npe = dim == 3 ? 8 : 4;
        for (int b = 0; b < npe; ++b) {
          const int bx = (b == 1 || b == 2 || b == 5 || b == 6) ? 1 : 0;
          const int by = (b == 2 || b == 3 || b == 6 || b == 7) ? 1 : 0;
          const int bz = b >= 4 ? 1 : 0;
          const i64 gj = (static_cast<i64>(cz + bz) * m.nny + (cy + by)) * m.nnx + (cx + bx);
          const i32 J = m.nindex[gj];
          if (J < 0) continue;
          float xj[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) xj[k] = k < dim ? static_cast<float>(x[static_cast<i64>(J) * dim + k]) : 0.0f;
#pragma unroll
          for (int ka = 0; ka < 3; ++ka) {
            if (ka < dim) {
              const float* row = ks + (dim * aI + ka) * ed + dim * b;
#pragma unroll
              for (int kb = 0; kb < 3; ++kb)
                if (kb < dim) acc[ka] = fmaf(row[kb], xj[kb], acc[ka]);
            }
          }
        }
#pragma unroll
        for (int ka = 0; ka < 3; ++ka) out[ka] = fmaf(s, acc[ka], out[ka]);
      }
}

// mode 0: y = A x ; 1: y = b - A x ; 2: y += A x
template <int MODE, class TX>
__global__ void __launch_bounds__(256) k_mf_apply(MfView m, i32 nodes, const TX* __restrict__ x, TX* __restrict__ y,
                                                  const TX* __restrict__ b) {
  __shared__ float ks[24 * 24];
  const int ed = m.dim == 3 ? 24 : 8;
  for (int k = threadIdx.x; k < ed * ed; k += blockDim.x) ks[k] = m.ke[k];
  __syncthreads();
  const i32 I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= nodes) return;
  float out[3];
  mf_node_apply<TX>(m, ks, I, x, out);
  for (int k = 0; k < m.dim; ++k) {
    const i64 row = static_cast<i64>(I) * m.dim + k;
    if (MODE == 0) y[row] = static_cast<TX>(out[k]);
    else if (MODE == 1) y[row] = b[row] - static_cast<TX>(out[k]);
    else y[row] += static_cast<TX>(out[k]);
  }
}

// Chebyshev step: r = r_in - A d ; dn = c1 d + c2 dinv r ; x = (x [+ d]) + dn
__global__ void __launch_bounds__(256) k_mf_cheb_step(MfView m, i32 nodes, const float* __restrict__ d,
                                                      const float* __restrict__ r_in, float* __restrict__ r,
                                                      float* __restrict__ dn, float* __restrict__ x,
                                                      const float* __restrict__ dinv,
                                                      const float* __restrict__ c12, int add_d) {
  __shared__ float ks[24 * 24];
  const int ed = m.dim == 3 ? 24 : 8;
  for (int k = threadIdx.x; k < ed * ed; k += blockDim.x) ks[k] = m.ke[k];
  __syncthreads();
  const i32 I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= nodes) return;
  float out[3];
  mf_node_apply<float>(m, ks, I, d, out);
  for (int k = 0; k < m.dim; ++k) {
    const i64 row = static_cast<i64>(I) * m.dim + k;
    const float ri = r_in[row] - out[k];
    r[row] = ri;
    const float di = c12[0] * d[row] + c12[1] * dinv[row] * ri;
    dn[row] = di;
    float xi = x[row];
    if (add_d) xi = xi + d[row];
    x[row] = xi + di;
  }
}

// r = b - A x ; d = dinv r / theta
__global__ void __launch_bounds__(256) k_mf_cheb_first(MfView m, i32 nodes, const float* __restrict__ x,
                                                       const float* __restrict__ b, float* __restrict__ r,
                                                       float* __restrict__ d, const float* __restrict__ dinv,
                                                       const float* __restrict__ inv_theta) {
  __shared__ float ks[24 * 24];
  const int ed = m.dim == 3 ? 24 : 8;
  for (int k = threadIdx.x; k < ed * ed; k += blockDim.x) ks[k] = m.ke[k];
  __syncthreads();
  const i32 I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= nodes) return;
  float out[3];
  mf_node_apply<float>(m, ks, I, x, out);
  for (int k = 0; k < m.dim; ++k) {
    const i64 row = static_cast<i64>(I) * m.dim + k;
    const float ri = b[row] - out[k];
    r[row] = ri;
    d[row] = dinv[row] * ri * *inv_theta;
  }
}

// ---------------------------------------------------------------------------
// Tiled 3-D variant: a block of 32 x 4 x 2 threads owns a 32 x 4 x (2 kNZ)
// tile of grid nodes (kNZ node layers per thread; two layers per thread
// measured slower at 192 x 96 x 96, 109 against 105 us); the tile's node
// values plus a one-node halo (one shared array per component) and the
// scales of the cells that touch it are staged in shared memory once (see
// MfHalo for the node values' layouts).  Each thread sums
// the 64 (cell, corner) 3 x 3 block products with K_e^0 taken from the kernel
// parameter (a __grid_constant__ struct indexed by compile-time constants,
// so its entries are constant-bank operands of the FMAs rather than loads).
// Modes: 0 y = A x, 1 y = b - A x, 3 Chebyshev step, 4 Chebyshev first step
// (same epilogues as the other operator kernels); and the pieces of the
// smoothed-prolongator transfers P = (I - w D^-1 A) P^ applied without P:
// 5 x_s += t - w D^-1 A t (t = P^ x_c, the input), 6 y = b - A x with
// dn = D^-1 y, 7 y = b - w A x (x = D^-1 r, b = r: the vector P^T maps to
// the coarse right-hand side); 8 y64 = A x in FP64 storage (the FP32 product
// as the CG operator of the matrix-free variant).
// ---------------------------------------------------------------------------
constexpr int kTX = 32, kTY = 4, kTZ = 2;  // threads per block axis (the default tile)
constexpr int kNZ = 1;                      // node layers per thread
// Tile shapes the launch-shape tuner chooses among (TX x TY x TZ threads,
// one node each), each with both halo layouts (variant v: shape v % 5, the
// float4 layout for v >= 5): every variant sums each node's cells and
// corners in the same order, so all give the same values bit for bit.
constexpr int kMfTiles = 10;
constexpr int kMfTileShape[5][3] = {{32, 4, 2}, {32, 8, 1}, {32, 2, 4}, {64, 2, 2}, {32, 4, 1}};

struct KeF32 {
  float k[24 * 24];  // K_e^0, row-major
};

struct MfArgs {
  const float* x;     // input (d for the Chebyshev step)
  float* y;           // mode 0/1: output
  const float* b;     // mode 1/4: right-hand side; mode 3: r_in
  float* r;           // mode 3/4: residual out
  float* dn;          // mode 3: new direction; mode 4: d out
  float* xs;          // mode 3: smoothed iterate (updated)
  const float* dinv;  // mode 3/4/5/6
  const float* coef;  // mode 3: (c1, c2); mode 4: 1 / theta; mode 5/7: w (device memory)
  int add_d;
  double* y64;        // mode 8: output
};

// The epilogue of a node's product o = (A x)_I (3 components) in each mode,
// in two parts: the node's operand loads (mf_node_load: right-hand side,
// inverse diagonal, smoothed iterate, as the mode reads them) and the
// arithmetic and stores (mf_node_store), so a kernel can issue the loads
// early.  self = the input x at node I itself (mode 3: the direction d,
// mode 5: t); c0, c1 = coef[0], coef[1] of the modes that read them.
struct MfNodeIn {
  float b[3], dinv[3], xs[3];
};

template <int MODE>
__device__ __forceinline__ void mf_node_load(const MfArgs& a, i32 I, MfNodeIn& in) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const i64 row = static_cast<i64>(I) * 3 + k;
    if (MODE == 1 || MODE == 3 || MODE == 4 || MODE == 6 || MODE == 7) in.b[k] = a.b[row];
    if (MODE == 3 || MODE == 4 || MODE == 5 || MODE == 6) in.dinv[k] = a.dinv[row];
    if (MODE == 3 || MODE == 5) in.xs[k] = a.xs[row];
  }
}

template <int MODE>
__device__ __forceinline__ void mf_node_store(const MfArgs& a, i32 I, const float (&o)[3], const float (&self)[3],
                                              const MfNodeIn& in, float c0, float c1) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const i64 row = static_cast<i64>(I) * 3 + k;
    if (MODE == 0) {
      a.y[row] = o[k];
    } else if (MODE == 1) {
      a.y[row] = in.b[k] - o[k];
    } else if (MODE == 3) {
      const float ri = in.b[k] - o[k];
      a.r[row] = ri;
      const float dv = self[k];
      const float di = c0 * dv + c1 * in.dinv[k] * ri;
      a.dn[row] = di;
      float xi = in.xs[k];
      if (a.add_d) xi = xi + dv;
      a.xs[row] = xi + di;
    } else if (MODE == 4) {
      const float ri = in.b[k] - o[k];
      a.r[row] = ri;
      a.dn[row] = in.dinv[k] * ri * c0;
    } else if (MODE == 5) {
      a.xs[row] = in.xs[k] + (self[k] - c0 * (in.dinv[k] * o[k]));
    } else if (MODE == 6) {
      const float ri = in.b[k] - o[k];
      a.y[row] = ri;
      a.dn[row] = in.dinv[k] * ri;
    } else if (MODE == 8) {
      a.y64[row] = static_cast<double>(o[k]);
    } else {
      a.y[row] = in.b[k] - c0 * o[k];
    }
  }
}

// coef[0], coef[1] of the modes that read them (device scalars)
template <int MODE>
__device__ __forceinline__ void mf_coefs(const MfArgs& a, float& c0, float& c1) {
  c0 = c1 = 0.0f;
  if (MODE == 3) {
    c0 = a.coef[0];
    c1 = a.coef[1];
  } else if (MODE == 4 || MODE == 5 || MODE == 7) {
    c0 = a.coef[0];
  }
}

template <int MODE>
__device__ __forceinline__ void mf_node_out(const MfArgs& a, i32 I, const float (&o)[3], const float (&self)[3]) {
  MfNodeIn in;
  mf_node_load<MODE>(a, I, in);
  float c0, c1;
  mf_coefs<MODE>(a, c0, c1);
  mf_node_store<MODE>(a, I, o, self, in, c0, c1);
}

// Node values of a tile in shared memory: one array per component (V4
// false: three 4-byte loads per corner, fewer registers) or (x, y, z,
// unused) per node (V4 true: one 16-byte load per corner).  The tuner picks;
// the arithmetic is the same.
template <bool V4, int NZ, int TY, int TX>
struct MfHalo;
template <int NZ, int TY, int TX>
struct MfHalo<false, NZ, TY, TX> {
  float v[3][NZ + 2][TY + 2][TX + 2];
  __device__ __forceinline__ void put(int z, int y, int x, float a, float b, float c) {
    v[0][z][y][x] = a;
    v[1][z][y][x] = b;
    v[2][z][y][x] = c;
  }
  __device__ __forceinline__ void get(int z, int y, int x, float (&o)[3]) const {
    o[0] = v[0][z][y][x];
    o[1] = v[1][z][y][x];
    o[2] = v[2][z][y][x];
  }
};
template <int NZ, int TY, int TX>
struct MfHalo<true, NZ, TY, TX> {
  float4 v[NZ + 2][TY + 2][TX + 2];
  __device__ __forceinline__ void put(int z, int y, int x, float a, float b, float c) {
    v[z][y][x] = make_float4(a, b, c, 0.0f);
  }
  __device__ __forceinline__ void get(int z, int y, int x, float (&o)[3]) const {
    const float4 t = v[z][y][x];
    o[0] = t.x;
    o[1] = t.y;
    o[2] = t.z;
  }
};

template <int MODE, int TX = kTX, int TY = kTY, int TZ = kTZ, bool V4 = false>
__global__ void __launch_bounds__(TX* TY* TZ) k_mf3_tile(MfView m, MfArgs a, const __grid_constant__ KeF32 ke) {
  constexpr int NZ = TZ * kNZ;  // node layers of the tile
  __shared__ MfHalo<V4, NZ, TY, TX> xh;
  __shared__ float sc[NZ + 1][TY + 1][TX + 1];
  const int tid = threadIdx.x;
  const i32 x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * NZ;
  const i32 nnz = m.nz + 1;
  // node values of the tile and its halo (zero outside the grid / clamped):
  // every thread first loads the free-node indices of all its halo entries,
  // then their values, so the loads of one thread are independent
  constexpr int kHalo = (NZ + 2) * (TY + 2) * (TX + 2);
  constexpr int kPer = (kHalo + TX * TY * TZ - 1) / (TX * TY * TZ);
  i32 hj[kPer];
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int e = tid + q * TX * TY * TZ;
    const int hx = e % (TX + 2), hy = (e / (TX + 2)) % (TY + 2), hz = e / ((TX + 2) * (TY + 2));
    const i32 gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = z0 - 1 + hz;
    hj[q] = -1;
    if (e < kHalo && gx >= 0 && gx < m.nnx && gy >= 0 && gy < m.nny && gz >= 0 && gz < nnz)
      hj[q] = m.nindex[(static_cast<i64>(gz) * m.nny + gy) * m.nnx + gx];
  }
  float hv[kPer][3];
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    hv[q][0] = hv[q][1] = hv[q][2] = 0.0f;
    if (hj[q] >= 0) {
      const float* p = a.x + static_cast<i64>(hj[q]) * 3;
      hv[q][0] = p[0];
      hv[q][1] = p[1];
      hv[q][2] = p[2];
    }
  }
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int e = tid + q * TX * TY * TZ;
    if (e < kHalo) {
      const int hx = e % (TX + 2), hy = (e / (TX + 2)) % (TY + 2), hz = e / ((TX + 2) * (TY + 2));
      xh.put(hz, hy, hx, hv[q][0], hv[q][1], hv[q][2]);
    }
  }
  // cell scales (zero outside the grid)
  for (int e = tid; e < (NZ + 1) * (TY + 1) * (TX + 1); e += TX * TY * TZ) {
    const int cx = e % (TX + 1), cy = (e / (TX + 1)) % (TY + 1), cz = e / ((TX + 1) * (TY + 1));
    const i32 gx = x0 - 1 + cx, gy = y0 - 1 + cy, gz = z0 - 1 + cz;
    float s = 0.0f;
    if (gx >= 0 && gx < m.nx && gy >= 0 && gy < m.ny && gz >= 0 && gz < m.nz)
      s = m.scale[(static_cast<i64>(gz) * m.ny + gy) * m.nx + gx];
    sc[cz][cy][cx] = s;
  }
  __syncthreads();
  const int tx = tid % TX, ty = (tid / TX) % TY, tz = tid / (TX * TY);
  const i32 gx = x0 + tx, gy = y0 + ty;
  if (gx >= m.nnx || gy >= m.nny) return;
  // kNZ consecutive node layers per thread: their neighbourhoods share
  // layers, so each shared value is loaded once per thread
#pragma unroll
  for (int q = 0; q < kNZ; ++q) {
    const int lz = tz * kNZ + q;  // node layer in the tile
    const i32 gz = z0 + lz;
    if (gz >= nnz) break;
    const i32 I = m.nindex[(static_cast<i64>(gz) * m.nny + gy) * m.nnx + gx];
    if (I < 0) continue;
    float out0 = 0.0f, out1 = 0.0f, out2 = 0.0f;
#pragma unroll
    for (int dz = -1; dz <= 0; ++dz)
#pragma unroll
      for (int dy = -1; dy <= 0; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 0; ++dx) {
          const float s = sc[lz + dz + 1][ty + dy + 1][tx + dx + 1];
          const int ox = -dx, oy = -dy, oz = -dz;
          const int aI = 4 * oz + (oy ? 3 - ox : ox);
          float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
#pragma unroll
          for (int b = 0; b < 8; ++b) {
            const int bx = (b == 1 || b == 2 || b == 5 || b == 6) ? 1 : 0;
            const int by = (b == 2 || b == 3 || b == 6 || b == 7) ? 1 : 0;
            const int bz = b >= 4 ? 1 : 0;
            float xb[3];
            xh.get(lz + dz + 1 + bz, ty + dy + 1 + by, tx + dx + 1 + bx, xb);
#pragma unroll
            for (int kb = 0; kb < 3; ++kb) {
              const float xv = xb[kb];
              a0 = fmaf(ke.k[(3 * aI + 0) * 24 + 3 * b + kb], xv, a0);
              a1 = fmaf(ke.k[(3 * aI + 1) * 24 + 3 * b + kb], xv, a1);
              a2 = fmaf(ke.k[(3 * aI + 2) * 24 + 3 * b + kb], xv, a2);
            }
          }
          out0 = fmaf(s, a0, out0);
          out1 = fmaf(s, a1, out1);
          out2 = fmaf(s, a2, out2);
        }
    const float o[3] = {out0, out1, out2};
    float self[3];
    xh.get(lz + 1, ty + 1, tx + 1, self);
    mf_node_out<MODE>(a, I, o, self);
  }
}

// FP64 variant of the tiled operator (same tile, halo and cell order): y =
// A x (MODE 0) or y = b - A x (MODE 1) with FP64 values, scales and K_e^0.
// It gives the matrix-free CG operator's true residuals, whose accuracy the
// FP32 products inside CG lack; FP64-pipe bound (576 multiply-adds per
// node), so it runs only at the restarts.
struct KeF64 {
  double k[24 * 24];
};

template <int MODE>
__global__ void __launch_bounds__(kTX* kTY* kTZ) k_mf3_tile64(MfView m, const double* __restrict__ scale,
                                                              const double* __restrict__ x, double* __restrict__ y,
                                                              const double* __restrict__ b,
                                                              const __grid_constant__ KeF64 ke) {
  constexpr int NZ = kTZ * kNZ;
  __shared__ double xh[3][NZ + 2][kTY + 2][kTX + 2];
  __shared__ double sc[NZ + 1][kTY + 1][kTX + 1];
  const int tid = threadIdx.x;
  const i32 x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY, z0 = blockIdx.z * NZ;
  const i32 nnz = m.nz + 1;
  constexpr int kHalo = (NZ + 2) * (kTY + 2) * (kTX + 2);
  for (int e = tid; e < kHalo; e += kTX * kTY * kTZ) {
    const int hx = e % (kTX + 2), hy = (e / (kTX + 2)) % (kTY + 2), hz = e / ((kTX + 2) * (kTY + 2));
    const i32 gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = z0 - 1 + hz;
    i32 j = -1;
    if (gx >= 0 && gx < m.nnx && gy >= 0 && gy < m.nny && gz >= 0 && gz < nnz)
      j = m.nindex[(static_cast<i64>(gz) * m.nny + gy) * m.nnx + gx];
    double v0 = 0.0, v1 = 0.0, v2 = 0.0;
    if (j >= 0) {
      const double* p = x + static_cast<i64>(j) * 3;
      v0 = p[0];
      v1 = p[1];
      v2 = p[2];
    }
    xh[0][hz][hy][hx] = v0;
    xh[1][hz][hy][hx] = v1;
    xh[2][hz][hy][hx] = v2;
  }
  for (int e = tid; e < (NZ + 1) * (kTY + 1) * (kTX + 1); e += kTX * kTY * kTZ) {
    const int cx = e % (kTX + 1), cy = (e / (kTX + 1)) % (kTY + 1), cz = e / ((kTX + 1) * (kTY + 1));
    const i32 gx = x0 - 1 + cx, gy = y0 - 1 + cy, gz = z0 - 1 + cz;
    double s = 0.0;
    if (gx >= 0 && gx < m.nx && gy >= 0 && gy < m.ny && gz >= 0 && gz < m.nz)
      s = scale[(static_cast<i64>(gz) * m.ny + gy) * m.nx + gx];
    sc[cz][cy][cx] = s;
  }
  __syncthreads();
  const int tx = tid % kTX, ty = (tid / kTX) % kTY, tz = tid / (kTX * kTY);
  const i32 gx = x0 + tx, gy = y0 + ty, gz = z0 + tz;
  if (gx >= m.nnx || gy >= m.nny || gz >= nnz) return;
  const i32 I = m.nindex[(static_cast<i64>(gz) * m.nny + gy) * m.nnx + gx];
  if (I < 0) return;
  double out0 = 0.0, out1 = 0.0, out2 = 0.0;
#pragma unroll
  for (int dz = -1; dz <= 0; ++dz)
#pragma unroll
    for (int dy = -1; dy <= 0; ++dy)
#pragma unroll
      for (int dx = -1; dx <= 0; ++dx) {
        const double s = sc[tz + dz + 1][ty + dy + 1][tx + dx + 1];
        const int ox = -dx, oy = -dy, oz = -dz;
        const int aI = 4 * oz + (oy ? 3 - ox : ox);
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
#pragma unroll
        for (int bb = 0; bb < 8; ++bb) {
          const int bx = (bb == 1 || bb == 2 || bb == 5 || bb == 6) ? 1 : 0;
          const int by = (bb == 2 || bb == 3 || bb == 6 || bb == 7) ? 1 : 0;
          const int bz = bb >= 4 ? 1 : 0;
#pragma unroll
          for (int kb = 0; kb < 3; ++kb) {
            const double xv = xh[kb][tz + dz + 1 + bz][ty + dy + 1 + by][tx + dx + 1 + bx];
            a0 = fma(ke.k[(3 * aI + 0) * 24 + 3 * bb + kb], xv, a0);
            a1 = fma(ke.k[(3 * aI + 1) * 24 + 3 * bb + kb], xv, a1);
            a2 = fma(ke.k[(3 * aI + 2) * 24 + 3 * bb + kb], xv, a2);
          }
        }
        out0 = fma(s, a0, out0);
        out1 = fma(s, a1, out1);
        out2 = fma(s, a2, out2);
      }
  const double o[3] = {out0, out1, out2};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const i64 row = static_cast<i64>(I) * 3 + k;
    if (MODE == 0) y[row] = o[k];
    else y[row] = b[row] - o[k];
  }
}

// The tentative prolongator P^ of level 0 (3 unknowns per node, B1 per
// aggregate; aggregate g owns coarse unknowns g B1 .. g B1 + B1 - 1; the row
// of fine unknown i is phat[phat_ptr[i] ...], B1 values, empty for a node in
// no aggregate).  t = P^ x_c, one thread per fine unknown.
template <int B1>
__global__ void __launch_bounds__(256) k_phat_prolong(i32 n, const i32* __restrict__ agg,
                                                      const i32* __restrict__ phat_ptr,
                                                      const float* __restrict__ phat, const float* __restrict__ xc,
                                                      float* __restrict__ t) {
  const i32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const i32 g = agg[i / 3];
  float s = 0.0f;
  if (g >= 0) {
    const float* ph = phat + phat_ptr[i];
    const float* xg = xc + static_cast<i64>(g) * B1;
#pragma unroll
    for (int j = 0; j < B1; ++j) s = fmaf(ph[j], xg[j], s);
  }
  t[i] = s;
}

// b_c = P^T t: one warp per aggregate; lane q takes the aggregate's member
// unknowns q, q + 32, ... (members ascending, 3 unknowns each) into B1 partial
// sums, reduced across the warp in a fixed butterfly order.
template <int B1>
__global__ void __launch_bounds__(256) k_phat_restrict(i32 naggs, const i32* __restrict__ mptr,
                                                       const i32* __restrict__ members,
                                                       const i32* __restrict__ phat_ptr,
                                                       const float* __restrict__ phat, const float* __restrict__ t,
                                                       float* __restrict__ bc) {
  const i32 g = static_cast<i32>((blockIdx.x * static_cast<i64>(blockDim.x) + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (g >= naggs) return;
  const i32 q0 = mptr[g], cnt = 3 * (mptr[g + 1] - q0);
  float acc[B1];
#pragma unroll
  for (int j = 0; j < B1; ++j) acc[j] = 0.0f;
  for (i32 q = lane; q < cnt; q += 32) {
    const i32 i = 3 * members[q0 + q / 3] + q % 3;
    const float ti = t[i];
    const float* ph = phat + phat_ptr[i];
#pragma unroll
    for (int j = 0; j < B1; ++j) acc[j] = fmaf(ph[j], ti, acc[j]);
  }
#pragma unroll
  for (int j = 0; j < B1; ++j)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
  if (lane < B1) {
    float v = acc[0];
#pragma unroll
    for (int j = 1; j < B1; ++j)
      if (lane == j) v = acc[j];
    bc[static_cast<i64>(g) * B1 + lane] = v;
  }
}

}  // namespace
}  // namespace simp
