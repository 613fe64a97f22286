// Coarsest-level direct solve in FP64 (src/fem/Multigrid.cpp:749-781, 859-865).
// The reference factors the dense coarse operator (LDL^T) and runs two
// triangular sweeps per V-cycle.  Here the SPD coarse operator is inverted
// once per setup by a blocked symmetric sweep (Gauss-Jordan elimination
// without pivoting, which is stable for SPD matrices because every pivot is a
// Schur complement's diagonal), and a V-cycle's coarse solve is one GEMV.
//
// Sweeping pivot block k of a symmetric M (P = M_kk^-1, U = M_{:,k}, V = U P):
//   M_ij <- M_ij - V_i U_j^T   (i, j outside k)
//   M_ik <- V_i,  M_kj <- V_j^T,  M_kk <- -P
// After all blocks M = -A^-1.  Only the lower triangle is stored and updated
// (GB300's FP64 rate makes the halved update worth the bookkeeping).  The
// scalar pivots met inside the pivot blocks are the squared Cholesky pivots
// (the D of A = L D L^T), recorded for the singularity check.
// Row-major n x n storage.
//
// The same sweep inverts the indefinite shifted pencil K - sigma G of the
// buckling spectral transformation (SIGNED pivots: any nonzero finite pivot
// is taken).  Its pivots are then the D of A = L D L^T in the natural order,
// so by Sylvester's law of inertia the count of negative pivots is the count
// of negative eigenvalues whenever no leading minor vanishes -- the number
// src/fem/Buckling.cpp:190-201 reads off its sparse LDL^T.
#pragma once

#include "common.h"

namespace simp {
namespace {

constexpr int kNB = 32;        // pivot block width = update tile width
constexpr int kSweepRows = 16;  // rows of U and V per block of k_sweep_pivot

// One launch per pivot block k0 (width kb <= kNB).  Every block sweeps the
// pivot block S = M[k0:k0+kb, k0:k0+kb] in shared memory into -S^-1 (the same
// few dozen microseconds of FP64 latency in every block, in parallel, so the
// panel needs no second launch), then writes U_i = M[i, k0:k0+kb] and
// V_i = U_i S^-1 for its rows i outside the block.  Block 0 records the
// pivots, the status (1 on a pivot that is not positive and finite; SIGNED:
// zero or not finite) and P.
template <bool SIGNED = false>
__global__ void __launch_bounds__(256) k_sweep_pivot(const double* __restrict__ m, int n, int k0, int kb,
                                                     double* __restrict__ u, double* __restrict__ v,
                                                     double* __restrict__ pout, double* __restrict__ piv,
                                                     int* __restrict__ status) {
  __shared__ double s[kNB][kNB + 1];
  __shared__ double urow[kNB], trow[kNB];
  __shared__ double pj;
  __shared__ double ush[8][kNB];
  const int tid = threadIdx.x;
  for (int e = tid; e < kNB * kNB; e += blockDim.x) {
    const int r = e / kNB, c = e % kNB;
    double val = r == c ? 1.0 : 0.0;
    if (r < kb && c < kb) val = m[(size_t)(k0 + max(r, c)) * n + k0 + min(r, c)];
    s[r][c] = val;
  }
  __syncthreads();
  for (int j = 0; j < kb; ++j) {
    if (tid < kNB) {
      const double d = s[j][j];
      const bool ok = (SIGNED ? d != 0.0 : d > 0.0) && isfinite(d);
      const double p = ok ? 1.0 / d : 1.0;
      const double uc = s[j][tid];
      urow[tid] = uc;
      trow[tid] = p * uc;
      if (tid == 0) {
        pj = p;
        if (blockIdx.x == 0) {
          piv[k0 + j] = d;
          if (!ok) *status = 1;
        }
      }
    }
    __syncthreads();
    for (int e = tid; e < kNB * kNB; e += blockDim.x) {
      const int r = e / kNB, c = e % kNB;
      if (r >= kb || c >= kb) continue;
      if (r != j && c != j) s[r][c] = fma(-urow[r], trow[c], s[r][c]);
      else if (r != j) s[r][j] = trow[r];
      else if (c != j) s[j][c] = trow[c];
      else s[j][j] = -pj;
    }
    __syncthreads();
  }
  // s = -S^-1
  if (blockIdx.x == 0)
    for (int e = tid; e < kb * kb; e += blockDim.x) pout[(e / kb) * kNB + e % kb] = -s[e / kb][e % kb];
  const int warp = tid >> 5, lane = tid & 31;
  const int i_end = min(n, (blockIdx.x + 1) * kSweepRows);
  for (int i = blockIdx.x * kSweepRows + warp; i < i_end; i += 8) {
    if (i >= k0 && i < k0 + kb) continue;
    double ui = 0.0;
    if (lane < kb) ui = i >= k0 + kb ? m[(size_t)i * n + k0 + lane] : m[(size_t)(k0 + lane) * n + i];
    ush[warp][lane] = ui;
    __syncwarp();
    double acc = 0.0;
    for (int d = 0; d < kb; ++d) acc = fma(ush[warp][d], s[d][lane], acc);
    if (lane < kb) {
      u[(size_t)i * kNB + lane] = ui;
      v[(size_t)i * kNB + lane] = -acc;
    }
    __syncwarp();
  }
}

// The update of pivot block k0 over the lower triangle, one 32 x 32 tile
// (I, J), J <= I, per block: a grid of nt x nt blocks, those above the
// diagonal return at once.  Reads only U, V, P and its own tile.
__global__ void __launch_bounds__(256) k_sweep_update(double* __restrict__ m, int n, int k0, int kb,
                                                      const double* __restrict__ u,
                                                      const double* __restrict__ v,
                                                      const double* __restrict__ p) {
  const int ti = blockIdx.y, tj = blockIdx.x;
  if (tj > ti) return;
  const int kt = k0 / kNB;
  const int r0 = ti * kNB, c0 = tj * kNB;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  __shared__ double vs[kNB][kNB + 1];
  __shared__ double us[kNB][kNB + 1];
  if (ti == kt && tj == kt) {
    for (int q = ty; q < kNB; q += 8)
      if (q < kb && tx < kb) m[(size_t)(k0 + q) * n + k0 + tx] = -p[q * kNB + tx];
    return;
  }
  if (ti == kt) {  // M_kj <- V_j^T for the columns j of tile J
    for (int q = ty; q < kNB; q += 8) {
      const int j = c0 + q;
      vs[q][tx] = (j < n && tx < kb) ? v[(size_t)j * kNB + tx] : 0.0;
    }
    __syncthreads();
    for (int q = ty; q < kb; q += 8)
      if (c0 + tx < n) m[(size_t)(k0 + q) * n + c0 + tx] = vs[tx][q];
    return;
  }
  if (tj == kt) {  // M_ik <- V_i for the rows i of tile I
    for (int q = ty; q < kNB; q += 8) {
      const int i = r0 + q;
      if (i < n && tx < kb) m[(size_t)i * n + k0 + tx] = v[(size_t)i * kNB + tx];
    }
    return;
  }
  for (int q = ty; q < kNB; q += 8) {
    const int i = r0 + q, j = c0 + q;
    vs[q][tx] = (i < n && tx < kb) ? v[(size_t)i * kNB + tx] : 0.0;
    us[q][tx] = (j < n && tx < kb) ? u[(size_t)j * kNB + tx] : 0.0;
  }
  __syncthreads();
  const int j = c0 + tx;
  if (j >= n) return;
#pragma unroll
  for (int qq = 0; qq < kNB / 8; ++qq) {
    const int q = ty + 8 * qq;
    const int i = r0 + q;
    if (i >= n || j > i) continue;
    double acc = 0.0;
#pragma unroll
    for (int d = 0; d < kNB; ++d) acc = fma(vs[q][d], us[tx][d], acc);
    m[(size_t)i * n + j] -= acc;
  }
}

// F = -M mirrored from the lower triangle to full storage: one 32 x 32 tile
// (I, J), J <= I, per block, written to (I, J) and (J, I).
__global__ void __launch_bounds__(256) k_sweep_finish(const double* __restrict__ m, double* __restrict__ f,
                                                      int n) {
  const int ti = blockIdx.y, tj = blockIdx.x;
  if (tj > ti) return;
  const int r0 = ti * kNB, c0 = tj * kNB;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  __shared__ double t[kNB][kNB + 1];
  for (int q = ty; q < kNB; q += 8) {
    const int i = r0 + q, j = c0 + tx;
    t[q][tx] = (i < n && j < n && (ti != tj || j <= i)) ? -m[(size_t)i * n + j] : 0.0;
  }
  __syncthreads();
  for (int q = ty; q < kNB; q += 8) {
    const int i = r0 + q, j = c0 + tx;
    if (i < n && j < n) f[(size_t)i * n + j] = ti != tj || tx <= q ? t[q][tx] : t[tx][q];
    if (ti != tj) {
      const int i2 = c0 + q, j2 = r0 + tx;
      if (i2 < n && j2 < n) f[(size_t)i2 * n + j2] = t[tx][q];
    }
  }
}

// y = M x for row-major M, one warp per row.
template <class TX, class TY>
__global__ void __launch_bounds__(256) k_gemv(const double* __restrict__ m, int n, const TX* __restrict__ x,
                                              TY* __restrict__ y) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const double* row = m + (size_t)warp * n;
  double s = 0.0;
  for (int c = lane; c < n; c += 32) s += row[c] * static_cast<double>(x[c]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[warp] = static_cast<TY>(s);
}

__global__ void k_dense_from_csr(int n, const i32* __restrict__ ptr, const i32* __restrict__ col,
                                 const double* __restrict__ val, double* __restrict__ a) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    for (i32 k = ptr[r]; k < ptr[r + 1]; ++k) a[(size_t)r * n + col[k]] = val[k];
}

// a = K - s G densely, K and G on the same CSR pattern (a zeroed before).
__global__ void k_dense_shifted(int n, const i32* __restrict__ ptr, const i32* __restrict__ col,
                                const double* __restrict__ kval, const double* __restrict__ gval, double s,
                                double* __restrict__ a) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    for (i32 k = ptr[r]; k < ptr[r + 1]; ++k) a[(size_t)r * n + col[k]] = kval[k] - s * gval[k];
}

// Z = F Y for a row-major n x n F and column-major n x q Y, Z: one 32 x 32
// tile (rows i0.., columns c0..) per block of 256 threads, the inner index
// staged 32 at a time; every output sums its terms in ascending inner order.
__global__ void __launch_bounds__(256) k_dense_gemm_cols(const double* __restrict__ f, int n, int q,
                                                         const double* __restrict__ y, double* __restrict__ z) {
  __shared__ double fs[kNB][kNB + 1];  // fs[i][k] = F[i0 + i][k0 + k]
  __shared__ double ys[kNB][kNB + 1];  // ys[c][k] = Y[k0 + k][c0 + c]
  const int i0 = blockIdx.x * kNB, c0 = blockIdx.y * kNB;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  double acc[kNB / 8] = {};
  for (int k0 = 0; k0 < n; k0 += kNB) {
    for (int q2 = ty; q2 < kNB; q2 += 8) {
      const int i = i0 + q2, k = k0 + tx, c = c0 + q2;
      fs[q2][tx] = (i < n && k < n) ? f[(size_t)i * n + k] : 0.0;
      ys[q2][tx] = (c < q && k < n) ? y[(size_t)c * n + k] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int qq = 0; qq < kNB / 8; ++qq) {
      const int c = ty + 8 * qq;
      double a = acc[qq];
#pragma unroll 8
      for (int k = 0; k < kNB; ++k) a = fma(fs[tx][k], ys[c][k], a);
      acc[qq] = a;
    }
    __syncthreads();
  }
#pragma unroll
  for (int qq = 0; qq < kNB / 8; ++qq) {
    const int i = i0 + tx, c = c0 + ty + 8 * qq;
    if (i < n && c < q) z[(size_t)c * n + i] = acc[qq];
  }
}

}  // namespace
}  // namespace simp
