// Coarsest-level direct solve in FP64 (src/fem/Multigrid.cpp:749-781, 859-865):
// blocked right-looking Cholesky A = L L^T, the explicit inverse factor
// W = L^-1, and the per-cycle solve x = W^T (W b) as two GEMVs, so a V-cycle
// spends a few microseconds at the coarsest level instead of a sequential
// triangular sweep.  Row-major n x n storage, lower triangle referenced.
#pragma once

#include "common.h"

namespace simp {
namespace {

constexpr int kNB = 32;  // panel width

// Unblocked Cholesky of the kb x kb diagonal block at (k0, k0).  piv[k0 + j]
// receives the pivot before its square root; status = 1 on a pivot that is
// not positive and finite.
__global__ void __launch_bounds__(256) k_potrf_diag(double* __restrict__ a, int n, int k0, int kb,
                                                    double* __restrict__ piv, int* __restrict__ status) {
  __shared__ double s[kNB][kNB + 1];
  for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
    const int i = e / kb, j = e % kb;
    s[i][j] = a[(size_t)(k0 + i) * n + k0 + j];
  }
  __syncthreads();
  for (int j = 0; j < kb; ++j) {
    __shared__ double djj;
    if (threadIdx.x == 0) {
      const double d = s[j][j];
      piv[k0 + j] = d;
      if (!(d > 0.0) || !isfinite(d)) {
        *status = 1;
        djj = 1.0;
      } else {
        djj = sqrt(d);
      }
      s[j][j] = djj;
    }
    __syncthreads();
    for (int i = j + 1 + threadIdx.x; i < kb; i += blockDim.x) s[i][j] /= djj;
    __syncthreads();
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
      const int i = e / kb, c = e % kb;
      if (c > j && i >= c) s[i][c] -= s[i][j] * s[c][j];
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
    const int i = e / kb, j = e % kb;
    if (j <= i) a[(size_t)(k0 + i) * n + k0 + j] = s[i][j];
  }
}

// Panel below the diagonal block: L21 = A21 L11^-T, one thread per row.
__global__ void __launch_bounds__(128) k_trsm_panel(double* __restrict__ a, int n, int k0, int kb) {
  __shared__ double l[kNB][kNB + 1];
  for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
    const int i = e / kb, j = e % kb;
    l[i][j] = j <= i ? a[(size_t)(k0 + i) * n + k0 + j] : 0.0;
  }
  __syncthreads();
  const int r = k0 + kb + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double x[kNB];
  double* row = a + (size_t)r * n + k0;
#pragma unroll
  for (int j = 0; j < kNB; ++j) x[j] = j < kb ? row[j] : 0.0;
#pragma unroll
  for (int j = 0; j < kNB; ++j) {
    if (j < kb) {
      double v = x[j];
#pragma unroll
      for (int c = 0; c < kNB; ++c)
        if (c < j) v -= x[c] * l[j][c];
      x[j] = v / l[j][j];
    }
  }
#pragma unroll
  for (int j = 0; j < kNB; ++j)
    if (j < kb) row[j] = x[j];
}

// C[r][c] -= sum_j A[r][j] * B(j, c) over 32 x 32 output tiles, with
// A(r, j) = a[r * n + ka + j] and B(j, c) = b[j * ldbj + c * ldbc].
// lower != 0 skips tiles strictly above the diagonal (and entries c > r).
__global__ void __launch_bounds__(256) k_tile_update(double* __restrict__ cmat, int n, int r0, int c0,
                                                     int rows, int cols, const double* __restrict__ amat,
                                                     int ka, const double* __restrict__ bmat, long ldbj,
                                                     long ldbc, int kb, int lower) {
  const int tr = blockIdx.y * 32, tc = blockIdx.x * 32;
  if (tr >= rows || tc >= cols) return;
  if (lower && r0 + tr + 31 < c0 + tc) return;
  __shared__ double as[32][kNB + 1];
  __shared__ double bs[kNB][33];
  for (int e = threadIdx.x; e < 32 * kNB; e += 256) {
    const int i = e / kNB, j = e % kNB;
    const int r = tr + i;
    as[i][j] = (r < rows && j < kb) ? amat[(size_t)(r0 + r) * n + ka + j] : 0.0;
    const int jj = e / 32, c = e % 32;
    bs[jj][c] = (tc + c < cols && jj < kb) ? bmat[(long)jj * ldbj + (long)(c0 + tc + c) * ldbc] : 0.0;
  }
  __syncthreads();
  const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;  // 8 rows of threads x 4 outputs
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = ty + 8 * q;
    const int r = tr + i, c = tc + tx;
    if (r >= rows || c >= cols) continue;
    if (lower && r0 + r < c0 + c) continue;
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < kNB; ++j) s += as[i][j] * bs[j][tx];
    cmat[(size_t)(r0 + r) * n + c0 + c] -= s;
  }
}

// Rows [k0, k0+kb) of W = L^-1: forward substitution of the updated right-hand
// sides with L11, one thread per column c < k0 + kb.
__global__ void __launch_bounds__(128) k_trsm_rows(double* __restrict__ w, const double* __restrict__ l,
                                                   int n, int k0, int kb) {
  __shared__ double lk[kNB][kNB + 1];
  for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
    const int i = e / kb, j = e % kb;
    lk[i][j] = j <= i ? l[(size_t)(k0 + i) * n + k0 + j] : 0.0;
  }
  __syncthreads();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k0 + kb) return;
  double x[kNB];
#pragma unroll
  for (int j = 0; j < kNB; ++j) x[j] = j < kb ? w[(size_t)(k0 + j) * n + c] : 0.0;
#pragma unroll
  for (int j = 0; j < kNB; ++j) {
    if (j < kb) {
      double v = x[j];
#pragma unroll
      for (int i = 0; i < kNB; ++i)
        if (i < j) v -= lk[j][i] * x[i];
      x[j] = v / lk[j][j];
    }
  }
#pragma unroll
  for (int j = 0; j < kNB; ++j)
    if (j < kb) w[(size_t)(k0 + j) * n + c] = x[j];
}

// y = M x for row-major M: one warp per row; `upper` restricts to c >= r,
// `lower_only` to c <= r.
template <class TX, class TY>
__global__ void __launch_bounds__(256) k_gemv(const double* __restrict__ m, int n, const TX* __restrict__ x,
                                              TY* __restrict__ y, int tri) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const int lo = tri == 2 ? warp : 0;         // 2: upper triangle (c >= r)
  const int hi = tri == 1 ? warp + 1 : n;     // 1: lower triangle (c <= r)
  const double* row = m + (size_t)warp * n;
  double s = 0.0;
  for (int c = lo + lane; c < hi; c += 32) s += row[c] * static_cast<double>(x[c]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[warp] = static_cast<TY>(s);
}

__global__ void k_dense_from_csr(int n, const i32* __restrict__ ptr, const i32* __restrict__ col,
                                 const double* __restrict__ val, double* __restrict__ a) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    for (i32 k = ptr[r]; k < ptr[r + 1]; ++k) a[(size_t)r * n + col[k]] = val[k];
}

__global__ void k_identity(double* __restrict__ a, int n) {
  const size_t total = (size_t)n * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
    a[e] = (e / n == e % n) ? 1.0 : 0.0;
}

__global__ void k_transpose(const double* __restrict__ a, double* __restrict__ t, int n) {
  __shared__ double tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = by + j, c = bx + threadIdx.x;
    tile[j][threadIdx.x] = (r < n && c < n) ? a[(size_t)r * n + c] : 0.0;
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = bx + j, c = by + threadIdx.x;
    if (r < n && c < n) t[(size_t)r * n + c] = tile[threadIdx.x][j];
  }
}

}  // namespace
}  // namespace simp
