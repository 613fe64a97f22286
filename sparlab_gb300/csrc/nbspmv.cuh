// Sparse operator applications of the AMG levels (A_l, P_l, R_l).
//
// Every level operator is a scalar CSR whose rows of one node share their
// length and column list (grouped by whole column nodes), stored back to
// back.  VS consecutive lanes own one row: they stride across its contiguous
// values (VS = 8 FP32 lanes read one 32-byte sector per step), then reduce
// with a fixed log2(VS)-step butterfly, so every output is written once by
// lane 0 of its group and the result does not depend on timing.
//
// Where every column node has the same width B (B = 2 or 3 on a level 0 whose
// nodes are fully free or fully clamped, B = 6 (3-D) or 3 (2-D) on coarse
// levels of full-rank aggregates), the column of entry w of a row is
// B * nbr[slot w / B] + w % B: the column array is not read and the index
// traffic is one slot record per block.
#pragma once

#include "kernels.cuh"

namespace simp {
namespace {

constexpr int kUnroll = 4;  // row steps whose loads a lane issues before their products

// Column of entry w of a row: column-free decode (B > 0) or the column array.
template <int B>
__device__ __forceinline__ i32 row_col(i32 w, i32 s0, const i32* __restrict__ nbr, const i32* __restrict__ cl) {
  if constexpr (B > 0) {
    const i32 t = w / B;
    return B * nbr[s0 + t] + (w - B * t);
  } else {
    return cl[w];
  }
}

// This lane's partial sum of one row, entries w = lane, lane + VS, ... in
// ascending order; kUnroll steps' loads are issued before their products so
// each lane keeps several independent loads in flight.
template <int VS, int B, class TV, class TX, class TA>
__device__ __forceinline__ TA lane_dot(i32 len, int lane, i32 s0, const i32* __restrict__ nbr,
                                       const i32* __restrict__ cl, const TV* __restrict__ v,
                                       const TX* __restrict__ x) {
  TA s = TA(0);
  i32 w = lane;
  for (; w + (kUnroll - 1) * VS < len; w += kUnroll * VS) {
    TV vv[kUnroll];
    TX xx[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      vv[u] = v[w + u * VS];
      xx[u] = x[row_col<B>(w + u * VS, s0, nbr, cl)];
    }
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) s += static_cast<TA>(vv[u]) * static_cast<TA>(xx[u]);
  }
  for (; w < len; w += VS) s += static_cast<TA>(v[w]) * static_cast<TA>(x[row_col<B>(w, s0, nbr, cl)]);
  return s;
}

// mode 0: y = A x ; 1: y = b - A x ; 2: y += A x.  TA is the arithmetic
// type (FP64 rows get VS = 4: GB300's FP64 rate is 1/64 of FP32, and a short
// reduction keeps the FP64 pipe on the products).
template <int VS, int B, int MODE, class TV, class TX, class TA>
__global__ void __launch_bounds__(256) k_rows_apply(const i32* __restrict__ node_of, NodeView pat,
                                                    const i32* __restrict__ rowptr, const i32* __restrict__ col,
                                                    const TV* __restrict__ val, const TX* __restrict__ x,
                                                    TX* __restrict__ y, const TX* __restrict__ b, i32 rows) {
  const i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 row = static_cast<i32>(t / VS);
  const int lane = static_cast<int>(t % VS);
  TA s = TA(0);
  if (row < rows) {
    const i32 k0 = rowptr[row], len = rowptr[row + 1] - k0;
    const i32 s0 = B > 0 ? pat.ptr[node_of[row]] : 0;
    s = lane_dot<VS, B, TV, TX, TA>(len, lane, s0, pat.nbr, col + k0, val + k0, x);
  }
#pragma unroll
  for (int o = VS / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, VS);
  if (row < rows && lane == 0) {
    if (MODE == 0) y[row] = static_cast<TX>(s);
    else if (MODE == 1) y[row] = b[row] - static_cast<TX>(s);
    else y[row] += static_cast<TX>(s);
  }
}

template <int VS, int B, class TV, class TX>
__device__ __forceinline__ TX rows_dot(i32 row, int lane, bool valid, const i32* __restrict__ node_of, NodeView pat,
                                       const i32* __restrict__ rowptr, const i32* __restrict__ col,
                                       const TV* __restrict__ val, const TX* __restrict__ x) {
  TX s = TX(0);
  if (valid) {
    const i32 k0 = rowptr[row], len = rowptr[row + 1] - k0;
    const i32 s0 = B > 0 ? pat.ptr[node_of[row]] : 0;
    s = lane_dot<VS, B, TV, TX, TX>(len, lane, s0, pat.nbr, col + k0, val + k0, x);
  }
#pragma unroll
  for (int o = VS / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, VS);
  return s;
}

// Chebyshev step: r = r_in - A d ; dn = c1 d + c2 dinv r ; x = (x [+ d]) + dn,
// (c1, c2) = c12[0..1] in device memory (the level's coefficients change with
// every setup; a captured launch keeps reading them)
template <int VS, int B, class T>
__global__ void __launch_bounds__(256) k_rows_cheb_step(i32 rows, const i32* __restrict__ node_of, NodeView pat,
                                                        const i32* __restrict__ rowptr, const i32* __restrict__ col,
                                                        const T* __restrict__ val, const T* __restrict__ d,
                                                        const T* __restrict__ r_in, T* __restrict__ r,
                                                        T* __restrict__ dn, T* __restrict__ x,
                                                        const T* __restrict__ dinv, const T* __restrict__ c12,
                                                        int add_d) {
  const i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 row = static_cast<i32>(t / VS);
  const int lane = static_cast<int>(t % VS);
  const bool valid = row < rows;
  const T s = rows_dot<VS, B, T, T>(row, lane, valid, node_of, pat, rowptr, col, val, d);
  if (valid && lane == 0) {
    const T ri = r_in[row] - s;
    r[row] = ri;
    const T di = c12[0] * d[row] + c12[1] * dinv[row] * ri;
    dn[row] = di;
    T xi = x[row];
    if (add_d) xi = xi + d[row];
    x[row] = xi + di;
  }
}

// r = b - A x ; d = dinv r / theta (1 / theta = *inv_theta, device memory)
template <int VS, int B, class T>
__global__ void __launch_bounds__(256) k_rows_cheb_first(i32 rows, const i32* __restrict__ node_of, NodeView pat,
                                                         const i32* __restrict__ rowptr, const i32* __restrict__ col,
                                                         const T* __restrict__ val, const T* __restrict__ x,
                                                         const T* __restrict__ b, T* __restrict__ r,
                                                         T* __restrict__ d, const T* __restrict__ dinv,
                                                         const T* __restrict__ inv_theta) {
  const i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 row = static_cast<i32>(t / VS);
  const int lane = static_cast<int>(t % VS);
  const bool valid = row < rows;
  const T s = rows_dot<VS, B, T, T>(row, lane, valid, node_of, pat, rowptr, col, val, x);
  if (valid && lane == 0) {
    const T ri = b[row] - s;
    r[row] = ri;
    d[row] = dinv[row] * ri * *inv_theta;
  }
}

// Double-float operator (mixed precision's CG operator): values stored as
// hi + lo float pairs, x as (hi, lo) pairs, products and sums in
// double-float arithmetic on the FP32 pipes, y in FP64.  About 2^-44 relative
// to the FP64 product, at FP32 instruction rates: bandwidth bound where the
// FP64 kernel is bound by GB300's FP64 rate.  mode 0: y = A x ; 1: y = b - A x.
// UNROLL: row steps whose loads a lane issues before their products (the
// products run in the same order for every UNROLL, so all give the same
// bits; the launch-shape tuner picks one).
template <int VS, int B, int MODE, int UNROLL = kUnroll>
__global__ void __launch_bounds__(256) k_rows_apply_df(const i32* __restrict__ node_of, NodeView pat,
                                                       const i32* __restrict__ rowptr, const i32* __restrict__ col,
                                                       const float2* __restrict__ v, const float2* __restrict__ x,
                                                       double* __restrict__ y,
                                                       const double* __restrict__ b, i32 rows) {
  const i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 row = static_cast<i32>(t / VS);
  const int lane = static_cast<int>(t % VS);
  float sh = 0.0f, sl = 0.0f;
  if (row < rows) {
    const i32 k0 = rowptr[row], len = rowptr[row + 1] - k0;
    const float2* vp = v + k0;  // (hi, lo) pairs: one 8-byte load per value
    const i32* cl = col + k0;
    const i32 s0 = B > 0 ? pat.ptr[node_of[row]] : 0;
    i32 w = lane;
    for (; w + (UNROLL - 1) * VS < len; w += UNROLL * VS) {
      float2 hv[UNROLL];
      float2 xv[UNROLL];
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        hv[u] = vp[w + u * VS];
        xv[u] = x[row_col<B>(w + u * VS, s0, pat.nbr, cl)];
      }
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) df_fma(hv[u].x, hv[u].y, xv[u].x, xv[u].y, sh, sl);
    }
    for (; w < len; w += VS) {
      const float2 xv = x[row_col<B>(w, s0, pat.nbr, cl)];
      const float2 hv = vp[w];
      df_fma(hv.x, hv.y, xv.x, xv.y, sh, sl);
    }
  }
#pragma unroll
  for (int o = VS / 2; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, sh, o, VS);
    const float ol = __shfl_xor_sync(0xffffffffu, sl, o, VS);
    float s, e;
    two_sum(sh, oh, s, e);
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(ol, e));
  }
  if (row < rows && lane == 0) {
    const double v = static_cast<double>(sh) + static_cast<double>(sl);
    if (MODE == 0) y[row] = v;
    else y[row] = b[row] - v;
  }
}

// y_k = A x_k for up to kMaxRhs right-hand sides of one double-float
// operator (the load cases of one problem): each (hi, lo) value pair of A is
// loaded once per row step for all of them, so A's bytes are read once for
// the k vectors.  A vector takes part while its flag *active[k] is nonzero
// (a solve that has stopped is skipped; null: always).  Every y_k is summed
// in exactly the lanes, steps and butterfly of k_rows_apply_df, so it equals
// that kernel's product bit for bit.
constexpr int kMaxRhs = 4;
struct MultiRhs {
  const float2* x[kMaxRhs];
  double* y[kMaxRhs];
  const int* active[kMaxRhs];
  int n;
};

template <int VS, int B>
__global__ void __launch_bounds__(256) k_rows_apply_df_multi(const i32* __restrict__ node_of, NodeView pat,
                                                             const i32* __restrict__ rowptr,
                                                             const i32* __restrict__ col,
                                                             const float2* __restrict__ v,
                                                             const __grid_constant__ MultiRhs m, i32 rows) {
  const i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 row = static_cast<i32>(t / VS);
  const int lane = static_cast<int>(t % VS);
  bool on[kMaxRhs];
  float sh[kMaxRhs], sl[kMaxRhs];
#pragma unroll
  for (int k = 0; k < kMaxRhs; ++k) {
    on[k] = k < m.n && (m.active[k] == nullptr || *m.active[k] != 0);
    sh[k] = sl[k] = 0.0f;
  }
  if (row < rows) {
    const i32 k0 = rowptr[row], len = rowptr[row + 1] - k0;
    const float2* vp = v + k0;
    const i32* cl = col + k0;
    const i32 s0 = B > 0 ? pat.ptr[node_of[row]] : 0;
    i32 w = lane;
    for (; w + (kUnroll - 1) * VS < len; w += kUnroll * VS) {
      float2 hv[kUnroll];
      i32 cw[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        hv[u] = vp[w + u * VS];
        cw[u] = row_col<B>(w + u * VS, s0, pat.nbr, cl);
      }
#pragma unroll
      for (int k = 0; k < kMaxRhs; ++k) {
        if (!on[k]) continue;
        float2 xv[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) xv[u] = m.x[k][cw[u]];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) df_fma(hv[u].x, hv[u].y, xv[u].x, xv[u].y, sh[k], sl[k]);
      }
    }
    for (; w < len; w += VS) {
      const float2 hv = vp[w];
      const i32 cw = row_col<B>(w, s0, pat.nbr, cl);
#pragma unroll
      for (int k = 0; k < kMaxRhs; ++k) {
        if (!on[k]) continue;
        const float2 xv = m.x[k][cw];
        df_fma(hv.x, hv.y, xv.x, xv.y, sh[k], sl[k]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kMaxRhs; ++k) {
    if (!on[k]) continue;  // the same for every thread
#pragma unroll
    for (int o = VS / 2; o > 0; o >>= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, sh[k], o, VS);
      const float ol = __shfl_xor_sync(0xffffffffu, sl[k], o, VS);
      float s, e;
      two_sum(sh[k], oh, s, e);
      sh[k] = s;
      sl[k] = __fadd_rn(sl[k], __fadd_rn(ol, e));
    }
    if (row < rows && lane == 0) m.y[k][row] = static_cast<double>(sh[k]) + static_cast<double>(sl[k]);
  }
}

}  // namespace
}  // namespace simp
