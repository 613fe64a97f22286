// Node-chunked sparse operator applications.
//
// Every level operator (A_l, P_l, R_l) is a scalar CSR whose rows of one
// node share their length and column list, and are stored back to back.  One
// warp owns one row node: for each of its (<= 6) rows the lanes stride across
// the row's contiguous values (coalesced loads), then the row sums are
// reduced with a fixed butterfly and lane r writes row r, so every output is
// written once and the result does not depend on timing.
//
// Level 0 of a grid whose nodes are all fully free or fully clamped has
// uniform B x B blocks (B = 2 or 3); there the column of entry w of a row is
// B * nbr[slot w / B] + w % B, so the column array is not read at all and the
// index traffic is one slot record per block.
#pragma once

#include "kernels.cuh"

namespace simp {
namespace {

constexpr int kMaxNode = 6;  // unknowns per node: 2-3 on level 0, rank <= 6 below

// Row sums of one row node; returns with acc[r] (r < nr) summed over the warp
// in every lane.  B > 0: uniform-block level 0 without the column array.
template <int B, class TV, class TX, class TA>
__device__ __forceinline__ void chunk_row_dots(i32 I, int lane, bool valid, const i32* __restrict__ row_first,
                                               NodeView pat, const i32* __restrict__ rowptr,
                                               const i32* __restrict__ col, const TV* __restrict__ val,
                                               const TX* __restrict__ x, int& nr, i32& r0, TA (&acc)[kMaxNode]) {
#pragma unroll
  for (int r = 0; r < kMaxNode; ++r) acc[r] = TA(0);
  nr = 0;
  r0 = 0;
  if (valid) {
    r0 = row_first[I];
    nr = row_first[I + 1] - r0;
    const i32 base = rowptr[r0];
    const i32 len = nr > 0 ? rowptr[r0 + 1] - base : 0;
    const i32 s0 = pat.ptr[I];
#pragma unroll
    for (int r = 0; r < kMaxNode; ++r) {
      if (r < nr) {
        const TV* v = val + base + r * len;
        TA s = TA(0);
        if constexpr (B > 0) {
          for (i32 w = lane; w < len; w += 32) {
            const i32 t = w / B;
            const i32 c = B * pat.nbr[s0 + t] + (w - B * t);
            s += static_cast<TA>(v[w]) * static_cast<TA>(x[c]);
          }
        } else {
          const i32* cl = col + base + r * len;
          for (i32 w = lane; w < len; w += 32) s += static_cast<TA>(v[w]) * static_cast<TA>(x[cl[w]]);
        }
        acc[r] = s;
      }
    }
  }
#pragma unroll
  for (int r = 0; r < kMaxNode; ++r) {
    if (r < nr) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
    }
  }
}

// mode 0: y = A x ; 1: y = b - A x ; 2: y += A x
template <int B, int MODE, class TV, class TX, class TA>
__global__ void __launch_bounds__(256) k_chunk_apply(i32 nodes, const i32* __restrict__ row_first, NodeView pat,
                                                     const i32* __restrict__ rowptr, const i32* __restrict__ col,
                                                     const TV* __restrict__ val, const TX* __restrict__ x,
                                                     TX* __restrict__ y, const TX* __restrict__ b) {
  const i32 I = static_cast<i32>((blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (I >= nodes) return;  // whole warps leave together
  TA acc[kMaxNode];
  int nr;
  i32 r0;
  chunk_row_dots<B, TV, TX, TA>(I, lane, true, row_first, pat, rowptr, col, val, x, nr, r0, acc);
#pragma unroll
  for (int r = 0; r < kMaxNode; ++r) {
    if (r < nr && lane == r) {
      const i32 row = r0 + r;
      if (MODE == 0) y[row] = static_cast<TX>(acc[r]);
      else if (MODE == 1) y[row] = b[row] - static_cast<TX>(acc[r]);
      else y[row] += static_cast<TX>(acc[r]);
    }
  }
}

// Chebyshev step: r = r_in - A d ; dn = c1 d + c2 dinv r ; x = (x [+ d]) + dn
template <int B, class T>
__global__ void __launch_bounds__(256) k_chunk_cheb_step(i32 nodes, const i32* __restrict__ first, NodeView pat,
                                                         const i32* __restrict__ rowptr, const i32* __restrict__ col,
                                                         const T* __restrict__ val, const T* __restrict__ d,
                                                         const T* __restrict__ r_in, T* __restrict__ r,
                                                         T* __restrict__ dn, T* __restrict__ x,
                                                         const T* __restrict__ dinv, T c1, T c2, int add_d) {
  const i32 I = static_cast<i32>((blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (I >= nodes) return;
  T acc[kMaxNode];
  int nr;
  i32 r0;
  chunk_row_dots<B, T, T, T>(I, lane, true, first, pat, rowptr, col, val, d, nr, r0, acc);
#pragma unroll
  for (int q = 0; q < kMaxNode; ++q) {
    if (q < nr && lane == q) {
      const i32 row = r0 + q;
      const T ri = r_in[row] - acc[q];
      r[row] = ri;
      const T di = c1 * d[row] + c2 * dinv[row] * ri;
      dn[row] = di;
      T xi = x[row];
      if (add_d) xi = xi + d[row];
      x[row] = xi + di;
    }
  }
}

// r = b - A x ; d = dinv r / theta
template <int B, class T>
__global__ void __launch_bounds__(256) k_chunk_cheb_first(i32 nodes, const i32* __restrict__ first, NodeView pat,
                                                          const i32* __restrict__ rowptr, const i32* __restrict__ col,
                                                          const T* __restrict__ val, const T* __restrict__ x,
                                                          const T* __restrict__ b, T* __restrict__ r,
                                                          T* __restrict__ d, const T* __restrict__ dinv,
                                                          T inv_theta) {
  const i32 I = static_cast<i32>((blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (I >= nodes) return;
  T acc[kMaxNode];
  int nr;
  i32 r0;
  chunk_row_dots<B, T, T, T>(I, lane, true, first, pat, rowptr, col, val, x, nr, r0, acc);
#pragma unroll
  for (int q = 0; q < kMaxNode; ++q) {
    if (q < nr && lane == q) {
      const i32 row = r0 + q;
      const T ri = b[row] - acc[q];
      r[row] = ri;
      d[row] = dinv[row] * ri * inv_theta;
    }
  }
}

// VS lanes per scalar row (VS = 4 or 8), for operators whose arithmetic is
// the bottleneck (FP64 on GB300 runs at 1/64 of the FP32 rate): a VS-lane
// reduction costs log2(VS) adds per row instead of five.  Lanes of a row
// read consecutive values (32-byte sectors fully used).
template <int VS, int B, int MODE, class TV, class TX, class TA>
__global__ void __launch_bounds__(256) k_rows_apply(i32 nodes, const i32* __restrict__ row_first,
                                                    const i32* __restrict__ node_of, NodeView pat,
                                                    const i32* __restrict__ rowptr, const i32* __restrict__ col,
                                                    const TV* __restrict__ val, const TX* __restrict__ x,
                                                    TX* __restrict__ y, const TX* __restrict__ b, i32 rows) {
  const i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 row = static_cast<i32>(t / VS);
  const int lane = static_cast<int>(t % VS);
  TA s = TA(0);
  if (row < rows) {
    const i32 k0 = rowptr[row], len = rowptr[row + 1] - k0;
    const TV* v = val + k0;
    if constexpr (B > 0) {
      const i32 s0 = pat.ptr[node_of[row]];
      for (i32 w = lane; w < len; w += VS) {
        const i32 tt = w / B;
        s += static_cast<TA>(v[w]) * static_cast<TA>(x[B * pat.nbr[s0 + tt] + (w - B * tt)]);
      }
    } else {
      const i32* cl = col + k0;
      for (i32 w = lane; w < len; w += VS) s += static_cast<TA>(v[w]) * static_cast<TA>(x[cl[w]]);
    }
  }
#pragma unroll
  for (int o = VS / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, VS);
  if (row < rows && lane == 0) {
    if (MODE == 0) y[row] = static_cast<TX>(s);
    else if (MODE == 1) y[row] = b[row] - static_cast<TX>(s);
    else y[row] += static_cast<TX>(s);
  }
  (void)row_first;
  (void)nodes;
}

template <int VS, int B, class TV, class TX>
__device__ __forceinline__ TX rows_dot(i32 row, int lane, bool valid, const i32* __restrict__ node_of, NodeView pat,
                                       const i32* __restrict__ rowptr, const i32* __restrict__ col,
                                       const TV* __restrict__ val, const TX* __restrict__ x) {
  TX s = TX(0);
  if (valid) {
    const i32 k0 = rowptr[row], len = rowptr[row + 1] - k0;
    const TV* v = val + k0;
    if constexpr (B > 0) {
      const i32 s0 = pat.ptr[node_of[row]];
      for (i32 w = lane; w < len; w += VS) {
        const i32 tt = w / B;
        s += static_cast<TX>(v[w]) * x[B * pat.nbr[s0 + tt] + (w - B * tt)];
      }
    } else {
      const i32* cl = col + k0;
      for (i32 w = lane; w < len; w += VS) s += static_cast<TX>(v[w]) * x[cl[w]];
    }
  }
#pragma unroll
  for (int o = VS / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, VS);
  return s;
}

// Chebyshev step with VS lanes per row (FP64 path).
template <int VS, int B, class T>
__global__ void __launch_bounds__(256) k_rows_cheb_step(i32 rows, const i32* __restrict__ node_of, NodeView pat,
                                                        const i32* __restrict__ rowptr, const i32* __restrict__ col,
                                                        const T* __restrict__ val, const T* __restrict__ d,
                                                        const T* __restrict__ r_in, T* __restrict__ r,
                                                        T* __restrict__ dn, T* __restrict__ x,
                                                        const T* __restrict__ dinv, T c1, T c2, int add_d) {
  const i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 row = static_cast<i32>(t / VS);
  const int lane = static_cast<int>(t % VS);
  const bool valid = row < rows;
  const T s = rows_dot<VS, B, T, T>(row, lane, valid, node_of, pat, rowptr, col, val, d);
  if (valid && lane == 0) {
    const T ri = r_in[row] - s;
    r[row] = ri;
    const T di = c1 * d[row] + c2 * dinv[row] * ri;
    dn[row] = di;
    T xi = x[row];
    if (add_d) xi = xi + d[row];
    x[row] = xi + di;
  }
}

template <int VS, int B, class T>
__global__ void __launch_bounds__(256) k_rows_cheb_first(i32 rows, const i32* __restrict__ node_of, NodeView pat,
                                                         const i32* __restrict__ rowptr, const i32* __restrict__ col,
                                                         const T* __restrict__ val, const T* __restrict__ x,
                                                         const T* __restrict__ b, T* __restrict__ r,
                                                         T* __restrict__ d, const T* __restrict__ dinv, T inv_theta) {
  const i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 row = static_cast<i32>(t / VS);
  const int lane = static_cast<int>(t % VS);
  const bool valid = row < rows;
  const T s = rows_dot<VS, B, T, T>(row, lane, valid, node_of, pat, rowptr, col, val, x);
  if (valid && lane == 0) {
    const T ri = b[row] - s;
    r[row] = ri;
    d[row] = dinv[row] * ri * inv_theta;
  }
}

}  // namespace
}  // namespace simp
