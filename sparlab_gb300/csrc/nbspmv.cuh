// Node-block sparse operator applications.
//
// Every level operator (A_l, P_l, R_l) is stored as scalar rows whose column
// lists are shared by all rows of a node and grouped by whole column nodes
// (see structure.h).  A group of G lanes owns one row node: lanes stride over
// its node-level slots, each lane multiplies the slot's (rows x cols) block by
// the column node's entries of x (loaded once for all rows of the node), and
// the per-row sums are reduced across the group with a fixed butterfly.  Index
// traffic is one slot record per block instead of one column per entry, and
// x is read once per block instead of once per row.
#pragma once

#include "kernels.cuh"

namespace simp {
namespace {

constexpr int kMaxNode = 6;  // unknowns per node: 2-3 on level 0, rank <= 6 below

template <class T>
struct Acc {
  using type = T;
};

// Per-row dot products of one row node; returns with acc[r] (r < nr) summed
// over the group in every lane.
template <int G, class TV, class TX, class TA>
__device__ __forceinline__ void nb_row_dots(i32 I, int lane, unsigned mask, bool valid, const i32* __restrict__ row_first,
                                            const i32* __restrict__ col_first, NodeView pat,
                                            const i32* __restrict__ rowptr, const TV* __restrict__ val,
                                            const TX* __restrict__ x, int& nr, i32& r0, TA (&acc)[kMaxNode]) {
#pragma unroll
  for (int r = 0; r < kMaxNode; ++r) acc[r] = TA(0);
  nr = 0;
  r0 = 0;
  if (valid) {
    r0 = row_first[I];
    nr = row_first[I + 1] - r0;
    i32 rp[kMaxNode];
#pragma unroll
    for (int r = 0; r < kMaxNode; ++r) rp[r] = r < nr ? rowptr[r0 + r] : 0;
    const i32 te = pat.ptr[I + 1];
    for (i32 t = pat.ptr[I] + lane; t < te; t += G) {
      const i32 J = pat.nbr[t];
      const i32 c0 = col_first[J];
      const int nc = col_first[J + 1] - c0;
      const i32 o = pat.off[t];
      TA xv[kMaxNode];
#pragma unroll
      for (int k = 0; k < kMaxNode; ++k) xv[k] = k < nc ? static_cast<TA>(x[c0 + k]) : TA(0);
#pragma unroll
      for (int r = 0; r < kMaxNode; ++r) {
        if (r < nr) {
          const TV* v = val + rp[r] + o;
#pragma unroll
          for (int k = 0; k < kMaxNode; ++k)
            if (k < nc) acc[r] += static_cast<TA>(v[k]) * xv[k];
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < kMaxNode; ++r) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(mask, acc[r], o, G);
  }
}

template <int G>
__device__ __forceinline__ unsigned group_mask() {
  if (G == 32) return 0xffffffffu;
  const int base = (threadIdx.x & 31) & ~(G - 1);
  return ((1u << G) - 1u) << base;
}

// mode 0: y = A x ; 1: y = b - A x ; 2: y += A x
template <int G, int MODE, class TV, class TX, class TA>
__global__ void __launch_bounds__(256) k_nb_apply(i32 nodes, const i32* __restrict__ row_first,
                                                  const i32* __restrict__ col_first, NodeView pat,
                                                  const i32* __restrict__ rowptr, const TV* __restrict__ val,
                                                  const TX* __restrict__ x, TX* __restrict__ y,
                                                  const TX* __restrict__ b) {
  const i64 t0 = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 I = static_cast<i32>(t0 / G);
  const int lane = static_cast<int>(t0 % G);
  const bool valid = I < nodes;
  TA acc[kMaxNode];
  int nr;
  i32 r0;
  nb_row_dots<G, TV, TX, TA>(I, lane, group_mask<G>(), valid, row_first, col_first, pat, rowptr, val, x, nr, r0,
                             acc);
  if (!valid) return;
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
template <int G, class TV, class TX>
__global__ void __launch_bounds__(256) k_nb_cheb_step(i32 nodes, const i32* __restrict__ first, NodeView pat,
                                                      const i32* __restrict__ rowptr, const TV* __restrict__ val,
                                                      const TX* __restrict__ d, const TX* __restrict__ r_in,
                                                      TX* __restrict__ r, TX* __restrict__ dn, TX* __restrict__ x,
                                                      const TX* __restrict__ dinv, TX c1, TX c2, int add_d) {
  const i64 t0 = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 I = static_cast<i32>(t0 / G);
  const int lane = static_cast<int>(t0 % G);
  const bool valid = I < nodes;
  TX acc[kMaxNode];
  int nr;
  i32 r0;
  nb_row_dots<G, TV, TX, TX>(I, lane, group_mask<G>(), valid, first, first, pat, rowptr, val, d, nr, r0, acc);
  if (!valid) return;
#pragma unroll
  for (int q = 0; q < kMaxNode; ++q) {
    if (q < nr && lane == q) {
      const i32 row = r0 + q;
      const TX ri = r_in[row] - acc[q];
      r[row] = ri;
      const TX di = c1 * d[row] + c2 * dinv[row] * ri;
      dn[row] = di;
      TX xi = x[row];
      if (add_d) xi = xi + d[row];
      x[row] = xi + di;
    }
  }
}

// r = b - A x ; d = dinv r / theta
template <int G, class TV, class TX>
__global__ void __launch_bounds__(256) k_nb_cheb_first(i32 nodes, const i32* __restrict__ first, NodeView pat,
                                                       const i32* __restrict__ rowptr, const TV* __restrict__ val,
                                                       const TX* __restrict__ x, const TX* __restrict__ b,
                                                       TX* __restrict__ r, TX* __restrict__ d,
                                                       const TX* __restrict__ dinv, TX inv_theta) {
  const i64 t0 = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 I = static_cast<i32>(t0 / G);
  const int lane = static_cast<int>(t0 % G);
  const bool valid = I < nodes;
  TX acc[kMaxNode];
  int nr;
  i32 r0;
  nb_row_dots<G, TV, TX, TX>(I, lane, group_mask<G>(), valid, first, first, pat, rowptr, val, x, nr, r0, acc);
  if (!valid) return;
#pragma unroll
  for (int q = 0; q < kMaxNode; ++q) {
    if (q < nr && lane == q) {
      const i32 row = r0 + q;
      const TX ri = b[row] - acc[q];
      r[row] = ri;
      d[row] = dinv[row] * ri * inv_theta;
    }
  }
}

}  // namespace
}  // namespace simp
