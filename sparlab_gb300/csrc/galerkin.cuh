// Galerkin products of the SA-AMG setup, one warp per row node with a dense
// row accumulator in shared memory (Gustavson's row-by-row product).
//
// The warp walks the left operand's slots of its row node in ascending order
// and adds each block product into the accumulator at positions found by a
// binary search of the (sorted) output slot list, so every output entry
// receives its terms in the same order as multiply_numeric in the reference
// (src/fem/Multigrid.cpp:121-180): ascending inner index, one rounded
// product and one rounded add per term.  Within one left slot the warp's
// lanes own distinct outputs; __syncwarp orders consecutive slots.
//
// Shared memory per warp: the accumulator (rows x row length of T), the
// output slots and their offsets, and the positions of the inner row's slots.
#pragma once

#include "amg.h"
#include "kernels.cuh"

namespace simp {
namespace {

template <class T>
__device__ __forceinline__ void warp_row_setup(const WarpRows& w, int warps, int warp, unsigned char* smem, T*& acc,
                                               i32*& sl, i32*& soff, i32*& upos) {
  acc = reinterpret_cast<T*>(smem) + static_cast<size_t>(warp) * w.acc;
  i32* base = reinterpret_cast<i32*>(reinterpret_cast<T*>(smem) + static_cast<size_t>(warps) * w.acc);
  sl = base + static_cast<size_t>(warp) * (2 * w.slots + w.inner);
  soff = sl + w.slots;
  upos = soff + w.slots;
}

// first index q of the sorted sl[0..ns) with sl[q] >= h (ns >= 1)
__device__ __forceinline__ int lower_slot(const i32* sl, int ns, i32 h) {
  int lo = 0, hi = ns - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (sl[mid] < h) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// position of column c of an inner row (slots of width b, or described by
// off when b == 0) in the accumulator row
__device__ __forceinline__ int inner_pos(int c, int b, const i32* __restrict__ off, i32 u0, i32 nu,
                                         const i32* upos) {
  if (b > 0) {
    const int u = c / b;
    return upos[u] + (c - u * b);
  }
  int u = 0;
  while (u + 1 < nu && off[u0 + u + 1] <= c) ++u;
  return upos[u] + (c - off[u0 + u]);
}

// AP = A P: warp per fine node I; inner rows are P's rows of I's neighbours J.
template <class T>
__global__ void __launch_bounds__(256) k_ap_rows(i32 nodes, WarpRows w, const i32* __restrict__ first, int b1,
                                                 NodeView a, const i32* __restrict__ arow,
                                                 const T* __restrict__ aval, NodeView p,
                                                 const i32* __restrict__ prow, const T* __restrict__ pval,
                                                 NodeView ap, const i32* __restrict__ aprow,
                                                 T* __restrict__ apval) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warps = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* acc;
  i32 *sl, *soff, *upos;
  warp_row_setup<T>(w, warps, warp, smem, acc, sl, soff, upos);
  for (i32 I = blockIdx.x * warps + warp; I < nodes; I += gridDim.x * warps) {
    const i32 r0 = first[I], nr = first[I + 1] - r0;
    const i32 s0 = ap.ptr[I], ns = ap.ptr[I + 1] - s0;
    if (nr == 0 || ns == 0) continue;
    const i32 L = aprow[r0 + 1] - aprow[r0];
    for (int q = lane; q < ns; q += 32) {
      sl[q] = ap.nbr[s0 + q];
      soff[q] = ap.off[s0 + q];
    }
    for (int q = lane; q < nr * L; q += 32) acc[q] = T(0);
    __syncwarp();
    for (i32 t = a.ptr[I]; t < a.ptr[I + 1]; ++t) {
      const i32 J = a.nbr[t];
      const i32 kj = first[J], sJ = first[J + 1] - kj;
      const i32 u0 = p.ptr[J], nu = p.ptr[J + 1] - u0;
      if (sJ == 0 || nu == 0) continue;
      for (int u = lane; u < nu; u += 32) upos[u] = soff[lower_slot(sl, ns, p.nbr[u0 + u])];
      __syncwarp();
      const i32 Lp = prow[kj + 1] - prow[kj];
      const i32 aoff = a.off[t];
      for (int q = lane; q < nr * Lp; q += 32) {
        const int ka = q / Lp, c = q - ka * Lp;
        const int pos = ka * L + inner_pos(c, b1, p.off, u0, nu, upos);
        const T* av = aval + arow[r0 + ka] + aoff;
        T v = acc[pos];
        for (int kb = 0; kb < sJ; ++kb) v = xadd(v, xmul(av[kb], pval[prow[kj + kb] + c]));
        acc[pos] = v;
      }
      __syncwarp();
    }
    for (int ka = 0; ka < nr; ++ka) {
      T* out = apval + aprow[r0 + ka];
      for (int q = lane; q < L; q += 32) out[q] = acc[ka * L + q];
    }
    __syncwarp();
  }
}

// RAW = R (AP): warp per coarse node g; inner rows are AP's rows of the
// fine nodes I of R's row g.
template <class T>
__global__ void __launch_bounds__(256) k_rap_rows(i32 nodes, WarpRows w, const i32* __restrict__ first1,
                                                  const i32* __restrict__ first, int b1, NodeView r,
                                                  const i32* __restrict__ rrow, const T* __restrict__ rval,
                                                  NodeView ap, const i32* __restrict__ aprow,
                                                  const T* __restrict__ apval, NodeView c,
                                                  const i32* __restrict__ crow, T* __restrict__ cval) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warps = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* acc;
  i32 *sl, *soff, *upos;
  warp_row_setup<T>(w, warps, warp, smem, acc, sl, soff, upos);
  for (i32 g = blockIdx.x * warps + warp; g < nodes; g += gridDim.x * warps) {
    const i32 r0 = first1[g], nr = first1[g + 1] - r0;
    const i32 s0 = c.ptr[g], ns = c.ptr[g + 1] - s0;
    if (nr == 0 || ns == 0) continue;
    const i32 L = crow[r0 + 1] - crow[r0];
    for (int q = lane; q < ns; q += 32) {
      sl[q] = c.nbr[s0 + q];
      soff[q] = c.off[s0 + q];
    }
    for (int q = lane; q < nr * L; q += 32) acc[q] = T(0);
    __syncwarp();
    for (i32 t = r.ptr[g]; t < r.ptr[g + 1]; ++t) {
      const i32 I = r.nbr[t];
      const i32 ki = first[I], sI = first[I + 1] - ki;
      const i32 u0 = ap.ptr[I], nu = ap.ptr[I + 1] - u0;
      if (sI == 0 || nu == 0) continue;
      for (int u = lane; u < nu; u += 32) upos[u] = soff[lower_slot(sl, ns, ap.nbr[u0 + u])];
      __syncwarp();
      const i32 La = aprow[ki + 1] - aprow[ki];
      const i32 roff = r.off[t];
      for (int q = lane; q < nr * La; q += 32) {
        const int kg = q / La, cc = q - kg * La;
        const int pos = kg * L + inner_pos(cc, b1, ap.off, u0, nu, upos);
        const T* rv = rval + rrow[r0 + kg] + roff;
        T v = acc[pos];
        for (int ka = 0; ka < sI; ++ka) v = xadd(v, xmul(rv[ka], apval[aprow[ki + ka] + cc]));
        acc[pos] = v;
      }
      __syncwarp();
    }
    for (int kg = 0; kg < nr; ++kg) {
      T* out = cval + crow[r0 + kg];
      for (int q = lane; q < L; q += 32) out[q] = acc[kg * L + q];
    }
    __syncwarp();
  }
}

// P = (I - omega D^-1 A) P-hat (src/fem/Multigrid.cpp:671-716): warp per
// fine node I; the inner rows are P-hat's rows of I's neighbours J, whose
// single slot is J's aggregate.
template <class T>
__global__ void __launch_bounds__(256) k_prolongator_rows(
    i32 nodes, WarpRows w, const i32* __restrict__ first, const i32* __restrict__ first1,
    const i32* __restrict__ agg, NodeView a, const i32* __restrict__ arow, const T* __restrict__ aval, NodeView p,
    const i32* __restrict__ prow, T* __restrict__ pval, const i32* __restrict__ phat_ptr,
    const T* __restrict__ phat, const double* __restrict__ dinv, double omega) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warps = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* acc;
  i32 *sl, *soff, *upos;
  warp_row_setup<T>(w, warps, warp, smem, acc, sl, soff, upos);
  for (i32 I = blockIdx.x * warps + warp; I < nodes; I += gridDim.x * warps) {
    const i32 r0 = first[I], nr = first[I + 1] - r0;
    const i32 s0 = p.ptr[I], ns = p.ptr[I + 1] - s0;
    if (nr == 0 || ns == 0) continue;
    const i32 L = prow[r0 + 1] - prow[r0];
    for (int q = lane; q < ns; q += 32) {
      sl[q] = p.nbr[s0 + q];
      soff[q] = p.off[s0 + q];
    }
    for (int q = lane; q < nr * L; q += 32) acc[q] = T(0);
    __syncwarp();
    for (i32 t = a.ptr[I]; t < a.ptr[I + 1]; ++t) {
      const i32 J = a.nbr[t];
      const i32 kj = first[J], sJ = first[J + 1] - kj;
      const i32 g = agg[J];
      if (sJ == 0 || g < 0) continue;
      const i32 rg = first1[g + 1] - first1[g];
      const int base = soff[lower_slot(sl, ns, g)];
      const i32 aoff = a.off[t];
      for (int q = lane; q < nr * rg; q += 32) {
        const int ka = q / rg, j = q - ka * rg;
        const int pos = ka * L + base + j;
        const T* av = aval + arow[r0 + ka] + aoff;
        T v = acc[pos];
        for (int kb = 0; kb < sJ; ++kb) v = xadd(v, xmul(av[kb], phat[phat_ptr[kj + kb] + j]));
        acc[pos] = v;
      }
      __syncwarp();
    }
    // P(i, :) = P-hat(i, :) - omega dinv_i (A P-hat)(i, :)
    const i32 gi = agg[I];
    const int own = gi >= 0 ? soff[lower_slot(sl, ns, gi)] : -1;
    for (int ka = 0; ka < nr; ++ka) {
      const T scale = static_cast<T>(omega * dinv[r0 + ka]);
      T* out = pval + prow[r0 + ka];
      const T* ph = phat + phat_ptr[r0 + ka];
      for (int q = lane; q < L; q += 32) {
        T v = xmul(acc[ka * L + q], -scale);
        if (own >= 0 && q >= own && q < own + (first1[gi + 1] - first1[gi])) v = xadd(v, ph[q - own]);
        out[q] = v;
      }
    }
    __syncwarp();
  }
  (void)upos;
}

}  // namespace
}  // namespace simp
