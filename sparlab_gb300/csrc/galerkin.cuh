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

constexpr int kChunk = 32;  // left-operand slots whose metadata a warp stages at once

// Per-warp shared memory: the accumulator (T), then int arrays: output slots
// and offsets, the chunk's slot metadata, and the (slot, inner slot) positions.
struct WarpSmem {
  int* sl;    // output slots (column nodes), ascending
  int* soff;  // their offsets in the output row
  int* mj;    // chunk: inner row node's first unknown
  int* msj;   // chunk: its unknown count
  int* mrow;  // chunk: start of its first inner row's values
  int* mlen;  // chunk: inner row length
  int* mu0;   // chunk: first inner slot
  int* mpre;  // chunk: exclusive prefix of inner slot counts (kChunk + 1)
  int* maux;  // chunk: left operand's slot offset (a.off / r.off)
  int* upos;  // pair positions in the accumulator row
};

constexpr int kMetaInts = 8 * kChunk + 1;

template <class T>
__device__ __forceinline__ T* warp_setup(const WarpRows& w, int warps, int warp, unsigned char* smem, WarpSmem& m) {
  T* acc = reinterpret_cast<T*>(smem) + static_cast<size_t>(warp) * w.acc;
  int* base = reinterpret_cast<int*>(reinterpret_cast<T*>(smem) + static_cast<size_t>(warps) * w.acc) +
              static_cast<size_t>(warp) * (2 * w.slots + kMetaInts + w.inner);
  m.sl = base;
  m.soff = m.sl + w.slots;
  m.mj = m.soff + w.slots;
  m.msj = m.mj + kChunk;
  m.mrow = m.msj + kChunk;
  m.mlen = m.mrow + kChunk;
  m.mu0 = m.mlen + kChunk;
  m.maux = m.mu0 + kChunk;
  m.mpre = m.maux + kChunk;
  m.upos = m.mpre + kChunk + 1;
  return acc;
}

// first index q of the sorted sl[0..ns) with sl[q] >= h (ns >= 1)
__device__ __forceinline__ int lower_slot(const int* sl, int ns, i32 h) {
  int lo = 0, hi = ns - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (sl[mid] < h) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Stage the output slots of a row node and zero its accumulator rows.
template <class T>
__device__ __forceinline__ void warp_begin(NodeView out, i32 node, int nrows, int len, int lane, const WarpSmem& m,
                                           T* acc) {
  const i32 s0 = out.ptr[node], ns = out.ptr[node + 1] - s0;
  for (int q = lane; q < ns; q += 32) {
    m.sl[q] = out.nbr[s0 + q];
    m.soff[q] = out.off[s0 + q];
  }
  for (int q = lane; q < nrows * len; q += 32) acc[q] = T(0);
  __syncwarp();
}

// Phase 1 + 2 for one chunk of the left operand's slots [t0, t0 + nt):
// metadata of each slot's inner row node (lanes over slots), then the
// accumulator position of every (slot, inner slot) pair (lanes over pairs).
// left: the left operand's node pattern; inner: the inner rows' pattern.
__device__ __forceinline__ void warp_chunk(NodeView left, i32 t0, int nt, const i32* __restrict__ first,
                                           NodeView inner, const i32* __restrict__ irow, int ns, int lane,
                                           const WarpSmem& m) {
  int nu = 0;
  if (lane < nt) {
    const i32 J = left.nbr[t0 + lane];
    const i32 kj = first[J], sJ = first[J + 1] - kj;
    const i32 u0 = inner.ptr[J];
    nu = sJ > 0 ? inner.ptr[J + 1] - u0 : 0;
    m.mj[lane] = kj;
    m.msj[lane] = sJ;
    m.mrow[lane] = sJ > 0 ? irow[kj] : 0;
    m.mlen[lane] = sJ > 0 ? irow[kj + 1] - irow[kj] : 0;
    m.mu0[lane] = u0;
    m.maux[lane] = left.off[t0 + lane];
  }
  int incl = nu;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane < nt) m.mpre[lane] = incl - nu;
  const int npairs = __shfl_sync(0xffffffffu, incl, 31);
  if (lane == 0) m.mpre[nt] = npairs;
  __syncwarp();
  for (int q = lane; q < npairs; q += 32) {
    int lo = 0, hi = nt - 1;  // the last slot t with mpre[t] <= q
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (m.mpre[mid] <= q) lo = mid;
      else hi = mid - 1;
    }
    const int u = q - m.mpre[lo];
    m.upos[q] = m.soff[lower_slot(m.sl, ns, inner.nbr[m.mu0[lo] + u])];
  }
  __syncwarp();
}

// Accumulator position of column c of the inner row of chunk slot t.
template <int B1>
__device__ __forceinline__ int pair_pos(int c, int t, const WarpSmem& m, const i32* __restrict__ ioff) {
  const int pb = m.mpre[t];
  if constexpr (B1 > 0) {
    const int u = c / B1;
    return m.upos[pb + u] + (c - u * B1);
  } else {
    const int nu = m.mpre[t + 1] - pb, u0 = m.mu0[t];
    int u = 0;
    while (u + 1 < nu && ioff[u0 + u + 1] <= c) ++u;
    return m.upos[pb + u] + (c - ioff[u0 + u]);
  }
}

// One product term: exact (rounded product, rounded add: the reference's
// order and rounding, FP64 setups) or fused (the FP32 reuse setups).
template <bool EXACT, class T>
__device__ __forceinline__ T term(T acc, T a, T b) {
  if constexpr (EXACT) return xadd(acc, xmul(a, b));
  else return fma(a, b, acc);
}

// Compile-time row widths: W > 0 fixes the count at W, W == 0 means "the
// runtime value n, at most 6".
template <int W>
__device__ __forceinline__ constexpr int wmax() { return W > 0 ? W : 6; }
template <int W>
__device__ __forceinline__ bool within(int k, int n) { return W > 0 ? true : k < n; }

// AP = A P: warp per fine node I; inner rows are P's rows of I's neighbours J.
// acc(ka, pos(c)) += sum_kb A((I,ka),(J,kb)) P((J,kb), c), kb ascending.
// NR: unknowns per node of this level (rows of I and of every J), B1: of the
// next level (0 = not uniform).
template <class T, bool EXACT, int NR, int B1>
__global__ void __launch_bounds__(256) k_ap_rows(i32 nodes, WarpRows w, const i32* __restrict__ first,
                                                 NodeView a, const i32* __restrict__ arow,
                                                 const T* __restrict__ aval, NodeView p,
                                                 const i32* __restrict__ prow, const T* __restrict__ pval,
                                                 NodeView ap, const i32* __restrict__ aprow,
                                                 T* __restrict__ apval) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int MR = wmax<NR>();
  const int warps = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpSmem m;
  T* acc = warp_setup<T>(w, warps, warp, smem, m);
  for (i32 I = blockIdx.x * warps + warp; I < nodes; I += gridDim.x * warps) {
    const i32 r0 = first[I], nr = NR > 0 ? NR : first[I + 1] - r0;
    const int ns = ap.ptr[I + 1] - ap.ptr[I];
    if (nr == 0 || ns == 0) continue;
    const i32 L = aprow[r0 + 1] - aprow[r0];
    const i32 abase = arow[r0], LA = arow[r0 + 1] - arow[r0];
    warp_begin<T>(ap, I, nr, L, lane, m, acc);
    for (i32 t0 = a.ptr[I]; t0 < a.ptr[I + 1]; t0 += kChunk) {
      const int nt = min(kChunk, a.ptr[I + 1] - t0);
      warp_chunk(a, t0, nt, first, p, prow, ns, lane, m);
      for (int t = 0; t < nt; ++t) {
        const int sJ = NR > 0 ? NR : m.msj[t], Lp = m.mlen[t];
        if (NR == 0 && sJ == 0) continue;
        T ar[MR][MR];
        const T* av = aval + abase + m.maux[t];
#pragma unroll
        for (int ka = 0; ka < MR; ++ka)
#pragma unroll
          for (int kb = 0; kb < MR; ++kb)
            ar[ka][kb] = (within<NR>(ka, nr) && within<NR>(kb, sJ)) ? av[ka * LA + kb] : T(0);
        const T* pv = pval + m.mrow[t];
        for (int c = lane; c < Lp; c += 32) {
          T pc[MR];
#pragma unroll
          for (int kb = 0; kb < MR; ++kb) pc[kb] = within<NR>(kb, sJ) ? pv[kb * Lp + c] : T(0);
          const int pos = pair_pos<B1>(c, t, m, p.off);
#pragma unroll
          for (int ka = 0; ka < MR; ++ka) {
            if (within<NR>(ka, nr)) {
              T v = acc[ka * L + pos];
#pragma unroll
              for (int kb = 0; kb < MR; ++kb)
                if (within<NR>(kb, sJ)) v = term<EXACT>(v, ar[ka][kb], pc[kb]);
              acc[ka * L + pos] = v;
            }
          }
        }
        __syncwarp();
      }
    }
    for (int ka = 0; ka < nr; ++ka) {
      T* out = apval + aprow[r0 + ka];
      for (int q = lane; q < L; q += 32) out[q] = acc[ka * L + q];
    }
    __syncwarp();
  }
}

// RAW = R (AP): warp per coarse node g; inner rows are AP's rows of the fine
// nodes I of R's row g.  acc(kg, pos(c)) += sum_ka R((g,kg),(I,ka)) AP((I,ka), c).
// NC: unknowns per coarse node (rows of g, and the AP column-node width),
// NF: per fine node (0 = not uniform).
template <class T, bool EXACT, int NC, int NF>
__global__ void __launch_bounds__(256) k_rap_rows(i32 nodes, WarpRows w, const i32* __restrict__ first1,
                                                  const i32* __restrict__ first, NodeView r,
                                                  const i32* __restrict__ rrow, const T* __restrict__ rval,
                                                  NodeView ap, const i32* __restrict__ aprow,
                                                  const T* __restrict__ apval, NodeView c,
                                                  const i32* __restrict__ crow, T* __restrict__ cval) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int MC = wmax<NC>(), MF = wmax<NF>();
  const int warps = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpSmem m;
  T* acc = warp_setup<T>(w, warps, warp, smem, m);
  for (i32 g = blockIdx.x * warps + warp; g < nodes; g += gridDim.x * warps) {
    const i32 r0 = first1[g], nr = NC > 0 ? NC : first1[g + 1] - r0;
    const int ns = c.ptr[g + 1] - c.ptr[g];
    if (nr == 0 || ns == 0) continue;
    const i32 L = crow[r0 + 1] - crow[r0];
    const i32 rbase = rrow[r0], LR = rrow[r0 + 1] - rrow[r0];
    warp_begin<T>(c, g, nr, L, lane, m, acc);
    for (i32 t0 = r.ptr[g]; t0 < r.ptr[g + 1]; t0 += kChunk) {
      const int nt = min(kChunk, r.ptr[g + 1] - t0);
      warp_chunk(r, t0, nt, first, ap, aprow, ns, lane, m);
      for (int t = 0; t < nt; ++t) {
        const int sI = NF > 0 ? NF : m.msj[t], La = m.mlen[t];
        if (NF == 0 && sI == 0) continue;
        T rr[MC][MF];
        const T* rv = rval + rbase + m.maux[t];
#pragma unroll
        for (int kg = 0; kg < MC; ++kg)
#pragma unroll
          for (int ka = 0; ka < MF; ++ka)
            rr[kg][ka] = (within<NC>(kg, nr) && within<NF>(ka, sI)) ? rv[kg * LR + ka] : T(0);
        const T* pv = apval + m.mrow[t];
        for (int cc = lane; cc < La; cc += 32) {
          T pc[MF];
#pragma unroll
          for (int ka = 0; ka < MF; ++ka) pc[ka] = within<NF>(ka, sI) ? pv[ka * La + cc] : T(0);
          const int pos = pair_pos<NC>(cc, t, m, ap.off);
#pragma unroll
          for (int kg = 0; kg < MC; ++kg) {
            if (within<NC>(kg, nr)) {
              T v = acc[kg * L + pos];
#pragma unroll
              for (int ka = 0; ka < MF; ++ka)
                if (within<NF>(ka, sI)) v = term<EXACT>(v, rr[kg][ka], pc[ka]);
              acc[kg * L + pos] = v;
            }
          }
        }
        __syncwarp();
      }
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
// single slot is J's aggregate.  Lanes own (ka, j) of one neighbour at a time.
template <class T, bool EXACT>
__global__ void __launch_bounds__(256) k_prolongator_rows(
    i32 nodes, WarpRows w, const i32* __restrict__ first, const i32* __restrict__ first1,
    const i32* __restrict__ agg, NodeView a, const i32* __restrict__ arow, const T* __restrict__ aval, NodeView p,
    const i32* __restrict__ prow, T* __restrict__ pval, const i32* __restrict__ phat_ptr,
    const T* __restrict__ phat, const double* __restrict__ dinv, double omega) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warps = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpSmem m;
  T* acc = warp_setup<T>(w, warps, warp, smem, m);
  for (i32 I = blockIdx.x * warps + warp; I < nodes; I += gridDim.x * warps) {
    const i32 r0 = first[I], nr = first[I + 1] - r0;
    const int ns = p.ptr[I + 1] - p.ptr[I];
    if (nr == 0 || ns == 0) continue;
    const i32 L = prow[r0 + 1] - prow[r0];
    const i32 abase = arow[r0], LA = arow[r0 + 1] - arow[r0];
    warp_begin<T>(p, I, nr, L, lane, m, acc);
    for (i32 t0 = a.ptr[I]; t0 < a.ptr[I + 1]; t0 += kChunk) {
      const int nt = min(kChunk, a.ptr[I + 1] - t0);
      // per neighbour: its unknowns, its aggregate's position and rank
      if (lane < nt) {
        const i32 J = a.nbr[t0 + lane];
        const i32 kj = first[J], sJ = first[J + 1] - kj;
        const i32 gJ = agg[J];
        const bool ok = sJ > 0 && gJ >= 0;
        m.mj[lane] = kj;
        m.msj[lane] = ok ? sJ : 0;
        m.mlen[lane] = ok ? first1[gJ + 1] - first1[gJ] : 0;
        m.mrow[lane] = ok ? m.soff[lower_slot(m.sl, ns, gJ)] : 0;
        m.maux[lane] = a.off[t0 + lane];
      }
      __syncwarp();
      for (int t = 0; t < nt; ++t) {
        const int sJ = m.msj[t], rg = m.mlen[t];
        if (sJ == 0) continue;
        const int base = m.mrow[t], kj = m.mj[t];
        const T* av = aval + abase + m.maux[t];
        for (int q = lane; q < nr * rg; q += 32) {
          const int ka = q / rg, j = q - ka * rg;
          const int pos = ka * L + base + j;
          T v = acc[pos];
          for (int kb = 0; kb < sJ; ++kb) v = term<EXACT>(v, av[ka * LA + kb], phat[phat_ptr[kj + kb] + j]);
          acc[pos] = v;
        }
        __syncwarp();
      }
    }
    // P(i, :) = P-hat(i, :) - omega dinv_i (A P-hat)(i, :)
    const i32 gi = agg[I];
    const int own = gi >= 0 ? m.soff[lower_slot(m.sl, ns, gi)] : -1;
    const int rown = gi >= 0 ? first1[gi + 1] - first1[gi] : 0;
    for (int ka = 0; ka < nr; ++ka) {
      const T scale = static_cast<T>(omega * dinv[r0 + ka]);
      T* out = pval + prow[r0 + ka];
      const T* ph = phat + phat_ptr[r0 + ka];
      for (int q = lane; q < L; q += 32) {
        const bool mine = own >= 0 && q >= own && q < own + rown;
        T v;
        if constexpr (EXACT) {
          v = xmul(acc[ka * L + q], -scale);
          if (mine) v = xadd(v, ph[q - own]);
        } else {
          v = mine ? fma(acc[ka * L + q], -scale, ph[q - own]) : acc[ka * L + q] * -scale;
        }
        out[q] = v;
      }
    }
    __syncwarp();
  }
}

// The same product by output entry, where every fine node has B0 unknowns
// and every aggregate B1: entry (ka, c) of fine node I's P row is slot
// s = c / B1, column j = c % B1; its contributors are the slots t of I's A
// row whose neighbour J lies in slot s's aggregate, ascending t, each stored
// as (offset of J's block in the A row, first P-hat value of J's rows) when
// the pattern is built.  Each entry sums its contributions in the warp
// kernel's order (t ascending, then kb) with the same arithmetic, so P is
// that kernel's bit for bit, without its per-neighbour passes and barriers.
template <class T, bool EXACT, int B0, int B1>
__global__ void __launch_bounds__(256) k_prolongator_gather(
    i32 nodes, const i32* __restrict__ agg, const i32* __restrict__ arow, const T* __restrict__ aval, NodeView p,
    const i32* __restrict__ prow, T* __restrict__ pval, const i32* __restrict__ phat_ptr,
    const T* __restrict__ phat, const double* __restrict__ dinv, double omega, const i32* __restrict__ pc_ptr,
    const int2* __restrict__ pc) {
  const int lane = threadIdx.x & 31;
  const i64 nwarps = (static_cast<i64>(gridDim.x) * blockDim.x) >> 5;
  for (i64 I = (blockIdx.x * static_cast<i64>(blockDim.x) + threadIdx.x) >> 5; I < nodes; I += nwarps) {
    const i32 r0 = B0 * static_cast<i32>(I);
    const i32 ps = p.ptr[I], ns = p.ptr[I + 1] - ps;
    if (ns == 0) continue;
    const i32 L = ns * B1;
    const i32 gi = agg[I];
    for (i32 q = lane; q < B0 * L; q += 32) {
      const i32 ka = q / L, c = q - ka * L;
      const i32 s = c / B1, j = c - s * B1;
      const i32 gs = ps + s;
      const T* ak = aval + arow[r0 + ka];
      T v = T(0);
      for (i32 k = pc_ptr[gs]; k < pc_ptr[gs + 1]; ++k) {
        const int2 e = pc[k];
        const T* av = ak + e.x;
        const T* ph = phat + e.y + j;
#pragma unroll
        for (int kb = 0; kb < B0; ++kb) v = term<EXACT>(v, av[kb], ph[kb * B1]);
      }
      const T scale = static_cast<T>(omega * dinv[r0 + ka]);
      const bool mine = gi >= 0 && p.nbr[gs] == gi;
      T out;
      if constexpr (EXACT) {
        out = xmul(v, -scale);
        if (mine) out = xadd(out, phat[phat_ptr[r0 + ka] + j]);
      } else {
        out = mine ? fma(v, -scale, phat[phat_ptr[r0 + ka] + j]) : v * -scale;
      }
      pval[prow[r0 + ka] + c] = out;
    }
  }
}

}  // namespace
}  // namespace simp
