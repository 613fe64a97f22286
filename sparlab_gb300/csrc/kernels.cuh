// Device kernels of the AMG-PCG solve: deterministic reductions, CSR
// operator applications with fused smoother epilogues, the Galerkin numeric
// products over node-level patterns, and the PCG vector updates.
//
// Determinism: every reduction has a fixed shape (grid, block, tree), every
// output entry is written by one thread that sums its terms in a fixed order,
// and no value path uses atomics, so results are bitwise reproducible run to
// run.  The setup products sum in exactly the order of the reference's
// multiply/multiply_numeric (src/fem/Multigrid.cpp:121-225) with rounded
// (unfused) multiply-adds, so their FP64 values equal the CPU oracle's.
#pragma once

#include "common.h"

#include <type_traits>

#include <cuda_runtime.h>

namespace simp {

// Scalar column indices of a CSR from its node pattern (defined in amg.cu).
__global__ void k_expand_columns(i32 n, const i32* __restrict__ node_of, NodeView p,
                                 const i32* __restrict__ col_first, const i32* __restrict__ rowptr,
                                 i32* __restrict__ col);

constexpr int kRedBlocks = 1024;   // fixed reduction grid
constexpr int kRedThreads = 256;

// Kernels below have internal linkage: every translation unit instantiates
// the ones it launches.
namespace {
// ---------------------------------------------------------------------------
// exact-order arithmetic (no contraction into FMA)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }

// Double-float arithmetic (a value is an unevaluated sum hi + lo of two
// floats, about 48 significant bits): Knuth's TwoSum and Dekker's product
// with a fused multiply-add for the exact product error.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (sh, sl) += (ah + al)(bh + bl), dropping al * bl
__device__ __forceinline__ void df_fma(float ah, float al, float bh, float bl, float& sh, float& sl) {
  const float p = __fmul_rn(ah, bh);
  float pe = __fmaf_rn(ah, bh, -p);
  pe = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, pe));
  float t, e;
  two_sum(sh, p, t, e);
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(e, pe));
}

// hi = fl32(v), lo = fl32(v - hi), both rounded to nearest even.  Where
// both halves are normal floats (v's exponent field in [949, 1149]: |v| in
// [2^-74, 2^127)), from v's bits with integer operations -- GB300 runs FP64
// conversions and arithmetic at 1/64 of its FP32 rate -- and otherwise by
// FP64 conversion.  The 53-bit significand M splits into its top 24 bits K
// and low 29 bits R; K rounds to nearest even on R (a carry out of K moves
// into the float exponent field), and v - hi is the remainder r = R or
// R - 2^29 in units of 2^(e - 1075), which one int -> float conversion
// rounds to 24 bits and a power of two scales exactly.
__device__ __forceinline__ void df_split(double v, float& hi, float& lo) {
  const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(v));
  const int e = static_cast<int>((u >> 52) & 0x7FFull);
  if (e >= 949 && e <= 1149) {
    const unsigned long long m = (u & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    unsigned k = static_cast<unsigned>(m >> 29);
    const int rr = static_cast<int>(m & 0x1FFFFFFFull);
    int r = rr;
    if (rr > 0x10000000 || (rr == 0x10000000 && (k & 1u))) {
      k += 1u;
      r = rr - 0x20000000;
    }
    const bool neg = (u >> 63) != 0;
    const unsigned bits = (static_cast<unsigned>(neg) << 31) | ((static_cast<unsigned>(e - 896) << 23) + (k - 0x800000u));
    hi = __uint_as_float(bits);
    lo = __int2float_rn(neg ? -r : r) * __uint_as_float(static_cast<unsigned>(e - 948) << 23);
    return;
  }
  hi = __double2float_rn(v);
  lo = __double2float_rn(v - static_cast<double>(hi));
}

__global__ void k_split_values(i64 n, const double* __restrict__ v, float* __restrict__ hi, float* __restrict__ lo) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    float h, l;
    df_split(v[i], h, l);
    if (hi) hi[i] = h;
    lo[i] = l;
  }
}

// hi = float(v) and the interleaved (hi, lo) pairs of the double-float operator
__global__ void k_split_values_pairs(i64 n, const double* __restrict__ v, float* __restrict__ hi,
                                     float2* __restrict__ pair) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    float h, l;
    df_split(v[i], h, l);
    hi[i] = h;
    pair[i] = make_float2(h, l);
  }
}

__global__ void k_split_pairs(i64 n, const double* __restrict__ v, float2* __restrict__ out) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    float h, l;
    df_split(v[i], h, l);
    out[i] = make_float2(h, l);
  }
}

template <class T>
__device__ __forceinline__ double todbl(T v) { return static_cast<double>(v); }

// Block-wide sum of one double per thread (fixed tree), valid in thread 0.
template <int BS>
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double warp_part[BS / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) warp_part[w] = v;
  __syncthreads();
  double s = 0.0;
  if (w == 0) {
    s = l < BS / 32 ? warp_part[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  __syncthreads();
  return s;
}

// ---------------------------------------------------------------------------
// elementwise
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_fill(T* __restrict__ x, T v, i64 n) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) x[i] = v;
}

template <class A, class B>
__global__ void k_convert(const A* __restrict__ a, B* __restrict__ b, i64 n) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    b[i] = static_cast<B>(a[i]);
}

// ---------------------------------------------------------------------------
// deterministic two-stage reductions
// ---------------------------------------------------------------------------
template <class TA, class TB>
__global__ void __launch_bounds__(kRedThreads) k_dot_partial(const TA* __restrict__ a,
                                                             const TB* __restrict__ b, i64 n,
                                                             double* __restrict__ part) {
  double s = 0.0;
  if constexpr (std::is_same<TA, float>::value && std::is_same<TB, float>::value) {
    // FP32 vectors (the reuse setups' Lanczos): each thread's products summed
    // in FP32 before the FP64 block sum (no per-element FP64 work)
    float sf = 0.0f;
    for (i64 i = blockIdx.x * (i64)kRedThreads + threadIdx.x; i < n; i += (i64)gridDim.x * kRedThreads)
      sf = fmaf(a[i], b[i], sf);
    s = static_cast<double>(sf);
  } else {
    for (i64 i = blockIdx.x * (i64)kRedThreads + threadIdx.x; i < n; i += (i64)gridDim.x * kRedThreads)
      s += todbl(a[i]) * todbl(b[i]);
  }
  s = block_sum<kRedThreads>(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// out = sum(part[0..m)) ; optional sqrt
__global__ void __launch_bounds__(kRedThreads) k_reduce_final(const double* __restrict__ part, int m,
                                                              double* __restrict__ out, int take_sqrt) {
  double s = 0.0;
  for (int i = threadIdx.x; i < m; i += kRedThreads) s += part[i];
  s = block_sum<kRedThreads>(s);
  if (threadIdx.x == 0) *out = take_sqrt ? sqrt(s) : s;
}

// ---------------------------------------------------------------------------
// PCG scalars and vector updates (FP64 CG scalars in device memory)
// ---------------------------------------------------------------------------
struct PcgScalars {
  double rz;       // r^T z of the current direction
  double pq;       // p^T A p
  double alpha, beta;
  double rr;       // ||r||^2 after the update
  double rz_new;
  int status;      // 0 ok, 2 breakdown (p^T A p <= 0 or non-finite)
  int pad;
};

__global__ void __launch_bounds__(kRedThreads) k_pcg_alpha(const double* __restrict__ part, int m,
                                                           PcgScalars* sc) {
  double s = 0.0;
  for (int i = threadIdx.x; i < m; i += kRedThreads) s += part[i];
  s = block_sum<kRedThreads>(s);
  if (threadIdx.x == 0) {
    sc->pq = s;
    if (!(s > 0.0) || !isfinite(s)) {
      sc->status = 2;
      sc->alpha = 0.0;
    } else {
      sc->alpha = sc->rz / s;
    }
  }
}

// rz_new = sum(part); beta = rz_new / rz; rz = rz_new
__global__ void __launch_bounds__(kRedThreads) k_pcg_beta(const double* __restrict__ part, int m,
                                                          PcgScalars* sc) {
  double s = 0.0;
  for (int i = threadIdx.x; i < m; i += kRedThreads) s += part[i];
  s = block_sum<kRedThreads>(s);
  if (threadIdx.x == 0) {
    sc->rz_new = s;
    sc->beta = s / sc->rz;
    sc->rz = s;
  }
}

// x += alpha p ; r -= alpha q ; partial ||r||^2
__global__ void __launch_bounds__(kRedThreads) k_pcg_update(double* __restrict__ x, double* __restrict__ r,
                                                            const double* __restrict__ p,
                                                            const double* __restrict__ q, i64 n,
                                                            const PcgScalars* __restrict__ sc,
                                                            double* __restrict__ part) {
  const double alpha = sc->alpha;
  double s = 0.0;
  for (i64 i = blockIdx.x * (i64)kRedThreads + threadIdx.x; i < n; i += (i64)gridDim.x * kRedThreads) {
    x[i] += alpha * p[i];
    const double ri = r[i] - alpha * q[i];
    r[i] = ri;
    s += ri * ri;
  }
  s = block_sum<kRedThreads>(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// p = z + beta p; with ps, also its double-float split (the next operator
// application's input in mixed precision); with p32, its FP32 copy (the
// input of the matrix-free CG operator)
__global__ void k_pcg_direction(double* __restrict__ p, const double* __restrict__ z, i64 n,
                                const PcgScalars* __restrict__ sc, float2* __restrict__ ps,
                                float* __restrict__ p32) {
  const double beta = sc->beta;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const double v = z[i] + beta * p[i];
    p[i] = v;
    if (ps) {
      float h, l;
      df_split(v, h, l);
      ps[i] = make_float2(h, l);
    }
    if (p32) p32[i] = __double2float_rn(v);
  }
}

// ---------------------------------------------------------------------------
// Chebyshev smoothing (Saad, Alg. 12.1 in D^-1 A; src/fem/Multigrid.cpp:
// 783-855): the operator steps live with the operator kernels (nbspmv.cuh,
// mfree.cuh); the zero-guess start needs no operator.
// ---------------------------------------------------------------------------
// zero guess: d = dinv b / theta ; x = d
template <class TX>
__global__ void k_cheb_zero(i64 n, const TX* __restrict__ b, const TX* __restrict__ dinv,
                            TX* __restrict__ d, TX* __restrict__ x, const TX* __restrict__ inv_theta) {
  const TX it = *inv_theta;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const TX di = dinv[i] * b[i] * it;
    d[i] = di;
    x[i] = di;
  }
}

// ---------------------------------------------------------------------------
// Lanczos pieces (src/fem/Multigrid.cpp:288-327)
// ---------------------------------------------------------------------------
// Lanczos vector kernels (FP64 scalars; vectors in T: FP64, or FP32 in the
// mixed-precision setups whose operator is FP32 anyway).
// w -= a v (a from device memory); block partials of ||w||^2
template <class T>
__global__ void __launch_bounds__(kRedThreads) k_axpy_norm(T* __restrict__ w, const T* __restrict__ v,
                                                           const double* __restrict__ a_dev, i64 n,
                                                           double* __restrict__ part) {
  const double a = *a_dev;
  double s = 0.0;
  if constexpr (std::is_same<T, float>::value) {
    // FP32 vectors: FP32 update, each thread's squares summed in FP32 before
    // the FP64 block sum (no per-element FP64 work)
    const float af = static_cast<float>(a);
    float sf = 0.0f;
    for (i64 i = blockIdx.x * (i64)kRedThreads + threadIdx.x; i < n; i += (i64)gridDim.x * kRedThreads) {
      const float wi = fmaf(-af, v[i], w[i]);
      w[i] = wi;
      sf = fmaf(wi, wi, sf);
    }
    s = static_cast<double>(sf);
  } else {
    for (i64 i = blockIdx.x * (i64)kRedThreads + threadIdx.x; i < n; i += (i64)gridDim.x * kRedThreads) {
      const T wi = static_cast<T>(todbl(w[i]) - a * todbl(v[i]));
      w[i] = wi;
      s += todbl(wi) * todbl(wi);
    }
  }
  s = block_sum<kRedThreads>(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// vp = v ; v = w / b ; tmp = s .* v
// (b from device memory; nothing once the breakdown test has stopped the steps)
template <class T>
__global__ void k_lanczos_shift(T* __restrict__ v, T* __restrict__ vp, const T* __restrict__ w,
                                const T* __restrict__ s, T* __restrict__ tmp,
                                const double* __restrict__ b, const double* __restrict__ stop, i64 n) {
  if (*stop != 0.0) return;
  const double bj = *b;
  if constexpr (std::is_same<T, float>::value) {
    // FP32 vectors: FP32 arithmetic with 1 / beta formed once per block
    __shared__ float inv_b;
    if (threadIdx.x == 0) inv_b = static_cast<float>(1.0 / bj);
    __syncthreads();
    const float ib = inv_b;
    for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
      vp[i] = v[i];
      const float vi = w[i] * ib;
      v[i] = vi;
      tmp[i] = s[i] * vi;
    }
  } else {
    for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
      vp[i] = v[i];
      const T vi = static_cast<T>(todbl(w[i]) / bj);
      v[i] = vi;
      tmp[i] = static_cast<T>(todbl(s[i]) * todbl(vi));
    }
  }
}

// v = v / nrm ; tmp = s .* v ; s = sqrt(dinv)
template <class T>
__global__ void k_lanczos_start(T* __restrict__ v, const double* __restrict__ nrm,
                                const double* __restrict__ dinv, T* __restrict__ s,
                                T* __restrict__ tmp, i64 n) {
  const double inv = *nrm;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const double si = sqrt(dinv[i]);
    s[i] = static_cast<T>(si);
    const double vi = todbl(v[i]) / inv;
    v[i] = static_cast<T>(vi);
    tmp[i] = static_cast<T>(todbl(static_cast<T>(si)) * todbl(static_cast<T>(vi)));
  }
}

// ---------------------------------------------------------------------------
// Setup numerics over node-level patterns
// ---------------------------------------------------------------------------
// 1 / diagonal; status 1 when a diagonal is not positive
template <class TV>
__global__ void k_inv_diag(i32 n, const i32* __restrict__ node_of, const i32* __restrict__ first,
                           const i32* __restrict__ self_slot, NodeView a, const i32* __restrict__ rowptr,
                           const TV* __restrict__ val, double* __restrict__ dinv, int* __restrict__ bad) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const i32 I = node_of[i];
    const i32 li = static_cast<i32>(i) - first[I];
    const double d = static_cast<double>(val[rowptr[i] + a.off[self_slot[I]] + li]);
    if (!(d > 0.0)) {
      atomicMin(bad, static_cast<int>(i));
      dinv[i] = 0.0;
    } else {
      dinv[i] = 1.0 / d;
    }
  }
}

// Block sums of squares per node-level slot (strength of connection,
// src/fem/Multigrid.cpp:460-513): rows of the row node in order, then the
// slot's columns in order.
__global__ void k_block_sumsq(i32 nnodes, const i32* __restrict__ first, NodeView a,
                              const i32* __restrict__ col_first, const i32* __restrict__ rowptr,
                              const double* __restrict__ val, double* __restrict__ acc) {
  for (i64 I = blockIdx.x * (i64)blockDim.x + threadIdx.x; I < nnodes; I += (i64)gridDim.x * blockDim.x) {
    for (i32 t = a.ptr[I]; t < a.ptr[I + 1]; ++t) {
      const i32 J = a.nbr[t];
      const i32 sz = col_first[J + 1] - col_first[J];
      double s = 0.0;
      for (i32 i = first[I]; i < first[I + 1]; ++i) {
        const double* v = val + rowptr[i] + a.off[t];
        for (i32 k = 0; k < sz; ++k) s = xadd(s, xmul(v[k], v[k]));
      }
      acc[t] = s;
    }
  }
}

// P = (I - omega D^-1 A) P-hat over P's node pattern
// (src/fem/Multigrid.cpp:671-716).  One TPR-lane group per fine row.
template <int TPR, class T>
__global__ void __launch_bounds__(256) k_prolongator(
    i32 n, const i32* __restrict__ node_of, const i32* __restrict__ first,
    const i32* __restrict__ first1, const i32* __restrict__ agg, NodeView a,
    const i32* __restrict__ arow, const T* __restrict__ aval, NodeView p,
    const i32* __restrict__ prow, T* __restrict__ pval, const i32* __restrict__ phat_ptr,
    const T* __restrict__ phat, const double* __restrict__ dinv, double omega) {
  const i64 t0 = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 i = static_cast<i32>(t0 / TPR);
  const int lane = static_cast<int>(t0 % TPR);
  if (i >= n) return;
  const i32 I = node_of[i];
  const T scale = static_cast<T>(omega * dinv[i]);
  const i32 aI = agg[I];
  for (i32 s = p.ptr[I] + lane; s < p.ptr[I + 1]; s += TPR) {
    const i32 g = p.nbr[s];
    const i32 rg = first1[g + 1] - first1[g];
    T acc[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
    for (i32 t = a.ptr[I]; t < a.ptr[I + 1]; ++t) {
      const i32 J = a.nbr[t];
      if (agg[J] != g) continue;
      const i32 sJ = first[J + 1] - first[J];
      const T* av = aval + arow[i] + a.off[t];
      for (i32 kb = 0; kb < sJ; ++kb) {
        const T v = av[kb];
        const T* ph = phat + phat_ptr[first[J] + kb];
#pragma unroll
        for (int j = 0; j < 6; ++j)
          if (j < rg) acc[j] = xadd(acc[j], xmul(v, ph[j]));
      }
    }
    T* out = pval + prow[i] + p.off[s];
    const T* own = phat + phat_ptr[i];
#pragma unroll
    for (int j = 0; j < 6; ++j)
      if (j < rg) {
        T v = xmul(acc[j], -scale);
        if (aI == g) v = xadd(v, own[j]);
        out[j] = v;
      }
  }
}

// R = P^T refill: R(c, (I, ka)) = P((I, ka), c)
template <int TPR, class T>
__global__ void __launch_bounds__(256) k_restriction(
    i32 nc, const i32* __restrict__ node_of1, const i32* __restrict__ first1,
    const i32* __restrict__ first, NodeView r, const i32* __restrict__ rrow, T* __restrict__ rval,
    const i32* __restrict__ r_to_p, NodeView p, const i32* __restrict__ prow,
    const T* __restrict__ pval) {
  const i64 t0 = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 c = static_cast<i32>(t0 / TPR);
  const int lane = static_cast<int>(t0 % TPR);
  if (c >= nc) return;
  const i32 g = node_of1[c];
  const i32 lc = c - first1[g];
  for (i32 t = r.ptr[g] + lane; t < r.ptr[g + 1]; t += TPR) {
    const i32 I = r.nbr[t];
    const i32 u = r_to_p[t];
    T* out = rval + rrow[c] + r.off[t];
    for (i32 ka = 0; ka < first[I + 1] - first[I]; ++ka) out[ka] = pval[prow[first[I] + ka] + p.off[u] + lc];
  }
}

// AP = A P over AP's node pattern (multiply_numeric order).
template <int TPR, class T>
__global__ void __launch_bounds__(256) k_product_ap(
    i32 n, const i32* __restrict__ node_of, const i32* __restrict__ first,
    const i32* __restrict__ first1, NodeView a, const i32* __restrict__ arow,
    const T* __restrict__ aval, NodeView p, const i32* __restrict__ prow,
    const T* __restrict__ pval, NodeView ap, const i32* __restrict__ aprow, T* __restrict__ apval) {
  const i64 t0 = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 i = static_cast<i32>(t0 / TPR);
  const int lane = static_cast<int>(t0 % TPR);
  if (i >= n) return;
  const i32 I = node_of[i];
  for (i32 s = ap.ptr[I] + lane; s < ap.ptr[I + 1]; s += TPR) {
    const i32 h = ap.nbr[s];
    const i32 rh = first1[h + 1] - first1[h];
    T acc[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
    for (i32 t = a.ptr[I]; t < a.ptr[I + 1]; ++t) {
      const i32 J = a.nbr[t];
      i32 u = p.ptr[J];
      const i32 ue = p.ptr[J + 1];
      while (u < ue && p.nbr[u] < h) ++u;
      if (u == ue || p.nbr[u] != h) continue;
      const i32 sJ = first[J + 1] - first[J];
      const T* av = aval + arow[i] + a.off[t];
      for (i32 kb = 0; kb < sJ; ++kb) {
        const T v = av[kb];
        const T* pv = pval + prow[first[J] + kb] + p.off[u];
#pragma unroll
        for (int j = 0; j < 6; ++j)
          if (j < rh) acc[j] = xadd(acc[j], xmul(v, pv[j]));
      }
    }
    T* out = apval + aprow[i] + ap.off[s];
#pragma unroll
    for (int j = 0; j < 6; ++j)
      if (j < rh) out[j] = acc[j];
  }
}

// RAW = R (AP) over the coarse node pattern (multiply_numeric order).
template <int TPR, class T>
__global__ void __launch_bounds__(256) k_product_rap(
    i32 nc, const i32* __restrict__ node_of1, const i32* __restrict__ first1,
    const i32* __restrict__ first, NodeView r, const i32* __restrict__ rrow,
    const T* __restrict__ rval, NodeView ap, const i32* __restrict__ aprow,
    const T* __restrict__ apval, NodeView c, const i32* __restrict__ crow, T* __restrict__ cval) {
  const i64 t0 = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  const i32 row = static_cast<i32>(t0 / TPR);
  const int lane = static_cast<int>(t0 % TPR);
  if (row >= nc) return;
  const i32 g = node_of1[row];
  for (i32 s = c.ptr[g] + lane; s < c.ptr[g + 1]; s += TPR) {
    const i32 h = c.nbr[s];
    const i32 rh = first1[h + 1] - first1[h];
    T acc[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
    for (i32 t = r.ptr[g]; t < r.ptr[g + 1]; ++t) {
      const i32 I = r.nbr[t];
      i32 u = ap.ptr[I];
      const i32 ue = ap.ptr[I + 1];
      while (u < ue && ap.nbr[u] < h) ++u;
      if (u == ue || ap.nbr[u] != h) continue;
      const i32 sI = first[I + 1] - first[I];
      const T* rv = rval + rrow[row] + r.off[t];
      for (i32 ka = 0; ka < sI; ++ka) {
        const T v = rv[ka];
        const T* apv = apval + aprow[first[I] + ka] + ap.off[u];
#pragma unroll
        for (int j = 0; j < 6; ++j)
          if (j < rh) acc[j] = xadd(acc[j], xmul(v, apv[j]));
      }
    }
    T* out = cval + crow[row] + c.off[s];
#pragma unroll
    for (int j = 0; j < 6; ++j)
      if (j < rh) out[j] = acc[j];
  }
}

// A_c = (RAW + RAW^T) / 2 on the (structurally symmetric) coarse pattern.
template <class T, class TO>
__global__ void k_symmetrize(i32 nc, const i32* __restrict__ node_of1, const i32* __restrict__ first1,
                             NodeView c, const i32* __restrict__ crow, const i32* __restrict__ tslot,
                             const T* __restrict__ raw, TO* __restrict__ out, double* __restrict__ out64) {
  for (i64 row = blockIdx.x * (i64)blockDim.x + threadIdx.x; row < nc; row += (i64)gridDim.x * blockDim.x) {
    const i32 g = node_of1[row];
    const i32 lc = static_cast<i32>(row) - first1[g];
    for (i32 s = c.ptr[g]; s < c.ptr[g + 1]; ++s) {
      const i32 h = c.nbr[s];
      const i32 st = tslot[s];
      const i32 base = crow[row] + c.off[s];
      for (i32 j = 0; j < first1[h + 1] - first1[h]; ++j) {
        const T a = raw[base + j];
        const T b = raw[crow[first1[h] + j] + c.off[st] + lc];
        const T v = xmul(T(0.5), xadd(a, b));
        out[base + j] = static_cast<TO>(v);
        if (out64) out64[base + j] = static_cast<double>(v);
      }
    }
  }
}

}  // namespace
}  // namespace simp
