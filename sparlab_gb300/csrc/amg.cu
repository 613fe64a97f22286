// GPU SA-AMG hierarchy, V-cycle and PCG (see amg.h).  Setup steps follow
// AmgPreconditioner::setup (src/fem/Multigrid.cpp:929-1111); the cycle
// follows Impl::cycle (:857-885) and Impl::smooth (:783-855); PCG follows
// pcg_solve (:1152-1237).
#include "amg.h"
#include "autotune.h"
#include "dense.cuh"
#include "galerkin.cuh"
#include "kernels.cuh"
#include "mfree.cuh"
#include "mfree_tc.cuh"
#include "nbspmv.cuh"

#include <cuda_profiler_api.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <thread>
#include <cmath>
#include <mutex>
#include <sstream>
#include <type_traits>
#include <unordered_map>

namespace simp {

std::atomic<int64_t> g_launches{0};
thread_local int64_t t_launches = 0;

void raise_dynamic_smem(const void* kernel, size_t bytes) {
  static std::mutex m;
  static std::unordered_map<const void*, size_t> limits;
  std::lock_guard<std::mutex> lock(m);
  size_t& cur = limits[kernel];
  if (bytes <= cur) return;
  SIMP_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)));
  cur = bytes;
}

void DevPattern::upload(const NodePattern& p, cudaStream_t s) {
  ptr.upload(p.ptr, s);
  nbr.upload(p.nbr, s);
  off.upload(p.off, s);
}

__global__ void k_expand_columns(i32 n, const i32* __restrict__ node_of, NodeView p,
                                 const i32* __restrict__ col_first, const i32* __restrict__ rowptr,
                                 i32* __restrict__ col) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const i32 I = node_of[i];
    i32 k = rowptr[i];
    for (i32 t = p.ptr[I]; t < p.ptr[I + 1]; ++t) {
      const i32 J = p.nbr[t];
      for (i32 c = col_first[J]; c < col_first[J + 1]; ++c) col[k++] = c;
    }
  }
}

namespace {

// w = s .* w - beta vp (beta from device memory); nothing once stopped.
// FP64 vectors: FP64 arithmetic; FP32 vectors (the reuse setups): FP32
// arithmetic, with beta rounded to FP32 (GB300 runs FP64 at 1/64 of the
// FP32 rate, so conversions and FP64 operations per element would bound
// these vector passes)
template <class T>
__global__ void k_lanczos_finish(T* __restrict__ w, const T* __restrict__ s, const T* __restrict__ vp,
                                 const double* __restrict__ beta, const double* __restrict__ stop, i64 n) {
  if (*stop != 0.0) return;
  const double bj = vp ? *beta : 0.0;
  if constexpr (std::is_same<T, float>::value) {
    const float bf = static_cast<float>(bj);
    for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
      float wi = w[i] * s[i];
      if (vp) wi = fmaf(-bf, vp[i], wi);
      w[i] = wi;
    }
  } else {
    for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
      double wi = todbl(w[i]) * todbl(s[i]);
      if (vp) wi -= bj * todbl(vp[i]);
      w[i] = static_cast<T>(wi);
    }
  }
}

// The reference's breakdown test of step j: stop when beta_j <= 1e-12 |alpha_j|
__global__ void k_lanczos_check(const double* __restrict__ ab, int j, double* __restrict__ stop) {
  if (threadIdx.x == 0 && blockIdx.x == 0 && !(ab[2 * j + 1] > 1.0e-12 * fabs(ab[2 * j]))) *stop = 1.0;
}

// Every operator application runs the VS-lanes-per-row kernels of
// nbspmv.cuh; (VS, B) come from the operator's shape: B = the uniform width of
// its column nodes (column-free decode) or 0, VS = the lanes per row chosen
// for the arithmetic type.
template <class TA, class F>
void with_shape(const NbOp& op, F&& f) {
  auto lanes = [&](auto b) {
    switch (std::is_same<TA, double>::value ? op.lanes64 : op.lanes32) {
      case 32: f(std::integral_constant<int, 32>{}, b); break;
      case 8: f(std::integral_constant<int, 8>{}, b); break;
      default: f(std::integral_constant<int, 4>{}, b); break;
    }
  };
  switch (op.block) {
    case 2: lanes(std::integral_constant<int, 2>{}); break;
    case 3: lanes(std::integral_constant<int, 3>{}); break;
    case 6: lanes(std::integral_constant<int, 6>{}); break;
    default: lanes(std::integral_constant<int, 0>{}); break;
  }
}

// The double-float operator's shape: its own lanes per row (2, 4 or 8) and
// the column-node width.
template <class F>
void with_shape_df(const NbOp& op, F&& f) {
  auto lanes = [&](auto b) {
    switch (op.lanes_df) {
      case 2: f(std::integral_constant<int, 2>{}, b); break;
      case 8: f(std::integral_constant<int, 8>{}, b); break;
      default: f(std::integral_constant<int, 4>{}, b); break;
    }
  };
  switch (op.block) {
    case 2: lanes(std::integral_constant<int, 2>{}); break;
    case 3: lanes(std::integral_constant<int, 3>{}); break;
    case 6: lanes(std::integral_constant<int, 6>{}); break;
    default: lanes(std::integral_constant<int, 0>{}); break;
  }
}

// One thread per (row, lane); no grid-stride loop in the row kernels.
unsigned rows_grid(const NbOp& op, int vs) {
  const i64 blocks = (static_cast<i64>(op.rows) * vs + 255) / 256;
  return static_cast<unsigned>(std::max<i64>(blocks, 1));
}

template <int MODE, class TV, class TX, class TA>
void nb_apply(const NbOp& op, const TV* val, const TX* x, TX* y, const TX* b, cudaStream_t s) {
  with_shape<TA>(op, [&](auto vs, auto blk) {
    constexpr int VS = decltype(vs)::value, B = decltype(blk)::value;
    k_rows_apply<VS, B, MODE, TV, TX, TA><<<rows_grid(op, VS), 256, 0, s>>>(
        op.node_of, op.pat, op.rowptr, op.col, val, x, y, b, op.rows);
  });
  SIMP_CHECK_LAUNCH();
}

template <class T>
void nb_cheb_step(const NbOp& op, const T* val, const T* d, const T* rin, T* r, T* dn, T* x, const T* dinv,
                  const T* c12, int add_d, cudaStream_t s) {
  with_shape<T>(op, [&](auto vs, auto blk) {
    constexpr int VS = decltype(vs)::value, B = decltype(blk)::value;
    k_rows_cheb_step<VS, B, T><<<rows_grid(op, VS), 256, 0, s>>>(
        op.rows, op.node_of, op.pat, op.rowptr, op.col, val, d, rin, r, dn, x, dinv, c12, add_d);
  });
  SIMP_CHECK_LAUNCH();
}

template <class T>
void nb_cheb_first(const NbOp& op, const T* val, const T* x, const T* b, T* r, T* d, const T* dinv,
                   const T* inv_theta, cudaStream_t s) {
  with_shape<T>(op, [&](auto vs, auto blk) {
    constexpr int VS = decltype(vs)::value, B = decltype(blk)::value;
    k_rows_cheb_first<VS, B, T><<<rows_grid(op, VS), 256, 0, s>>>(
        op.rows, op.node_of, op.pat, op.rowptr, op.col, val, x, b, r, d, dinv, inv_theta);
  });
  SIMP_CHECK_LAUNCH();
}

// Width B of every column node (node J's unknowns at B*J .. B*J+B-1), or 0:
// the column-free decode of nbspmv.cuh needs it.
int uniform_block(const std::vector<i32>& col_first) {
  for (int b : {6, 3, 2}) {
    bool ok = !col_first.empty();
    for (size_t J = 0; ok && J < col_first.size(); ++J) ok = col_first[J] == b * static_cast<i32>(J);
    if (ok) return b;
  }
  return 0;
}

// Lanes per row: FP64 products are arithmetic bound on GB300 (1/64 of the
// FP32 rate), so FP64 rows get few lanes and short reductions; FP32 rows are
// bandwidth bound and get 8 lanes (one 32-byte sector per step) or a whole
// warp for long rows.
template <class T>
int row_lanes(const DevCsr& c) {
  const i64 avg = c.rows > 0 ? c.nnz / c.rows : 0;
  if (std::is_same<T, double>::value) return avg > 100 ? 8 : 4;
  // short rows (the prolongators, ~30 values): 4 lanes put twice the rows in
  // flight per warp, which the per-row index chain (row -> node -> slots ->
  // x) needs to hide its latency (P_0 at 192x96x96: 93 against 150 us)
  return avg >= 256 ? 32 : (avg >= 64 ? 8 : 4);
}

// Per-precision views of a level's arrays.
template <class T>
struct V;
template <>
struct V<double> {
  static const double* a(const DevCsr& c) { return c.v64.p; }
  static double* x(LevelWork& l) { return l.x64.p; }
  static double* b(LevelWork& l) { return l.b64.p; }
  static double* r(LevelWork& l) { return l.r64.p; }
  static double* d(LevelWork& l) { return l.d64.p; }
  static double* e(LevelWork& l) { return l.e64.p; }
  static const double* dinv(Level& l) { return l.dinv64.p; }
  static const double* cheb(Level& l) { return l.cheb64.p; }
};
template <>
struct V<float> {
  static const float* a(const DevCsr& c) { return c.v32.p; }
  static float* x(LevelWork& l) { return l.x32.p; }
  static float* b(LevelWork& l) { return l.b32.p; }
  static float* r(LevelWork& l) { return l.r32.p; }
  static float* d(LevelWork& l) { return l.d32.p; }
  static float* e(LevelWork& l) { return l.e32.p; }
  static const float* dinv(Level& l) { return l.dinv32.p; }
  static const float* cheb(Level& l) { return l.cheb32.p; }
};

template <class A, class B>
void convert(const A* a, B* b, i64 n, cudaStream_t s) {
  k_convert<A, B><<<grid_for(n, 256, 4096), 256, 0, s>>>(a, b, n);
  SIMP_CHECK_LAUNCH();
}

MfView mf_view(const MfOp& o) {
  MfView v;
  v.dim = o.dim;
  v.nx = o.nx;
  v.ny = o.ny;
  v.nz = o.nz;
  v.nnx = o.nnx;
  v.nny = o.nny;
  v.gnode = o.gnode;
  v.nindex = o.nindex;
  v.ke = o.ke;
  v.scale = o.scale;
  return v;
}

template <int MODE>
void mf3_64(const MfOp& mf, const double* x, double* y, const double* b, cudaStream_t s) {
  const dim3 grid((mf.nnx + kTX - 1) / kTX, (mf.nny + kTY - 1) / kTY, (mf.nz + 1 + kTZ * kNZ - 1) / (kTZ * kNZ));
  KeF64 ke;
  std::copy(mf.ke64_host, mf.ke64_host + 24 * 24, ke.k);
  k_mf3_tile64<MODE><<<grid, kTX * kTY * kTZ, 0, s>>>(mf_view(mf), mf.scale64, x, y, b, ke);
  SIMP_CHECK_LAUNCH();
}

template <int MODE, int TX, int TY, int TZ>
void mf3_shape(const MfOp& mf, const MfArgs& a, const KeF32& ke, cudaStream_t s, bool v4) {
  const dim3 grid((mf.nnx + TX - 1) / TX, (mf.nny + TY - 1) / TY, (mf.nz + 1 + TZ - 1) / TZ);
  if (v4) k_mf3_tile<MODE, TX, TY, TZ, true><<<grid, TX * TY * TZ, 0, s>>>(mf_view(mf), a, ke);
  else k_mf3_tile<MODE, TX, TY, TZ, false><<<grid, TX * TY * TZ, 0, s>>>(mf_view(mf), a, ke);
  SIMP_CHECK_LAUNCH();
}

// The tensor-core kernel: CTAs of 31 x 7 node columns, each marching
// `layers` node layers (mf.tc_layers; every chunking gives the same values).
template <int MODE>
void mf3_tc(const MfOp& mf, const MfArgs& a, const KeF32& ke, cudaStream_t s) {
  const i32 nnz = mf.nz + 1;
  const int layers = mf.tc_layers > 0 ? std::min<i32>(mf.tc_layers, nnz) : nnz;
  const dim3 grid((mf.nnx + kTcNodesX - 1) / kTcNodesX, (mf.nny + kTcNodesY - 1) / kTcNodesY,
                  (nnz + layers - 1) / layers);
  raise_dynamic_smem(reinterpret_cast<const void*>(&k_mf3_tc<MODE>), kTcSmemBytes);
  k_mf3_tc<MODE><<<grid, kTcThreads, kTcSmemBytes, s>>>(mf_view(mf), a, ke, layers, mf.status);
  SIMP_CHECK_LAUNCH();
}

// The tiled matrix-free kernel in the variant the tuner chose for the mode
// (mf.tile[MODE]: shape kMfTileShape[tile % 5], float4 halo for tile >= 5;
// every variant gives the same values), or the
// tensor-core kernel (mf.tensor).
template <int MODE>
void mf3(const MfOp& mf, const MfArgs& a, cudaStream_t s) {
  KeF32 ke;
  std::copy(mf.ke_host, mf.ke_host + 24 * 24, ke.k);
  if (mf.tensor) {
    mf3_tc<MODE>(mf, a, ke, s);
    return;
  }
  static_assert(kMfTiles == 10, "tile table");
  const int tile = mf.tile[MODE];
  const bool v4 = tile >= 5;
  switch (tile % 5) {
    case 1: mf3_shape<MODE, 32, 8, 1>(mf, a, ke, s, v4); break;
    case 2: mf3_shape<MODE, 32, 2, 4>(mf, a, ke, s, v4); break;
    case 3: mf3_shape<MODE, 64, 2, 2>(mf, a, ke, s, v4); break;
    case 4: mf3_shape<MODE, 32, 4, 1>(mf, a, ke, s, v4); break;
    default: mf3_shape<MODE, 32, 4, 2>(mf, a, ke, s, v4); break;
  }
}

// Matrix-free level-0 pieces of the FP32 cycle (tiled in 3-D).
void mf_cheb_first(const MfOp& mf, i32 nodes, const float* x, const float* b, float* r, float* d,
                   const float* dinv, const float* inv_theta, cudaStream_t s) {
  if (mf.dim == 3) {
    MfArgs a{};
    a.x = x;
    a.b = b;
    a.r = r;
    a.dn = d;
    a.dinv = dinv;
    a.coef = inv_theta;
    mf3<4>(mf, a, s);
    return;
  }
  k_mf_cheb_first<<<grid_for(nodes, 256), 256, 0, s>>>(mf_view(mf), nodes, x, b, r, d, dinv, inv_theta);
  SIMP_CHECK_LAUNCH();
}

void mf_cheb_step(const MfOp& mf, i32 nodes, const float* d, const float* rin, float* r, float* dn, float* x,
                  const float* dinv, const float* c12, int add_d, cudaStream_t s) {
  if (mf.dim == 3) {
    MfArgs a{};
    a.x = d;
    a.b = rin;
    a.r = r;
    a.dn = dn;
    a.xs = x;
    a.dinv = dinv;
    a.coef = c12;
    a.add_d = add_d;
    mf3<3>(mf, a, s);
    return;
  }
  k_mf_cheb_step<<<grid_for(nodes, 256), 256, 0, s>>>(mf_view(mf), nodes, d, rin, r, dn, x, dinv, c12, add_d);
  SIMP_CHECK_LAUNCH();
}

void mf_apply(const MfOp& mf, i32 nodes, const float* x, float* y, cudaStream_t s) {
  if (mf.dim == 3) {
    MfArgs a{};
    a.x = x;
    a.y = y;
    mf3<0>(mf, a, s);
    return;
  }
  k_mf_apply<0, float><<<grid_for(nodes, 256), 256, 0, s>>>(mf_view(mf), nodes, x, y, nullptr);
  SIMP_CHECK_LAUNCH();
}

void mf_residual(const MfOp& mf, i32 nodes, const float* x, float* r, const float* b, cudaStream_t s) {
  if (mf.dim == 3) {
    MfArgs a{};
    a.x = x;
    a.y = r;
    a.b = b;
    mf3<1>(mf, a, s);
    return;
  }
  k_mf_apply<1, float><<<grid_for(nodes, 256), 256, 0, s>>>(mf_view(mf), nodes, x, r, b);
  SIMP_CHECK_LAUNCH();
}

// Level-0 transfers of the FP32 cycle without the stored R and P
// (3-D tiled operator): with P = (I - w D^-1 A) P^ and A, D symmetric,
//   restriction  b_c = P^T (r - w A D^-1 r)   from x and b (r = b - A x),
//   prolongation x  += t - w D^-1 A t,  t = P^ x_c.
// u and t are scratch vectors of the level (n floats).
void mf_restrict(const MfOp& mf, const Level& lv, const float* x, const float* b, float* r, float* u, float* bc,
                 cudaStream_t s) {
  MfArgs a{};
  a.x = x;
  a.b = b;
  a.y = r;
  a.dn = u;
  a.dinv = lv.dinv32.p;
  mf3<6>(mf, a, s);
  MfArgs c{};
  c.x = u;
  c.b = r;
  c.y = r;
  c.coef = lv.omega32.p;
  mf3<7>(mf, c, s);
  const i64 th = static_cast<i64>(lv.naggs) * 32;
  k_phat_restrict<6><<<grid_for(th, 256), 256, 0, s>>>(lv.naggs, lv.d_members_ptr.p, lv.d_members.p,
                                                         lv.phat_ptr.p, lv.phat32.p, r, bc);
  SIMP_CHECK_LAUNCH();
}

void mf_prolong(const MfOp& mf, const Level& lv, const float* xc, float* t, float* x, cudaStream_t s) {
  k_phat_prolong<6><<<grid_for(lv.n, 256), 256, 0, s>>>(lv.n, lv.d_agg.p, lv.phat_ptr.p, lv.phat32.p, xc, t);
  SIMP_CHECK_LAUNCH();
  MfArgs a{};
  a.x = t;
  a.xs = x;
  a.dinv = lv.dinv32.p;
  a.coef = lv.omega32.p;
  mf3<5>(mf, a, s);
}

// Node layers per CTA of the tensor-core matrix-free kernel: chunkings of
// the z march for about 2 (variant 0), 4, 1 or 8 CTAs per SM.
constexpr int kTcChunkings = 4;
int tc_layers_of(const MfOp& mf, int variant) {
  int dev = 0, sms = 0;
  SIMP_CUDA(cudaGetDevice(&dev));
  SIMP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const i64 nnz = mf.nz + 1;
  const i64 xy = static_cast<i64>((mf.nnx + kTcNodesX - 1) / kTcNodesX) * ((mf.nny + kTcNodesY - 1) / kTcNodesY);
  static const int per_sm[kTcChunkings] = {2, 4, 1, 8};
  i64 chunks = std::max<i64>(1, (static_cast<i64>(per_sm[variant]) * sms + xy / 2) / xy);
  chunks = std::min(chunks, nnz);
  return static_cast<int>((nnz + chunks - 1) / chunks);
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

// Each context owns a stream, so contexts driven from different host threads
// (independent problem instances) run concurrently.  It is a blocking
// stream: work on the legacy default stream (one-time uploads, a caller's
// own kernels on device pointers it passes in) stays ordered with it.
GpuAmg::GpuAmg(const AmgOptions& o) : opt(o) {
  SIMP_CUDA(cudaStreamCreate(&stream));
  part.alloc(kRedBlocks);
  scal.alloc(16);
  dstatus.alloc(4);
  mf_status.alloc(1);
  SIMP_CUDA(cudaMemset(mf_status.p, 0, sizeof(int)));
  main_.stream = stream;
}

void GpuAmg::check_mf_status(cudaStream_t s) {
  if (!mf.tensor) return;
  int h = 0;
  SIMP_CUDA(cudaMemcpyAsync(&h, mf_status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  SIMP_CUDA(cudaStreamSynchronize(s));
  if (h != 0) {
    SIMP_CUDA(cudaMemsetAsync(mf_status.p, 0, sizeof(int), s));
    throw Error(kCudaError, "matrix-free tensor-core operator: an MMA completion wait ran out");
  }
}

GpuAmg::~GpuAmg() {
  together_forget(this);
  extra_.clear();
  if (stream) {
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
  }
}

SolveWork::~SolveWork() {
  if (body) cudaGraphExecDestroy(body);
  if (own_stream && stream) {
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
  }
}

SolveWork& GpuAmg::work(int k) {
  if (k == 0) return main_;
  while (static_cast<int>(extra_.size()) < k) {
    std::unique_ptr<SolveWork> w(new SolveWork());
    SIMP_CUDA(cudaStreamCreate(&w->stream));
    w->own_stream = true;
    extra_.push_back(std::move(w));
  }
  return *extra_[static_cast<size_t>(k - 1)];
}

// FP32 vector of length n, zero-filled when (re)allocated
void GpuAmg::alloc32(DBuf<float>& v, i64 n, cudaStream_t s) {
  if (v.n == static_cast<size_t>(n) && v.p) return;
  v.alloc(static_cast<size_t>(n));
  SIMP_CUDA(cudaMemsetAsync(v.p, 0, sizeof(float) * n, s));
}

// Sizes a workspace for the current hierarchy (nothing is reallocated while
// the sizes stay the same).
void GpuAmg::ensure(SolveWork& w) {
  w.lv.resize(levels.size());
  for (size_t l = 0; l < levels.size(); ++l) {
    const i64 n = levels[l]->n;
    LevelWork& v = w.lv[l];
    if (mixed()) {
      for (DBuf<float>* b : {&v.x32, &v.b32, &v.r32, &v.d32, &v.e32}) alloc32(*b, n, w.stream);
    } else {
      for (DBuf<double>* b : {&v.x64, &v.b64, &v.r64, &v.d64, &v.e64}) b->alloc(static_cast<size_t>(n));
    }
  }
  const size_t n0 = levels.empty() ? 0 : static_cast<size_t>(levels.front()->n);
  w.part.alloc(kRedBlocks);
  w.scal.alloc(16);
  for (DBuf<double>* b : {&w.pr, &w.pz, &w.pp, &w.pq}) b->alloc(n0);
  if (mixed()) w.xsplit.alloc(n0);
}

Level& GpuAmg::level0() {
  if (levels.empty()) levels.emplace_back(new Level());
  return *levels.front();
}

double GpuAmg::dot(SolveWork& w, const double* a, const double* b, i64 n) {
  // the context's own workspace uses the context's reduction buffers, so a
  // dot works before ensure() (setup's Lanczos)
  double* pt = &w == &main_ ? part.p : w.part.p;
  double* sc = &w == &main_ ? scal.p : w.scal.p;
  k_dot_partial<double, double><<<kRedBlocks, kRedThreads, 0, w.stream>>>(a, b, n, pt);
  SIMP_CHECK_LAUNCH();
  k_reduce_final<<<1, kRedThreads, 0, w.stream>>>(pt, kRedBlocks, sc, 0);
  SIMP_CHECK_LAUNCH();
  double h = 0.0;
  SIMP_CUDA(cudaMemcpyAsync(&h, sc, sizeof(double), cudaMemcpyDeviceToHost, w.stream));
  SIMP_CUDA(cudaStreamSynchronize(w.stream));
  return h;
}

void GpuAmg::make_ops(size_t l) {
  Level& lv = *levels[l];
  lv.opA.nodes = lv.nnodes;
  lv.opA.row_first = lv.d_first.p;
  lv.opA.pat = lv.d_apat.view();
  lv.opA.rowptr = lv.a.ptr.p;
  lv.opA.col = lv.a.col.p;
  lv.opA.block = uniform_block(lv.first);
  lv.opA.node_of = lv.d_node_of.p;
  lv.opA.rows = lv.n;
  lv.opA.lanes32 = row_lanes<float>(lv.a);
  lv.opA.lanes64 = row_lanes<double>(lv.a);
  if (l + 1 < levels.size()) {
    Level& nv = *levels[l + 1];
    lv.opP.nodes = lv.nnodes;
    lv.opP.row_first = lv.d_first.p;
    lv.opP.pat = lv.d_ppat.view();
    lv.opP.rowptr = lv.p.ptr.p;
    lv.opP.col = lv.p.col.p;
    lv.opP.block = uniform_block(nv.first);
    lv.opP.node_of = lv.d_node_of.p;
    lv.opP.rows = lv.n;
    lv.opP.lanes32 = row_lanes<float>(lv.p);
    lv.opP.lanes64 = row_lanes<double>(lv.p);
    lv.opR.nodes = nv.nnodes;
    lv.opR.row_first = nv.d_first.p;
    lv.opR.pat = lv.d_rpat.view();
    lv.opR.rowptr = lv.r.ptr.p;
    lv.opR.col = lv.r.col.p;
    lv.opR.block = uniform_block(lv.first);
    lv.opR.node_of = nv.d_node_of.p;
    lv.opR.rows = nv.n;
    lv.opR.lanes32 = row_lanes<float>(lv.r);
    lv.opR.lanes64 = row_lanes<double>(lv.r);
  }
}

void GpuAmg::op0(SolveWork& w, const double* x, double* y, const double* rhs, bool split_ready) {
  Level& l0 = *levels.front();
  const NbOp& op = l0.opA;
  const cudaStream_t stream = w.stream;
  if (mf_cg()) {  // the FP64 matrix-free product (true residuals)
    if (rhs) mf3_64<1>(mf, x, y, rhs, stream);
    else mf3_64<0>(mf, x, y, nullptr, stream);
    return;
  }
  if (!mixed()) {
    if (rhs) nb_apply<1, double, double, double>(op, l0.a.v64.p, x, y, rhs, stream);
    else nb_apply<0, double, double, double>(op, l0.a.v64.p, x, y, nullptr, stream);
    return;
  }
  w.xsplit.alloc(static_cast<size_t>(l0.n));
  float2* xsplit = w.xsplit.p;
  if (!split_ready) {
    k_split_pairs<<<grid_for(l0.n, 256, 8192), 256, 0, stream>>>(l0.n, x, xsplit);
    SIMP_CHECK_LAUNCH();
  }
  df_apply(xsplit, y, rhs, stream);
}

// The double-float level-0 product, row by row (k_rows_apply_df), with the
// tuned unroll (df_unroll_: 4 or 8 row steps in flight per lane, the same
// bits).
void GpuAmg::df_apply(const float2* xsplit, double* y, const double* rhs, cudaStream_t stream) {
  df_apply_unroll(xsplit, y, rhs, stream, df_unroll_);
}

void GpuAmg::df_apply_unroll(const float2* xsplit, double* y, const double* rhs, cudaStream_t stream, int unroll) {
  Level& l0 = *levels.front();
  const NbOp& op = l0.opA;
  with_shape_df(op, [&](auto vs, auto blk) {
    constexpr int VS = decltype(vs)::value, B = decltype(blk)::value;
    const unsigned grid = rows_grid(op, VS);
    auto go = [&](auto ur) {
      constexpr int U = decltype(ur)::value;
      if (rhs)
        k_rows_apply_df<VS, B, 1, U><<<grid, 256, 0, stream>>>(op.node_of, op.pat, op.rowptr, op.col, l0.a.v2.p,
                                                               xsplit, y, rhs, op.rows);
      else
        k_rows_apply_df<VS, B, 0, U><<<grid, 256, 0, stream>>>(op.node_of, op.pat, op.rowptr, op.col, l0.a.v2.p,
                                                               xsplit, y, nullptr, op.rows);
    };
    if (unroll == 8) go(std::integral_constant<int, 8>{});
    else go(std::integral_constant<int, 4>{});
  });
  SIMP_CHECK_LAUNCH();
}

// The double-float operator's unroll for this level 0: the faster of 4 and
// 8 row steps in flight per lane on y = A x (the same bits), before the
// first CUDA graph capture of a structure.
void GpuAmg::tune_df() {
  if (!mixed() || mf_cg()) return;
  Level& l0 = *levels.front();
  const i32 n = l0.n;
  DBuf<float2> xs(static_cast<size_t>(n));
  DBuf<double> ys(static_cast<size_t>(n));
  SIMP_CUDA(cudaMemsetAsync(xs.p, 0, sizeof(float2) * n, stream));
  std::ostringstream key;
  key << "df0:" << n << "x" << l0.a.nnz << "x" << l0.opA.lanes_df;
  const int v = tune_pick(key.str(), 2, [&](int c) { df_apply_unroll(xs.p, ys.p, nullptr, stream, c ? 8 : 4); },
                          stream, 0, 5);
  df_unroll_ = v ? 8 : 4;
  SIMP_CUDA(cudaStreamSynchronize(stream));
}

cudaGraphNode_t GpuAmg::add_op0_multi(cudaGraph_t g, const std::vector<SolveWork*>& ws,
                                      const std::vector<cudaGraphNode_t>& deps) {
  Level& l0 = *levels.front();
  const NbOp& op = l0.opA;
  MultiRhs m{};
  m.n = static_cast<int>(ws.size());
  for (size_t k = 0; k < ws.size() && k < static_cast<size_t>(kMaxRhs); ++k) {
    m.x[k] = ws[k]->xsplit.p;
    m.y[k] = ws[k]->pq.p;
    m.active[k] = ws[k]->loop.p;
  }
  cudaGraphNode_t node = nullptr;
  with_shape_df(op, [&](auto vs, auto blk) {
    constexpr int VS = decltype(vs)::value, B = decltype(blk)::value;
    const i32* node_of = op.node_of;
    NodeView pat = op.pat;
    const i32* rowptr = op.rowptr;
    const i32* col = op.col;
    const float2* v = l0.a.v2.p;
    i32 rows = op.rows;
    void* args[] = {&node_of, &pat, &rowptr, &col, &v, &m, &rows};
    cudaGraphNodeParams kp = {};
    kp.type = cudaGraphNodeTypeKernel;
    kp.kernel.func = reinterpret_cast<void*>(&k_rows_apply_df_multi<VS, B>);
    kp.kernel.gridDim = dim3(rows_grid(op, VS));
    kp.kernel.blockDim = dim3(256);
    kp.kernel.sharedMemBytes = 0;
    kp.kernel.kernelParams = args;
    kp.kernel.extra = nullptr;
    SIMP_CUDA(cudaGraphAddNode(&node, g, deps.data(), nullptr, deps.size(), &kp));
  });
  return node;
}

void GpuAmg::spmv0_fast(const double* x, double* y) {
  Level& l0 = *levels.front();
  if (!mixed()) {
    op0(work(0), x, y, nullptr);
    return;
  }
  const i32 n = l0.n;
  LevelWork& v = work(0).lv.front();  // the cycle's level-0 vectors are free between solves
  convert(x, v.d32.p, n, stream);
  if (mf.enabled) {
    mf_apply(mf, l0.nnodes, v.d32.p, v.e32.p, stream);
  } else {
    nb_apply<0, float, float, float>(l0.opA, l0.a.v32.p, v.d32.p, v.e32.p, nullptr, stream);
  }
  convert(v.e32.p, y, n, stream);
}

void GpuAmg::cg_op(SolveWork& w, const double* p, double* q, bool p32_ready) {
  if (!mf_cg()) {
    op0(w, p, q, nullptr, p32_ready);
    return;
  }
  const i32 n = levels.front()->n;
  w.p32.alloc(static_cast<size_t>(n));
  if (!p32_ready) convert(p, w.p32.p, n, w.stream);
  MfArgs a{};
  a.x = w.p32.p;
  a.y64 = q;
  mf3<8>(mf, a, w.stream);
}

void GpuAmg::apply_values0(SolveWork& w, const double* values, const double* x, double* y) {
  nb_apply<0, double, double, double>(levels.front()->opA, values, x, y, nullptr, w.stream);
}

// CUDA-event time of the level-0 CG operator (op0: FP64 values in fp64
// mode, double-float values in mixed mode) on this context's stream, and its
// compulsory bytes (8 per value either way).
void GpuAmg::time_operator(int reps, double* ms, double* bytes) {
  if (!ready_) throw Error(kBadInput, "the operator is built by the first setup");
  Level& l0 = *levels.front();
  const i32 n = l0.n;
  DBuf<double> x64(n), y64(n);
  k_fill<double><<<grid_for(n, 256), 256, 0, stream>>>(x64.p, 1.0, n);
  SIMP_CHECK_LAUNCH();
  // In mixed mode the CG writes the operand's hi/lo split inside its
  // direction update, so the operator kernel runs alone: split once here and
  // time the operator kernel the same way.
  op0(main_, x64.p, y64.p, nullptr);
  auto launch = [&]() { op0(main_, x64.p, y64.p, nullptr, true); };
  for (int k = 0; k < 3; ++k) launch();
  // the timed launches are the profiler's capture window when one is attached
  cudaProfilerStart();
  cudaEvent_t e0, e1;
  SIMP_CUDA(cudaEventCreate(&e0));
  SIMP_CUDA(cudaEventCreate(&e1));
  SIMP_CUDA(cudaEventRecord(e0, stream));
  for (int k = 0; k < reps; ++k) launch();
  SIMP_CUDA(cudaEventRecord(e1, stream));
  SIMP_CUDA(cudaEventSynchronize(e1));
  cudaProfilerStop();
  float t = 0.0f;
  SIMP_CUDA(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = t / std::max(reps, 1);
  // values, then the index data the kernel reads: one slot record per block
  // with the column-free decode (else a column per value), row pointers,
  // row -> node map and node pointers; then x once and y once
  const double index = l0.opA.block > 0 ? static_cast<double>(l0.apat.slots()) * 4.0
                                        : static_cast<double>(l0.a.nnz) * 4.0;
  *bytes = static_cast<double>(l0.a.nnz) * 8.0 + index + static_cast<double>(n + 1) * 4.0 +
           static_cast<double>(n) * 4.0 + static_cast<double>(l0.nnodes + 1) * 4.0 + 2.0 * static_cast<double>(n) * 8.0;
}

void GpuAmg::refresh_level0_fp32() {
  Level& l0 = *levels.front();
  l0.a.v32.alloc(static_cast<size_t>(l0.a.nnz));
  l0.a.v2.alloc(static_cast<size_t>(l0.a.nnz));
  k_split_values_pairs<<<grid_for(l0.a.nnz, 256, 8192), 256, 0, stream>>>(l0.a.nnz, l0.a.v64.p, l0.a.v32.p,
                                                                           l0.a.v2.p);
  SIMP_CHECK_LAUNCH();
}

template <class T>
struct LzBufs;
template <>
struct LzBufs<double> {
  static DBuf<double>* get(Level& l) { return l.lz; }
};
template <>
struct LzBufs<float> {
  static DBuf<float>* get(Level& l) { return l.lz32; }
};

// The m Lanczos steps of a level (Multigrid.cpp:288-327).  T = double: FP64
// vectors and operator.  T = float (the FP32 reuse setups): FP32 vectors and
// the FP32 operator the smoother uses (matrix-free on a structured level 0),
// with the scalars and the sums of the dot products in FP64.
template <class T>
void GpuAmg::lanczos(size_t l, int m, double* ab) {
  Level& lv = *levels[l];
  const i32 n = lv.n;
  double* stop = ab + 2 * m;
  DBuf<T>* bufs = LzBufs<T>::get(lv);
  for (int k = 0; k < 5; ++k) bufs[k].alloc(static_cast<size_t>(n));
  T* v = bufs[0].p;
  T* vp = bufs[1].p;
  T* w = bufs[2].p;
  T* s = bufs[3].p;
  T* tmp = bufs[4].p;
  if constexpr (std::is_same<T, double>::value)
    SIMP_CUDA(cudaMemcpyAsync(v, lv.lz_start.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
  else
    convert(lv.lz_start.p, v, n, stream);
  k_lanczos_start<T><<<grid_for(n, 256), 256, 0, stream>>>(v, scal.p + 1, lv.dinv64.p, s, tmp, n);
  SIMP_CHECK_LAUNCH();
  for (int j = 0; j < m; ++j) {
    if constexpr (std::is_same<T, float>::value) {
      if (l == 0 && mf.enabled) mf_apply(mf, lv.nnodes, tmp, w, stream);
      else nb_apply<0, float, float, float>(lv.opA, lv.a.v32.p, tmp, w, nullptr, stream);
    } else {
      nb_apply<0, double, double, double>(lv.opA, lv.a.v64.p, tmp, w, nullptr, stream);
    }
    k_lanczos_finish<T><<<grid_for(n, 256), 256, 0, stream>>>(w, s, j > 0 ? vp : nullptr,
                                                             j > 0 ? ab + 2 * j - 1 : nullptr, stop, n);
    SIMP_CHECK_LAUNCH();
    k_dot_partial<T, T><<<kRedBlocks, kRedThreads, 0, stream>>>(w, v, n, part.p);
    SIMP_CHECK_LAUNCH();
    k_reduce_final<<<1, kRedThreads, 0, stream>>>(part.p, kRedBlocks, ab + 2 * j, 0);
    SIMP_CHECK_LAUNCH();
    if (j + 1 == m) break;  // beta of the last step is not used
    k_axpy_norm<T><<<kRedBlocks, kRedThreads, 0, stream>>>(w, v, ab + 2 * j, n, part.p);
    SIMP_CHECK_LAUNCH();
    k_reduce_final<<<1, kRedThreads, 0, stream>>>(part.p, kRedBlocks, ab + 2 * j + 1, 1);
    SIMP_CHECK_LAUNCH();
    k_lanczos_check<<<1, 32, 0, stream>>>(ab, j, stop);
    SIMP_CHECK_LAUNCH();
    k_lanczos_shift<T><<<grid_for(n, 256), 256, 0, stream>>>(v, vp, w, s, tmp, ab + 2 * j + 1, stop, n);
    SIMP_CHECK_LAUNCH();
  }
}

// inverse diagonal and lambda_max(D^-1 A) of one level (Multigrid.cpp:718-747)
void GpuAmg::numeric_level(size_t l) {
  Level& lv = *levels[l];
  const i32 n = lv.n;
  const bool fp32 = mixed() && ready_ && lv.a.v32.p != nullptr;
  make_ops(l);
  lv.dinv64.alloc(n);
  SIMP_CUDA(cudaMemsetAsync(dstatus.p, 0x7f, sizeof(int), stream));
  if (fp32)
    k_inv_diag<float><<<grid_for(n, 256), 256, 0, stream>>>(n, lv.d_node_of.p, lv.d_first.p, lv.d_self.p,
                                                            lv.d_apat.view(), lv.a.ptr.p, lv.a.v32.p, lv.dinv64.p,
                                                            dstatus.p);
  else
    k_inv_diag<double><<<grid_for(n, 256), 256, 0, stream>>>(n, lv.d_node_of.p, lv.d_first.p, lv.d_self.p,
                                                             lv.d_apat.view(), lv.a.ptr.p, lv.a.v64.p, lv.dinv64.p,
                                                             dstatus.p);
  SIMP_CHECK_LAUNCH();
  // the diagonal's status is read with the Lanczos coefficients below (one
  // host round trip per level); a bad diagonal only makes them garbage
  if (mixed()) {
    lv.dinv32.alloc(n);
    convert(lv.dinv64.p, lv.dinv32.p, n, stream);
  }
  // Lanczos on D^-1/2 A D^-1/2 with the reference's start vector (its norm
  // made once per size); alpha_j, beta_j stay in device memory (lz_ab_[2j],
  // [2j+1]; [2m] = the stop flag of the breakdown test): the steps after a
  // breakdown change nothing, and the host reads all coefficients once
  if (lv.lz_start.n != static_cast<size_t>(n)) {
    std::vector<double> h(static_cast<size_t>(n));
    for (i32 i = 0; i < n; ++i) h[i] = 1.0 + 0.5 * std::sin(1.7 * static_cast<double>(i) + 0.3);
    lv.lz_start.upload(h, stream);
    lv.lz_norm = std::sqrt(dot(lv.lz_start.p, lv.lz_start.p, n));
  }
  const int m = std::max(1, std::min<int>(opt.lanczos_steps, n));
  lz_ab_.alloc(static_cast<size_t>(2 * m + 1));
  double* ab = lz_ab_.p;
  SIMP_CUDA(cudaMemsetAsync(ab + 2 * m, 0, sizeof(double), stream));
  SIMP_CUDA(cudaMemcpyAsync(scal.p + 1, &lv.lz_norm, sizeof(double), cudaMemcpyHostToDevice, stream));
  if (fp32) lanczos<float>(l, m, ab);
  else lanczos<double>(l, m, ab);
  int bad = 0;
  std::vector<double> hab(static_cast<size_t>(2 * m));
  SIMP_CUDA(cudaMemcpyAsync(hab.data(), ab, sizeof(double) * 2 * m, cudaMemcpyDeviceToHost, stream));
  SIMP_CUDA(cudaMemcpyAsync(&bad, dstatus.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
  SIMP_CUDA(cudaStreamSynchronize(stream));
  if (bad != 0x7f7f7f7f) {
    std::ostringstream os;
    os << "multigrid level " << l << ": diagonal entry " << bad
       << " is not positive; a stiffness matrix must have a positive diagonal. The model has an "
          "unconnected degree of freedom or a non-positive stiffness";
    throw Error(kBreakdown, os.str());
  }
  std::vector<double> alpha, beta;
  for (int j = 0; j < m; ++j) {
    const double aj = hab[2 * j], bj = hab[2 * j + 1];
    alpha.push_back(aj);
    if (j + 1 == m || !(bj > 1.0e-12 * std::abs(aj))) break;
    beta.push_back(bj);
  }
  std::vector<double> off(beta.begin(), beta.begin() + static_cast<long>(alpha.size() - 1));
  lv.lambda = tridiagonal_max_eigenvalue(alpha, off);
  if (!(lv.lambda > 0.0) || !std::isfinite(lv.lambda)) {
    std::ostringstream os;
    os << "multigrid level " << l << ": the spectral estimate of D^-1 A is " << lv.lambda
       << "; the matrix is not positive definite";
    throw Error(kBreakdown, os.str());
  }
  // Chebyshev coefficients on [lambda / ratio, 1.1 lambda] (Multigrid.cpp:812-853)
  const double upper = 1.1 * lv.lambda, lower = upper / opt.cheb_ratio;
  const double theta = 0.5 * (upper + lower), delta = 0.5 * (upper - lower);
  const double sigma = theta / delta;
  double rho = 1.0 / sigma;
  lv.inv_theta = 1.0 / theta;
  lv.c1.clear();
  lv.c2.clear();
  for (int k = 1; k < opt.degree; ++k) {
    const double rn = 1.0 / (2.0 * sigma - rho);
    lv.c1.push_back(rn * rho);
    lv.c2.push_back(2.0 * rn / delta);
    rho = rn;
  }
  // the kernels read them from device memory: [1 / theta, c1_0, c2_0, ...,
  // 0, 0] (the closing pair is the degree-1 step's)
  std::vector<double> coef{lv.inv_theta};
  for (size_t k = 0; k < lv.c1.size(); ++k) {
    coef.push_back(lv.c1[k]);
    coef.push_back(lv.c2[k]);
  }
  coef.push_back(0.0);
  coef.push_back(0.0);
  const std::vector<float> coef32(coef.begin(), coef.end());
  lv.cheb64.upload(coef, stream);
  lv.cheb32.upload(coef32, stream);
  const std::vector<float> omega{static_cast<float>(opt.damping / lv.lambda)};
  lv.omega32.upload(omega, stream);
}

// Aggregates, tentative prolongator and symbolic patterns of level l -> l+1.
// Returns with levels[l+1] created, or leaves the hierarchy unchanged when
// coarsening stalls.
void GpuAmg::build_transfer(size_t l) {
  Level& lv = *levels[l];
  // strength of connection from the FP64 values (block sums of squares)
  DBuf<double> acc(static_cast<size_t>(lv.apat.slots()));
  k_block_sumsq<<<grid_for(lv.nnodes, 128), 128, 0, stream>>>(lv.nnodes, lv.d_first.p, lv.d_apat.view(),
                                                               lv.d_first.p, lv.a.ptr.p, lv.a.v64.p, acc.p);
  SIMP_CHECK_LAUNCH();
  const std::vector<double> hacc = acc.to_host(stream);
  const std::vector<i32> self = pattern_self_slots(lv.apat);
  std::vector<double> bdiag(static_cast<size_t>(lv.nnodes));
  for (i32 I = 0; I < lv.nnodes; ++I) bdiag[I] = self[I] >= 0 ? std::sqrt(hacc[self[I]]) : 0.0;
  lv.naggs = aggregate_nodes(lv.apat, hacc, bdiag, opt.theta, lv.agg);
  const int m = static_cast<int>(lv.null.size() / std::max<i32>(lv.n, 1));
  Tentative t = tentative_prolongator(lv.first, lv.agg, lv.naggs, lv.null, m);
  const i32 nc = t.next_first.back();
  if (nc >= static_cast<i32>(0.85 * static_cast<double>(lv.n)) || nc == 0) {
    lv.agg.clear();
    lv.naggs = 0;
    return;
  }
  std::unique_ptr<Level> nx(new Level());
  Level& nv = *nx;
  nv.first = std::move(t.next_first);
  nv.nnodes = lv.naggs;
  nv.n = nc;
  nv.null = std::move(t.next_null);
  nv.d_first.upload(nv.first, stream);
  nv.d_node_of.upload(node_of_unknowns(nv.first), stream);
  lv.d_agg.upload(lv.agg, stream);
  lv.phat_ptr.upload(t.phat_ptr, stream);
  lv.phat64.upload(t.phat, stream);
  if (mixed()) {
    lv.phat32.alloc(t.phat.size());
    convert(lv.phat64.p, lv.phat32.p, static_cast<i64>(t.phat.size()), stream);
  }
  lv.mf_transfer = false;
  if (mixed() && l == 0 && uniform_block(lv.first) == 3 && uniform_block(nv.first) == 6) {
    std::vector<i32> mptr(static_cast<size_t>(lv.naggs) + 1, 0), members(static_cast<size_t>(lv.nnodes));
    bool all = true;
    for (i32 I = 0; I < lv.nnodes; ++I) {
      if (lv.agg[I] < 0) all = false;
      else ++mptr[lv.agg[I] + 1];
    }
    if (all) {
      for (i32 g = 0; g < lv.naggs; ++g) mptr[g + 1] += mptr[g];
      std::vector<i32> fill(mptr.begin(), mptr.end() - 1);
      for (i32 I = 0; I < lv.nnodes; ++I) members[fill[lv.agg[I]]++] = I;
      lv.d_members_ptr.upload(mptr, stream);
      lv.d_members.upload(members, stream);
      lv.mf_transfer = true;
    }
  }
  // symbolic patterns
  lv.ppat = pattern_prolongator(lv.apat, lv.agg, lv.naggs);
  finish_offsets(lv.ppat, nv.first);
  if (mixed()) {
    // contributors of each P slot: the A slots t of the same row node whose
    // neighbour lies in the slot's aggregate, ascending (k_prolongator_gather)
    std::vector<i32> pc_ptr(static_cast<size_t>(lv.ppat.slots()) + 1, 0), count;
    std::vector<int2> pc_t;
    pc_t.reserve(static_cast<size_t>(lv.apat.slots()));
    for (i32 I = 0; I < lv.apat.rows; ++I) {
      const i32 p0 = lv.ppat.ptr[I], ns = lv.ppat.ptr[I + 1] - p0;
      const i32* pn = lv.ppat.nbr.data() + p0;
      count.assign(static_cast<size_t>(ns) + 1, 0);
      auto slot_of = [&](i32 g) { return static_cast<i32>(std::lower_bound(pn, pn + ns, g) - pn); };
      for (i32 sa = lv.apat.ptr[I]; sa < lv.apat.ptr[I + 1]; ++sa) {
        const i32 g = lv.agg[lv.apat.nbr[sa]];
        if (g >= 0) ++count[slot_of(g) + 1];
      }
      for (i32 s = 0; s < ns; ++s) count[s + 1] += count[s];
      const size_t base = pc_t.size();
      pc_t.resize(base + count[ns]);
      std::vector<i32> fill(count.begin(), count.end() - 1);
      for (i32 sa = lv.apat.ptr[I]; sa < lv.apat.ptr[I + 1]; ++sa) {
        const i32 J = lv.apat.nbr[sa];
        const i32 g = lv.agg[J];
        if (g >= 0) pc_t[base + fill[slot_of(g)]++] = make_int2(lv.apat.off[sa], t.phat_ptr[lv.first[J]]);
      }
      for (i32 s = 0; s < ns; ++s) pc_ptr[p0 + s + 1] = static_cast<i32>(base + count[s + 1]);
    }
    lv.d_pc_ptr.upload(pc_ptr, stream);
    lv.d_pc.upload(pc_t, stream);
  }
  std::vector<i32> r_to_p;
  lv.rpat = pattern_transpose(lv.ppat, &r_to_p);
  finish_offsets(lv.rpat, lv.first);
  lv.appat = pattern_product(lv.apat, lv.ppat);
  finish_offsets(lv.appat, nv.first);
  nv.apat = pattern_product(lv.rpat, lv.appat);
  finish_offsets(nv.apat, nv.first);
  const std::vector<i32> sym_t = pattern_transpose_slots(nv.apat);
  // shared-memory shapes of the warp-per-node products: accumulator rows,
  // output slots, and (slot, inner slot) pairs per chunk of left slots
  auto shape = [](const NodePattern& out, const std::vector<i32>& row_first, const NodePattern& left,
                  const NodePattern* inner) {
    WarpRows w;
    for (i32 I = 0; I < out.rows; ++I) {
      const i64 acc = static_cast<i64>(row_first[I + 1] - row_first[I]) * out.rowlen[I];
      w.acc = static_cast<int>(std::max<i64>(w.acc, std::min<i64>(acc, 1 << 30)));
      w.slots = std::max(w.slots, out.ptr[I + 1] - out.ptr[I]);
    }
    if (inner)
      for (i32 I = 0; I < left.rows; ++I)
        for (i32 t0 = left.ptr[I]; t0 < left.ptr[I + 1]; t0 += kChunk) {
          int pairs = 0;
          for (i32 t = t0; t < std::min(t0 + kChunk, left.ptr[I + 1]); ++t)
            pairs += inner->ptr[left.nbr[t] + 1] - inner->ptr[left.nbr[t]];
          w.inner = std::max(w.inner, pairs);
        }
    return w;
  };
  lv.wr_p = shape(lv.ppat, lv.first, lv.apat, nullptr);
  lv.wr_ap = shape(lv.appat, lv.first, lv.apat, &lv.ppat);
  lv.wr_rap = shape(nv.apat, nv.first, lv.rpat, &lv.appat);
  lv.d_ppat.upload(lv.ppat, stream);
  lv.d_rpat.upload(lv.rpat, stream);
  lv.d_appat.upload(lv.appat, stream);
  nv.d_apat.upload(nv.apat, stream);
  lv.d_r_to_p.upload(r_to_p, stream);
  lv.d_sym_t.upload(sym_t, stream);
  nv.d_self.upload(pattern_self_slots(nv.apat), stream);
  // scalar CSR structures
  auto make = [&](DevCsr& c, const NodePattern& pat, const std::vector<i32>& row_first,
                  const std::vector<i32>& col_first, const DBuf<i32>& row_node_of, const DevPattern& dpat,
                  const DBuf<i32>& d_col_first) {
    const std::vector<i32> ptr = scalar_rowptr(pat, row_first);
    c.rows = row_first.back();
    c.cols = col_first.back();
    c.nnz = ptr.back();
    c.ptr.upload(ptr, stream);
    c.col.alloc(static_cast<size_t>(c.nnz));
    k_expand_columns<<<grid_for(c.rows, 256), 256, 0, stream>>>(c.rows, row_node_of.p, dpat.view(),
                                                                d_col_first.p, c.ptr.p, c.col.p);
    SIMP_CHECK_LAUNCH();
    c.v64.alloc(static_cast<size_t>(c.nnz));
    if (mixed()) c.v32.alloc(static_cast<size_t>(c.nnz));
  };
  make(lv.p, lv.ppat, lv.first, nv.first, lv.d_node_of, lv.d_ppat, nv.d_first);
  make(lv.r, lv.rpat, nv.first, lv.first, nv.d_node_of, lv.d_rpat, lv.d_first);
  make(lv.ap, lv.appat, lv.first, nv.first, lv.d_node_of, lv.d_appat, nv.d_first);
  make(nv.a, nv.apat, nv.first, nv.first, nv.d_node_of, nv.d_apat, nv.d_first);
  lv.raw64.alloc(static_cast<size_t>(nv.a.nnz));
  if (mixed()) lv.raw32.alloc(static_cast<size_t>(nv.a.nnz));
  levels.push_back(std::move(nx));
}

// Launches a warp-per-row-node product with its shared-memory shape; false
// (nothing launched) when one warp's accumulator would not fit.
template <class T, class... KArgs, class... Args>
bool launch_rows(const char* name, void (*kernel)(i32, WarpRows, KArgs...), i32 nodes, const WarpRows& w,
                 cudaStream_t s, Args... args) {
  const size_t per_warp =
      static_cast<size_t>(w.acc) * sizeof(T) + static_cast<size_t>(2 * w.slots + kMetaInts + w.inner) * 4;
  if (per_warp > 200 * 1024) return false;
  // variants: at most 8, 4 or 2 warps (row nodes) per block within a 96 KB
  // (variant 0: the untuned launch) or 192 KB shared-memory budget; a row
  // node's products run in one warp in the same order in every variant
  auto launch = [&](int v) {
    static constexpr int kMaxWarps[4] = {8, 4, 2, 8};
    const size_t budget = v == 3 ? 192 * 1024 : 96 * 1024;
    const int warps = static_cast<int>(
        std::min<size_t>(static_cast<size_t>(kMaxWarps[v]), std::max<size_t>(1, budget / per_warp)));
    const size_t smem = per_warp * warps;
    if (smem > 48 * 1024) raise_dynamic_smem(reinterpret_cast<const void*>(kernel), smem);
    const i64 blocks = std::max<i64>(1, std::min<i64>((static_cast<i64>(nodes) + warps - 1) / warps, 152 * 64));
    kernel<<<static_cast<unsigned>(blocks), warps * 32, smem, s>>>(nodes, w, args...);
    SIMP_CHECK_LAUNCH();
  };
  std::ostringstream key;
  key << name << (sizeof(T) == 4 ? "32:" : "64:") << nodes << "x" << w.acc << "x" << w.slots;
  launch(tune_pick(key.str(), 4, launch, s, 0));
  return true;
}

// Numeric P, R, AP, RAP and symmetrisation (Multigrid.cpp:671-716, 1047-1055).
template <class T>
static void galerkin_t(GpuAmg& g, Level& lv, Level& nv, bool last, cudaStream_t stream) {
  const bool f32 = sizeof(T) == 4;
  auto A = [&](DevCsr& c) -> T* { return f32 ? reinterpret_cast<T*>(c.v32.p) : reinterpret_cast<T*>(c.v64.p); };
  const T* phat = f32 ? reinterpret_cast<const T*>(lv.phat32.p) : reinterpret_cast<const T*>(lv.phat64.p);
  T* raw = f32 ? reinterpret_cast<T*>(lv.raw32.p) : reinterpret_cast<T*>(lv.raw64.p);
  const double omega = g.opt.damping / lv.lambda;
  const int b1 = uniform_block(nv.first);
  constexpr bool kExact = std::is_same<T, double>::value;
  const int bf = uniform_block(lv.first);
  auto gather = [&](auto kernel) {
    const i64 blocks = std::max<i64>(1, std::min<i64>((static_cast<i64>(lv.nnodes) * 32 + 255) / 256, 152 * 64));
    kernel<<<static_cast<unsigned>(blocks), 256, 0, stream>>>(lv.nnodes, lv.d_agg.p, lv.a.ptr.p, A(lv.a),
                                                              lv.d_ppat.view(), lv.p.ptr.p, A(lv.p), lv.phat_ptr.p,
                                                              phat, lv.dinv64.p, omega, lv.d_pc_ptr.p, lv.d_pc.p);
    SIMP_CHECK_LAUNCH();
  };
  // FP32 reuse setups take the gather form (3.7 % of a 192x96x96 iteration
  // faster, same bits); the exact FP64 products stay on the warp kernel,
  // which is the faster of the two with rounded operations
  if (!kExact && bf == 3 && b1 == 6) {
    gather(k_prolongator_gather<T, kExact, 3, 6>);
  } else if (!kExact && bf == 2 && b1 == 3) {
    gather(k_prolongator_gather<T, kExact, 2, 3>);
  } else if (!kExact && bf == 6 && b1 == 6) {
    gather(k_prolongator_gather<T, kExact, 6, 6>);
  } else if (!kExact && bf == 3 && b1 == 3) {
    gather(k_prolongator_gather<T, kExact, 3, 3>);
  } else if (!launch_rows<T>("prolongator_rows", k_prolongator_rows<T, kExact>, lv.nnodes, lv.wr_p, stream,
                             lv.d_first.p, nv.d_first.p,
                             lv.d_agg.p, lv.d_apat.view(), lv.a.ptr.p, A(lv.a), lv.d_ppat.view(), lv.p.ptr.p,
                             A(lv.p), lv.phat_ptr.p, phat, lv.dinv64.p, omega)) {
    const i64 th = static_cast<i64>(lv.n) * 8;
    k_prolongator<8, T><<<grid_for(th, 256), 256, 0, stream>>>(
        lv.n, lv.d_node_of.p, lv.d_first.p, nv.d_first.p, lv.d_agg.p, lv.d_apat.view(), lv.a.ptr.p, A(lv.a),
        lv.d_ppat.view(), lv.p.ptr.p, A(lv.p), lv.phat_ptr.p, phat, lv.dinv64.p, omega);
    SIMP_CHECK_LAUNCH();
  }
  {
    const i64 th = static_cast<i64>(nv.n) * 32;
    k_restriction<32, T><<<grid_for(th, 256), 256, 0, stream>>>(
        nv.n, nv.d_node_of.p, nv.d_first.p, lv.d_first.p, lv.d_rpat.view(), lv.r.ptr.p, A(lv.r), lv.d_r_to_p.p,
        lv.d_ppat.view(), lv.p.ptr.p, A(lv.p));
    SIMP_CHECK_LAUNCH();
  }
  auto ap_rows = [&](auto kernel) {
    return launch_rows<T>("ap_rows", kernel, lv.nnodes, lv.wr_ap, stream, lv.d_first.p, lv.d_apat.view(), lv.a.ptr.p,
                          A(lv.a),
                          lv.d_ppat.view(), lv.p.ptr.p, A(lv.p), lv.d_appat.view(), lv.ap.ptr.p, A(lv.ap));
  };
  auto rap_rows = [&](auto kernel) {
    return launch_rows<T>("rap_rows", kernel, nv.nnodes, lv.wr_rap, stream, nv.d_first.p, lv.d_first.p,
                          lv.d_rpat.view(),
                          lv.r.ptr.p, A(lv.r), lv.d_appat.view(), lv.ap.ptr.p, A(lv.ap), nv.d_apat.view(),
                          nv.a.ptr.p, raw);
  };
  // compile-time node widths for the common shapes: 3-D level 0 (3 -> 6),
  // coarse 3-D (6 -> 6), 2-D level 0 (2 -> 3), coarse 2-D (3 -> 3)
  constexpr bool X = std::is_same<T, double>::value;
  const int b0 = uniform_block(lv.first);
  const bool ap_done = (b0 == 3 && b1 == 6)   ? ap_rows(k_ap_rows<T, X, 3, 6>)
                       : (b0 == 6 && b1 == 6) ? ap_rows(k_ap_rows<T, X, 6, 6>)
                       : (b0 == 2 && b1 == 3) ? ap_rows(k_ap_rows<T, X, 2, 3>)
                       : (b0 == 3 && b1 == 3) ? ap_rows(k_ap_rows<T, X, 3, 3>)
                                              : ap_rows(k_ap_rows<T, X, 0, 0>);
  if (!ap_done) {
    const i64 th = static_cast<i64>(lv.n) * 32;
    k_product_ap<32, T><<<grid_for(th, 256), 256, 0, stream>>>(
        lv.n, lv.d_node_of.p, lv.d_first.p, nv.d_first.p, lv.d_apat.view(), lv.a.ptr.p, A(lv.a),
        lv.d_ppat.view(), lv.p.ptr.p, A(lv.p), lv.d_appat.view(), lv.ap.ptr.p, A(lv.ap));
    SIMP_CHECK_LAUNCH();
  }
  const bool rap_done = (b1 == 6 && b0 == 3)   ? rap_rows(k_rap_rows<T, X, 6, 3>)
                        : (b1 == 6 && b0 == 6) ? rap_rows(k_rap_rows<T, X, 6, 6>)
                        : (b1 == 3 && b0 == 2) ? rap_rows(k_rap_rows<T, X, 3, 2>)
                        : (b1 == 3 && b0 == 3) ? rap_rows(k_rap_rows<T, X, 3, 3>)
                                               : rap_rows(k_rap_rows<T, X, 0, 0>);
  if (!rap_done) {
    const i64 th = static_cast<i64>(nv.n) * 32;
    k_product_rap<32, T><<<grid_for(th, 256), 256, 0, stream>>>(
        nv.n, nv.d_node_of.p, nv.d_first.p, lv.d_first.p, lv.d_rpat.view(), lv.r.ptr.p, A(lv.r),
        lv.d_appat.view(), lv.ap.ptr.p, A(lv.ap), nv.d_apat.view(), nv.a.ptr.p, raw);
    SIMP_CHECK_LAUNCH();
  }
  // FP64 copy of the coarse operator where the FP64 path or the coarse
  // factorisation needs it
  double* out64 = (!f32 || last) ? nv.a.v64.p : nullptr;
  k_symmetrize<T, T><<<grid_for(nv.n, 128), 128, 0, stream>>>(nv.n, nv.d_node_of.p, nv.d_first.p, nv.d_apat.view(),
                                                              nv.a.ptr.p, lv.d_sym_t.p, raw, A(nv.a), f32 ? out64 : nullptr);
  SIMP_CHECK_LAUNCH();
}

void GpuAmg::galerkin(size_t l, bool fp32) {
  Level& lv = *levels[l];
  Level& nv = *levels[l + 1];
  const bool last = l + 2 == levels.size();
  if (fp32) {
    galerkin_t<float>(*this, lv, nv, last, stream);
  } else {
    galerkin_t<double>(*this, lv, nv, last, stream);
    if (mixed()) {
      convert(lv.p.v64.p, lv.p.v32.p, lv.p.nnz, stream);
      convert(lv.r.v64.p, lv.r.v32.p, lv.r.nnz, stream);
      convert(nv.a.v64.p, nv.a.v32.p, nv.a.nnz, stream);
    }
  }
}

// Dense FP64 inverse of the coarsest operator by the blocked symmetric sweep
// (dense.cuh), with the squared Cholesky pivots as the singularity check.
void GpuAmg::coarse_factorize() {
  Level& lv = *levels.back();
  const i32 n = lv.n;
  if (n > 16000) {
    std::ostringstream os;
    os << "multigrid: the coarsest level has " << n
       << " unknowns, beyond the dense direct solve (16000); raise max_levels";
    throw Error(kBadInput, os.str());
  }
  nc_ = n;
  const size_t nn = static_cast<size_t>(n) * n;
  dense_.alloc(nn);
  swept_.alloc(nn);
  piv_.alloc(n);
  panel_.alloc(2 * static_cast<size_t>(n) * kNB + kNB * kNB);
  double* pu = panel_.p;
  double* pv = pu + static_cast<size_t>(n) * kNB;
  double* pp = pv + static_cast<size_t>(n) * kNB;
  SIMP_CUDA(cudaMemsetAsync(swept_.p, 0, nn * sizeof(double), stream));
  k_dense_from_csr<<<grid_for(n, 128), 128, 0, stream>>>(n, lv.a.ptr.p, lv.a.col.p, lv.a.v64.p, swept_.p);
  SIMP_CHECK_LAUNCH();
  SIMP_CUDA(cudaMemsetAsync(dstatus.p, 0, sizeof(int), stream));
  const int nt = (n + kNB - 1) / kNB;
  const dim3 tiles(nt, nt);
  for (int k0 = 0; k0 < n; k0 += kNB) {
    const int kb = std::min(kNB, n - k0);
    k_sweep_pivot<false><<<(n + kSweepRows - 1) / kSweepRows, 256, 0, stream>>>(swept_.p, n, k0, kb, pu, pv,
                                                                                 pp, piv_.p, dstatus.p);
    SIMP_CHECK_LAUNCH();
    k_sweep_update<<<tiles, 256, 0, stream>>>(swept_.p, n, k0, kb, pu, pv, pp);
    SIMP_CHECK_LAUNCH();
  }
  int status = 0;
  SIMP_CUDA(cudaMemcpyAsync(&status, dstatus.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
  const std::vector<double> piv = piv_.to_host(stream);
  double mx = 0.0, mn = std::numeric_limits<double>::max();
  for (double v : piv) {
    mx = std::max(mx, std::abs(v));
    mn = std::min(mn, v);
  }
  const double ratio = mx > 0.0 ? mn / mx : 0.0;
  stats.pivot_ratio = ratio;
  if (status != 0 || !(ratio > opt.pivot_tol)) {
    std::ostringstream os;
    os << "multigrid: the coarsest operator (" << n << " unknowns) is singular or indefinite "
       << "(smallest / largest pivot " << ratio << "). A rigid-body mode survived to the coarse "
       << "level, so the model is under-constrained: too few supports, or a part connected to nothing";
    throw Error(kUnderConstrained, os.str());
  }
  k_sweep_finish<<<tiles, 256, 0, stream>>>(swept_.p, dense_.p, n);
  SIMP_CHECK_LAUNCH();
}

// x = A_c^-1 b at the coarsest level: one GEMV with the FP64 inverse
template <class T>
void GpuAmg::coarse_solve(SolveWork& w, size_t l) {
  const int n = nc_;
  const i64 th = static_cast<i64>(n) * 32;
  LevelWork& v = w.lv[l];
  k_gemv<T, T><<<grid_for(th, 256), 256, 0, w.stream>>>(dense_.p, n, V<T>::b(v), V<T>::x(v));
  SIMP_CHECK_LAUNCH();
}

void GpuAmg::setup(bool structure_changed) {
  const auto t0 = std::chrono::steady_clock::now();
  const bool reuse = opt.reuse && !structure_changed && ready_;
  if (mf.enabled) {
    mf.status = mf_status.p;
    mf.tensor = mf.dim == 3 && opt.tensor_cores != 0;
    if (mf.tensor && mf.tc_layers <= 0) mf.tc_layers = tc_layers_of(mf, 0);
  }
  if (!reuse) {
    while (levels.size() > 1) levels.pop_back();
    Level& l0 = *levels.front();
    l0.agg.clear();
    l0.naggs = 0;
    ready_ = false;
  }
  // Reused structure in mixed mode: FP32 numerics; a new structure is set up
  // in FP64 so the aggregates come from the FP64 values.
  const bool fp32 = mixed() && reuse;
  if (mixed() && !level0_fp32_fresh) refresh_level0_fp32();
  level0_fp32_fresh = false;
  const size_t reused_levels = levels.size();
  size_t l = 0;
  while (true) {
    numeric_level(l);
    Level& lv = *levels[l];
    const bool stop = reuse ? (l + 1 == reused_levels)
                            : (lv.n <= opt.coarse_size || static_cast<int>(l) + 1 >= opt.max_levels);
    if (stop) break;
    if (!reuse) {
      build_transfer(l);
      if (levels.size() == l + 1) break;  // coarsening stalled
    }
    galerkin(l, fp32);
    ++l;
  }
  levels.resize(l + 1);
  for (size_t k = 0; k < levels.size(); ++k) make_ops(k);
  coarse_factorize();
  ensure(main_);
  for (auto& w : extra_) ensure(*w);
  if (!reuse) {
    tune_level0();
    tune_df();
  }
  ready_ = true;
  // captured iteration bodies stay valid across reuse setups: their launches
  // take only workspace and level pointers, which a reuse setup keeps
  if (!reuse) ++epoch_;
  stats.reused = reuse;
  compute_stats();
  SIMP_CUDA(cudaStreamSynchronize(stream));
  stats.setup_seconds = seconds_since(t0);
}

// The matrix-free operator's launch shape for this grid: the fastest of the
// shapes in kMfTileShape (FMA kernel) or of the z-chunkings of the tensor-
// core kernel, on y = A x with the current cell scales (each family gives
// the same values in every shape).  Before the first CUDA graph capture of a
// structure.
void GpuAmg::tune_level0() {
  if (!(mf.enabled && mf.dim == 3) || !mf.scale) return;
  const i32 n = levels.front()->n;
  DBuf<float> tx(static_cast<size_t>(n)), ty(static_cast<size_t>(n));
  k_fill<float><<<grid_for(n, 256), 256, 0, stream>>>(tx.p, 1.0f, n);
  SIMP_CHECK_LAUNCH();
  if (mf.tensor) {
    std::ostringstream key;
    key << "mf3tc:" << mf.nnx << "x" << mf.nny << "x" << (mf.nz + 1);
    const int v = tune_pick(key.str(), kTcChunkings,
                            [&](int c) {
                              MfOp m = mf;
                              m.tc_layers = tc_layers_of(mf, c);
                              MfArgs a{};
                              a.x = tx.p;
                              a.y = ty.p;
                              mf3<0>(m, a, stream);
                            },
                            stream, 0, 5);
    mf.tc_layers = tc_layers_of(mf, v);
    check_mf_status(stream);
    return;
  }
  // each mode's epilogue reads and writes different vectors: tune each one
  // on scratch vectors (the values do not matter to the timing)
  DBuf<float> tb(static_cast<size_t>(n)), tr(static_cast<size_t>(n)), td(static_cast<size_t>(n)),
      ts(static_cast<size_t>(n)), coef(2);
  DBuf<double> t64(static_cast<size_t>(n));
  for (DBuf<float>* v : {&tb, &tr, &td, &ts})
    k_fill<float><<<grid_for(n, 256), 256, 0, stream>>>(v->p, 1.0f, n);
  k_fill<float><<<1, 32, 0, stream>>>(coef.p, 0.5f, 2);
  SIMP_CHECK_LAUNCH();
  MfArgs a{};
  a.x = tx.p;
  a.y = ty.p;
  a.b = tb.p;
  a.r = tr.p;
  a.dn = td.p;
  a.xs = ts.p;
  a.dinv = tb.p;
  a.coef = coef.p;
  a.y64 = t64.p;
  auto tune_mode = [&](int mode, auto launch) {
    std::ostringstream key;
    key << "mf3:" << mf.nnx << "x" << mf.nny << "x" << (mf.nz + 1) << ":m" << mode;
    mf.tile[mode] = tune_pick(key.str(), kMfTiles,
                              [&](int v) {
                                MfOp m = mf;
                                m.tile[mode] = v;
                                launch(m);
                              },
                              stream, 0, 5);
  };
  tune_mode(0, [&](const MfOp& m) { mf3<0>(m, a, stream); });
  tune_mode(1, [&](const MfOp& m) { mf3<1>(m, a, stream); });
  tune_mode(3, [&](const MfOp& m) { mf3<3>(m, a, stream); });
  tune_mode(4, [&](const MfOp& m) { mf3<4>(m, a, stream); });
  tune_mode(5, [&](const MfOp& m) { mf3<5>(m, a, stream); });
  tune_mode(6, [&](const MfOp& m) { mf3<6>(m, a, stream); });
  tune_mode(7, [&](const MfOp& m) { mf3<7>(m, a, stream); });
  if (mf_cg()) tune_mode(8, [&](const MfOp& m) { mf3<8>(m, a, stream); });
  SIMP_CUDA(cudaStreamSynchronize(stream));
}

void GpuAmg::compute_stats() {
  stats.num_levels = static_cast<int>(levels.size());
  double nz = 0, rows = 0, stored = 0;
  for (size_t k = 0; k < levels.size(); ++k) {
    const Level& lv = *levels[k];
    nz += static_cast<double>(lv.a.nnz);
    rows += lv.n;
    if (k > 0) stored += static_cast<double>(lv.a.nnz);
    if (k + 1 < levels.size())
      stored += static_cast<double>(lv.p.nnz + lv.r.nnz + lv.ap.nnz + levels[k + 1]->a.nnz + lv.phat64.n);
  }
  stored += static_cast<double>(nc_) * nc_;
  stats.operator_complexity = nz / static_cast<double>(levels.front()->a.nnz);
  stats.grid_complexity = rows / static_cast<double>(levels.front()->n);
  stats.storage = static_cast<i64>(std::min(stored, 2.0e9));
}

// Chebyshev smoothing of x (Multigrid.cpp:783-855) on level l.
template <class T>
void GpuAmg::smooth(SolveWork& w, size_t l, bool zero_guess) {
  Level& lv = *levels[l];
  LevelWork& v = w.lv[l];
  const cudaStream_t stream = w.stream;
  const i32 n = lv.n;
  const T* A = V<T>::a(lv.a);
  T* x = V<T>::x(v);
  T* b = V<T>::b(v);
  T* r = V<T>::r(v);
  T* d = V<T>::d(v);
  T* e = V<T>::e(v);
  const T* dinv = V<T>::dinv(lv);
  bool matrix_free = false;
  if constexpr (std::is_same<T, float>::value) matrix_free = l == 0 && mf.enabled;
  if (zero_guess) {
    k_cheb_zero<T><<<grid_for(n, 256), 256, 0, stream>>>(n, b, dinv, d, x, V<T>::cheb(lv));
    SIMP_CHECK_LAUNCH();
  } else if (matrix_free) {
    if constexpr (std::is_same<T, float>::value)
      mf_cheb_first(mf, lv.nnodes, x, b, r, d, dinv, lv.cheb32.p, stream);
  } else {
    nb_cheb_first<T>(lv.opA, A, x, b, r, d, dinv, V<T>::cheb(lv), stream);
  }
  for (int k = 1; k < opt.degree; ++k) {
    const T* rin = (k == 1 && zero_guess) ? b : r;
    const int add_d = (k == 1 && !zero_guess) ? 1 : 0;
    if (matrix_free) {
      if constexpr (std::is_same<T, float>::value)
        mf_cheb_step(mf, lv.nnodes, d, rin, r, e, x, dinv, lv.cheb32.p + 2 * k - 1, add_d, stream);
    } else {
      nb_cheb_step<T>(lv.opA, A, d, rin, r, e, x, dinv, V<T>::cheb(lv) + 2 * k - 1, add_d, stream);
    }
    std::swap(d, e);
  }
  if (opt.degree == 1 && !zero_guess) nb_cheb_step<T>(lv.opA, A, d, r, r, e, x, dinv, V<T>::cheb(lv) + 1, 1, stream);
}

template <class T>
void GpuAmg::cycle(SolveWork& w, size_t l) {
  Level& lv = *levels[l];
  if (l + 1 == levels.size()) {
    coarse_solve<T>(w, l);
    return;
  }
  LevelWork& v = w.lv[l];
  LevelWork& nv = w.lv[l + 1];
  const cudaStream_t stream = w.stream;
  smooth<T>(w, l, true);
  bool matrix_free = false;
  if constexpr (std::is_same<T, float>::value) {
    matrix_free = l == 0 && mf.enabled;
    if (matrix_free && mf.dim == 3 && lv.mf_transfer && opt.mf_transfer) {
      // residual, restriction, coarse cycle and prolongation without the
      // stored R and P (d32 and e32 are free between the smoothing sweeps)
      mf_restrict(mf, lv, v.x32.p, v.b32.p, v.r32.p, v.d32.p, nv.b32.p, stream);
      cycle<T>(w, l + 1);
      mf_prolong(mf, lv, nv.x32.p, v.e32.p, v.x32.p, stream);
      smooth<T>(w, l, false);
      return;
    }
  }
  if (matrix_free) {  // residual
    if constexpr (std::is_same<T, float>::value)
      mf_residual(mf, lv.nnodes, V<T>::x(v), V<T>::r(v), V<T>::b(v), stream);
  } else {
    nb_apply<1, T, T, T>(lv.opA, V<T>::a(lv.a), V<T>::x(v), V<T>::r(v), V<T>::b(v), stream);
  }
  nb_apply<0, T, T, T>(lv.opR, V<T>::a(lv.r), V<T>::r(v), V<T>::b(nv), nullptr, stream);      // restrict
  cycle<T>(w, l + 1);
  nb_apply<2, T, T, T>(lv.opP, V<T>::a(lv.p), V<T>::x(nv), V<T>::x(v), nullptr, stream);      // x += P x_c
  smooth<T>(w, l, false);
}

void GpuAmg::apply(SolveWork& w, const double* r, double* z) {
  if (!ready_) throw Error(kBadInput, "multigrid: apply() called before setup()");
  Level& f = *levels.front();
  LevelWork& v = w.lv.front();
  if (mixed()) {
    convert(r, v.b32.p, f.n, w.stream);
    cycle<float>(w, 0);
    convert(v.x32.p, z, f.n, w.stream);
  } else {
    SIMP_CUDA(cudaMemcpyAsync(v.b64.p, r, sizeof(double) * f.n, cudaMemcpyDeviceToDevice, w.stream));
    cycle<double>(w, 0);
    SIMP_CUDA(cudaMemcpyAsync(z, v.x64.p, sizeof(double) * f.n, cudaMemcpyDeviceToDevice, w.stream));
  }
}

// Preconditioned CG on A x = b (FP64 operator and vectors) from the guess in
// x; `restarts` follows the reference's true-residual restarts.  Stops when
// the recursive residual reaches `target` or the iteration `budget` is spent.
// PCG iteration k > 1, second half of k - 1 and first half of k: z = M r,
// beta, p = z + beta p (and p's double-float split), then q = A p, alpha,
// x += alpha p, r -= alpha q, ||r||^2 -- no host value in between.
void GpuAmg::pcg_tail(SolveWork& w, float2* psplit) {
  const i32 n = levels.front()->n;
  const cudaStream_t stream = w.stream;
  PcgScalars* sc = reinterpret_cast<PcgScalars*>(w.scal.p + 8);
  apply(w, w.pr.p, w.pz.p);
  k_dot_partial<double, double><<<kRedBlocks, kRedThreads, 0, stream>>>(w.pr.p, w.pz.p, n, w.part.p);
  SIMP_CHECK_LAUNCH();
  k_pcg_beta<<<1, kRedThreads, 0, stream>>>(w.part.p, kRedBlocks, sc);
  SIMP_CHECK_LAUNCH();
  k_pcg_direction<<<grid_for(n, 256), 256, 0, stream>>>(w.pp.p, w.pz.p, n, sc, psplit,
                                                         mf_cg() ? w.p32.p : nullptr);
  SIMP_CHECK_LAUNCH();
}

void GpuAmg::pcg_head(SolveWork& w, double* x, bool split_ready, bool op_done) {
  const i32 n = levels.front()->n;
  const cudaStream_t stream = w.stream;
  PcgScalars* sc = reinterpret_cast<PcgScalars*>(w.scal.p + 8);
  if (!op_done) cg_op(w, w.pp.p, w.pq.p, split_ready);
  k_dot_partial<double, double><<<kRedBlocks, kRedThreads, 0, stream>>>(w.pp.p, w.pq.p, n, w.part.p);
  SIMP_CHECK_LAUNCH();
  k_pcg_alpha<<<1, kRedThreads, 0, stream>>>(w.part.p, kRedBlocks, sc);
  SIMP_CHECK_LAUNCH();
  k_pcg_update<<<kRedBlocks, kRedThreads, 0, stream>>>(x, w.pr.p, w.pp.p, w.pq.p, n, sc, w.part.p);
  SIMP_CHECK_LAUNCH();
  k_reduce_final<<<1, kRedThreads, 0, stream>>>(w.part.p, kRedBlocks, &sc->rr, 0);
  SIMP_CHECK_LAUNCH();
}

// pcg_tail + pcg_head as one graph launch: captured on the first use after a
// setup (thread-local capture, so other threads' solves go on), then
// replayed; every pointer is the workspace's, x included (w.px).
void GpuAmg::pcg_body(SolveWork& w, double* x, float2* psplit) {
  if (w.body && w.body_epoch == epoch_) {
    SIMP_CUDA(cudaGraphLaunch(w.body, w.stream));
    g_launches.fetch_add(w.body_kernels, std::memory_order_relaxed);
    return;
  }
  if (w.body) {
    SIMP_CUDA(cudaGraphExecDestroy(w.body));
    w.body = nullptr;
  }
  SIMP_CUDA(cudaStreamBeginCapture(w.stream, cudaStreamCaptureModeThreadLocal));
  const int64_t before = t_launches;
  cudaGraph_t graph = nullptr;
  try {
    pcg_tail(w, psplit);
    pcg_head(w, x, psplit != nullptr || mf_cg());
  } catch (...) {
    cudaStreamEndCapture(w.stream, &graph);
    if (graph) cudaGraphDestroy(graph);
    throw;
  }
  const int64_t kernels = t_launches - before;
  SIMP_CUDA(cudaStreamEndCapture(w.stream, &graph));
  const cudaError_t e = cudaGraphInstantiate(&w.body, graph, 0);
  cudaGraphDestroy(graph);
  SIMP_CUDA(e);
  // the captured launches ran nothing: count them when the graph runs
  g_launches.fetch_sub(kernels, std::memory_order_relaxed);
  w.body_kernels = kernels;
  w.body_epoch = epoch_;
  SIMP_CUDA(cudaGraphLaunch(w.body, w.stream));
  g_launches.fetch_add(kernels, std::memory_order_relaxed);
}

GpuAmg::PcgResult GpuAmg::pcg(SolveWork& w, const double* b, double* x_out, double target, int budget,
                              bool restarts, double bnorm) {
  Level& f = *levels.front();
  const i32 n = f.n;
  const cudaStream_t stream = w.stream;
  // the iterate lives in the workspace while CG runs (a fixed address for
  // the captured iteration body)
  w.px.alloc(static_cast<size_t>(n));
  double* x = w.px.p;
  SIMP_CUDA(cudaMemcpyAsync(x, x_out, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
  DBuf<double>& pr = w.pr;
  DBuf<double>& pz = w.pz;
  DBuf<double>& pp = w.pp;
  PcgResult res;
  PcgScalars* sc = reinterpret_cast<PcgScalars*>(w.scal.p + 8);
  static_assert(sizeof(PcgScalars) <= 8 * sizeof(double), "scalar block");
  auto op = [&](const double* in, double* out, const double* rhs) { op0(w, in, out, rhs, false); };
  auto dot = [&](const double* a, const double* c, i64 m) { return this->dot(w, a, c, m); };
  auto apply = [&](const double* r, double* z) { this->apply(w, r, z); };
  // mixed: the direction update also writes p's double-float split (or,
  // with the matrix-free CG operator, its FP32 copy)
  float2* psplit = mixed() && !mf_cg() ? w.xsplit.p : nullptr;
  if (mf_cg()) w.p32.alloc(static_cast<size_t>(n));
  const bool p_copy = psplit != nullptr || mf_cg();
  bool p_split = false;
  int total = 0;
  bool rec_conv = false;
  double best = std::numeric_limits<double>::max();
  // the FP32 products of the matrix-free CG operator make each restart a
  // step of iterative refinement on the FP64 true residual: allow more
  const int rounds = restarts ? (mf_cg() ? 12 : 3) : 1;
  for (int restart = 0; restart < rounds; ++restart) {
    op(x, pr.p, b);
    double rnorm = std::sqrt(dot(pr.p, pr.p, n));
    res.relres = rnorm / bnorm;
    if (rnorm <= target) { res.converged = true; break; }
    apply(pr.p, pz.p);
    SIMP_CUDA(cudaMemcpyAsync(pp.p, pz.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
    const double rz = dot(pr.p, pz.p, n);
    {
      PcgScalars h{};
      h.rz = rz;
      SIMP_CUDA(cudaMemcpyAsync(sc, &h, sizeof(h), cudaMemcpyHostToDevice, stream));
    }
    bool conv = false;
    p_split = false;
    bool first = true;
    while (total < budget) {
      if (first) {
        pcg_head(w, x, false);
        first = false;
      } else if (opt.graphs) {
        pcg_body(w, x, psplit);
      } else {
        pcg_tail(w, psplit);
        pcg_head(w, x, p_split);
      }
      PcgScalars h{};
      SIMP_CUDA(cudaMemcpyAsync(&h, sc, sizeof(h), cudaMemcpyDeviceToHost, stream));
      SIMP_CUDA(cudaStreamSynchronize(stream));
      if (h.status != 0) {
        std::ostringstream os;
        os << "preconditioned CG broke down at iteration " << total + 1 << " (p^T A p = " << h.pq
           << "): the stiffness matrix or the multigrid preconditioner is not positive definite. "
              "Check the supports, or use a direct solver to confirm";
        throw Error(kBreakdown, os.str());
      }
      ++total;
      rnorm = std::sqrt(h.rr);
      if (rnorm <= target) { conv = true; break; }
      p_split = p_copy;
    }
    if (!restarts) {
      res.converged = conv;
      res.relres = rnorm / bnorm;
      break;
    }
    op(x, pr.p, b);
    res.relres = std::sqrt(dot(pr.p, pr.p, n)) / bnorm;
    if (res.relres * bnorm <= target) { res.converged = true; break; }
    if (!conv) break;
    rec_conv = true;
    if (!(res.relres < 0.5 * best)) break;
    best = res.relres;
  }
  if (!res.converged && rec_conv) res.converged = true;
  res.iterations = total;
  check_mf_status(stream);
  SIMP_CUDA(cudaMemcpyAsync(x_out, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
  return res;
}

// ---------------------------------------------------------------------------
// Several PCG solves advanced together (solve_together).
// ---------------------------------------------------------------------------
namespace {

// Sets a system's conditionals from its loop flag (first node of its
// branch): h guards its iteration body (or, with a fused CG operator, the
// part before it) and h2, when `two`, the part after the fused operator.
__global__ void k_arm(cudaGraphConditionalHandle h, cudaGraphConditionalHandle h2, int two,
                      const int* __restrict__ loop) {
  const unsigned v = loop[0] != 0 ? 1u : 0u;
  cudaGraphSetConditional(h, v);
  if (two) cudaGraphSetConditional(h2, v);
}

// K_ff size (double-float value pairs, bytes) from which the CG products of
// load cases sharing a hierarchy are fused in the lock-step graph (GB300's
// L2 holds 126 MB)
constexpr double kFuseBytes = 128.0 * 1024 * 1024;

// Sets a fused operator's conditional: on while any of its systems iterates.
__global__ void k_arm_any(cudaGraphConditionalHandle h, const int* __restrict__ l0, const int* __restrict__ l1,
                          const int* __restrict__ l2, const int* __restrict__ l3) {
  const bool on = (l0 && l0[0] != 0) || (l1 && l1[0] != 0) || (l2 && l2[0] != 0) || (l3 && l3[0] != 0);
  cudaGraphSetConditional(h, on ? 1u : 0u);
}

// After an iteration body: count the iteration and apply GpuAmg::pcg's test
// (no breakdown, sqrt(||r||^2) above the stopping norm, budget left); the
// flag is the host's view of whether the system iterates on, flag[n] counts
// the bodies that ran since the host last cleared it.
__global__ void k_loop_test(const PcgScalars* __restrict__ sc, int* __restrict__ loop,
                            const double* __restrict__ target, int* __restrict__ flag, int n) {
  const int total = loop[1] + 1;
  loop[1] = total;
  const bool go = sc->status == 0 && !(sqrt(sc->rr) <= target[0]) && total < loop[2];
  loop[0] = go ? 1 : 0;
  flag[0] = go ? 1 : 0;
  flag[n] += 1;
}

}  // namespace

// One graph over a set of (hierarchy, workspace) pairs: per pair an arm
// kernel and a conditional node whose body is the pair's PCG iteration
// (pcg_tail + pcg_head, as pcg_body captures it) and its loop test.
// Mixed-precision pairs that share a hierarchy (the load cases of one
// problem) have their CG operator fused: each one's body is split at the
// operator into two conditional nodes, and between them one multi-RHS
// launch (k_rows_apply_df_multi, up to kMaxRhs pairs) applies the shared
// double-float K_ff to every pair still iterating -- K_ff is read once for
// all of them, each product equal bit for bit to the pair's own.
struct TogetherGraph {
  std::vector<std::pair<GpuAmg*, SolveWork*>> members;
  std::vector<uint64_t> epochs;
  std::vector<int64_t> kernels;  // kernels of each member's body (without a fused operator)
  int64_t fused_nodes = 0;       // fused operators (one arm kernel each per graph launch)
  std::vector<std::vector<int>> fused_members;  // members of each fused operator
  cudaGraphExec_t exec = nullptr;
  cudaStream_t stream = nullptr;
  DBuf<int> flags;
  TogetherGraph() = default;
  TogetherGraph(const TogetherGraph&) = delete;
  TogetherGraph& operator=(const TogetherGraph&) = delete;
  ~TogetherGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (stream) cudaStreamDestroy(stream);
  }

  bool matches(const std::vector<std::pair<GpuAmg*, SolveWork*>>& m) const {
    if (m != members) return false;
    for (size_t i = 0; i < m.size(); ++i)
      if (m[i].first->epoch_ != epochs[i]) return false;
    return true;
  }

  // conditional node after `dep` guarded by h; `body` is captured into it on
  // w's stream.  Returns the node; adds the captured kernels to `count`.
  template <class F>
  static cudaGraphNode_t add_conditional(cudaGraph_t g, cudaGraphNode_t dep, cudaGraphConditionalHandle h,
                                         SolveWork& w, int64_t& count, F&& body) {
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    cudaGraphNode_t cond = nullptr;
    SIMP_CUDA(cudaGraphAddNode(&cond, g, &dep, nullptr, 1, &cp));
    SIMP_CUDA(cudaStreamBeginCaptureToGraph(w.stream, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                            cudaStreamCaptureModeThreadLocal));
    const int64_t before = t_launches;
    try {
      body();
    } catch (...) {
      cudaGraph_t tmp = nullptr;
      cudaStreamEndCapture(w.stream, &tmp);
      throw;
    }
    const int64_t k = t_launches - before;
    cudaGraph_t tmp = nullptr;
    SIMP_CUDA(cudaStreamEndCapture(w.stream, &tmp));
    // captured launches ran nothing: counted when the graph runs
    g_launches.fetch_sub(k, std::memory_order_relaxed);
    count += k;
    return cond;
  }

  void build() {
    const size_t n = members.size();
    if (!stream) SIMP_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    flags.alloc(2 * n);  // [0, n) iterate-on flags, [n, 2n) bodies run
    kernels.assign(n, 0);
    fused_nodes = 0;
    fused_members.clear();
    epochs.clear();
    // pairs whose CG operator is fused: double-float operators of a hierarchy
    // that two or more pairs share, in member order, where K_ff's value pairs
    // do not fit in L2 (kFuseBytes): reading them once per launch instead of
    // once per system then saves DRAM traffic, while below that size the
    // values stay in L2 and the join of the systems' bodies at the fused
    // launch costs more concurrency than it saves
    std::vector<std::vector<size_t>> groups;
    std::vector<char> fused(n, 0);
    for (size_t i = 0; i < n; ++i) {
      GpuAmg* a = members[i].first;
      if (!a->mixed() || a->mf_cg()) continue;
      if (static_cast<double>(a->levels.front()->a.nnz) * 8.0 < kFuseBytes) continue;
      bool placed = false;
      for (auto& grp : groups)
        if (members[grp.front()].first == a) {
          grp.push_back(i);
          placed = true;
        }
      if (!placed) groups.push_back({i});
    }
    for (auto& grp : groups)
      if (grp.size() > 1)
        for (size_t i : grp) fused[i] = 1;
    cudaGraph_t g = nullptr;
    SIMP_CUDA(cudaGraphCreate(&g, 0));
    try {
      std::vector<cudaGraphNode_t> first(n, nullptr);
      std::vector<cudaGraphConditionalHandle> second(n);
      for (size_t i = 0; i < n; ++i) {
        GpuAmg& a = *members[i].first;
        SolveWork& w = *members[i].second;
        epochs.push_back(a.epoch_);
        cudaGraphConditionalHandle h, h2 = 0;
        SIMP_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
        if (fused[i]) SIMP_CUDA(cudaGraphConditionalHandleCreate(&h2, g, 0, 0));
        second[i] = h2;
        const int* loop = w.loop.p;
        int two = fused[i];
        void* args[] = {&h, &h2, &two, &loop};
        cudaGraphNodeParams kp = {};
        kp.type = cudaGraphNodeTypeKernel;
        kp.kernel.func = reinterpret_cast<void*>(k_arm);
        kp.kernel.gridDim = dim3(1);
        kp.kernel.blockDim = dim3(1);
        kp.kernel.sharedMemBytes = 0;
        kp.kernel.kernelParams = args;
        kp.kernel.extra = nullptr;
        cudaGraphNode_t arm = nullptr;
        SIMP_CUDA(cudaGraphAddNode(&arm, g, nullptr, nullptr, 0, &kp));
        first[i] = add_conditional(g, arm, h, w, kernels[i], [&] {
          float2* ps = a.psplit_of(w);
          a.pcg_tail(w, ps);
          if (fused[i]) return;
          a.pcg_head(w, w.px.p, ps != nullptr || a.mf_cg());
          k_loop_test<<<1, 1, 0, w.stream>>>(reinterpret_cast<const PcgScalars*>(w.scal.p + 8), w.loop.p,
                                             w.loopd.p, flags.p + i, static_cast<int>(n));
          SIMP_CHECK_LAUNCH();
        });
      }
      for (auto& grp : groups) {
        if (grp.size() < 2) continue;
        GpuAmg& a = *members[grp.front()].first;
        for (size_t c0 = 0; c0 < grp.size(); c0 += kMaxRhs) {
          const size_t c1 = std::min(grp.size(), c0 + kMaxRhs);
          std::vector<SolveWork*> ws;
          std::vector<cudaGraphNode_t> deps;
          const int* loops[kMaxRhs] = {nullptr, nullptr, nullptr, nullptr};
          fused_members.emplace_back();
          for (size_t c = c0; c < c1; ++c) {
            ws.push_back(members[grp[c]].second);
            deps.push_back(first[grp[c]]);
            loops[c - c0] = members[grp[c]].second->loop.p;
            fused_members.back().push_back(static_cast<int>(grp[c]));
          }
          // the fused launch runs only while one of its systems iterates
          cudaGraphConditionalHandle hf;
          SIMP_CUDA(cudaGraphConditionalHandleCreate(&hf, g, 0, 0));
          void* aargs[] = {&hf, &loops[0], &loops[1], &loops[2], &loops[3]};
          cudaGraphNodeParams ap = {};
          ap.type = cudaGraphNodeTypeKernel;
          ap.kernel.func = reinterpret_cast<void*>(k_arm_any);
          ap.kernel.gridDim = dim3(1);
          ap.kernel.blockDim = dim3(1);
          ap.kernel.sharedMemBytes = 0;
          ap.kernel.kernelParams = aargs;
          ap.kernel.extra = nullptr;
          cudaGraphNode_t arm_f = nullptr;
          SIMP_CUDA(cudaGraphAddNode(&arm_f, g, deps.data(), nullptr, deps.size(), &ap));
          cudaGraphNodeParams cp = {};
          cp.type = cudaGraphNodeTypeConditional;
          cp.conditional.handle = hf;
          cp.conditional.type = cudaGraphCondTypeIf;
          cp.conditional.size = 1;
          cudaGraphNode_t op = nullptr;
          SIMP_CUDA(cudaGraphAddNode(&op, g, &arm_f, nullptr, 1, &cp));
          a.add_op0_multi(cp.conditional.phGraph_out[0], ws, {});
          ++fused_nodes;
          for (size_t c = c0; c < c1; ++c) {
            const size_t i = grp[c];
            SolveWork& w = *members[i].second;
            add_conditional(g, op, second[i], w, kernels[i], [&] {
              a.pcg_head(w, w.px.p, true, true);
              k_loop_test<<<1, 1, 0, w.stream>>>(reinterpret_cast<const PcgScalars*>(w.scal.p + 8), w.loop.p,
                                                 w.loopd.p, flags.p + i, static_cast<int>(n));
              SIMP_CHECK_LAUNCH();
            });
          }
        }
      }
      if (exec) {
        cudaGraphExecDestroy(exec);
        exec = nullptr;
      }
      SIMP_CUDA(cudaGraphInstantiate(&exec, g, 0));
    } catch (...) {
      cudaGraphDestroy(g);
      throw;
    }
    cudaGraphDestroy(g);
  }
};

namespace {
std::mutex g_together_mu;
std::vector<std::unique_ptr<TogetherGraph>> g_together;  // most recent last

// The graph of a member set (built or rebuilt on demand); the caller holds
// g_together_mu.
TogetherGraph& together_graph(const std::vector<std::pair<GpuAmg*, SolveWork*>>& m) {
  for (auto& t : g_together)
    if (t->members == m) {
      if (!t->matches(m)) t->build();
      return *t;
    }
  if (g_together.size() >= 8) g_together.erase(g_together.begin());
  g_together.emplace_back(new TogetherGraph());
  g_together.back()->members = m;
  g_together.back()->build();
  return *g_together.back();
}
}  // namespace

// drops the cached graphs that hold a hierarchy about to be destroyed
void together_forget(const GpuAmg* a) {
  std::lock_guard<std::mutex> lock(g_together_mu);
  for (size_t i = 0; i < g_together.size();) {
    bool hit = false;
    for (auto& m : g_together[i]->members) hit = hit || m.first == a;
    if (hit) g_together.erase(g_together.begin() + static_cast<long>(i));
    else ++i;
  }
}

// fn(i) for i in [0, n) from a pool of host threads (each on the caller's
// device); every task's work goes to its own stream
template <class F>
void each_task(size_t n, F&& fn) {
  const size_t workers = std::max<size_t>(1, std::min<size_t>(n, std::thread::hardware_concurrency()));
  if (workers <= 1) {
    for (size_t i = 0; i < n; ++i) fn(i);
    return;
  }
  int dev = 0;
  SIMP_CUDA(cudaGetDevice(&dev));
  std::atomic<size_t> next{0};
  std::vector<std::thread> pool;
  for (size_t k = 0; k < workers; ++k)
    pool.emplace_back([&] {
      cudaSetDevice(dev);
      for (size_t i = next++; i < n; i = next++) fn(i);
    });
  for (auto& t : pool) t.join();
}

std::vector<GpuAmg::TaskResult> GpuAmg::solve_together(std::vector<SolveTask>& tasks) {
  struct St {
    double bnorm = 0, target = 0, best = std::numeric_limits<double>::max();
    int total = 0, round = 0, rounds = 3;
    bool done = false, rec_conv = false, conv = false, looping = false, ran = false;
  };
  const size_t n = tasks.size();
  std::vector<TaskResult> out(n);
  std::vector<St> st(n);
  auto fail = [&](size_t i, const Error& e) {
    out[i].error_code = e.code;
    out[i].error = e.what();
    st[i].done = true;
  };
  auto finish = [&](size_t i) {
    GpuAmg& a = *tasks[i].amg;
    SolveWork& w = *tasks[i].w;
    if (!out[i].r.converged && st[i].rec_conv) out[i].r.converged = true;
    out[i].r.iterations = st[i].total;
    const i32 nn = a.levels.front()->n;
    SIMP_CUDA(cudaMemcpyAsync(tasks[i].x, w.px.p, sizeof(double) * nn, cudaMemcpyDeviceToDevice, w.stream));
    st[i].done = true;
  };
  auto breakdown = [&](size_t i, const PcgScalars& h) {
    std::ostringstream os;
    os << "preconditioned CG broke down at iteration " << st[i].total + 1 << " (p^T A p = " << h.pq
       << "): the stiffness matrix or the multigrid preconditioner is not positive definite. "
          "Check the supports, or use a direct solver to confirm";
    fail(i, Error(kBreakdown, os.str()));
  };
  // set-up: as solve() does
  for (size_t i = 0; i < n; ++i) {
    GpuAmg& a = *tasks[i].amg;
    SolveWork& w = *tasks[i].w;
    if (!a.ready_) throw Error(kBadInput, "solve called before factorize");
    a.ensure(w);
    w.loop.alloc(4);
    w.loopd.alloc(2);
    const i32 nn = a.levels.front()->n;
    st[i].bnorm = std::sqrt(a.dot(w, tasks[i].b, tasks[i].b, nn));
    if (st[i].bnorm == 0.0) {
      SIMP_CUDA(cudaMemsetAsync(tasks[i].x, 0, sizeof(double) * nn, w.stream));
      out[i].r.converged = true;
      st[i].done = true;
      continue;
    }
    st[i].target = a.opt.rtol * st[i].bnorm;
    st[i].rounds = a.mf_cg() ? 12 : 3;
    w.px.alloc(static_cast<size_t>(nn));
    if (a.mf_cg()) w.p32.alloc(static_cast<size_t>(nn));
    SIMP_CUDA(cudaMemcpyAsync(w.px.p, tasks[i].x, sizeof(double) * nn, cudaMemcpyDeviceToDevice, w.stream));
  }
  while (true) {
    bool any = false;
    for (size_t i = 0; i < n; ++i) any = any || !st[i].done;
    if (!any) break;
    // round start and each round's first iteration, per system (host
    // threads: each system's host round trips overlap the others')
    each_task(n, [&](size_t i) {
      St& s = st[i];
      s.ran = false;
      s.looping = false;
      if (s.done) return;
      GpuAmg& a = *tasks[i].amg;
      SolveWork& w = *tasks[i].w;
      const i32 nn = a.levels.front()->n;
      try {
        a.op0(w, w.px.p, w.pr.p, tasks[i].b, false);
        const double rnorm = std::sqrt(a.dot(w, w.pr.p, w.pr.p, nn));
        out[i].r.relres = rnorm / s.bnorm;
        if (rnorm <= s.target) {
          out[i].r.converged = true;
          finish(i);
          return;
        }
        a.apply(w, w.pr.p, w.pz.p);
        SIMP_CUDA(cudaMemcpyAsync(w.pp.p, w.pz.p, sizeof(double) * nn, cudaMemcpyDeviceToDevice, w.stream));
        const double rz = a.dot(w, w.pr.p, w.pz.p, nn);
        PcgScalars* sc = reinterpret_cast<PcgScalars*>(w.scal.p + 8);
        PcgScalars h{};
        h.rz = rz;
        SIMP_CUDA(cudaMemcpyAsync(sc, &h, sizeof(h), cudaMemcpyHostToDevice, w.stream));
        s.conv = false;
        s.ran = true;
        if (s.total < a.opt.maxit) {
          a.pcg_head(w, w.px.p, false);
          SIMP_CUDA(cudaMemcpyAsync(&h, sc, sizeof(h), cudaMemcpyDeviceToHost, w.stream));
          SIMP_CUDA(cudaStreamSynchronize(w.stream));
          if (h.status != 0) {
            breakdown(i, h);
            return;
          }
          ++s.total;
          if (std::sqrt(h.rr) <= s.target) s.conv = true;
          else if (s.total < a.opt.maxit) s.looping = true;
        }
        if (s.looping) {
          const int hl[4] = {1, s.total, a.opt.maxit, 0};
          const double ht[2] = {s.target, 0.0};
          SIMP_CUDA(cudaMemcpyAsync(w.loop.p, hl, sizeof(hl), cudaMemcpyHostToDevice, w.stream));
          SIMP_CUDA(cudaMemcpyAsync(w.loopd.p, ht, sizeof(ht), cudaMemcpyHostToDevice, w.stream));
          SIMP_CUDA(cudaStreamSynchronize(w.stream));
        }
      } catch (const Error& e) {
        fail(i, e);
      }
    });
    // the later iterations of the round: all looping systems together
    std::vector<size_t> idx;
    for (size_t i = 0; i < n; ++i)
      if (st[i].looping) idx.push_back(i);
    if (!idx.empty()) {
      std::vector<std::pair<GpuAmg*, SolveWork*>> members;
      for (size_t i : idx) members.emplace_back(tasks[i].amg, tasks[i].w);
      std::lock_guard<std::mutex> lock(g_together_mu);
      TogetherGraph& tg = together_graph(members);
      // one launch per host check (several launches per check measured
      // slower: the launches after a system stops still run every member's
      // arm and conditional); the bodies that ran are counted on the device
      const size_t m = idx.size();
      std::vector<int> hf(2 * m, 1);
      std::vector<int> active(m, 1);
      size_t alive = m;
      SIMP_CUDA(cudaMemsetAsync(tg.flags.p + m, 0, sizeof(int) * m, tg.stream));
      std::vector<int> seen(m, 0);
      const int per_check = 1;
      while (alive > 0) {
        for (int r = 0; r < per_check; ++r) SIMP_CUDA(cudaGraphLaunch(tg.exec, tg.stream));
        SIMP_CUDA(cudaMemcpyAsync(hf.data(), tg.flags.p, sizeof(int) * 2 * m, cudaMemcpyDeviceToHost, tg.stream));
        SIMP_CUDA(cudaStreamSynchronize(tg.stream));
        int64_t launched = static_cast<int64_t>(per_check) * (tg.fused_nodes + static_cast<int64_t>(m));
        // a fused operator ran in every launch in which one of its systems ran a body
        for (const auto& fm : tg.fused_members) {
          int most = 0;
          for (int k : fm) most = std::max(most, hf[m + k] - seen[k]);
          launched += most;
        }
        alive = 0;
        for (size_t k = 0; k < m; ++k) {
          launched += static_cast<int64_t>(hf[m + k] - seen[k]) * tg.kernels[k];
          seen[k] = hf[m + k];
          active[k] = active[k] && hf[k];
          alive += active[k] ? 1 : 0;
        }
        g_launches.fetch_add(launched, std::memory_order_relaxed);
      }
      for (size_t k = 0; k < idx.size(); ++k) {
        const size_t i = idx[k];
        SolveWork& w = *tasks[i].w;
        PcgScalars h{};
        int hl[4] = {0, 0, 0, 0};
        SIMP_CUDA(cudaMemcpyAsync(&h, w.scal.p + 8, sizeof(h), cudaMemcpyDeviceToHost, w.stream));
        SIMP_CUDA(cudaMemcpyAsync(hl, w.loop.p, sizeof(hl), cudaMemcpyDeviceToHost, w.stream));
        SIMP_CUDA(cudaStreamSynchronize(w.stream));
        if (h.status != 0) {
          st[i].total = hl[1] - 1;  // the iteration that broke down is not counted
          breakdown(i, h);
          continue;
        }
        st[i].total = hl[1];
        st[i].conv = std::sqrt(h.rr) <= st[i].target;
      }
    }
    // round end, per system: true residual and the restart decision
    each_task(n, [&](size_t i) {
      St& s = st[i];
      if (s.done || !s.ran) return;
      GpuAmg& a = *tasks[i].amg;
      SolveWork& w = *tasks[i].w;
      const i32 nn = a.levels.front()->n;
      try {
        a.op0(w, w.px.p, w.pr.p, tasks[i].b, false);
        out[i].r.relres = std::sqrt(a.dot(w, w.pr.p, w.pr.p, nn)) / s.bnorm;
        if (out[i].r.relres * s.bnorm <= s.target) {
          out[i].r.converged = true;
          finish(i);
          return;
        }
        if (!s.conv) {
          finish(i);
          return;
        }
        s.rec_conv = true;
        if (!(out[i].r.relres < 0.5 * s.best)) {
          finish(i);
          return;
        }
        s.best = out[i].r.relres;
        if (++s.round >= s.rounds) finish(i);
      } catch (const Error& e) {
        fail(i, e);
      }
    });
  }
  for (size_t i = 0; i < n; ++i) SIMP_CUDA(cudaStreamSynchronize(tasks[i].w->stream));
  for (size_t i = 0; i < n; ++i) {
    if (out[i].error_code != 0) continue;
    try {
      tasks[i].amg->check_mf_status(tasks[i].w->stream);
    } catch (const Error& e) {
      out[i].error_code = e.code;
      out[i].error = e.what();
    }
  }
  return out;
}

GpuAmg::PcgResult GpuAmg::solve(SolveWork& w, const double* b, double* x) {
  if (!ready_) throw Error(kBadInput, "solve called before factorize");
  ensure(w);
  Level& f = *levels.front();
  const i32 n = f.n;
  const double bnorm = std::sqrt(dot(w, b, b, n));
  if (bnorm == 0.0) {
    SIMP_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, w.stream));
    PcgResult r;
    r.converged = true;
    return r;
  }
  const double target = opt.rtol * bnorm;
  // The CG operator and the true-residual restarts are FP64 in both modes; in
  // mixed precision the preconditioner (V-cycle) runs in FP32.  CG with an
  // FP32 operator converges towards the FP32 matrix's solution: with the SIMP
  // stiffness contrast it needed up to twice the CG iterations even with
  // FP64 residual replacement, so the outer operator stays FP64.
  return pcg(w, b, x, target, opt.maxit, true, bnorm);
}

}  // namespace simp
