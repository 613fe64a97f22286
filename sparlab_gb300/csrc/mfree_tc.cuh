// Matrix-free level-0 operator of a structured Hex8 grid on the fifth-
// generation tensor cores: the element products F_e = K_e^0 x_e of a layer
// of cells as one GEMM per 128 cells (tcgen05.mma kind::tf32, FP32
// accumulation in tensor memory).
//
// Element-major form of the tiled operator in mfree.cuh: y_I = sum over the
// cells e around node I of s_e (K_e^0 x_e)[rows of I's corner].  A CTA owns
// a column of 31 x 7 nodes and marches it along z over a chunk of node
// layers.  Per cell layer it
//   1. gathers each cell's 24 corner values (8 corners x 3) as TF32 hi + lo
//      pairs (v = hi + lo to about 2^-22, each rounded to nearest) from a
//      ring of four node layers with a one-node halo in shared memory (a
//      node's values are split once, when its layer enters the ring), and
//      writes the cell's row of A = [A_hi | A_lo] (K = 48) in the plain
//      canonical K-major layout;
//   2. one thread issues, per 128-cell M tile, six K = 8 steps of
//      A · B^T with B = [[K_hi, K_hi], [K_lo, 0]] (N = 48): columns 0-23
//      accumulate A_hi K_hi + A_lo K_hi and columns 24-47 A_hi K_lo, all in
//      FP32 in tensor memory (3 x TF32: the dropped A_lo K_lo term is about
//      2^-22 relative);
//   3. every thread reads its cell's 48 accumulator columns back, forms
//      F_e = s_e (D[0:24] + D[24:48]) and stores its bottom-corner and
//      top-corner halves (the node layers below and above the cell centre)
//      in shared memory;
//   4. while the next cell layer's MMA runs, the threads of the owned nodes
//      finish the node layer below the last cell layer (the partial sum of
//      its four cells below, carried in registers, plus the bottom corners
//      of its four cells above) and start the next one (the top corners of
//      the cells below it), each in a fixed order (cells below first, then
//      dy, dx ascending), then apply the mode's epilogue (mf_node_store; the
//      node's free index, operands and own input value are loaded two and
//      one layers ahead).
// Every node's value is summed by one thread from the same F rows whatever
// the chunking, so the result does not depend on the launch shape.
// One thread waits for each MMA; the others wait at the barrier after it.
// Node values are loaded in two stages (free-node indices, then values) and
// enter the ring three layers ahead of the layer that reads them.
//
// The cells of a CTA's layer are 32 x 8 = 256 (two M = 128 tiles: TMEM
// lanes = cells, columns 0-47 and 64-111); the CTA owns their 31 x 7
// interior nodes, so neighbouring CTAs recompute one cell row / column (the
// halo).  Thread t owns cell (t % 32, t / 32) of every layer; warp w reads
// TMEM lanes 32 (w % 4) .. + 31 of M tile w / 4, which are exactly its
// threads' cells.
//
// The MMA completion is waited on with the bounded mbarrier wait of tc.cuh;
// a wait that runs out sets *status (kTcTimeout) and all threads leave the
// march together (the barrier after the wait ORs the failure), wait once
// more for the MMA in flight and free the tensor memory.
#pragma once

#include "mfree.cuh"
#include "tc.cuh"

namespace simp {
namespace {

constexpr int kTcCellsX = 32, kTcCellsY = 8;                        // cells of a layer per CTA
constexpr int kTcNodesX = kTcCellsX - 1, kTcNodesY = kTcCellsY - 1;  // nodes a CTA owns per layer
constexpr int kTcHaloX = kTcCellsX + 1, kTcHaloY = kTcCellsY + 1;    // node values a cell layer reads
constexpr int kTcHalo = kTcHaloX * kTcHaloY;                         // 297
constexpr int kTcThreads = kTcCellsX * kTcCellsY;                    // one cell per thread
constexpr int kTcRing = 4;                                           // node layers in shared memory
constexpr int kTcHaloPer = (kTcHalo + kTcThreads - 1) / kTcThreads;  // halo entries per thread (2)
constexpr int kTcN = 48;                                             // GEMM N (see B)

// Shared memory (bytes from a 128-byte aligned base).  A: 256 rows x 48
// TF32 (hi in K 0-23, lo in K 24-47), element (r, k) at (k / 4) 4096 +
// (r / 8) 128 + (r % 8) 16 + (k % 4) 4 (leading-dimension offset 4096,
// stride 128).  B: 48 rows x 48, (n, k) at (k / 4) 768 + (n / 8) 128 +
// (n % 8) 16 + (k % 4) 4.  Then the node ring (per node: (hi_x, hi_y, hi_z,
// lo_x) as a float4 and (lo_y, lo_z) as a float2, two arrays), the corner
// rows of F ([12][256] floats, bottom then top), the mbarrier and the
// tensor-memory address.
constexpr int kTcALbo = kTcThreads / 8 * 128;  // 4,096
constexpr int kTcBLbo = kTcN / 8 * 128;        // 768
constexpr int kTcOffB = 12 * kTcALbo;          // 49,152
constexpr int kTcOffRingA = kTcOffB + 12 * kTcBLbo;
constexpr int kTcOffRingB = kTcOffRingA + kTcRing * kTcHalo * 16;
constexpr int kTcOffF = kTcOffRingB + kTcRing * kTcHalo * 8;
constexpr int kTcOffBar = kTcOffF + 24 * kTcThreads * 4;
constexpr int kTcSmemBytes = kTcOffBar + 16 + 128;  // + alignment slack (111,600: two CTAs per SM)
constexpr uint32_t kTcTmemCols = 128;               // two tiles of 48 columns at 0 and 64

// Corner b of a cell (the K_e^0 column block 3 b .. 3 b + 2): offsets
// (bx, by, bz) = (0,0,0) (1,0,0) (1,1,0) (0,1,0) and the same at z + 1.
__device__ __forceinline__ constexpr int corner_x(int b) { return (b == 1 || b == 2 || b == 5 || b == 6) ? 1 : 0; }
__device__ __forceinline__ constexpr int corner_y(int b) { return (b == 2 || b == 3 || b == 6 || b == 7) ? 1 : 0; }

template <int MODE>
__global__ void __launch_bounds__(kTcThreads, 2)
    k_mf3_tc(MfView m, MfArgs a, const __grid_constant__ KeF32 ke, int layers, int* status) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  float4* ring_a = reinterpret_cast<float4*>(smem + kTcOffRingA);
  float2* ring_b = reinterpret_cast<float2*>(smem + kTcOffRingB);
  float* fb = reinterpret_cast<float*>(smem + kTcOffF);  // bottom corners (rows 0-11)
  float* ft = fb + 12 * kTcThreads;                      // top corners (rows 12-23)
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kTcOffBar);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kTcOffBar + 8);
  const int tid = threadIdx.x, warp = tid >> 5;
  const i32 gx0 = blockIdx.x * kTcNodesX, gy0 = blockIdx.y * kTcNodesY;
  const i32 nnz = m.nz + 1;
  const i32 nz0 = blockIdx.z * layers;
  const i32 nz1 = min(nz0 + layers, nnz);
  const int ncl = nz1 - nz0 + 1;  // cell layers nz0 - 1 .. nz1 - 1
  const i64 node_layer = static_cast<i64>(m.nnx) * m.nny, cell_layer = static_cast<i64>(m.nx) * m.ny;

  // B = [[K_hi, K_hi], [K_lo, 0]] (K_e^0 is symmetric: row n of B's blocks
  // is row n of K)
  for (int e = tid; e < kTcN * 48; e += kTcThreads) {
    const int n = e / 48, k = e % 48;
    const int r = n % 24, c = k % 24;
    const float v = ke.k[r * 24 + c];
    const uint32_t hi = tc::tf32_round(v);
    const uint32_t lo = tc::tf32_round(v - __uint_as_float(hi));
    const uint32_t w = n < 24 ? hi : (k < 24 ? lo : 0u);
    const int off = (k >> 2) * kTcBLbo + (n >> 3) * 128 + (n & 7) * 16 + (k & 3) * 4;
    *reinterpret_cast<uint32_t*>(smem + kTcOffB + off) = w;
  }
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::fence_mbar_init();
  }
  __syncwarp();
  if (warp == 0) tc::tmem_alloc(tslot, kTcTmemCols);

  // This thread's halo entries (tid, tid + 256 of the 33 x 9 node layer):
  // their in-layer offsets, or -1 outside the grid.  Node values arrive in
  // two stages: the free-node indices of a layer one iteration before its
  // values (hj), the values one iteration before they enter the ring (pv).
  i64 h2d[kTcHaloPer];
#pragma unroll
  for (int q = 0; q < kTcHaloPer; ++q) {
    const int e = tid + q * kTcThreads;
    const i32 gx = gx0 - 1 + e % kTcHaloX, gy = gy0 - 1 + e / kTcHaloX;
    h2d[q] = (e < kTcHalo && gx >= 0 && gx < m.nnx && gy >= 0 && gy < m.nny) ? static_cast<i64>(gy) * m.nnx + gx
                                                                               : -1;
  }
  auto indices = [&](i32 L, i32 (&j)[kTcHaloPer]) {
#pragma unroll
    for (int q = 0; q < kTcHaloPer; ++q)
      j[q] = (h2d[q] >= 0 && L >= 0 && L < nnz) ? m.nindex[L * node_layer + h2d[q]] : -1;
  };
  auto values = [&](const i32 (&j)[kTcHaloPer], float4 (&v)[kTcHaloPer]) {
#pragma unroll
    for (int q = 0; q < kTcHaloPer; ++q) {
      v[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (j[q] >= 0) {
        const float* p = a.x + static_cast<i64>(j[q]) * 3;
        v[q].x = p[0];
        v[q].y = p[1];
        v[q].z = p[2];
      }
    }
  };
  // a layer enters the ring split into TF32 hi + lo
  auto put = [&](int slot, const float4 (&v)[kTcHaloPer]) {
#pragma unroll
    for (int q = 0; q < kTcHaloPer; ++q) {
      const int e = tid + q * kTcThreads;
      if (e < kTcHalo) {
        const float c[3] = {v[q].x, v[q].y, v[q].z};
        float h[3], l[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          h[k] = __uint_as_float(tc::tf32_round(c[k]));
          l[k] = __uint_as_float(tc::tf32_round(c[k] - h[k]));
        }
        ring_a[slot * kTcHalo + e] = make_float4(h[0], h[1], h[2], l[0]);
        ring_b[slot * kTcHalo + e] = make_float2(l[1], l[2]);
      }
    }
  };
  // this thread's cell: its in-layer offset or -1 outside the grid
  const int cxl = tid % kTcCellsX, cyl = tid / kTcCellsX;
  const i32 cgx = gx0 - 1 + cxl, cgy = gy0 - 1 + cyl;
  const i64 c2d = (cgx >= 0 && cgx < m.nx && cgy >= 0 && cgy < m.ny) ? static_cast<i64>(cgy) * m.nx + cgx : -1;
  auto scale_of = [&](i32 cz) { return (c2d >= 0 && cz >= 0 && cz < m.nz) ? m.scale[cz * cell_layer + c2d] : 0.0f; };
  // this thread's node of the sums (threads 32 .. 248, so warp 0, whose
  // thread 0 issues the MMAs, has none): in-layer offset or -1; its free
  // index and epilogue operands are loaded two and one iterations ahead of
  // its sum
  const int nt = tid - 32;
  const int nxl = nt % kTcNodesX, nyl = nt / kTcNodesX;
  const i64 n2d = (nt >= 0 && nt < kTcNodesX * kTcNodesY && gx0 + nxl < m.nnx && gy0 + nyl < m.nny)
                      ? static_cast<i64>(gy0 + nyl) * m.nnx + gx0 + nxl
                      : -1;
  auto node_of = [&](i32 L) { return (n2d >= 0 && L >= nz0 && L < nz1) ? m.nindex[L * node_layer + n2d] : -1; };
  auto load_node = [&](i32 I, MfNodeIn& in, float (&self)[3]) {
    mf_node_load<MODE>(a, I, in);
    if (MODE == 3 || MODE == 5) {
#pragma unroll
      for (int k = 0; k < 3; ++k) self[k] = a.x[static_cast<i64>(I) * 3 + k];
    }
  };
  float c0, c1;
  mf_coefs<MODE>(a, c0, c1);

  // prologue: node layers nz0 - 1 .. nz0 + 1 in ring slots 0 .. 2 (layer L
  // sits in slot (L - nz0 + 1) % 4); indices of layer nz0 + 2; node indices
  // of the first two summed layers and the first one's operands
  {
    i32 j[kTcHaloPer];
    float4 v[kTcHaloPer];
    for (int r = 0; r < 3; ++r) {
      indices(nz0 - 1 + r, j);
      values(j, v);
      put(r, v);
    }
  }
  i32 hj[kTcHaloPer];
  indices(nz0 + 2, hj);
  float s_cur = scale_of(nz0 - 1);
  i32 I_cur = node_of(nz0), I_next = node_of(nz0 + 1);
  MfNodeIn in_cur;
  float self_cur[3] = {0.0f, 0.0f, 0.0f};
  if (I_cur >= 0) load_node(I_cur, in_cur, self_cur);
  float part[3] = {0.0f, 0.0f, 0.0f};  // the cells below the next summed node layer
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc::idesc_tf32(128, kTcN);
  const uint64_t a_desc = tc::smem_desc_plain(tc::smem_u32(smem), kTcALbo, 128);
  const uint64_t b_desc = tc::smem_desc_plain(tc::smem_u32(smem + kTcOffB), kTcBLbo, 128);
  // this thread's A row: (r / 8) 128 + (r % 8) 16 within each 16-byte column group
  uint8_t* arow = smem + (tid >> 3) * 128 + (tid & 7) * 16;

  // the corner rows of the node's cells in the last cell layer (F holds it):
  // the bottom corners finish the node layer below it, the top corners start
  // the node layer above it
  auto finish = [&]() {
    if (I_cur < 0) return;
    float o[3] = {part[0], part[1], part[2]};
#pragma unroll
    for (int dy = -1; dy <= 0; ++dy)
#pragma unroll
      for (int dx = -1; dx <= 0; ++dx) {
        const int c = (nyl + dy + 1) * kTcCellsX + nxl + dx + 1;
        const int aI = -dy ? 3 + dx : -dx;  // the node's bottom corner in the cell
#pragma unroll
        for (int k = 0; k < 3; ++k) o[k] += fb[(3 * aI + k) * kTcThreads + c];
      }
    mf_node_store<MODE>(a, I_cur, o, self_cur, in_cur, c0, c1);
  };
  auto start = [&]() {
    part[0] = part[1] = part[2] = 0.0f;
    if (n2d < 0) return;
#pragma unroll
    for (int dy = -1; dy <= 0; ++dy)
#pragma unroll
      for (int dx = -1; dx <= 0; ++dx) {
        const int c = (nyl + dy + 1) * kTcCellsX + nxl + dx + 1;
        const int aI = -dy ? 3 + dx : -dx;  // the node's top corner in the cell is 4 + aI
#pragma unroll
        for (int k = 0; k < 3; ++k) part[k] += ft[(3 * aI + k) * kTcThreads + c];
      }
  };

  bool ok = true;
  int it = 0;
  for (; it < ncl; ++it) {
    const i32 cz = nz0 - 1 + it;
    // 1. A rows of this cell from node layers cz (slot it % 4) and cz + 1
    {
      const int s0 = (it % kTcRing) * kTcHalo, s1 = ((it + 1) % kTcRing) * kTcHalo;
      float hv[24], lv[24];
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        const int e = (b < 4 ? s0 : s1) + (cyl + corner_y(b)) * kTcHaloX + cxl + corner_x(b);
        const float4 u = ring_a[e];
        const float2 w = ring_b[e];
        hv[3 * b + 0] = u.x;
        hv[3 * b + 1] = u.y;
        hv[3 * b + 2] = u.z;
        lv[3 * b + 0] = u.w;
        lv[3 * b + 1] = w.x;
        lv[3 * b + 2] = w.y;
      }
#pragma unroll
      for (int g = 0; g < 6; ++g) {
        *reinterpret_cast<float4*>(arow + g * kTcALbo) =
            make_float4(hv[4 * g], hv[4 * g + 1], hv[4 * g + 2], hv[4 * g + 3]);
        *reinterpret_cast<float4*>(arow + (6 + g) * kTcALbo) =
            make_float4(lv[4 * g], lv[4 * g + 1], lv[4 * g + 2], lv[4 * g + 3]);
      }
    }
    tc::fence_proxy_async_smem();
    __syncthreads();
    // 2. D = A B^T for the two 128-cell tiles (six K = 8 steps each);
    // descriptors advance by (byte offset >> 4) in their start-address field
    if (tid == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const uint32_t d = tmem + static_cast<uint32_t>(mt * 64);
#pragma unroll
        for (int s = 0; s < 6; ++s) {
          const uint64_t ao = static_cast<uint64_t>((s * 2 * kTcALbo + mt * 16 * 128) >> 4);
          const uint64_t bo = static_cast<uint64_t>((s * 2 * kTcBLbo) >> 4);
          tc::mma_tf32(d, a_desc + ao, b_desc + bo, idesc, s > 0 ? 1u : 0u);
        }
      }
      tc::mma_commit(bar);
    }
    // meanwhile: the node layer below the last cell layer, the partial sums
    // of the one above it, and the loads of later layers
    if (it >= 2) finish();
    if (it >= 1) start();
    const bool more = it + 3 <= ncl;  // node layer cz + 3 is still read
    float4 pv[kTcHaloPer];
    if (more) values(hj, pv);
    if (it + 4 <= ncl) indices(cz + 4, hj);
    const float s_next = it + 1 < ncl ? scale_of(cz + 1) : 0.0f;
    if (it >= 2) {
      I_cur = I_next;
      I_next = node_of(nz0 + it);  // summed in iteration it + 2
      if (I_cur >= 0) load_node(I_cur, in_cur, self_cur);  // summed in iteration it + 1
    }
    // 3. wait for the MMA (one thread), then every thread's row of F
    if (tid == 0) ok = tc::mbar_wait(bar, static_cast<uint32_t>(it & 1), status);
    if (__syncthreads_or(!ok)) break;
    tc::fence_after_sync();
    {
      uint32_t r[48];
      tc::tmem_ld48_start(tmem + (static_cast<uint32_t>((warp & 3) * 32) << 16) +
                              static_cast<uint32_t>((warp >> 2) * 64),
                          r);
      if (more) put((it + 3) % kTcRing, pv);
      tc::tmem_ld48_wait(r);
#pragma unroll
      for (int jj = 0; jj < 12; ++jj) {
        fb[jj * kTcThreads + tid] = s_cur * (__uint_as_float(r[jj]) + __uint_as_float(r[jj + 24]));
        ft[jj * kTcThreads + tid] = s_cur * (__uint_as_float(r[12 + jj]) + __uint_as_float(r[36 + jj]));
      }
    }
    s_cur = s_next;
    tc::fence_before_sync();
  }
  if (it == ncl) {
    // the last node layer, nz1 - 1
    __syncthreads();
    finish();
  } else if (tid == 0) {
    tc::mbar_wait(bar, static_cast<uint32_t>(it & 1), nullptr);  // the MMA in flight
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kTcTmemCols);
  }
}

}  // namespace
}  // namespace simp
