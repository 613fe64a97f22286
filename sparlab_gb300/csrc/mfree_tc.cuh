// Matrix-free level-0 operator of a structured Hex8 grid on the fifth-
// generation tensor cores: the element products F_e = K_e^0 x_e of a layer
// of cells as one GEMM per 128 cells (tcgen05.mma kind::tf32, FP32
// accumulation in tensor memory).
//
// Element-major form of the tiled operator in mfree.cuh: y_I = sum over the
// cells e around node I of s_e (K_e^0 x_e)[rows of I's corner].  A CTA owns
// a column of 31 x 7 nodes and marches it along z over a chunk of node
// layers.  Per cell layer it
//   1. gathers each cell's 24 corner values (8 corners x 3) from the node
//      values of the two node layers the cells span (a ring of four node
//      layers with a one-node halo, staged in shared memory), splits each
//      value into TF32 hi + lo (v = hi + lo exactly, lo rounded to TF32), and
//      writes the rows of A (256 cells x 24) in the plain canonical K-major
//      layout;
//   2. one thread issues, per 128-cell M tile, the 3 x TF32 products
//      A_lo K_hi + A_hi K_lo + A_hi K_hi (K = 8 per instruction, N = 32 with
//      rows 24..31 of B zero) into 32 tensor-memory columns: about FP32
//      accuracy (the dropped A_lo K_lo term is ~2^-22 relative);
//   3. every thread reads its cell's row of F from tensor memory, scales it
//      by s_e and stores the bottom-corner half (the node layer below the
//      cell's centre) and the top-corner half (the layer above) in shared
//      memory;
//   4. while the next cell layer's MMA runs, the threads of the node layer
//      between the last two cell layers sum their 8 cells' corner rows in a
//      fixed order (cells below first, then dy, dx ascending) and apply the
//      mode's epilogue (mf_node_store; the node's free index and operands
//      are loaded two and one layers ahead).
// One thread waits for each MMA; the others wait at the barrier after it.
// Node values are loaded in two stages (free-node indices, then values) and
// enter the ring three layers ahead of the layer that reads them.
// Every node's value is summed by one thread from the same F rows whatever
// the chunking, so the result does not depend on the launch shape.
//
// The cells of a CTA's layer are 32 x 8 = 256 (two M = 128 tiles: TMEM
// lanes = cells, columns 0-31 and 32-63); the CTA owns their 31 x 7 interior
// nodes, so neighbouring CTAs recompute one cell row / column (the halo).
// Thread t owns cell (t % 32, t / 32) of every layer; warp w reads TMEM lanes
// 32 (w % 4) .. + 31 of M tile w / 4, which are exactly its threads' cells.
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

// Shared memory (bytes from a 128-byte aligned base).  A: two parts (hi, lo)
// of 256 rows x 24 TF32, element (r, j) at (j / 4) 4096 + (r / 8) 128 +
// (r % 8) 16 + (j % 4) 4 (leading-dimension offset 4096, stride 128).  B: two
// parts of 32 rows x 24, (n, k) at (k / 4) 512 + (n / 8) 128 + (n % 8) 16 +
// (k % 4) 4.  Then the node ring (float4 per node), the bottom-corner rows
// of F ([12][256] floats) and the top-corner rows of the last two cell layers
// ([2][12][256]), the mbarrier and the tensor-memory address.
constexpr int kTcAPart = kTcThreads * 24 * 4;  // 24,576
constexpr int kTcBPart = 32 * 24 * 4;          // 3,072
constexpr int kTcALbo = kTcThreads / 8 * 128;  // 4,096
constexpr int kTcBLbo = 32 / 8 * 128;          // 512
constexpr int kTcOffB = 2 * kTcAPart;
constexpr int kTcOffRing = kTcOffB + 2 * kTcBPart;
constexpr int kTcOffF0 = kTcOffRing + kTcRing * kTcHalo * 16;
constexpr int kTcOffF1 = kTcOffF0 + 12 * kTcThreads * 4;
constexpr int kTcOffBar = kTcOffF1 + 2 * 12 * kTcThreads * 4;
constexpr int kTcSmemBytes = kTcOffBar + 16 + 128;  // + alignment slack (111,312: two CTAs per SM)
constexpr uint32_t kTcTmemCols = 64;

// Corner b of a cell (the K_e^0 column block 3 b .. 3 b + 2): offsets
// (bx, by, bz) = (0,0,0) (1,0,0) (1,1,0) (0,1,0) and the same at z + 1.
__device__ __forceinline__ constexpr int corner_x(int b) { return (b == 1 || b == 2 || b == 5 || b == 6) ? 1 : 0; }
__device__ __forceinline__ constexpr int corner_y(int b) { return (b == 2 || b == 3 || b == 6 || b == 7) ? 1 : 0; }

template <int MODE>
__global__ void __launch_bounds__(kTcThreads, 2)
    k_mf3_tc(MfView m, MfArgs a, const __grid_constant__ KeF32 ke, int layers, int* status) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  float4* ring = reinterpret_cast<float4*>(smem + kTcOffRing);
  float* f0 = reinterpret_cast<float*>(smem + kTcOffF0);
  float* f1 = reinterpret_cast<float*>(smem + kTcOffF1);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kTcOffBar);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kTcOffBar + 8);
  const int tid = threadIdx.x, warp = tid >> 5;
  const i32 gx0 = blockIdx.x * kTcNodesX, gy0 = blockIdx.y * kTcNodesY;
  const i32 nnz = m.nz + 1;
  const i32 nz0 = blockIdx.z * layers;
  const i32 nz1 = min(nz0 + layers, nnz);
  const int ncl = nz1 - nz0 + 1;  // cell layers nz0 - 1 .. nz1 - 1
  const i64 node_layer = static_cast<i64>(m.nnx) * m.nny, cell_layer = static_cast<i64>(m.nx) * m.ny;

  // B = K_e^0 (symmetric: row n of B is row n of K) as TF32 hi + lo
  for (int e = tid; e < 32 * 24; e += kTcThreads) {
    const int n = e / 24, k = e % 24;
    const float v = n < 24 ? ke.k[n * 24 + k] : 0.0f;
    const uint32_t hi = tc::tf32_round(v);
    const uint32_t lo = tc::tf32_round(v - __uint_as_float(hi));
    const int off = (k >> 2) * kTcBLbo + (n >> 3) * 128 + (n & 7) * 16 + (k & 3) * 4;
    *reinterpret_cast<uint32_t*>(smem + kTcOffB + off) = hi;
    *reinterpret_cast<uint32_t*>(smem + kTcOffB + kTcBPart + off) = lo;
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
  auto put = [&](int slot, const float4 (&v)[kTcHaloPer]) {
#pragma unroll
    for (int q = 0; q < kTcHaloPer; ++q) {
      const int e = tid + q * kTcThreads;
      if (e < kTcHalo) ring[slot * kTcHalo + e] = v[q];
    }
  };
  // this thread's cell: its in-layer offset or -1 outside the grid
  const int cxl = tid % kTcCellsX, cyl = tid / kTcCellsX;
  const i32 cgx = gx0 - 1 + cxl, cgy = gy0 - 1 + cyl;
  const i64 c2d = (cgx >= 0 && cgx < m.nx && cgy >= 0 && cgy < m.ny) ? static_cast<i64>(cgy) * m.nx + cgx : -1;
  auto scale_of = [&](i32 cz) { return (c2d >= 0 && cz >= 0 && cz < m.nz) ? m.scale[cz * cell_layer + c2d] : 0.0f; };
  // this thread's node of the sums (threads < 217): in-layer offset or -1;
  // its free index and epilogue operands are loaded two and one iterations
  // ahead of its sum
  const int nxl = tid % kTcNodesX, nyl = tid / kTcNodesX;
  const i64 n2d = (tid < kTcNodesX * kTcNodesY && gx0 + nxl < m.nnx && gy0 + nyl < m.nny)
                      ? static_cast<i64>(gy0 + nyl) * m.nnx + gx0 + nxl
                      : -1;
  auto node_of = [&](i32 L) { return (n2d >= 0 && L >= nz0 && L < nz1) ? m.nindex[L * node_layer + n2d] : -1; };
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
  if (I_cur >= 0) mf_node_load<MODE>(a, I_cur, in_cur);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc::idesc_tf32(128, 32);
  const uint64_t a_desc = tc::smem_desc_plain(tc::smem_u32(smem), kTcALbo, 128);
  const uint64_t b_desc = tc::smem_desc_plain(tc::smem_u32(smem + kTcOffB), kTcBLbo, 128);
  // this thread's A row: (r / 8) 128 + (r % 8) 16 within each 16-byte column group
  uint8_t* arow = smem + (tid >> 3) * 128 + (tid & 7) * 16;

  // Node layer nz0 - 2 + it is summed in iteration it (it >= 2) while the
  // MMA of cell layer it runs, from the bottom-corner rows of cell layer
  // it - 1 (f0) and the top-corner rows of it - 2 (f1); the last node layer
  // after the march.
  auto node_sum = [&](int it) {
    if (I_cur < 0) return;
    const float* below = f1 + (it & 1) * 12 * kTcThreads;  // cell layer it - 2
    float o[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int dz = -1; dz <= 0; ++dz)
#pragma unroll
      for (int dy = -1; dy <= 0; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 0; ++dx) {
          const int c = (nyl + dy + 1) * kTcCellsX + nxl + dx + 1;
          const int ox = -dx, oy = -dy, oz = -dz;
          const int aI = 4 * oz + (oy ? 3 - ox : ox);  // the node's corner in the cell
          const float* src = oz ? below + (3 * aI - 12) * kTcThreads : f0 + 3 * aI * kTcThreads;
#pragma unroll
          for (int k = 0; k < 3; ++k) o[k] += src[k * kTcThreads + c];
        }
    const float4 sv = ring[((it - 1) % kTcRing) * kTcHalo + (nyl + 1) * kTcHaloX + nxl + 1];
    const float self[3] = {sv.x, sv.y, sv.z};
    mf_node_store<MODE>(a, I_cur, o, self, in_cur, c0, c1);
  };

  bool ok = true;
  int it = 0;
  for (; it < ncl; ++it) {
    const i32 cz = nz0 - 1 + it;
    // 1. A rows of this cell from node layers cz (slot it % 3) and cz + 1
    {
      const float4* r0 = ring + (it % kTcRing) * kTcHalo;
      const float4* r1 = ring + ((it + 1) % kTcRing) * kTcHalo;
      float xv[24];
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        const float4 v = (b < 4 ? r0 : r1)[(cyl + corner_y(b)) * kTcHaloX + cxl + corner_x(b)];
        xv[3 * b + 0] = v.x;
        xv[3 * b + 1] = v.y;
        xv[3 * b + 2] = v.z;
      }
#pragma unroll
      for (int g = 0; g < 6; ++g) {
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          hi[q] = tc::tf32_round(xv[4 * g + q]);
          lo[q] = tc::tf32_round(xv[4 * g + q] - __uint_as_float(hi[q]));
        }
        *reinterpret_cast<uint4*>(arow + g * kTcALbo) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<uint4*>(arow + kTcAPart + g * kTcALbo) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
      }
    }
    tc::fence_proxy_async_smem();
    __syncthreads();
    // 2. F = A K^T for the two 128-cell tiles (3 x TF32); descriptors advance
    // by (byte offset >> 4) in their start-address field
    if (tid == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const uint32_t d = tmem + static_cast<uint32_t>(mt * 32);
#pragma unroll
        for (int s = 0; s < 3; ++s) {
          const uint64_t ao = static_cast<uint64_t>((s * 2 * kTcALbo + mt * 16 * 128) >> 4);
          const uint64_t bo = static_cast<uint64_t>((s * 2 * kTcBLbo) >> 4);
          const uint64_t ahi = a_desc + ao, alo = a_desc + ao + (kTcAPart >> 4);
          const uint64_t bhi = b_desc + bo, blo = b_desc + bo + (kTcBPart >> 4);
          tc::mma_tf32(d, alo, bhi, idesc, s > 0 ? 1u : 0u);
          tc::mma_tf32(d, ahi, blo, idesc, 1u);
          tc::mma_tf32(d, ahi, bhi, idesc, 1u);
        }
      }
      tc::mma_commit(bar);
    }
    // meanwhile: the sums of node layer cz - 1, and the loads of later layers
    // (node values of layer cz + 3 enter the ring after this iteration's
    // second barrier, so the next iteration's first barrier orders them
    // before the A rows of iteration it + 2 read them)
    if (it >= 2) node_sum(it);
    const bool more = it + 3 <= ncl;  // node layer cz + 3 is still read
    float4 pv[kTcHaloPer];
    if (more) values(hj, pv);
    if (it + 4 <= ncl) indices(cz + 4, hj);
    const float s_next = it + 1 < ncl ? scale_of(cz + 1) : 0.0f;
    if (it >= 2) {
      I_cur = I_next;
      I_next = node_of(nz0 + it);  // summed in iteration it + 2
      if (I_cur >= 0) mf_node_load<MODE>(a, I_cur, in_cur);  // summed in iteration it + 1
    }
    // 3. wait for the MMA (one thread), then every thread's row of F
    if (tid == 0) ok = tc::mbar_wait(bar, static_cast<uint32_t>(it & 1), status);
    if (__syncthreads_or(!ok)) break;
    tc::fence_after_sync();
    {
      float fv[24];
      tc::tmem_ld24(tmem + (static_cast<uint32_t>((warp & 3) * 32) << 16) + static_cast<uint32_t>((warp >> 2) * 32),
                    fv);
      float* top = f1 + (it & 1) * 12 * kTcThreads;
#pragma unroll
      for (int jj = 0; jj < 12; ++jj) {
        f0[jj * kTcThreads + tid] = s_cur * fv[jj];
        top[jj * kTcThreads + tid] = s_cur * fv[12 + jj];
      }
    }
    if (more) put((it + 3) % kTcRing, pv);
    s_cur = s_next;
    tc::fence_before_sync();
  }
  if (it == ncl) {
    // the last node layer, nz1 - 1
    __syncthreads();
    node_sum(it);
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
