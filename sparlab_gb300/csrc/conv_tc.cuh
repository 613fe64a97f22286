// 3 x 3 x 3 convolutions of the displacement surrogate on the fifth-
// generation tensor cores (BF16 operands, FP32 accumulation in tensor memory).
//
// Activations are channels-last BF16 on the nodal grid ([z][y][x][c], c a
// multiple of 16).  A convolution is an implicit GEMM: a CTA owns an output
// tile of 32 x 4 x 1 nodes (M = 128 GEMM rows, x fastest); for each of the 27
// taps one TMA 4-D box (c, 32, 4, 1) of the input, shifted by the tap's
// offset, lands in shared memory in the K-major swizzled layout the MMA reads
// (coordinates outside the grid read zero: the convolution's zero padding),
// together with the tap's weight block (N x c, K-major).  One thread issues
// the MMAs (K = 16 per instruction) into an FP32 accumulator of N tensor-
// memory columns; a 4-stage mbarrier pipeline overlaps the loads of later
// taps with the MMAs of earlier ones.  The four warps then read the
// accumulator (one GEMM row per thread), add the bias, apply ReLU and store
// the row.
//
// The same kernel computes the data gradient of a convolution: with `flip`
// the tap offsets are negated and the weights are the transposed blocks
// W_t^T, so out[u] = sum_t W_t^T in[u - o_t].
//
// Inputs may have two segments (a concatenation: upsampled features and a
// skip connection), each with its own tensor map and swizzle; outputs may be
// split into two column segments (the data gradient of a concatenated input).
#pragma once

#include "tc.cuh"

namespace simp {
namespace conv {

constexpr int kThreads = 128;
constexpr int kStages = 4;
constexpr int kTileX = 32, kTileY = 4;

struct ConvArgs {
  int nx, ny, nz;       // grid (nodes): input and output
  int nseg;             // input segments (1 or 2)
  int cseg[2];          // channels of each input segment (16, 32 or 64)
  int n;                // GEMM N: output columns (multiple of 16, <= 128)
  int flip;             // 1: tap t reads the offset -o_t (data gradient)
  const float* bias;    // n values, or null
  int relu;             // 1: max(0, .)
  int nout;             // output segments (1 or 2): columns [0, out_c[0]), [out_c[0], + out_c[1])
  int out_c[2];         // columns of each output segment
  int out_pitch[2];     // channels per node of each output tensor
  int out_f32[2];       // 1: FP32 output tensor, 0: BF16
  void* out[2];
  int* status;          // set on a wait that ran out
};

__host__ __device__ constexpr int round1024(int b) { return (b + 1023) & ~1023; }

__host__ __device__ inline int stage_bytes(const ConvArgs& p, int* a0, int* a1, int* b0, int* b1) {
  *a0 = kTileX * kTileY * p.cseg[0] * 2;
  *a1 = p.nseg > 1 ? kTileX * kTileY * p.cseg[1] * 2 : 0;
  *b0 = round1024(p.n * p.cseg[0] * 2);
  *b1 = p.nseg > 1 ? round1024(p.n * p.cseg[1] * 2) : 0;
  return *a0 + *a1 + *b0 + *b1;
}

__host__ __device__ inline size_t smem_bytes(const ConvArgs& p) {
  int a0, a1, b0, b1;
  const int st = stage_bytes(p, &a0, &a1, &b0, &b1);
  return 1024 + static_cast<size_t>(kStages) * st + 256;
}

__host__ __device__ inline uint32_t tmem_cols(int n) {
  uint32_t c = 32;
  while (c < static_cast<uint32_t>(n)) c <<= 1;
  return c;
}

__device__ __forceinline__ void tap_offset(int t, int flip, int& dx, int& dy, int& dz) {
  dz = t / 9 - 1;
  dy = (t / 3) % 3 - 1;
  dx = t % 3 - 1;
  if (flip) {
    dx = -dx;
    dy = -dy;
    dz = -dz;
  }
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&v);
}

__global__ void __launch_bounds__(kThreads) k_conv_tc(const __grid_constant__ CUtensorMap a0map,
                                                      const __grid_constant__ CUtensorMap a1map,
                                                      const __grid_constant__ CUtensorMap b0map,
                                                      const __grid_constant__ CUtensorMap b1map, const ConvArgs p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  int abytes0, abytes1, bbytes0, bbytes1;
  const int stage = stage_bytes(p, &abytes0, &abytes1, &bbytes0, &bbytes1);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * stage);
  uint64_t* empty = full + kStages;
  uint64_t* done = empty + kStages;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int x0 = blockIdx.x * kTileX, y0 = blockIdx.y * kTileY, z0 = blockIdx.z;
  const uint32_t ncols = tmem_cols(p.n);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(done, 1);
    tc::fence_mbar_init();
    tc::prefetch_map(&a0map);
    tc::prefetch_map(&b0map);
    if (p.nseg > 1) {
      tc::prefetch_map(&a1map);
      tc::prefetch_map(&b1map);
    }
  }
  if (warp == 0) tc::tmem_alloc(tslot, ncols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;

  const uint32_t tx_bytes = static_cast<uint32_t>(kTileX * kTileY * 2 * (p.cseg[0] + (p.nseg > 1 ? p.cseg[1] : 0)) +
                                                  p.n * 2 * (p.cseg[0] + (p.nseg > 1 ? p.cseg[1] : 0)));
  if (warp == 0 && lane == 0) {
    // producer: the 27 taps' input boxes and weight blocks
    for (int t = 0; t < 27; ++t) {
      const int s = t % kStages, use = t / kStages;
      if (use > 0 && !tc::mbar_wait(&empty[s], (use - 1) & 1, p.status)) break;
      uint8_t* st = smem + s * stage;
      int dx, dy, dz;
      tap_offset(t, p.flip, dx, dy, dz);
      tc::mbar_arrive_expect_tx(&full[s], tx_bytes);
      tc::tma_load_4d(st, &a0map, 0, x0 + dx, y0 + dy, z0 + dz, &full[s]);
      if (p.nseg > 1) tc::tma_load_4d(st + abytes0, &a1map, 0, x0 + dx, y0 + dy, z0 + dz, &full[s]);
      tc::tma_load_2d(st + abytes0 + abytes1, &b0map, 0, t * p.n, &full[s]);
      if (p.nseg > 1) tc::tma_load_2d(st + abytes0 + abytes1 + bbytes0, &b1map, p.cseg[0], t * p.n, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    const uint32_t idesc = tc::idesc_bf16(128, p.n);
    for (int t = 0; t < 27; ++t) {
      const int s = t % kStages, use = t / kStages;
      if (!tc::mbar_wait(&full[s], use & 1, p.status)) break;
      tc::fence_after_sync();
      const uint32_t base = tc::smem_u32(smem + s * stage);
      for (int seg = 0; seg < p.nseg; ++seg) {
        const uint32_t a_addr = base + (seg ? abytes0 : 0);
        const uint32_t b_addr = base + abytes0 + abytes1 + (seg ? bbytes0 : 0);
        const int rb = p.cseg[seg] * 2;
        for (int kk = 0; kk < p.cseg[seg] / 16; ++kk)
          tc::mma_bf16(tmem, tc::smem_desc(a_addr + kk * 32, rb), tc::smem_desc(b_addr + kk * 32, rb), idesc,
                       (t | seg | kk) != 0 ? 1u : 0u);
      }
      tc::mma_commit(&empty[s]);
    }
    tc::mma_commit(done);
  }
  __syncwarp();

  // epilogue: thread (warp, lane) owns GEMM row 32 warp + lane
  const bool ok = tc::mbar_wait(done, 0, p.status);
  tc::fence_after_sync();
  const int row = warp * 32 + lane;
  const int gx = x0 + (row % kTileX), gy = y0 + row / kTileX, gz = z0;
  const bool valid = ok && gx < p.nx && gy < p.ny && gz < p.nz;
  const long long node = (static_cast<long long>(gz) * p.ny + gy) * p.nx + gx;
  for (int c0 = 0; c0 < p.n; c0 += 16) {
    float v[16];
    tc::tmem_ld16(tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c0), v);
    if (!valid) continue;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      if (p.bias) v[k] += p.bias[c0 + k];
      if (p.relu) v[k] = fmaxf(v[k], 0.0f);
    }
    const int seg = (p.nout > 1 && c0 >= p.out_c[0]) ? 1 : 0;
    const int lc = c0 - (seg ? p.out_c[0] : 0);
    if (lc >= p.out_c[seg]) continue;
    if (p.out_f32[seg]) {
      float* o = static_cast<float*>(p.out[seg]) + node * p.out_pitch[seg] + lc;
      for (int k = 0; k < 16 && lc + k < p.out_c[seg]; ++k) o[k] = v[k];
    } else {
      uint4* o = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(p.out[seg]) + node * p.out_pitch[seg] + lc);
      o[0] = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
      o[1] = make_uint4(pack_bf16(v[8], v[9]), pack_bf16(v[10], v[11]), pack_bf16(v[12], v[13]),
                        pack_bf16(v[14], v[15]));
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, ncols);
  }
}

}  // namespace conv
}  // namespace simp
