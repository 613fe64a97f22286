// The displacement surrogate network: a four-level 3-D encoder-decoder on the
// nodal grid (channels 16 / 32 / 64 / 64, 3 x 3 x 3 convolutions, BF16
// weights and activations, FP32 accumulation), trained on (filtered density,
// load) -> displacement pairs from solver runs and used as a PCG start.
//
// Levels: the grid of level l + 1 has n / 2 + 1 nodes per axis for n on
// level l; features move down by full-weighting restriction R = P^T / 8 and
// up by the trilinear nodal prolongation P (weights 1, 1/2 per axis), so
// every convolution is stride 1.  Layers (input channels -> output):
//   e0a 16 -> 16, e0b 16 -> 16 = s0        (input: density, load x y z, zeros)
//   e1a 16 -> 32, e1b 32 -> 32 = s1        (on R s0)
//   e2a 32 -> 64, e2b 64 -> 64 = s2        (on R s1)
//   e3a 64 -> 64, e3b 64 -> 64 = b3        (on R s2)
//   d2 [P b3 | s2] 128 -> 64, d1 [P d2 | s1] 96 -> 32, d0 [P d1 | s0] 48 -> 16
//   head 16 -> 3 (no activation; FP32 output, padded to 16 columns)
// ReLU after every layer but the head.  The input's density channel is the
// mean of the cell densities around a node; the load channels are the nodal
// load divided by its largest component.  The target is the displacement
// divided by its largest component: the network predicts the shape, and the
// PCG start takes the energy-optimal multiple (with the previous
// displacements) under the current stiffness.
#include "../../include/simp_gpu.h"

#include "kernels.cuh"
#include "problem.h"
#include "surrogate.h"
#include "surrogate_net.h"
#include "topopt.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <sstream>

namespace simp {
namespace sg {

namespace {

constexpr int kIn = 16;  // input channels (4 used)

struct LayerDef {
  int nin;      // input segments
  int cin[2];   // channels per segment
  int cout;     // output channels (3 for the head)
  int relu;
};

// e0a e0b e1a e1b e2a e2b e3a e3b d2 d1 d0 head
const LayerDef kLayers[kNumLayers] = {
    {1, {16, 0}, 16, 1}, {1, {16, 0}, 16, 1}, {1, {16, 0}, 32, 1}, {1, {32, 0}, 32, 1},
    {1, {32, 0}, 64, 1}, {1, {64, 0}, 64, 1}, {1, {64, 0}, 64, 1}, {1, {64, 0}, 64, 1},
    {2, {64, 64}, 64, 1}, {2, {64, 32}, 32, 1}, {2, {32, 16}, 16, 1}, {1, {16, 0}, 3, 0}};

int npad(int c) { return (c + 15) / 16 * 16; }
int cin_total(const LayerDef& L) { return L.cin[0] + (L.nin > 1 ? L.cin[1] : 0); }

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

// fine = scale * P coarse (+ fine when accumulate): trilinear nodal weights
__global__ void k_prolong(int C, int nx, int ny, int nz, int cx, int cy, int cz, const __nv_bfloat16* __restrict__ coarse,
                          __nv_bfloat16* __restrict__ fine, float scale, int accumulate) {
  const long long total = static_cast<long long>(nx) * ny * nz * C;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int c = static_cast<int>(e % C);
    const long long v = e / C;
    const int x = static_cast<int>(v % nx), y = static_cast<int>((v / nx) % ny),
              z = static_cast<int>(v / (static_cast<long long>(nx) * ny));
    int ix[2], iy[2], iz[2];
    float wx[2], wy[2], wz[2];
    int nxs = 1, nys = 1, nzs = 1;
    ix[0] = x >> 1; wx[0] = 1.0f;
    if (x & 1) { ix[1] = ix[0] + 1; wx[0] = wx[1] = 0.5f; nxs = 2; }
    iy[0] = y >> 1; wy[0] = 1.0f;
    if (y & 1) { iy[1] = iy[0] + 1; wy[0] = wy[1] = 0.5f; nys = 2; }
    iz[0] = z >> 1; wz[0] = 1.0f;
    if (z & 1) { iz[1] = iz[0] + 1; wz[0] = wz[1] = 0.5f; nzs = 2; }
    float s = 0.0f;
    for (int a = 0; a < nzs; ++a)
      for (int b = 0; b < nys; ++b)
        for (int d = 0; d < nxs; ++d)
          if (ix[d] < cx && iy[b] < cy && iz[a] < cz)
            s += wz[a] * wy[b] * wx[d] * bf(coarse[((static_cast<long long>(iz[a]) * cy + iy[b]) * cx + ix[d]) * C + c]);
    s *= scale;
    if (accumulate) s += bf(fine[e]);
    fine[e] = __float2bfloat16_rn(s);
  }
}

// coarse = scale * P^T fine (full weighting with scale 1/8)
__global__ void k_restrict(int C, int nx, int ny, int nz, int cx, int cy, int cz, const __nv_bfloat16* __restrict__ fine,
                           __nv_bfloat16* __restrict__ coarse, float scale) {
  const long long total = static_cast<long long>(cx) * cy * cz * C;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int c = static_cast<int>(e % C);
    const long long V = e / C;
    const int X = static_cast<int>(V % cx), Y = static_cast<int>((V / cx) % cy),
              Z = static_cast<int>(V / (static_cast<long long>(cx) * cy));
    float s = 0.0f;
    for (int dz = -1; dz <= 1; ++dz) {
      const int z = 2 * Z + dz;
      if (z < 0 || z >= nz) continue;
      const float wz = dz ? 0.5f : 1.0f;
      for (int dy = -1; dy <= 1; ++dy) {
        const int y = 2 * Y + dy;
        if (y < 0 || y >= ny) continue;
        const float wy = dy ? 0.5f : 1.0f;
        for (int dx = -1; dx <= 1; ++dx) {
          const int x = 2 * X + dx;
          if (x < 0 || x >= nx) continue;
          const float wx = dx ? 0.5f : 1.0f;
          s += wz * wy * wx * bf(fine[((static_cast<long long>(z) * ny + y) * nx + x) * C + c]);
        }
      }
    }
    coarse[e] = __float2bfloat16_rn(s * scale);
  }
}

// g = a > 0 ? g : 0
__global__ void k_relu_bwd(long long n, const __nv_bfloat16* __restrict__ a, __nv_bfloat16* __restrict__ g) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    if (!(bf(a[e]) > 0.0f)) g[e] = __float2bfloat16_rn(0.0f);
}

// a += b
__global__ void k_add(long long n, __nv_bfloat16* __restrict__ a, const __nv_bfloat16* __restrict__ b) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    a[e] = __float2bfloat16_rn(bf(a[e]) + bf(b[e]));
}

// 4 stored input channels -> the 16-channel network input
__global__ void k_expand_input(long long nodes, const __nv_bfloat16* __restrict__ in4, __nv_bfloat16* __restrict__ in16) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nodes; v += (long long)gridDim.x * blockDim.x) {
    uint4 lo, hi = make_uint4(0, 0, 0, 0);
    const uint2 src = *reinterpret_cast<const uint2*>(in4 + v * 4);
    lo = make_uint4(src.x, src.y, 0, 0);
    uint4* dst = reinterpret_cast<uint4*>(in16 + v * kIn);
    dst[0] = lo;
    dst[1] = hi;
  }
}

// Squared error of the prediction at the free components against the target
// (block partials) and its gradient 2 (pred - target) / count into the head's
// 16-column output gradient (BF16; unused columns zero).
__global__ void __launch_bounds__(256) k_loss(long long nodes, const float* __restrict__ pred,
                                              const __nv_bfloat16* __restrict__ target,
                                              const uint8_t* __restrict__ mask, float inv_count,
                                              __nv_bfloat16* __restrict__ grad, double* __restrict__ part) {
  double s = 0.0;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nodes; v += (long long)gridDim.x * blockDim.x) {
    float g[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (mask[v] & (1 << k)) {
        const float d = pred[v * 3 + k] - bf(target[v * 3 + k]);
        s += static_cast<double>(d) * d;
        g[k] = 2.0f * d * inv_count;
      }
    }
    const __nv_bfloat162 p01 = __floats2bfloat162_rn(g[0], g[1]), p23 = __floats2bfloat162_rn(g[2], g[3]);
    uint4* dst = reinterpret_cast<uint4*>(grad + v * 16);
    dst[0] = make_uint4(*reinterpret_cast<const uint32_t*>(&p01), *reinterpret_cast<const uint32_t*>(&p23), 0u, 0u);
    dst[1] = make_uint4(0u, 0u, 0u, 0u);
  }
  s = block_sum<256>(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Adam step on the FP32 master parameters, then the BF16 weight copies:
// forward [27][npad][cin] and transposed (data gradient) [27][cin][npad].
__global__ void k_adam(long long n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float c1, float c2, float eps, float gscale) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float gi = g[e] * gscale;
    const float mi = b1 * m[e] + (1.0f - b1) * gi;
    const float vi = b2 * v[e] + (1.0f - b2) * gi * gi;
    m[e] = mi;
    v[e] = vi;
    w[e] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  }
}

__global__ void k_pack_weights(int cout, int np, int cin, const float* __restrict__ w, __nv_bfloat16* __restrict__ wf,
                               __nv_bfloat16* __restrict__ wt) {
  const int total = 27 * np * cin;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int t = e / (np * cin), r = (e / cin) % np, c = e % cin;
    const float val = r < cout ? w[(t * cout + r) * cin + c] : 0.0f;
    const __nv_bfloat16 b = __float2bfloat16_rn(val);
    wf[e] = b;
    wt[(t * cin + c) * np + r] = b;
  }
}

// network input from a problem's state: channel 0 the mean density of the
// cells around a node, 1..3 the nodal load / its largest component (zero on
// clamped components); 4 channels per node
__global__ void k_problem_input(GridView g, const double* __restrict__ rho, const double* __restrict__ f,
                                const i32* __restrict__ free_index, double inv_fmax, __nv_bfloat16* __restrict__ in4) {
  const long long nodes = static_cast<long long>(g.nnx) * g.nny * g.nnz;
  for (long long nd = blockIdx.x * (long long)blockDim.x + threadIdx.x; nd < nodes;
       nd += (long long)gridDim.x * blockDim.x) {
    const int ix = static_cast<int>(nd % g.nnx), iy = static_cast<int>((nd / g.nnx) % g.nny),
              iz = static_cast<int>(nd / (static_cast<long long>(g.nnx) * g.nny));
    double s = 0.0;
    int cnt = 0;
    const int zlo = g.dim == 3 ? -1 : 0;
    for (int dz = zlo; dz <= 0; ++dz)
      for (int dy = -1; dy <= 0; ++dy)
        for (int dx = -1; dx <= 0; ++dx) {
          const int cx = ix + dx, cy = iy + dy, cz = iz + dz;
          if (cx < 0 || cx >= g.nx || cy < 0 || cy >= g.ny || cz < 0 || cz >= g.nz) continue;
          s += rho[(static_cast<long long>(cz) * g.ny + cy) * g.nx + cx];
          ++cnt;
        }
    float val[4] = {cnt ? static_cast<float>(s / cnt) : 0.0f, 0.0f, 0.0f, 0.0f};
    for (int k = 0; k < 3; ++k) {
      if (k < g.dim) {
        const i32 fi = free_index[nd * g.dim + k];
        if (fi >= 0) val[1 + k] = static_cast<float>(f[fi] * inv_fmax);
      }
    }
    const __nv_bfloat162 p01 = __floats2bfloat162_rn(val[0], val[1]), p23 = __floats2bfloat162_rn(val[2], val[3]);
    *reinterpret_cast<uint2*>(in4 + nd * 4) =
        make_uint2(*reinterpret_cast<const uint32_t*>(&p01), *reinterpret_cast<const uint32_t*>(&p23));
  }
}

// training target: u / max|u| at free components (BF16, 3 per node) and the
// free-component mask
__global__ void k_problem_target(long long nodes, int dim, const double* __restrict__ u, const i32* __restrict__ free_index,
                                 double inv_umax, __nv_bfloat16* __restrict__ tgt, uint8_t* __restrict__ mask) {
  for (long long nd = blockIdx.x * (long long)blockDim.x + threadIdx.x; nd < nodes;
       nd += (long long)gridDim.x * blockDim.x) {
    uint8_t mk = 0;
    for (int k = 0; k < 3; ++k) {
      float val = 0.0f;
      if (k < dim) {
        const i32 fi = free_index[nd * dim + k];
        if (fi >= 0) {
          val = static_cast<float>(u[fi] * inv_umax);
          mk |= static_cast<uint8_t>(1 << k);
        }
      }
      tgt[nd * 3 + k] = __float2bfloat16_rn(val);
    }
    mask[nd] = mk;
  }
}

// prediction (FP32, 3 per node) -> free-DOF vector
__global__ void k_prediction_to_dofs(long long nodes, int dim, const float* __restrict__ pred,
                                     const i32* __restrict__ free_index, double* __restrict__ u) {
  for (long long nd = blockIdx.x * (long long)blockDim.x + threadIdx.x; nd < nodes;
       nd += (long long)gridDim.x * blockDim.x)
    for (int k = 0; k < dim; ++k) {
      const i32 fi = free_index[nd * dim + k];
      if (fi >= 0) {
        const float p = pred[nd * 3 + k];
        u[fi] = isfinite(p) ? static_cast<double>(p) : 0.0;
      }
    }
}

__global__ void __launch_bounds__(256) k_absmax(long long n, const double* __restrict__ a, double* __restrict__ part) {
  double s = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    s = fmax(s, fabs(a[e]));
  for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
  __shared__ double wm[8];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int k = 0; k < 8; ++k) m = fmax(m, wm[k]);
    part[blockIdx.x] = m;
  }
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

inline int blocks_for(long long n) { return static_cast<int>(std::min<long long>((n + 255) / 256, 4096)); }

}  // namespace

// ---------------------------------------------------------------------------
Net::Net(uint64_t seed) {
  size_t off = 0;
  for (int l = 0; l < kNumLayers; ++l) {
    const LayerDef& L = kLayers[l];
    woff[l] = off;
    off += static_cast<size_t>(27) * L.cout * cin_total(L);
    boff[l] = off;
    off += static_cast<size_t>(L.cout);
  }
  nparams = off;
  master.alloc(nparams);
  grad.alloc(nparams);
  m1.alloc(nparams);
  m2.alloc(nparams);
  m1.zero();
  m2.zero();
  grad.zero();
  // He-uniform initial weights (fan-in 27 cin), zero biases; seeded
  std::vector<float> h(nparams, 0.0f);
  uint64_t s = seed;
  for (int l = 0; l < kNumLayers; ++l) {
    const LayerDef& L = kLayers[l];
    const double fan = 27.0 * cin_total(L);
    const double a = std::sqrt(6.0 / fan) * (l == kNumLayers - 1 ? 0.1 : 1.0);
    for (size_t k = 0; k < static_cast<size_t>(27) * L.cout * cin_total(L); ++k) {
      const double r = static_cast<double>(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
      h[woff[l] + k] = static_cast<float>((2.0 * r - 1.0) * a);
    }
  }
  master.upload(h);
  for (int l = 0; l < kNumLayers; ++l) {
    const LayerDef& L = kLayers[l];
    wf[l].alloc(static_cast<size_t>(27) * npad(L.cout) * cin_total(L));
    wt[l].alloc(static_cast<size_t>(27) * npad(L.cout) * cin_total(L));
  }
  size_t maxpart = 0;
  for (int l = 0; l < kNumLayers; ++l) maxpart = std::max(maxpart, wgrad_partial_floats(npad(kLayers[l].cout), cin_total(kLayers[l])));
  wpart.alloc(maxpart);
  status.alloc(1);
  status.zero();
  lpart.alloc(4096);
  SIMP_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  pack();
}

Net::~Net() {
  if (stream) cudaStreamDestroy(stream);
}

void Net::pack() {
  for (int l = 0; l < kNumLayers; ++l) {
    const LayerDef& L = kLayers[l];
    k_pack_weights<<<64, 256, 0, stream>>>(L.cout, npad(L.cout), cin_total(L), master.p + woff[l], wf[l].p, wt[l].p);
    SIMP_CHECK_LAUNCH();
  }
}

void Net::set_params(const float* host) {
  SIMP_CUDA(cudaMemcpyAsync(master.p, host, sizeof(float) * nparams, cudaMemcpyHostToDevice, stream));
  pack();
  SIMP_CUDA(cudaStreamSynchronize(stream));
}

void Net::get_params(float* host) {
  SIMP_CUDA(cudaMemcpyAsync(host, master.p, sizeof(float) * nparams, cudaMemcpyDeviceToHost, stream));
  SIMP_CUDA(cudaStreamSynchronize(stream));
}

void Net::shape(int nx, int ny, int nz) {
  if (nx == gx[0] && ny == gy[0] && nz == gz[0]) return;
  gx[0] = nx;
  gy[0] = ny;
  gz[0] = nz;
  for (int k = 1; k < 4; ++k) {
    gx[k] = gx[k - 1] / 2 + 1;
    gy[k] = gy[k - 1] / 2 + 1;
    gz[k] = gz[k - 1] / 2 + 1;
  }
  auto nodes = [&](int k) { return static_cast<size_t>(gx[k]) * gy[k] * gz[k]; };
  in16.alloc(nodes(0) * kIn);
  // activations (outputs of each layer) and grid-transfer results
  const int lvl[kNumLayers] = {0, 0, 1, 1, 2, 2, 3, 3, 2, 1, 0, 0};
  for (int l = 0; l < kNumLayers; ++l) {
    lvl_of[l] = lvl[l];
    if (l == kNumLayers - 1) continue;
    act[l].alloc(nodes(lvl[l]) * kLayers[l].cout);
    gact[l].alloc(nodes(lvl[l]) * kLayers[l].cout);
  }
  out.alloc(nodes(0) * 3);
  gout.alloc(nodes(0) * 16);
  for (int k = 1; k < 4; ++k) {  // R s_{k-1} on level k, and its gradient
    const int c = kLayers[2 * k - 1].cout;
    down[k].alloc(nodes(k) * c);
    gdown[k].alloc(nodes(k) * c);
  }
  for (int k = 0; k < 3; ++k) {  // P (decoder input from level k + 1) on level k, and its gradient
    const int c = k == 2 ? 64 : kLayers[8 + (1 - k)].cout;  // P b3 (64), P d2 (64), P d1 (32)
    up[k].alloc(nodes(k) * c);
    gup[k].alloc(nodes(k) * c);
  }
}

void Net::conv(int l, const void* in0, const void* in1, void* outp, int out_f32, bool data_grad, void* gout0,
               void* gout1) {
  const LayerDef& L = kLayers[l];
  const int lv = lvl_of[l];
  ConvSpec s;
  s.nx = gx[lv];
  s.ny = gy[lv];
  s.nz = gz[lv];
  s.status = status.p;
  if (!data_grad) {
    s.nseg = L.nin;
    s.in[0] = in0;
    s.in[1] = in1;
    s.cseg[0] = L.cin[0];
    s.cseg[1] = L.nin > 1 ? L.cin[1] : 0;
    s.w = wf[l].p;
    s.n = npad(L.cout);
    s.bias = master.p + boff[l];
    s.relu = L.relu;
    s.nout = 1;
    s.out[0] = outp;
    s.out_c[0] = L.cout;
    s.out_pitch[0] = out_f32 ? 3 : L.cout;
    s.out_f32[0] = out_f32;
    if (L.cout % 16) {  // the head: the bias has 3 entries, so add none here and fold it below
      s.bias = nullptr;
    }
  } else {
    // data gradient: in = the output gradient (npad(cout) channels), out =
    // the input segments' gradients
    s.nseg = 1;
    s.in[0] = in0;
    s.cseg[0] = npad(L.cout);
    s.w = wt[l].p;
    s.n = cin_total(L);
    s.flip = 1;
    s.nout = L.nin;
    s.out[0] = gout0;
    s.out[1] = gout1;
    s.out_c[0] = L.cin[0];
    s.out_c[1] = L.nin > 1 ? L.cin[1] : 0;
    s.out_pitch[0] = L.cin[0];
    s.out_pitch[1] = L.nin > 1 ? L.cin[1] : 0;
  }
  conv_launch(s, stream);
}

// head bias (3 values) added to the FP32 output
__global__ void k_head_bias(long long nodes, const float* __restrict__ b, float* __restrict__ out) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nodes; v += (long long)gridDim.x * blockDim.x)
    for (int k = 0; k < 3; ++k) out[v * 3 + k] += b[k];
}

void Net::transfer_down(int k, const __nv_bfloat16* fine, __nv_bfloat16* coarse, int c, float scale) {
  const long long n = static_cast<long long>(gx[k]) * gy[k] * gz[k] * c;
  k_restrict<<<blocks_for(n), 256, 0, stream>>>(c, gx[k - 1], gy[k - 1], gz[k - 1], gx[k], gy[k], gz[k], fine, coarse,
                                                scale);
  SIMP_CHECK_LAUNCH();
}

void Net::transfer_up(int k, const __nv_bfloat16* coarse, __nv_bfloat16* fine, int c, float scale, int acc) {
  const long long n = static_cast<long long>(gx[k]) * gy[k] * gz[k] * c;
  k_prolong<<<blocks_for(n), 256, 0, stream>>>(c, gx[k], gy[k], gz[k], gx[k + 1], gy[k + 1], gz[k + 1], coarse, fine,
                                               scale, acc);
  SIMP_CHECK_LAUNCH();
}

void Net::forward() {
  using B = __nv_bfloat16;
  conv(0, in16.p, nullptr, act[0].p, 0);
  conv(1, act[0].p, nullptr, act[1].p, 0);                   // s0
  transfer_down(1, act[1].p, down[1].p, 16, 0.125f);
  conv(2, down[1].p, nullptr, act[2].p, 0);
  conv(3, act[2].p, nullptr, act[3].p, 0);                   // s1
  transfer_down(2, act[3].p, down[2].p, 32, 0.125f);
  conv(4, down[2].p, nullptr, act[4].p, 0);
  conv(5, act[4].p, nullptr, act[5].p, 0);                   // s2
  transfer_down(3, act[5].p, down[3].p, 64, 0.125f);
  conv(6, down[3].p, nullptr, act[6].p, 0);
  conv(7, act[6].p, nullptr, act[7].p, 0);                   // b3
  transfer_up(2, act[7].p, up[2].p, 64, 1.0f, 0);
  conv(8, up[2].p, act[5].p, act[8].p, 0);                   // d2
  transfer_up(1, act[8].p, up[1].p, 64, 1.0f, 0);
  conv(9, up[1].p, act[3].p, act[9].p, 0);                   // d1
  transfer_up(0, act[9].p, up[0].p, 32, 1.0f, 0);
  conv(10, up[0].p, act[1].p, act[10].p, 0);                 // d0
  conv(11, act[10].p, nullptr, out.p, 1);                    // head (FP32)
  const long long n0 = static_cast<long long>(gx[0]) * gy[0] * gz[0];
  k_head_bias<<<blocks_for(n0), 256, 0, stream>>>(n0, master.p + boff[11], out.p);
  SIMP_CHECK_LAUNCH();
  (void)sizeof(B);
}

void Net::wgrad(int l, const void* x0, const void* x1, const void* dy) {
  const LayerDef& L = kLayers[l];
  const int lv = lvl_of[l];
  WgradSpec s;
  s.nx = gx[lv];
  s.ny = gy[lv];
  s.nz = gz[lv];
  s.nseg = L.nin;
  s.x0 = static_cast<const __nv_bfloat16*>(x0);
  s.c0 = L.cin[0];
  s.x1 = static_cast<const __nv_bfloat16*>(x1);
  s.c1 = L.nin > 1 ? L.cin[1] : 0;
  s.dy = static_cast<const __nv_bfloat16*>(dy);
  s.cdy = npad(L.cout);
  s.cout = L.cout;
  s.gw = grad.p + woff[l];
  s.gb = grad.p + boff[l];
  wgrad_launch(s, wpart.p, stream);
}

// Backward pass from gout (the head's output gradient, 16 columns per node):
// parameter gradients are added to `grad`.
void Net::backward() {
  auto relu_bwd = [&](int l, __nv_bfloat16* g) {
    const long long n = static_cast<long long>(gx[lvl_of[l]]) * gy[lvl_of[l]] * gz[lvl_of[l]] * kLayers[l].cout;
    k_relu_bwd<<<blocks_for(n), 256, 0, stream>>>(n, act[l].p, g);
    SIMP_CHECK_LAUNCH();
  };
  auto add = [&](int l, __nv_bfloat16* a, const __nv_bfloat16* b) {
    const long long n = static_cast<long long>(gx[lvl_of[l]]) * gy[lvl_of[l]] * gz[lvl_of[l]] * kLayers[l].cout;
    k_add<<<blocks_for(n), 256, 0, stream>>>(n, a, b);
    SIMP_CHECK_LAUNCH();
  };
  // head
  wgrad(11, act[10].p, nullptr, gout.p);
  conv(11, gout.p, nullptr, nullptr, 0, true, gact[10].p, nullptr);
  relu_bwd(10, gact[10].p);
  // d0 = conv([P d1 | s0]) -> g(P d1) in gup[0], g s0 (decoder part) in gact[1]
  wgrad(10, up[0].p, act[1].p, gact[10].p);
  conv(10, gact[10].p, nullptr, nullptr, 0, true, gup[0].p, gact[1].p);
  transfer_down(1, gup[0].p, gact[9].p, 32, 1.0f);           // g d1 = P^T g(P d1)
  relu_bwd(9, gact[9].p);
  wgrad(9, up[1].p, act[3].p, gact[9].p);
  conv(9, gact[9].p, nullptr, nullptr, 0, true, gup[1].p, gact[3].p);
  transfer_down(2, gup[1].p, gact[8].p, 64, 1.0f);           // g d2
  relu_bwd(8, gact[8].p);
  wgrad(8, up[2].p, act[5].p, gact[8].p);
  conv(8, gact[8].p, nullptr, nullptr, 0, true, gup[2].p, gact[5].p);
  transfer_down(3, gup[2].p, gact[7].p, 64, 1.0f);           // g b3
  // bottom
  relu_bwd(7, gact[7].p);
  wgrad(7, act[6].p, nullptr, gact[7].p);
  conv(7, gact[7].p, nullptr, nullptr, 0, true, gact[6].p, nullptr);
  relu_bwd(6, gact[6].p);
  wgrad(6, down[3].p, nullptr, gact[6].p);
  conv(6, gact[6].p, nullptr, nullptr, 0, true, gdown[3].p, nullptr);
  // s2 = e2b: decoder gradient (gact[5]) + R^T of the bottom input gradient
  transfer_up(2, gdown[3].p, gact[5].p, 64, 0.125f, 1);
  relu_bwd(5, gact[5].p);
  wgrad(5, act[4].p, nullptr, gact[5].p);
  conv(5, gact[5].p, nullptr, nullptr, 0, true, gact[4].p, nullptr);
  relu_bwd(4, gact[4].p);
  wgrad(4, down[2].p, nullptr, gact[4].p);
  conv(4, gact[4].p, nullptr, nullptr, 0, true, gdown[2].p, nullptr);
  transfer_up(1, gdown[2].p, gact[3].p, 32, 0.125f, 1);      // s1
  relu_bwd(3, gact[3].p);
  wgrad(3, act[2].p, nullptr, gact[3].p);
  conv(3, gact[3].p, nullptr, nullptr, 0, true, gact[2].p, nullptr);
  relu_bwd(2, gact[2].p);
  wgrad(2, down[1].p, nullptr, gact[2].p);
  conv(2, gact[2].p, nullptr, nullptr, 0, true, gdown[1].p, nullptr);
  transfer_up(0, gdown[1].p, gact[1].p, 16, 0.125f, 1);      // s0
  relu_bwd(1, gact[1].p);
  wgrad(1, act[0].p, nullptr, gact[1].p);
  conv(1, gact[1].p, nullptr, nullptr, 0, true, gact[0].p, nullptr);
  relu_bwd(0, gact[0].p);
  wgrad(0, in16.p, nullptr, gact[0].p);
  (void)add;
}

double Net::loss(const __nv_bfloat16* target, const uint8_t* mask, long long count) {
  const long long n0 = static_cast<long long>(gx[0]) * gy[0] * gz[0];
  const int blocks = std::min(blocks_for(n0), 4096);
  k_loss<<<blocks, 256, 0, stream>>>(n0, out.p, target, mask, 1.0f / static_cast<float>(std::max(1LL, count)), gout.p,
                                     lpart.p);
  SIMP_CHECK_LAUNCH();
  std::vector<double> h(static_cast<size_t>(blocks));
  SIMP_CUDA(cudaMemcpyAsync(h.data(), lpart.p, sizeof(double) * blocks, cudaMemcpyDeviceToHost, stream));
  SIMP_CUDA(cudaStreamSynchronize(stream));
  double s = 0.0;
  for (double v : h) s += v;
  return s / static_cast<double>(std::max(1LL, count));
}

void Net::adam_step(float lr, float gscale) {
  ++adam_t;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f / (1.0f - std::pow(b1, static_cast<float>(adam_t)));
  const float c2 = 1.0f / (1.0f - std::pow(b2, static_cast<float>(adam_t)));
  k_adam<<<blocks_for(static_cast<long long>(nparams)), 256, 0, stream>>>(static_cast<long long>(nparams), master.p, grad.p,
                                                                          m1.p, m2.p, lr, b1, b2, c1, c2, 1e-8f, gscale);
  SIMP_CHECK_LAUNCH();
  grad.zero(stream);
  pack();
}

void Net::check_status() {
  int h = 0;
  SIMP_CUDA(cudaMemcpyAsync(&h, status.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
  SIMP_CUDA(cudaStreamSynchronize(stream));
  if (h) throw Error(kCudaError, "surrogate: a tensor-core pipeline wait timed out");
}

// ---------------------------------------------------------------------------
// Samples and the problem-facing operations
// ---------------------------------------------------------------------------
static double device_absmax(const double* a, long long n, DBuf<double>& part, cudaStream_t s) {
  const int blocks = 512;
  part.alloc(blocks);
  k_absmax<<<blocks, 256, 0, s>>>(n, a, part.p);
  SIMP_CHECK_LAUNCH();
  std::vector<double> h(blocks);
  SIMP_CUDA(cudaMemcpyAsync(h.data(), part.p, sizeof(double) * blocks, cudaMemcpyDeviceToHost, s));
  SIMP_CUDA(cudaStreamSynchronize(s));
  return *std::max_element(h.begin(), h.end());
}

void Surrogate::input_of(GpuProblem& p, int load, __nv_bfloat16* in4) {
  GridView g;
  g.dim = p.d.dim;
  g.nx = p.d.nx;
  g.ny = p.d.ny;
  g.nz = p.d.dim == 3 ? p.d.nz : 1;
  g.nnx = p.d.nx + 1;
  g.nny = p.d.ny + 1;
  g.nnz = p.d.dim == 3 ? p.d.nz + 1 : 1;
  const double* f = p.b.p + static_cast<size_t>(load) * p.nfree;
  // the loads do not change: their largest component is taken once per problem
  if (p.load_absmax.size() != static_cast<size_t>(p.d.nloads))
    p.load_absmax.assign(static_cast<size_t>(p.d.nloads), -1.0);
  double& fmax = p.load_absmax[static_cast<size_t>(load)];
  if (fmax < 0.0) fmax = device_absmax(f, p.nfree, scratch, net.stream);
  const long long nodes = static_cast<long long>(g.nnx) * g.nny * g.nnz;
  k_problem_input<<<blocks_for(nodes), 256, 0, net.stream>>>(g, p.rho.p, f, p.dof_map.p,
                                                             fmax > 0.0 ? 1.0 / fmax : 0.0, in4);
  SIMP_CHECK_LAUNCH();
}

void Surrogate::add_sample(GpuProblem& p, int load) {
  if (p.d.dim != 3) throw Error(kBadInput, "the surrogate serves 3-D (Hex8) problems");
  if (!p.evaluated) throw Error(kBadInput, "add a surrogate sample after an evaluation (it needs a displacement)");
  SIMP_CUDA(cudaStreamSynchronize(p.amg.stream));
  Sample s;
  s.nx = p.d.nx + 1;
  s.ny = p.d.ny + 1;
  s.nz = p.d.nz + 1;
  const long long nodes = static_cast<long long>(s.nx) * s.ny * s.nz;
  s.in4.alloc(static_cast<size_t>(nodes) * 4);
  s.target.alloc(static_cast<size_t>(nodes) * 3);
  s.mask.alloc(static_cast<size_t>(nodes));
  input_of(p, load, s.in4.p);
  const double* u = p.u.p + static_cast<size_t>(load) * p.nfree;
  const double umax = device_absmax(u, p.nfree, scratch, net.stream);
  k_problem_target<<<blocks_for(nodes), 256, 0, net.stream>>>(nodes, 3, u, p.dof_map.p,
                                                              umax > 0.0 ? 1.0 / umax : 0.0, s.target.p, s.mask.p);
  SIMP_CHECK_LAUNCH();
  s.count = p.nfree;
  SIMP_CUDA(cudaStreamSynchronize(net.stream));
  samples.push_back(std::move(s));
}

double Surrogate::train(int epochs, double lr0, int batch, uint64_t seed) {
  if (samples.empty()) throw Error(kBadInput, "the surrogate has no training samples");
  std::vector<size_t> order(samples.size());
  std::iota(order.begin(), order.end(), 0);
  uint64_t s = seed;
  const long long steps = static_cast<long long>(epochs) * static_cast<long long>(samples.size());
  long long step = 0;
  double epoch_loss = 0.0;
  for (int ep = 0; ep < epochs; ++ep) {
    for (size_t k = order.size(); k > 1; --k) std::swap(order[k - 1], order[splitmix(s) % k]);
    double sum = 0.0;
    int in_batch = 0;
    for (size_t q = 0; q < order.size(); ++q, ++step) {
      Sample& smp = samples[order[q]];
      net.shape(smp.nx, smp.ny, smp.nz);
      const long long nodes = static_cast<long long>(smp.nx) * smp.ny * smp.nz;
      k_expand_input<<<blocks_for(nodes), 256, 0, net.stream>>>(nodes, smp.in4.p, net.in16.p);
      SIMP_CHECK_LAUNCH();
      net.forward();
      sum += net.loss(smp.target.p, smp.mask.p, smp.count);
      net.backward();
      if (++in_batch == batch || q + 1 == order.size()) {
        // cosine decay from lr0 to lr0 / 20
        const double frac = static_cast<double>(step) / std::max(1LL, steps - 1);
        const double lr = lr0 * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(3.141592653589793 * frac)));
        net.adam_step(static_cast<float>(lr), 1.0f / static_cast<float>(in_batch));
        in_batch = 0;
      }
    }
    net.check_status();
    epoch_loss = sum / static_cast<double>(order.size());
    losses.push_back(epoch_loss);
  }
  return epoch_loss;
}

Surrogate::~Surrogate() {
  if (after) cudaEventDestroy(after);
}

void Surrogate::predict(GpuProblem& p, int load, double* u_out) {
  std::lock_guard<std::mutex> lock(mu);
  // the problem's state is written on its own stream
  SIMP_CUDA(cudaStreamSynchronize(p.amg.stream));
  enqueue(p, load, u_out);
  SIMP_CUDA(cudaStreamSynchronize(net.stream));
  net.check_status();
}

void Surrogate::predict_async(GpuProblem& p, int load, double* u_out, cudaEvent_t ready) {
  std::lock_guard<std::mutex> lock(mu);
  if (!after) SIMP_CUDA(cudaEventCreateWithFlags(&after, cudaEventDisableTiming));
  SIMP_CUDA(cudaEventRecord(after, p.amg.stream));
  SIMP_CUDA(cudaStreamWaitEvent(net.stream, after, 0));
  enqueue(p, load, u_out);
  SIMP_CUDA(cudaEventRecord(ready, net.stream));
}

void Surrogate::enqueue(GpuProblem& p, int load, double* u_out) {
  if (p.d.dim != 3) throw Error(kBadInput, "the surrogate serves 3-D (Hex8) problems");
  net.shape(p.d.nx + 1, p.d.ny + 1, p.d.nz + 1);
  const long long nodes = static_cast<long long>(p.d.nx + 1) * (p.d.ny + 1) * (p.d.nz + 1);
  in4.alloc(static_cast<size_t>(nodes) * 4);
  input_of(p, load, in4.p);
  k_expand_input<<<blocks_for(nodes), 256, 0, net.stream>>>(nodes, in4.p, net.in16.p);
  SIMP_CHECK_LAUNCH();
  net.forward();
  SIMP_CUDA(cudaMemsetAsync(u_out, 0, sizeof(double) * p.nfree, net.stream));
  k_prediction_to_dofs<<<blocks_for(nodes), 256, 0, net.stream>>>(nodes, 3, net.out.p, p.dof_map.p, u_out);
  SIMP_CHECK_LAUNCH();
}

}  // namespace sg
}  // namespace simp
