// The displacement surrogate: a 3-D convolutional encoder-decoder on the
// nodal grid whose prediction joins the PCG start (warm_start = 3).  This
// file holds its layer kernels (tensor-core convolutions from conv_tc.cuh,
// the weight gradient, grid transfers, activations, the loss and the Adam
// step) and the host side that builds tensor maps and launches them.
#include "../../include/simp_gpu.h"

#include "common.h"
#include "conv_tc.cuh"
#include "surrogate.h"

#include <cudaTypedefs.h>

#include <cmath>
#include <mutex>
#include <sstream>

namespace simp {
namespace sg {

// ---------------------------------------------------------------------------
// Tensor maps
// ---------------------------------------------------------------------------
namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    err = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
    if (err == cudaSuccess && q == cudaDriverEntryPointSuccess) fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  if (!fn) throw Error(kCudaError, "cuTensorMapEncodeTiled is not available from the driver");
  return fn;
}

CUtensorMapSwizzle swizzle_for(int row_bytes) {
  switch (row_bytes) {
    case 32: return CU_TENSOR_MAP_SWIZZLE_32B;
    case 64: return CU_TENSOR_MAP_SWIZZLE_64B;
    case 128: return CU_TENSOR_MAP_SWIZZLE_128B;
    default: throw Error(kBadInput, "surrogate: channel counts must be 16, 32 or 64 per tensor");
  }
}

void check_encode(CUresult r, const char* what) {
  if (r != CUDA_SUCCESS) {
    std::ostringstream os;
    os << "cuTensorMapEncodeTiled failed for the " << what << " (error " << static_cast<int>(r) << ")";
    throw Error(kCudaError, os.str());
  }
}

}  // namespace

// Channels-last BF16 activations [nz][ny][nx][c]: boxes of (c, 32, 4, 1).
CUtensorMap act_map(const void* base, int c, int nx, int ny, int nz) {
  if (reinterpret_cast<uintptr_t>(base) % 16) throw Error(kBadInput, "surrogate: activations must be 16-byte aligned");
  CUtensorMap m;
  const cuuint64_t dims[4] = {static_cast<cuuint64_t>(c), static_cast<cuuint64_t>(nx), static_cast<cuuint64_t>(ny),
                              static_cast<cuuint64_t>(nz)};
  const cuuint64_t strides[3] = {static_cast<cuuint64_t>(c) * 2, static_cast<cuuint64_t>(c) * 2 * nx,
                                 static_cast<cuuint64_t>(c) * 2 * nx * ny};
  const cuuint32_t box[4] = {static_cast<cuuint32_t>(c), conv::kTileX, conv::kTileY, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  check_encode(encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(c * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE),
               "activations");
  return m;
}

// Weights [27 n rows][k] (K contiguous): boxes of (c, n) at column offset k0.
CUtensorMap weight_map(const void* base, int k, int n, int c) {
  if (reinterpret_cast<uintptr_t>(base) % 16) throw Error(kBadInput, "surrogate: weights must be 16-byte aligned");
  CUtensorMap m;
  const cuuint64_t dims[2] = {static_cast<cuuint64_t>(k), static_cast<cuuint64_t>(27) * n};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(k) * 2};
  const cuuint32_t box[2] = {static_cast<cuuint32_t>(c), static_cast<cuuint32_t>(n)};
  const cuuint32_t estr[2] = {1, 1};
  check_encode(encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(c * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE),
               "weights");
  return m;
}

// One convolution (or its data gradient) on the tensor cores.
void conv_launch(const ConvSpec& s, cudaStream_t stream) {
  conv::ConvArgs p{};
  p.nx = s.nx;
  p.ny = s.ny;
  p.nz = s.nz;
  p.nseg = s.nseg;
  p.n = s.n;
  p.flip = s.flip;
  p.bias = s.bias;
  p.relu = s.relu;
  p.nout = s.nout;
  p.status = s.status;
  int ktot = 0;
  for (int k = 0; k < s.nseg; ++k) {
    if (s.cseg[k] != 16 && s.cseg[k] != 32 && s.cseg[k] != 64)
      throw Error(kBadInput, "surrogate: input segments must have 16, 32 or 64 channels");
    p.cseg[k] = s.cseg[k];
    ktot += s.cseg[k];
  }
  if (s.n % 16 || s.n < 16 || s.n > 128) throw Error(kBadInput, "surrogate: output columns must be 16..128, step 16");
  for (int k = 0; k < s.nout; ++k) {
    p.out_c[k] = s.out_c[k];
    p.out_pitch[k] = s.out_pitch[k];
    p.out_f32[k] = s.out_f32[k];
    p.out[k] = s.out[k];
  }
  if (s.nout > 1 && s.out_c[0] % 16) throw Error(kBadInput, "surrogate: split outputs at a multiple of 16 columns");
  const CUtensorMap a0 = act_map(s.in[0], s.cseg[0], s.nx, s.ny, s.nz);
  const CUtensorMap a1 = s.nseg > 1 ? act_map(s.in[1], s.cseg[1], s.nx, s.ny, s.nz) : a0;
  const CUtensorMap b0 = weight_map(s.w, ktot, s.n, s.cseg[0]);
  const CUtensorMap b1 = s.nseg > 1 ? weight_map(s.w, ktot, s.n, s.cseg[1]) : b0;
  const size_t smem = conv::smem_bytes(p);
  raise_dynamic_smem(reinterpret_cast<const void*>(conv::k_conv_tc), smem);
  const dim3 grid((s.nx + conv::kTileX - 1) / conv::kTileX, (s.ny + conv::kTileY - 1) / conv::kTileY, s.nz);
  conv::k_conv_tc<<<grid, conv::kThreads, smem, stream>>>(a0, a1, b0, b1, p);
  SIMP_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// Weight and bias gradients on the CUDA cores (FP32 accumulation):
// dW_t[co][ci] = sum_v dY[v][co] X[v + o_t][ci], db[co] = sum_v dY[v][co].
// Block (tap t, group g) sums the voxel chunks g, g + G, ... of 128 nodes in
// a fixed order into its partial; k_wgrad_sum adds the G partials in order.
// ---------------------------------------------------------------------------
constexpr int kWgChunk = 128;
constexpr int kWgGroups = 64;
constexpr int kWgThreads = 256;

__global__ void __launch_bounds__(kWgThreads) k_wgrad_partial(int nx, int ny, int nz, int nseg, const __nv_bfloat16* x0,
                                                              int c0, const __nv_bfloat16* x1, int c1,
                                                              const __nv_bfloat16* dy, int cdy, int cout,
                                                              float* __restrict__ part) {
  extern __shared__ float wsm[];
  const int t = blockIdx.y;  // tap; t == 27: the bias gradient
  const int g = blockIdx.x;
  const int cin = c0 + (nseg > 1 ? c1 : 0);
  float* sdy = wsm;                       // [kWgChunk][cout]
  float* sx = wsm + kWgChunk * cout;      // [kWgChunk][cin]
  const int dz = t < 27 ? t / 9 - 1 : 0, dyo = t < 27 ? (t / 3) % 3 - 1 : 0, dx = t < 27 ? t % 3 - 1 : 0;
  const long long nodes = static_cast<long long>(nx) * ny * nz;
  const long long chunks = (nodes + kWgChunk - 1) / kWgChunk;
  const int outs = t < 27 ? cout * cin : cout;
  constexpr int kPer = 32;  // outputs per thread (up to 64 x 128 = 8192 = 256 x 32)
  float acc[kPer];
#pragma unroll
  for (int q = 0; q < kPer; ++q) acc[q] = 0.0f;
  for (long long ch = g; ch < chunks; ch += gridDim.x) {
    const long long v0 = ch * kWgChunk;
    __syncthreads();
    for (int e = threadIdx.x; e < kWgChunk * cout; e += kWgThreads) {
      const int r = e / cout, c = e % cout;
      const long long v = v0 + r;
      sdy[e] = (v < nodes && c < cdy) ? __bfloat162float(dy[v * cdy + c]) : 0.0f;
    }
    if (t < 27) {
      for (int e = threadIdx.x; e < kWgChunk * cin; e += kWgThreads) {
        const int r = e / cin, c = e % cin;
        const long long v = v0 + r;
        float val = 0.0f;
        if (v < nodes) {
          const int vx = static_cast<int>(v % nx), vy = static_cast<int>((v / nx) % ny),
                    vz = static_cast<int>(v / (static_cast<long long>(nx) * ny));
          const int ux = vx + dx, uy = vy + dyo, uz = vz + dz;
          if (ux >= 0 && ux < nx && uy >= 0 && uy < ny && uz >= 0 && uz < nz) {
            const long long u = (static_cast<long long>(uz) * ny + uy) * nx + ux;
            val = c < c0 ? __bfloat162float(x0[u * c0 + c]) : __bfloat162float(x1[u * c1 + (c - c0)]);
          }
        }
        sx[e] = val;
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      const int o = threadIdx.x + q * kWgThreads;
      if (o < outs) {
        float s = acc[q];
        if (t < 27) {
          const int co = o / cin, ci = o % cin;
          for (int r = 0; r < kWgChunk; ++r) s = fmaf(sdy[r * cout + co], sx[r * cin + ci], s);
        } else {
          for (int r = 0; r < kWgChunk; ++r) s += sdy[r * cout + o];
        }
        acc[q] = s;
      }
    }
  }
  float* out = part + (static_cast<long long>(t) * gridDim.x + g) * (cout * cin > cout ? cout * cin : cout);
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int o = threadIdx.x + q * kWgThreads;
    if (o < outs) out[o] = acc[q];
  }
}

// gw[t][co][ci] += sum_g part[t][g][co ci]; gb[co] += sum_g part[27][g][co]
__global__ void k_wgrad_sum(int cout, int cin, int groups, const float* __restrict__ part, float* __restrict__ gw,
                            float* __restrict__ gb) {
  const int stride = cout * cin;
  const int total = 27 * stride + cout;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int t = e < 27 * stride ? e / stride : 27;
    const int o = e < 27 * stride ? e % stride : e - 27 * stride;
    float s = 0.0f;
    for (int g = 0; g < groups; ++g) s += part[(static_cast<long long>(t) * groups + g) * stride + o];
    if (t < 27) gw[e] += s;
    else gb[o] += s;
  }
}

void wgrad_launch(const WgradSpec& s, float* part, cudaStream_t stream) {
  const int cin = s.c0 + (s.nseg > 1 ? s.c1 : 0);
  if (s.cout * cin > kWgThreads * 32) throw Error(kBadInput, "surrogate: weight block too large for the gradient kernel");
  const size_t smem = sizeof(float) * kWgChunk * (s.cout + cin);
  raise_dynamic_smem(reinterpret_cast<const void*>(k_wgrad_partial), smem);
  k_wgrad_partial<<<dim3(kWgGroups, 28), kWgThreads, smem, stream>>>(s.nx, s.ny, s.nz, s.nseg, s.x0, s.c0, s.x1, s.c1,
                                                                    s.dy, s.cdy, s.cout, part);
  SIMP_CHECK_LAUNCH();
  k_wgrad_sum<<<grid_for(27 * s.cout * cin + s.cout, 256, 1024), 256, 0, stream>>>(s.cout, cin, kWgGroups, part, s.gw,
                                                                                   s.gb);
  SIMP_CHECK_LAUNCH();
}

size_t wgrad_partial_floats(int cout, int cin) { return static_cast<size_t>(28) * kWgGroups * cout * cin; }

}  // namespace sg
}  // namespace simp

// ---------------------------------------------------------------------------
// C ABI: single layers on device pointers (the surrogate's building blocks)
// ---------------------------------------------------------------------------
using namespace simp;

namespace simp {
namespace sg {
std::string& last_error() {
  thread_local std::string e;
  return e;
}
}  // namespace sg
}  // namespace simp

namespace {
template <class F>
int sg_guard(F&& f) {
  try {
    f();
    return kOk;
  } catch (const Error& e) {
    sg::last_error() = e.what();
    return e.code;
  } catch (const std::exception& e) {
    sg::last_error() = e.what();
    return kBadInput;
  }
}

int read_status(int* dstatus, cudaStream_t s) {
  int h = 0;
  SIMP_CUDA(cudaMemcpyAsync(&h, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
  SIMP_CUDA(cudaStreamSynchronize(s));
  return h;
}
}  // namespace

extern "C" {

const char* simp_surrogate_last_error(void) { return sg::last_error().c_str(); }

int simp_conv3d_bf16(int32_t nx, int32_t ny, int32_t nz, int32_t nseg, const void* const* in, const int32_t* cseg,
                     const void* weights, int32_t n, const float* bias, int32_t relu, int32_t flip, int32_t nout,
                     void* const* out, const int32_t* out_c, const int32_t* out_pitch, const int32_t* out_f32) {
  return sg_guard([&] {
    if (nx < 1 || ny < 1 || nz < 1 || nseg < 1 || nseg > 2 || nout < 1 || nout > 2)
      throw Error(kBadInput, "simp_conv3d_bf16: bad sizes");
    sg::ConvSpec s{};
    s.nx = nx;
    s.ny = ny;
    s.nz = nz;
    s.nseg = nseg;
    for (int k = 0; k < nseg; ++k) {
      s.in[k] = in[k];
      s.cseg[k] = cseg[k];
    }
    s.w = weights;
    s.n = n;
    s.bias = bias;
    s.relu = relu;
    s.flip = flip;
    s.nout = nout;
    for (int k = 0; k < nout; ++k) {
      s.out[k] = out[k];
      s.out_c[k] = out_c[k];
      s.out_pitch[k] = out_pitch[k];
      s.out_f32[k] = out_f32[k];
    }
    DBuf<int> st(1);
    st.zero();
    s.status = st.p;
    sg::conv_launch(s, 0);
    if (read_status(st.p, 0)) throw Error(kCudaError, "simp_conv3d_bf16: a pipeline wait timed out");
  });
}

int simp_conv3d_wgrad(int32_t nx, int32_t ny, int32_t nz, int32_t nseg, const void* const* in, const int32_t* cseg,
                      const void* dy, int32_t cdy, int32_t cout, float* gw, float* gb) {
  return sg_guard([&] {
    sg::WgradSpec s{};
    s.nx = nx;
    s.ny = ny;
    s.nz = nz;
    s.nseg = nseg;
    s.x0 = static_cast<const __nv_bfloat16*>(in[0]);
    s.c0 = cseg[0];
    s.x1 = nseg > 1 ? static_cast<const __nv_bfloat16*>(in[1]) : nullptr;
    s.c1 = nseg > 1 ? cseg[1] : 0;
    s.dy = static_cast<const __nv_bfloat16*>(dy);
    s.cdy = cdy;
    s.cout = cout;
    s.gw = gw;
    s.gb = gb;
    DBuf<float> part(sg::wgrad_partial_floats(cout, s.c0 + s.c1));
    sg::wgrad_launch(s, part.p, 0);
    SIMP_CUDA(cudaStreamSynchronize(0));
  });
}

}  // extern "C"
