// Layer launches of the displacement surrogate (surrogate.cu) and the
// network that chains them (surrogate_net.cu).
#pragma once

#include "common.h"

#include <cuda.h>
#include <cuda_bf16.h>

#include <string>

namespace simp {
namespace sg {

// One convolution on the tensor cores (see conv_tc.cuh).
struct ConvSpec {
  int nx = 0, ny = 0, nz = 0;
  int nseg = 1;
  const void* in[2] = {nullptr, nullptr};  // BF16 channels-last inputs
  int cseg[2] = {0, 0};
  const void* w = nullptr;                 // BF16 [27][n][sum cseg]
  int n = 0;
  const float* bias = nullptr;
  int relu = 0;
  int flip = 0;
  int nout = 1;
  void* out[2] = {nullptr, nullptr};
  int out_c[2] = {0, 0};
  int out_pitch[2] = {0, 0};
  int out_f32[2] = {0, 0};
  int* status = nullptr;
};

// Weight and bias gradient of one convolution (FP32, added to gw / gb).
struct WgradSpec {
  int nx = 0, ny = 0, nz = 0;
  int nseg = 1;
  const __nv_bfloat16* x0 = nullptr;
  int c0 = 0;
  const __nv_bfloat16* x1 = nullptr;
  int c1 = 0;
  const __nv_bfloat16* dy = nullptr;
  int cdy = 0;   // channels per node of dy
  int cout = 0;  // output channels whose gradient is formed (<= cdy)
  float* gw = nullptr;  // [27][cout][c0 + c1]
  float* gb = nullptr;  // [cout]
};

CUtensorMap act_map(const void* base, int c, int nx, int ny, int nz);
CUtensorMap weight_map(const void* base, int k, int n, int c);
void conv_launch(const ConvSpec& s, cudaStream_t stream);
void wgrad_launch(const WgradSpec& s, float* part, cudaStream_t stream);
size_t wgrad_partial_floats(int cout, int cin);
// message of the last failed surrogate call on this thread
std::string& last_error();

}  // namespace sg
}  // namespace simp
