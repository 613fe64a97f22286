// The displacement surrogate (surrogate_net.cu): network state, training
// samples and the operations a problem uses.
#pragma once

#include "common.h"
#include "surrogate.h"

#include <cuda_bf16.h>

#include <mutex>
#include <vector>

namespace simp {

class GpuProblem;

namespace sg {

constexpr int kNumLayers = 12;

// Parameters (FP32 master copy, its gradient, Adam moments), the BF16 weight
// copies the tensor-core kernels read, and the activations of one grid size.
class Net {
 public:
  explicit Net(uint64_t seed);
  ~Net();
  Net(const Net&) = delete;
  Net& operator=(const Net&) = delete;

  size_t nparams = 0;
  size_t woff[kNumLayers] = {}, boff[kNumLayers] = {};
  DBuf<float> master, grad, m1, m2;
  DBuf<__nv_bfloat16> wf[kNumLayers], wt[kNumLayers];  // [27][npad][cin] and [27][cin][npad]
  cudaStream_t stream = nullptr;
  DBuf<__nv_bfloat16> in16;  // network input, 16 channels per node
  DBuf<float> out;           // prediction, 3 per node
  DBuf<__nv_bfloat16> gout;  // its gradient, 16 columns per node
  long long adam_t = 0;

  void shape(int nx, int ny, int nz);  // nodes per axis of level 0
  void forward();
  void backward();  // from gout; adds to grad
  double loss(const __nv_bfloat16* target, const uint8_t* mask, long long count);  // also writes gout
  void adam_step(float lr, float gscale);
  void set_params(const float* host);
  void get_params(float* host);
  void check_status();
  int grid(int level, int axis) const { return axis == 0 ? gx[level] : axis == 1 ? gy[level] : gz[level]; }

 private:
  int gx[4] = {0, 0, 0, 0}, gy[4] = {0, 0, 0, 0}, gz[4] = {0, 0, 0, 0};
  int lvl_of[kNumLayers] = {};
  DBuf<__nv_bfloat16> act[kNumLayers], gact[kNumLayers];
  DBuf<__nv_bfloat16> down[4], gdown[4], up[3], gup[3];
  DBuf<float> wpart;
  DBuf<int> status;
  DBuf<double> lpart;
  void pack();
  void conv(int l, const void* in0, const void* in1, void* out, int out_f32, bool data_grad = false,
            void* gout0 = nullptr, void* gout1 = nullptr);
  void wgrad(int l, const void* x0, const void* x1, const void* dy);
  void transfer_down(int k, const __nv_bfloat16* fine, __nv_bfloat16* coarse, int c, float scale);
  void transfer_up(int k, const __nv_bfloat16* coarse, __nv_bfloat16* fine, int c, float scale, int acc);
};

// One (input, target) pair on the device: 4 input channels and the
// normalised displacement (3 per node), with the free-component mask.
struct Sample {
  int nx = 0, ny = 0, nz = 0;  // nodes per axis
  DBuf<__nv_bfloat16> in4, target;
  DBuf<uint8_t> mask;
  long long count = 0;  // free components
};

class Surrogate {
 public:
  explicit Surrogate(uint64_t seed) : net(seed) {}
  ~Surrogate();
  Surrogate(const Surrogate&) = delete;
  Surrogate& operator=(const Surrogate&) = delete;
  Net net;
  std::vector<Sample> samples;
  std::vector<double> losses;  // mean loss of each training epoch
  // the problem's current physical density and load case `load` with its
  // displacement of the last evaluation
  void add_sample(GpuProblem& p, int load);
  // Adam over the samples (shuffled, seeded), `batch` samples per step,
  // cosine-decayed learning rate; returns the last epoch's mean loss
  double train(int epochs, double lr0, int batch, uint64_t seed);
  // predicted displacement of load case `load` at the problem's current
  // physical density, as a free-DOF vector (device, nfree doubles; the
  // network's scale, a shape only)
  void predict(GpuProblem& p, int load, double* u_device);
  // the same, enqueued on the network's stream after the work the problem's
  // stream holds so far, without waiting for it: `ready` is recorded when the
  // prediction is written (the caller makes its stream wait on it)
  void predict_async(GpuProblem& p, int load, double* u_device, cudaEvent_t ready);

 private:
  DBuf<__nv_bfloat16> in4;
  DBuf<double> scratch;
  std::mutex mu;          // one caller at a time issues work on the network's buffers
  cudaEvent_t after = nullptr;
  void input_of(GpuProblem& p, int load, __nv_bfloat16* in4);
  void enqueue(GpuProblem& p, int load, double* u_device);
};

}  // namespace sg
}  // namespace simp
