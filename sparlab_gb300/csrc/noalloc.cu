// Filtered design volume with no device allocation.
//
// simp_filter_volume_noalloc computes the physical density of a structured
// problem -- rho = clamp(H x, 0, 1), Heaviside-projected at the current beta
// and the objective's threshold when the problem has the projection on -- and
// its volume sum_e v_e rho_e, as simp_evaluate does, but it allocates nothing: the per-chunk partial
// sums live in a file-scope device array instead of a buffer from cudaMalloc.
// It is meant for callers that cannot allocate device memory at the point of
// the call: an optimiser loop that evaluates the volume of many trial designs
// per iteration and must not synchronise the device through cudaMalloc /
// cudaFree, or an application whose device memory is owned by its own pool
// under a fixed budget.
//
// Limits and behaviour:
//  * at most kMaxChunks * kChunk = 67,108,864 elements; larger problems are
//    rejected with SIMP_BAD_INPUT;
//  * the scratch array (kMaxChunks doubles, 128 KiB) is held by every GPU
//    that loads the library until the process exits;
//  * the first call on a device looks up the array's device address with that
//    device current and caches it, so make the first call before any stream
//    capture on that device; a cudaDeviceReset after that first call is not
//    supported (the cached address would be stale);
//  * every call shares the one array: calls whose kernels overlap on the GPU
//    (other streams, other threads) race on it.  Each call overwrites every
//    partial it reads, so nothing has to start at zero.
#include "../../include/simp_gpu.h"

#include "kernels.cuh"
#include "problem.h"
#include "topopt.cuh"

#include <mutex>
#include <sstream>

namespace simp {
namespace {

constexpr int kChunk = 4096;        // elements summed by one block
constexpr int kMaxChunks = 16384;   // partial sums the scratch array holds
constexpr int kChunkThreads = 256;

static __device__ __align__(256) double g_volume_scratch[kMaxChunks];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
double* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once
// per device, with that device current).
double* scratch_address() {
  int dev = 0;
  SIMP_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) throw Error(kBadInput, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[dev]) {
    double* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&ptr), g_volume_scratch);
    if (e != cudaSuccess)
      throw Error(kCudaError, std::string("cudaGetSymbolAddress of the volume scratch: ") + cudaGetErrorString(e));
    g_scratch_addr[dev] = ptr;
  }
  return g_scratch_addr[dev];
}

// One block per chunk: rho for the chunk's elements and its volume partial.
// project != 0: rho is the Heaviside projection of the clamped filtered
// density at (beta, eta), as simp_evaluate's k_project computes it.
__global__ void __launch_bounds__(kChunkThreads) k_volume_chunks(GridView g, const Stencil* __restrict__ st,
                                                                 const double* __restrict__ w, i64 ne,
                                                                 const double* __restrict__ x,
                                                                 double* __restrict__ rho,
                                                                 const double* __restrict__ vols,
                                                                 int project, double beta, double eta,
                                                                 double* __restrict__ partial) {
  const i64 lo = static_cast<i64>(blockIdx.x) * kChunk;
  const i64 hi = lo + kChunk < ne ? lo + kChunk : ne;
  double vs = 0.0;
  for (i64 e = lo + threadIdx.x; e < hi; e += kChunkThreads) {
    const i32 ex = static_cast<i32>(e % g.nx), ey = static_cast<i32>((e / g.nx) % g.ny),
              ez = static_cast<i32>(e / ((i64)g.nx * g.ny));
    double s = 0.0;
    for (int k = 0; k < st->count; ++k) {
      const i32 qx = ex + st->dx[k], qy = ey + st->dy[k], qz = ez + st->dz[k];
      if (!in_grid(g, qx, qy, qz)) continue;
      const i64 q = (static_cast<i64>(qz) * g.ny + qy) * g.nx + qx;
      s = xadd(s, xmul(w[k * ne + e], x[q]));
    }
    s = fmin(fmax(s, 0.0), 1.0);
    if (project) {
      double deriv;
      s = project_one(s, beta, eta, deriv);
    }
    rho[e] = s;
    vs += s * vols[e];
  }
  vs = block_sum<kChunkThreads>(vs);
  if (threadIdx.x == 0) partial[blockIdx.x] = vs;
}

// Sum of the chunk partials in a fixed order into out.
__global__ void __launch_bounds__(kChunkThreads) k_sum_chunks(const double* __restrict__ partial, int chunks,
                                                              double* __restrict__ out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < chunks; i += kChunkThreads) s += partial[i];
  s = block_sum<kChunkThreads>(s);
  if (threadIdx.x == 0) *out = s;
}

}  // namespace

// Launches the two kernels of the no-allocation volume on the problem's stream.
void filter_volume_noalloc(GpuProblem& p, const double* x, double* rho, double* volume) {
  if (p.ne > static_cast<i64>(kChunk) * kMaxChunks) {
    std::ostringstream os;
    os << "simp_filter_volume_noalloc: " << p.ne << " elements exceed the scratch capacity of "
       << static_cast<i64>(kChunk) * kMaxChunks << " elements";
    throw Error(kBadInput, os.str());
  }
  if (!x || !rho || !volume) throw Error(kBadInput, "simp_filter_volume_noalloc: NULL device pointer");
  double* scratch = scratch_address();
  const int chunks = static_cast<int>((p.ne + kChunk - 1) / kChunk);
  GridView g;
  g.dim = p.d.dim;
  g.nx = p.d.nx;
  g.ny = p.d.ny;
  g.nz = p.d.dim == 3 ? p.d.nz : 1;
  g.nnx = p.d.nx + 1;
  g.nny = p.d.ny + 1;
  g.nnz = p.d.dim == 3 ? p.d.nz + 1 : 1;
  k_volume_chunks<<<chunks, kChunkThreads, 0, p.amg.stream>>>(g, static_cast<const Stencil*>(p.stencil_d), p.hw.p,
                                                              p.ne, x, rho, p.vols.p, p.d.projection ? 1 : 0,
                                                              p.beta, p.d.objective_eta(), scratch);
  SIMP_CHECK_LAUNCH();
  k_sum_chunks<<<1, kChunkThreads, 0, p.amg.stream>>>(scratch, chunks, volume);
  SIMP_CHECK_LAUNCH();
}

}  // namespace simp
