// Shared definitions of the GB300 SIMP library: status codes, errors, device
// buffers and launch accounting.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace simp {

using i32 = int32_t;
using i64 = int64_t;

enum Status : int {
  kOk = 0,
  kBadInput = 1,
  kBreakdown = 2,
  kUnderConstrained = 3,
  kMaxIter = 4,
  kNonFinite = 5,
  kCudaError = 6
};

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define SIMP_CUDA(expr)                                                                   \
  do {                                                                                    \
    cudaError_t e_ = (expr);                                                              \
    if (e_ != cudaSuccess)                                                                \
      throw ::simp::Error(::simp::kCudaError, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Kernel launches are counted (the library's own kernels only); the
// per-thread count lets a stream capture tell how many kernels it recorded.
extern std::atomic<int64_t> g_launches;
extern thread_local int64_t t_launches;
#define SIMP_LAUNCHED() (++::simp::t_launches, ::simp::g_launches.fetch_add(1, std::memory_order_relaxed))
#define SIMP_CHECK_LAUNCH()             \
  do {                                  \
    SIMP_LAUNCHED();                    \
    SIMP_CUDA(cudaGetLastError());      \
  } while (0)

// Owning device array (move-only).
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  explicit DBuf(size_t count) { alloc(count); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count == n && p) return;
    release();
    if (count) SIMP_CUDA(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void upload(const T* h, size_t count, cudaStream_t s = 0) {
    alloc(count);
    if (count) SIMP_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void upload(const std::vector<T>& h, cudaStream_t s = 0) { upload(h.data(), h.size(), s); }
  void download(T* h, size_t count, cudaStream_t s = 0) const {
    if (count) SIMP_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
  }
  std::vector<T> to_host(cudaStream_t s = 0) const {
    std::vector<T> h(n);
    download(h.data(), n, s);
    SIMP_CUDA(cudaStreamSynchronize(s));
    return h;
  }
  void zero(cudaStream_t s = 0) {
    if (n) SIMP_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
  size_t bytes() const { return n * sizeof(T); }
};

// Raises a kernel's dynamic shared-memory limit to at least `bytes` and never
// lowers it: the limit is one value per kernel, shared by every host thread,
// so a thread that set a smaller value could make another thread's larger
// launch fail between its set and its launch.
void raise_dynamic_smem(const void* kernel, size_t bytes);

// dst = a device copy of src (same length)
template <class T>
void copy_device(DBuf<T>& dst, const DBuf<T>& src, cudaStream_t s = 0) {
  dst.alloc(src.n);
  if (src.n) SIMP_CUDA(cudaMemcpyAsync(dst.p, src.p, src.n * sizeof(T), cudaMemcpyDeviceToDevice, s));
}

// Device view of a node-level pattern (see structure.h).
struct NodeView {
  const i32* ptr;   // row-node slot pointer
  const i32* nbr;   // column node per slot
  const i32* off;   // offset of the slot within a scalar row
};

inline int grid_for(i64 work, int block, int max_blocks = 1 << 20) {
  i64 g = (work + block - 1) / block;
  if (g < 1) g = 1;
  if (g > max_blocks) g = max_blocks;
  return static_cast<int>(g);
}

}  // namespace simp
