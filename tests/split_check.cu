// Checks df_split (kernels.cuh) against FP64 conversion on the device, bit
// for bit: hi = fl32(v), lo = fl32(v - hi).  Doubles from a fixed
// xorshift stream over exponent fields 0..2046 (zero, subnormal, normal,
// out of float range), with forced ties and carries in the rounded bits.
// Prints the number of mismatches; exits 0 when there are none.
#include <cstdio>
#include <cstring>
#include <vector>

#include "kernels.cuh"

using namespace simp;

__global__ void k_check(const double* __restrict__ v, long long n, unsigned long long* __restrict__ bad) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float h, l;
    df_split(v[i], h, l);
    const float rh = __double2float_rn(v[i]);
    const float rl = __double2float_rn(v[i] - static_cast<double>(rh));
    const bool nan = v[i] != v[i];
    if (!nan && (__float_as_uint(h) != __float_as_uint(rh) || __float_as_uint(l) != __float_as_uint(rl)))
      atomicAdd(bad, 1ull);
  }
}

int main() {
  const long long n = 1 << 24;
  std::vector<double> h(n);
  unsigned long long s = 0x9E3779B97F4A7C15ull;
  for (long long i = 0; i < n; ++i) {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    unsigned long long u = s;
    const unsigned long long e = (u >> 40) % 2047ull;      // exponent field 0 .. 2046
    u = (u & 0x800FFFFFFFFFFFFFull) | (e << 52);
    if (i % 8 == 1) u = (u & ~0x1FFFFFFFull) | 0x10000000ull;  // a tie in the 29 rounded bits
    if (i % 8 == 2) u |= 0xFFFFFFFFFFFFFull;                  // rounds up into the exponent
    double d;
    memcpy(&d, &u, sizeof d);
    h[i] = d;
  }
  double* dv = nullptr;
  unsigned long long* dbad = nullptr;
  if (cudaMalloc(&dv, n * sizeof(double)) != cudaSuccess || cudaMalloc(&dbad, sizeof(unsigned long long)) != cudaSuccess)
    return 2;
  cudaMemcpy(dv, h.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemset(dbad, 0, sizeof(unsigned long long));
  k_check<<<1024, 256>>>(dv, n, dbad);
  unsigned long long bad = 0;
  if (cudaMemcpy(&bad, dbad, sizeof bad, cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
  printf("mismatches %llu of %lld\n", bad, n);
  cudaFree(dv);
  cudaFree(dbad);
  return bad == 0 ? 0 : 1;
}
