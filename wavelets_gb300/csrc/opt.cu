// Error of a restored 8-bit cubelet against its original: the squared
// differences of the parameter sweep (computeErrorRatesAfterDequant,
// test_compress_common.cc:616-694: u8 pixels, |a - b| squared, summed in
// double).  Each CTA sums a grid-strided share in 64-bit integers (the
// squares are exact) and adds it to one accumulator.
#include <cuda_runtime.h>

#include "wl_internal.h"

namespace wl {
namespace {

constexpr int kErrThreads = 256;

__global__ void __launch_bounds__(kErrThreads)
sq_err_u8_kernel(const uint8_t *__restrict__ a, const uint8_t *__restrict__ b, long long n,
                 unsigned long long *__restrict__ out) {
  __shared__ unsigned long long part[kErrThreads / 32];
  unsigned long long s = 0;
  const long long stride = (long long)gridDim.x * kErrThreads;
  for (long long i = blockIdx.x * (long long)kErrThreads + threadIdx.x; i < n; i += stride) {
    const int d = (int)a[i] - (int)b[i];
    s += (unsigned long long)(d * d);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < kErrThreads / 32; w++) t += part[w];
    if (t) atomicAdd(out, t);
  }
}

}  // namespace

void launch_sq_err_u8(const uint8_t *a, const uint8_t *b, long long n, unsigned long long *out,
                      cudaStream_t s) {
  cudaMemsetAsync(out, 0, sizeof(unsigned long long), s);
  if (n <= 0) return;
  long long blocks = (n + kErrThreads * 16 - 1) / (kErrThreads * 16);
  if (blocks > 152 * 8) blocks = 152 * 8;
  sq_err_u8_kernel<<<(unsigned)blocks, kErrThreads, 0, s>>>(a, b, n, out);
}

}  // namespace wl
