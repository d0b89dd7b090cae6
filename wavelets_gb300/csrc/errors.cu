// Error metrics of a restored cubelet against its original (the reference's
// -err option): ErrorAccumulator (test_compress_common.h:90-160) fed as
// computeErrorRatesAfterDequant does (test_compress_common.cc:616-694).
//
// Every pair (a, b) adds, in double, a, a*a, |a - b| and |a - b|^2, where the
// products and the difference are float operations like the reference's
// add(float, float).  a is the original value as a float; b is the restored
// float converted the way the reference compares it:
//   UINT8    floatToByte: <= 0 -> 0, >= 255 -> 255, else truncated;
//   INT32    floatToInt (IntInputDataUnchanged): (int)(f + 0.5f); 16-bit data
//            travels as INT32 and is compared the same way;
//   FLOAT32  (int)f, converted back to float (the reference's own cast).
// Each CTA sums a grid-strided share; the per-CTA partial sums are added on
// the host in CTA order, so the result does not depend on scheduling.
#include <cuda_runtime.h>

#include "wl_internal.h"

namespace wl {
namespace {

constexpr int kThreads = 256;

template <typename T>
__device__ __forceinline__ float original_value(const T *p, long long i) {
  return (float)p[i];
}

__device__ __forceinline__ float compared_value(float f, int dtype) {
  if (dtype == WL_U8) return f <= 0.f ? 0.f : (f >= 255.f ? 255.f : (float)(unsigned char)f);
  if (dtype == WL_F32) return (float)(int)f;
  return (float)(int)__fadd_rn(f, 0.5f);  // INT32 and 16-bit
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
err_sums_kernel(const T *__restrict__ orig, const float *__restrict__ rest, long long n,
                int dtype, double4 *__restrict__ part) {
  __shared__ double4 sh[kThreads / 32];
  double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  const long long stride = (long long)gridDim.x * kThreads;
  for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n; i += stride) {
    const float a = original_value(orig, i);
    const float b = compared_value(rest[i], dtype);
    const float d = fabsf(__fsub_rn(a, b));
    s0 += (double)a;
    s1 += (double)__fmul_rn(a, a);
    s2 += (double)d;
    s3 += (double)__fmul_rn(d, d);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    s3 += __shfl_xor_sync(0xffffffffu, s3, o);
  }
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = make_double4(s0, s1, s2, s3);
  __syncthreads();
  if (threadIdx.x == 0) {
    double4 t = sh[0];
    for (int w = 1; w < kThreads / 32; w++) {
      t.x += sh[w].x;
      t.y += sh[w].y;
      t.z += sh[w].z;
      t.w += sh[w].w;
    }
    part[blockIdx.x] = t;
  }
}

}  // namespace

int err_sums_blocks(long long n) {
  long long blocks = (n + kThreads * 16 - 1) / (kThreads * 16);
  if (blocks < 1) blocks = 1;
  if (blocks > 152 * 8) blocks = 152 * 8;
  return (int)blocks;
}

void launch_err_sums(const void *orig, int dtype, const float *rest, long long n,
                     double *part, int blocks, cudaStream_t s) {
  double4 *p = reinterpret_cast<double4 *>(part);
  switch (dtype) {
    case WL_U8:
      err_sums_kernel<<<blocks, kThreads, 0, s>>>(static_cast<const uint8_t *>(orig), rest, n,
                                                  dtype, p);
      break;
    case WL_U16:
      err_sums_kernel<<<blocks, kThreads, 0, s>>>(static_cast<const uint16_t *>(orig), rest, n,
                                                  dtype, p);
      break;
    case WL_I32:
      err_sums_kernel<<<blocks, kThreads, 0, s>>>(static_cast<const int32_t *>(orig), rest, n,
                                                  dtype, p);
      break;
    default:
      err_sums_kernel<<<blocks, kThreads, 0, s>>>(static_cast<const float *>(orig), rest, n,
                                                  dtype, p);
      break;
  }
}

}  // namespace wl
