// Threshold selection for callers that cannot allocate device memory.
//
// Some callers of this library are not allowed to call cudaMalloc: code that
// runs while a stream is being captured (allocation is an illegal operation
// there), hosts that hand the library a fixed memory budget or their own
// memory pool and account for every byte, and real-time serving loops that
// must not stall on the allocator.  wl_select_threshold_noalloc gives them
// the radix-select threshold of select.cu without any allocation: its
// scratch lives in the file-scope array below, which every GPU that loads the
// library holds until the process exits.
//
// The kernels are a variant of select.cu's: per-chunk extremes go to a
// scratch slot per chunk (reduced by one CTA) instead of atomics on a
// per-cubelet state record, and the digit histogram lives in the static
// array.  The result is the same k-th smallest |coefficient| (k =
// (int)(fraction * n) in float arithmetic, 0 replaced by 1e-16).
#include <cfloat>
#include <mutex>

#include "wl_internal.h"

namespace wl {
namespace {

constexpr int kThreads = kChunkThreads;
constexpr int kPer = kChunk / kThreads;
constexpr long long kNoallocMaxChunks = WL_NOALLOC_MAX_ELEMENTS / kChunk;

struct NoallocScratch {
  unsigned hist[kSelectBins];
  unsigned prefix;
  unsigned pad0;
  unsigned long long rank;
  uint4 part[kNoallocMaxChunks];  // per chunk: minOrd, maxOrd, top |c|, second |c|
};

// The scratch.  Host code must not take its address directly (the host-side
// symbol is a stand-in, not a device address): noalloc_scratch_ptr() looks up
// the device address once per device with cudaGetSymbolAddress.
static __device__ __align__(256) NoallocScratch g_noalloc;

__device__ __forceinline__ unsigned ord_enc(float f) {
  unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord_dec(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}
__device__ __forceinline__ void top2(unsigned &a1, unsigned &a2, unsigned b1, unsigned b2) {
  unsigned t1 = max(a1, b1), t2 = max(min(a1, b1), max(a2, b2));
  a1 = t1;
  a2 = t2;
}

__global__ void noalloc_clear(NoallocScratch *s) {
  for (int i = threadIdx.x; i < kSelectBins; i += blockDim.x) s->hist[i] = 0;
  if (threadIdx.x == 0) { s->prefix = 0; s->rank = 0; }
}

template <int PASS>
__global__ void __launch_bounds__(kThreads)
noalloc_pass(const float *__restrict__ c, long long n, NoallocScratch *s) {
  __shared__ unsigned hist[kSelectBins];
  __shared__ uint4 wpart[kThreads / 32];
  const long long start = (long long)blockIdx.x * kChunk;
  const int len = (int)min((long long)kChunk, n - start);
  for (int i = threadIdx.x; i < kSelectBins; i += kThreads) hist[i] = 0;
  const unsigned prefix = s->prefix;
  __syncthreads();
  unsigned mn = 0xffffffffu, mx = 0u, a1 = 0u, a2 = 0u;
  for (int k = 0; k < kPer; k++) {
    const int i = threadIdx.x + k * kThreads;
    if (i >= len) break;
    const float v = c[start + i];
    const unsigned a = __float_as_uint(v) & 0x7fffffffu;
    if (PASS == 0) {
      atomicAdd(&hist[a >> 20], 1u);
      mn = min(mn, ord_enc(v));
      mx = max(mx, ord_enc(v));
      top2(a1, a2, a, 0u);
    } else if (PASS == 1) {
      if ((a >> 20) == prefix) atomicAdd(&hist[(a >> 8) & 0xfffu], 1u);
    } else {
      if ((a >> 8) == prefix) atomicAdd(&hist[a & 0xffu], 1u);
    }
  }
  if (PASS == 0) {
    for (int off = 16; off > 0; off >>= 1) {
      mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, off));
      mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
      const unsigned b1 = __shfl_xor_sync(0xffffffffu, a1, off);
      const unsigned b2 = __shfl_xor_sync(0xffffffffu, a2, off);
      top2(a1, a2, b1, b2);
    }
    if ((threadIdx.x & 31) == 0) wpart[threadIdx.x >> 5] = make_uint4(mn, mx, a1, a2);
  }
  __syncthreads();
  const int nb = PASS == 2 ? 256 : kSelectBins;
  for (int i = threadIdx.x; i < nb; i += kThreads)
    if (hist[i]) atomicAdd(&s->hist[i], hist[i]);
  if (PASS == 0 && threadIdx.x == 0) {
    uint4 r = wpart[0];
    for (int w = 1; w < kThreads / 32; w++) {
      r.x = min(r.x, wpart[w].x);
      r.y = max(r.y, wpart[w].y);
      top2(r.z, r.w, wpart[w].z, wpart[w].w);
    }
    s->part[blockIdx.x] = r;
  }
}

// One CTA: find the bucket holding the remaining rank; clear the histogram.
// PASS 0 also reduces the per-chunk extremes; PASS 2 writes the result.
template <int PASS>
__global__ void __launch_bounds__(1024)
noalloc_resolve(long long n, int nChunks, float fraction, NoallocScratch *s, float *out) {
  __shared__ unsigned long long part[1024];
  __shared__ uint4 red[32];
  const int nb = PASS == 2 ? 256 : kSelectBins;
  const int per = (nb + 1023) / 1024;
  unsigned long long rank;
  if (PASS == 0) {
    const float kf = __fmul_rn(fraction, __ll2float_rn(n));
    long long k = (long long)__float2ll_rz(kf);
    if (k >= n) k = n - 1;
    if (k < 0) k = 0;
    rank = (unsigned long long)k;
    // Traverse starts min at FLT_MAX and max at FLT_MIN (thresh_cpu.cc:67-68)
    uint4 r = make_uint4(ord_enc(FLT_MAX), ord_enc(FLT_MIN), 0u, 0u);
    for (int i = threadIdx.x; i < nChunks; i += 1024) {
      const uint4 q = s->part[i];
      r.x = min(r.x, q.x);
      r.y = max(r.y, q.y);
      top2(r.z, r.w, q.z, q.w);
    }
    for (int off = 16; off > 0; off >>= 1) {
      r.x = min(r.x, __shfl_xor_sync(0xffffffffu, r.x, off));
      r.y = max(r.y, __shfl_xor_sync(0xffffffffu, r.y, off));
      const unsigned b1 = __shfl_xor_sync(0xffffffffu, r.z, off);
      const unsigned b2 = __shfl_xor_sync(0xffffffffu, r.w, off);
      top2(r.z, r.w, b1, b2);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = r;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint4 t = red[0];
      for (int w = 1; w < 32; w++) {
        t.x = min(t.x, red[w].x);
        t.y = max(t.y, red[w].y);
        top2(t.z, t.w, red[w].z, red[w].w);
      }
      out[1] = ord_dec(t.x);
      out[2] = ord_dec(t.y);
      out[3] = __uint_as_float(t.z);
      out[4] = __uint_as_float(t.w);
    }
  } else {
    rank = s->rank;
  }
  unsigned long long sum = 0;
  for (int j = 0; j < per; j++) {
    const int i = threadIdx.x * per + j;
    if (i < nb) sum += s->hist[i];
  }
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const unsigned long long v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  const unsigned long long incl = part[threadIdx.x], excl = incl - sum;
  if (rank >= excl && rank < incl) {
    unsigned long long c = excl;
    for (int j = 0; j < per; j++) {
      const int i = threadIdx.x * per + j;
      const unsigned h = i < nb ? s->hist[i] : 0;
      if (rank < c + h) {
        const unsigned rem = (unsigned)(rank - c);
        if (PASS == 0) {
          s->prefix = (unsigned)i;
          s->rank = rem;
        } else if (PASS == 1) {
          s->prefix = (s->prefix << 12) | (unsigned)i;
          s->rank = rem;
        } else {
          float t = __uint_as_float((s->prefix << 8) | (unsigned)i);
          if (t == 0.0f) t = 1e-16f;  // thresh_cpu.cc:98
          out[0] = t;
        }
        break;
      }
      c += h;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kSelectBins; i += 1024) s->hist[i] = 0;
}

// Device address of g_noalloc for the current device, looked up once per
// device (the first call on a device does the lookup).
constexpr int kMaxDevices = 64;
std::mutex g_mu;
NoallocScratch *g_ptr[kMaxDevices] = {};

cudaError_t noalloc_scratch_ptr(NoallocScratch **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc);
    if (e != cudaSuccess) return e;
    g_ptr[dev] = static_cast<NoallocScratch *>(p);
  }
  *out = g_ptr[dev];
  return cudaSuccess;
}

}  // namespace
}  // namespace wl

extern "C" wl_status wl_select_threshold_noalloc(const float *coeffs, long long n,
                                                 float fraction, void *stream, float *out) {
  using namespace wl;
  if (!coeffs || !out || n < 1) return WL_EINVAL;
  if (n > WL_NOALLOC_MAX_ELEMENTS) return WL_EINVAL;
  if (!(fraction >= 0.f && fraction <= 1.f)) return WL_EINVAL;
  NoallocScratch *s = nullptr;
  if (noalloc_scratch_ptr(&s) != cudaSuccess) return WL_ECUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nChunks = (int)((n + kChunk - 1) / kChunk);
  // Each launch's own status is checked (cudaLaunchKernel returns it), so an
  // error left pending by earlier, unrelated work is neither reported here
  // nor cleared.
  const float *cp = coeffs;
  long long nn = n;
  int nc = nChunks;
  float fr = fraction;
  float *op = out;
  void *aClear[] = {&s};
  void *aPass[] = {&cp, &nn, &s};
  void *aRes[] = {&nn, &nc, &fr, &s, &op};
  const dim3 one(1), big(1024), grid(nChunks), blk(kThreads);
  cudaError_t e = cudaLaunchKernel((const void *)noalloc_clear, one, big, aClear, 0, st);
  if (e == cudaSuccess) e = cudaLaunchKernel((const void *)noalloc_pass<0>, grid, blk, aPass, 0, st);
  if (e == cudaSuccess) e = cudaLaunchKernel((const void *)noalloc_resolve<0>, one, big, aRes, 0, st);
  if (e == cudaSuccess) e = cudaLaunchKernel((const void *)noalloc_pass<1>, grid, blk, aPass, 0, st);
  if (e == cudaSuccess) e = cudaLaunchKernel((const void *)noalloc_resolve<1>, one, big, aRes, 0, st);
  if (e == cudaSuccess) e = cudaLaunchKernel((const void *)noalloc_pass<2>, grid, blk, aPass, 0, st);
  if (e == cudaSuccess) e = cudaLaunchKernel((const void *)noalloc_resolve<2>, one, big, aRes, 0, st);
  return e == cudaSuccess ? WL_OK : WL_ECUDA;
}
