// Threshold selection without a sort: exact radix select of the k-th smallest
// |coefficient| for every cubelet of a batch.
//
// Reference: thresh_cpu(CubeFloat*) (thresh_cpu.cc:80-109) builds |c|, tracks
// min/max, std::sorts all N values and takes sorted[(int)(frac*N)], replacing
// 0 by 1e-16; min starts at FLT_MAX and max at FLT_MIN (the smallest positive
// float, thresh_cpu.cc:67-68).  Non-negative floats order like their bit
// patterns, so the k-th smallest |c| is found digit by digit: 12 bits
// (31..20), 12 bits (19..8), 8 bits (7..0), one histogram pass per digit over
// the coefficients that still match the prefix.  The first pass also reduces
// min, max and the two largest |c| (the second largest feeds the Lloyd
// codebook, test_compress_cpu.cc:422).
#include <cfloat>

#include "wl_internal.h"

namespace wl {
namespace {

constexpr int kThreads = kChunkThreads;
constexpr int kPerThread = kChunk / kThreads;

// float -> unsigned with the same order (for atomicMin/Max on signed values)
__device__ __forceinline__ unsigned ord_enc(float f) {
  unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord_dec(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ int find_cubelet(const long long *prefix, int n, long long c) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= c) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// top-2 merge of multisets {a1,a2} and {b1,b2} (a1>=a2, b1>=b2)
__device__ __forceinline__ void top2_merge(unsigned &a1, unsigned &a2, unsigned b1, unsigned b2) {
  unsigned t1 = max(a1, b1);
  unsigned t2 = max(min(a1, b1), max(a2, b2));
  a1 = t1;
  a2 = t2;
}

template <int PASS>
__global__ void __launch_bounds__(kThreads)
select_pass(DevBatch b, const float *__restrict__ coef) {
  __shared__ unsigned hist[kSelectBins];
  __shared__ unsigned sMin[kThreads / 32], sMax[kThreads / 32], sA1[kThreads / 32], sA2[kThreads / 32];
  const long long chunk = blockIdx.x;
  const int ci = find_cubelet(b.chunkPrefix, b.n, chunk);
  const CubeletDev cd = b.cub[ci];
  const long long start = (chunk - cd.chunkBase) * (long long)kChunk;
  const int len = (int)min((long long)kChunk, cd.n - start);
  const float *src = coef + cd.coefOff + start;
  CubeletState *st = b.state + ci;

  for (int i = threadIdx.x; i < kSelectBins; i += kThreads) hist[i] = 0;
  unsigned prefix = 0;
  if (PASS > 0) prefix = st->prefix;
  __syncthreads();

  unsigned mn = 0xffffffffu, mx = 0u, a1 = 0u, a2 = 0u;
  for (int k = 0; k < kPerThread; k++) {
    const int i = threadIdx.x + k * kThreads;
    if (i >= len) break;
    const float v = src[i];
    const unsigned a = __float_as_uint(v) & 0x7fffffffu;
    if (PASS == 0) {
      atomicAdd(&hist[a >> 20], 1u);
      mn = min(mn, ord_enc(v));
      mx = max(mx, ord_enc(v));
      top2_merge(a1, a2, a, 0u);
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
      unsigned b1 = __shfl_xor_sync(0xffffffffu, a1, off);
      unsigned b2 = __shfl_xor_sync(0xffffffffu, a2, off);
      top2_merge(a1, a2, b1, b2);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { sMin[w] = mn; sMax[w] = mx; sA1[w] = a1; sA2[w] = a2; }
  }
  __syncthreads();
  const int nb = PASS == 2 ? 256 : kSelectBins;
  unsigned *g = b.selHist + (size_t)ci * kSelectBins;
  for (int i = threadIdx.x; i < nb; i += kThreads)
    if (hist[i]) atomicAdd(&g[i], hist[i]);
  if (PASS == 0 && threadIdx.x == 0) {
    for (int w = 1; w < kThreads / 32; w++) {
      mn = min(mn, sMin[w]);
      mx = max(mx, sMax[w]);
      top2_merge(a1, a2, sA1[w], sA2[w]);
    }
    mn = min(mn, sMin[0]); mx = max(mx, sMax[0]);
    top2_merge(a1, a2, sA1[0], sA2[0]);
    atomicMin(&st->minOrd, mn);
    atomicMax(&st->maxOrd, mx);
    // merge the pair into (absMax, absMax2) with a 64-bit CAS loop
    unsigned long long *pair = reinterpret_cast<unsigned long long *>(&st->absMax);
    unsigned long long old = *pair, assumed;
    do {
      assumed = old;
      unsigned c1 = (unsigned)(assumed & 0xffffffffu), c2 = (unsigned)(assumed >> 32);
      unsigned n1 = c1, n2 = c2;
      top2_merge(n1, n2, a1, a2);
      unsigned long long nv = ((unsigned long long)n2 << 32) | n1;
      if (nv == assumed) break;
      old = atomicCAS(pair, assumed, nv);
    } while (old != assumed);
  }
}

// Find the digit bucket holding the remaining rank; one CTA per cubelet.
template <int PASS>
__global__ void __launch_bounds__(1024) select_resolve(DevBatch b) {
  __shared__ unsigned long long part[1024];
  const int ci = blockIdx.x;
  CubeletState *st = b.state + ci;
  const CubeletDev cd = b.cub[ci];
  unsigned *g = b.selHist + (size_t)ci * kSelectBins;
  const int nb = PASS == 2 ? 256 : kSelectBins;
  const int per = (nb + 1023) / 1024;

  unsigned long long rank;
  if (PASS == 0) {
    // k = (int)(frac * N) in float arithmetic (thresh_cpu.cc:96); k == N
    // (frac == 1) reads past the array in the reference and is clamped here
    const float kf = __fmul_rn(cd.frac, __ll2float_rn(cd.n));
    long long k = (long long)__float2ll_rz(kf);
    if (k >= cd.n) k = cd.n - 1;
    if (k < 0) k = 0;
    rank = (unsigned long long)k;
  } else {
    rank = st->rank;
  }
  // per-thread sums of `per` consecutive bins, then an exclusive scan
  unsigned long long s = 0;
  for (int j = 0; j < per; j++) {
    int i = threadIdx.x * per + j;
    if (i < nb) s += g[i];
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    unsigned long long v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  const unsigned long long incl = part[threadIdx.x];
  const unsigned long long excl = incl - s;
  if (rank >= excl && rank < incl) {
    unsigned long long c = excl;
    for (int j = 0; j < per; j++) {
      int i = threadIdx.x * per + j;
      unsigned h = i < nb ? g[i] : 0;
      if (rank < c + h) {
        const unsigned rem = (unsigned)(rank - c);
        if (PASS == 0) {
          st->prefix = (unsigned)i;
          st->rank = rem;
          st->minVal = ord_dec(st->minOrd);
          st->maxVal = ord_dec(st->maxOrd);
          st->maxAbs = __uint_as_float(st->absMax);
          st->maxAbs2 = __uint_as_float(st->absMax2);
        } else if (PASS == 1) {
          st->prefix = (st->prefix << 12) | (unsigned)i;
          st->rank = rem;
        } else {
          const unsigned bits = (st->prefix << 8) | (unsigned)i;
          float t = __uint_as_float(bits);
          if (t == 0.0f) t = 1e-16f;  // thresh_cpu.cc:98
          st->threshold = t;
        }
        break;
      }
      c += h;
    }
  }
  __syncthreads();
  // clear the histogram for the next digit
  for (int i = threadIdx.x; i < kSelectBins; i += 1024) g[i] = 0;
}

__global__ void select_init(DevBatch b) {
  const int ci = blockIdx.x * blockDim.x + threadIdx.x;
  if (ci >= b.n) return;
  CubeletState *st = b.state + ci;
  // Traverse starts min at FLT_MAX and max at FLT_MIN (thresh_cpu.cc:67-68)
  st->minOrd = ord_enc(FLT_MAX);
  st->maxOrd = ord_enc(FLT_MIN);
  st->absMax = 0u;
  st->absMax2 = 0u;
}

}  // namespace

void launch_select(DevBatch &b, const float *coef, cudaStream_t s) {
  select_init<<<(b.n + 127) / 128, 128, 0, s>>>(b);
  const unsigned chunks = (unsigned)b.totalChunks;
  select_pass<0><<<chunks, kThreads, 0, s>>>(b, coef);
  select_resolve<0><<<b.n, 1024, 0, s>>>(b);
  select_pass<1><<<chunks, kThreads, 0, s>>>(b, coef);
  select_resolve<1><<<b.n, 1024, 0, s>>>(b);
  select_pass<2><<<chunks, kThreads, 0, s>>>(b, coef);
  select_resolve<2><<<b.n, 1024, 0, s>>>(b);
}

}  // namespace wl
