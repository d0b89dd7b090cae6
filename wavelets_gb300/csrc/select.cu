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
//
// Only the first pass reads the whole volume for the first digit; a second
// full pass compacts the coefficients of the threshold's 12-bit bucket (a few
// percent of them) into the cubelet's region of the free second coefficient
// buffer, and the last two digits are histogrammed over those candidates
// alone.  The compaction pass also builds the Lloyd histogram of every
// |c| above the bucket, so the Lloyd quantizer needs no pass of its own.
#include <cfloat>
#include <type_traits>

#include "select_common.cuh"
#include "wl_internal.h"

namespace wl {
namespace {

constexpr int kThreads = kChunkThreads;
constexpr int kPerThread = kChunk / kThreads;
static_assert(kPerThread == 16, "load_chunk assumes four float4 per thread");

using selc::ord_dec;
using selc::ord_enc;
using selc::top2_merge;

// element of the chunk held in v[k] by this thread: float4 j = threadIdx.x +
// kThreads * (k / 4), so every warp load is 512 contiguous bytes
__device__ __forceinline__ int chunk_index(int k) {
  return 4 * (threadIdx.x + kThreads * (k >> 2)) + (k & 3);
}
// all loads of the thread issued before any use; elements past len read 0
__device__ __forceinline__ void load_chunk(const float *src, int len, float (&v)[kPerThread]) {
  if (len == kChunk && (reinterpret_cast<size_t>(src) & 15) == 0) {
    const float4 *s4 = reinterpret_cast<const float4 *>(src);
#pragma unroll
    for (int j = 0; j < kPerThread / 4; j++) {
      const float4 q = s4[threadIdx.x + kThreads * j];
      v[4 * j] = q.x; v[4 * j + 1] = q.y; v[4 * j + 2] = q.z; v[4 * j + 3] = q.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kPerThread; k++) {
      const int i = chunk_index(k);
      v[k] = i < len ? src[i] : 0.f;
    }
  }
}

// First digit (bits 31..20 of |c|) plus min, max and the two largest |c|.
// A CTA takes kQuantGroup consecutive chunks of one cubelet (one histogram
// flush per group); a thread's 16 loads of a chunk are issued together, and
// six CTAs per SM keep enough of them in flight.
__global__ void __launch_bounds__(kThreads, 6)
select_pass0(DevBatch b, const float *__restrict__ coef) {
  __shared__ unsigned hist[kSelectBins];
  const int ci = b.groupCub[blockIdx.x];
  const CubeletDev cd = b.cub[ci];
  if (cd.selFused) return;  // the last transform pass gathered these already
  const int c0 = ((int)blockIdx.x - cd.groupBase) * kQuantGroup;
  const int nc = min(kQuantGroup, cd.nChunks - c0);
  auto chunk_len = [&](int k) {
    return (int)min((long long)kChunk, cd.n - (long long)(c0 + k) * kChunk);
  };
  auto chunk_src = [&](int k) { return coef + cd.coefOff + (long long)(c0 + k) * kChunk; };

  selc::clear_hist<kThreads>(hist);
  __syncthreads();
  selc::SelAcc acc{hist};
  for (int k = 0; k < nc; k++) {
    const int len = chunk_len(k);
    float v[kPerThread];
    load_chunk(chunk_src(k), len, v);
    if (len == kChunk) {
#pragma unroll
      for (int j = 0; j < kPerThread; j++) acc.visit(v[j]);
    } else {
#pragma unroll
      for (int j = 0; j < kPerThread; j++)
        if (chunk_index(j) < len) acc.visit(v[j]);
    }
  }
  selc::flush<kThreads>(acc, b.selHist + (size_t)ci * kSelectBins, b.state + ci);
}

// Second full pass: compact the coefficients of the threshold bucket
// (|c| >> 20 == prefix) into the cubelet's candidate region, and add every
// |c| above the bucket to the Lloyd histogram (those are above the threshold
// whatever its low 20 bits turn out to be).  Chunk groups as in pass 0.
__global__ void __launch_bounds__(kThreads, 6)
select_compact(DevBatch b, const float *__restrict__ coef, unsigned *__restrict__ cand) {
  __shared__ unsigned lh[kLloydBins];
  const int ci = b.groupCub[blockIdx.x];
  const CubeletDev cd = b.cub[ci];
  const int c0 = ((int)blockIdx.x - cd.groupBase) * kQuantGroup;
  const int nc = min(kQuantGroup, cd.nChunks - c0);
  CubeletState *st = b.state + ci;
  const unsigned prefix = st->prefix;
  const bool lloyd = cd.quantAlg == WL_LLOYD && !st->lloydDeferred;
  const unsigned lbase = st->lloydBase, lhi = st->lloydHiBits;
  const int lshift = st->lloydShift;
  auto chunk_len = [&](int k) {
    return (int)min((long long)kChunk, cd.n - (long long)(c0 + k) * kChunk);
  };
  auto chunk_src = [&](int k) { return coef + cd.coefOff + (long long)(c0 + k) * kChunk; };
  if (lloyd)
    for (int i = threadIdx.x; i < kLloydBins; i += kThreads) lh[i] = 0;
  __syncthreads();

  const int lane = threadIdx.x & 31;
  unsigned *dst = cand + cd.coefOff;
  for (int k = 0; k < nc; k++) {
    const int len = chunk_len(k);
    float v[kPerThread];
    load_chunk(chunk_src(k), len, v);
    unsigned m = 0;  // candidates among this thread's values
    auto scan = [&](auto full) {
#pragma unroll
      for (int j = 0; j < kPerThread; j++) {
        const unsigned a = __float_as_uint(v[j]) & 0x7fffffffu;
        const bool in = decltype(full)::value || chunk_index(j) < len;
        if (in && (a >> 20) == prefix) m |= 1u << j;
        if (lloyd && in && (a >> 20) > prefix && a <= lhi)
          atomicAdd(&lh[(a - lbase) >> lshift], 1u);
      }
    };
    if (len == kChunk) scan(std::true_type());
    else scan(std::false_type());
    // warp-wide exclusive count of candidates, one reservation per warp and
    // chunk (the candidates' order does not matter: they are only counted)
    const unsigned cnt = __popc(m);
    unsigned inc = cnt;
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned t = __shfl_up_sync(0xffffffffu, inc, off);
      if (lane >= off) inc += t;
    }
    unsigned base = 0;
    if (lane == 31 && inc) base = atomicAdd(&st->candCount, inc);
    unsigned o = __shfl_sync(0xffffffffu, base, 31) + inc - cnt;
#pragma unroll
    for (int j = 0; j < kPerThread; j++)
      if ((m >> j) & 1u) dst[o++] = __float_as_uint(v[j]) & 0x7fffffffu;
  }
  __syncthreads();  // every thread's Lloyd histogram counts are in
  if (lloyd) {
    unsigned *g = reinterpret_cast<unsigned *>(b.lloydHist) + (size_t)ci * kLloydBins;
    for (int i = threadIdx.x; i < kLloydBins; i += kThreads)
      if (lh[i]) atomicAdd(&g[i], lh[i]);
  }
}

// Digit histograms over the candidates: PASS 1 bits 19..8, PASS 2 bits 7..0
// of the candidates that match the 24-bit prefix.  blockIdx.y = cubelet.
template <int PASS>
__global__ void __launch_bounds__(kThreads)
cand_hist(DevBatch b, const unsigned *__restrict__ cand) {
  __shared__ unsigned hist[kSelectBins];
  const int ci = blockIdx.y;
  const CubeletDev cd = b.cub[ci];
  const CubeletState *st = b.state + ci;
  const unsigned n = st->candCount;
  if ((unsigned)blockIdx.x * kThreads >= n) return;
  const unsigned prefix = st->prefix;
  const int nb = PASS == 2 ? 256 : kSelectBins;
  for (int i = threadIdx.x; i < nb; i += kThreads) hist[i] = 0;
  __syncthreads();
  const unsigned *src = cand + cd.coefOff;
  for (unsigned i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const unsigned a = src[i];
    if (PASS == 1) atomicAdd(&hist[(a >> 8) & 0xfffu], 1u);
    else if ((a >> 8) == prefix) atomicAdd(&hist[a & 0xffu], 1u);
  }
  __syncthreads();
  unsigned *g = b.selHist + (size_t)ci * kSelectBins;
  for (int i = threadIdx.x; i < nb; i += kThreads)
    if (hist[i]) atomicAdd(&g[i], hist[i]);
}

// Lloyd histogram bins for threshold < |c| <= hi: bin = (bits - base) >> shift,
// the shift the smallest that keeps the range inside kLloydBins bins
__device__ __forceinline__ void set_lloyd_bins(CubeletState *st, unsigned base, unsigned hiBits) {
  const unsigned span = hiBits > base ? hiBits - base : 0u;
  int shift = 0;
  while ((span >> shift) >= (unsigned)kLloydBins) shift++;
  st->lloydBase = base;
  st->lloydHiBits = hiBits;
  st->lloydShift = shift;
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
          if (cd.quantAlg == WL_LLOYD) {
            // Lloyd range top: the second largest |c| unless it is not above
            // the threshold (test_compress_cpu.cc:419-422).  Decidable from
            // the bucket alone unless it lies in the bucket; bucket 0 may
            // hold a zero threshold, which becomes 1e-16.
            const unsigned P = (unsigned)i, a2 = st->absMax2;
            int deferred = 0;
            unsigned hiBits = 0;
            if (P == 0 || (a2 >> 20) == P) deferred = 1;
            else hiBits = (a2 >> 20) > P ? a2 : st->absMax;
            st->lloydDeferred = deferred;
            if (!deferred) set_lloyd_bins(st, P << 20, hiBits);
          }
        } else if (PASS == 1) {
          st->prefix = (st->prefix << 12) | (unsigned)i;
          st->rank = rem;
        } else {
          const unsigned bits = (st->prefix << 8) | (unsigned)i;
          float t = __uint_as_float(bits);
          if (t == 0.0f) t = 1e-16f;  // thresh_cpu.cc:98
          st->threshold = t;
          if (cd.quantAlg == WL_LLOYD && st->lloydDeferred) {
            const float hi = st->maxAbs2 > t ? st->maxAbs2 : st->maxAbs;
            set_lloyd_bins(st, __float_as_uint(t), __float_as_uint(hi));
          }
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

// cubelet index of every chunk (and quantize group), so chunk kernels start
// with one load
__global__ void chunk_map_kernel(DevBatch b) {
  const CubeletDev cd = b.cub[blockIdx.x];
  for (int j = threadIdx.x; j < cd.nChunks; j += blockDim.x)
    b.chunkCub[cd.chunkBase + j] = (int)blockIdx.x;
  const int groups = (cd.nChunks + kQuantGroup - 1) / kQuantGroup;
  for (int j = threadIdx.x; j < groups; j += blockDim.x)
    b.groupCub[cd.groupBase + j] = (int)blockIdx.x;
  const int enc = (int)(((long long)cd.nChunks * b.encF + kEncThreads - 1) / kEncThreads);
  for (int j = threadIdx.x; j < enc; j += blockDim.x) b.encCub[cd.encBase + j] = (int)blockIdx.x;
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
  st->candCount = 0u;
  st->lloydDeferred = 0;
}

}  // namespace

void launch_select_init(DevBatch &b, cudaStream_t s) {
  select_init<<<(b.n + 127) / 128, 128, 0, s>>>(b);
}

void launch_select(DevBatch &b, const float *coef, bool pass0, cudaStream_t s) {
  chunk_map_kernel<<<b.n, 256, 0, s>>>(b);
  unsigned *cand = reinterpret_cast<unsigned *>(b.coef2);
  const unsigned groups = (unsigned)b.totalGroups;
  if (pass0) select_pass0<<<groups, kThreads, 0, s>>>(b, coef);
  select_resolve<0><<<b.n, 1024, 0, s>>>(b);
  select_compact<<<groups, kThreads, 0, s>>>(b, coef, cand);
  cand_hist<1><<<dim3(kCandSlices, b.n), kThreads, 0, s>>>(b, cand);
  select_resolve<1><<<b.n, 1024, 0, s>>>(b);
  cand_hist<2><<<dim3(kCandSlices, b.n), kThreads, 0, s>>>(b, cand);
  select_resolve<2><<<b.n, 1024, 0, s>>>(b);
}

}  // namespace wl
