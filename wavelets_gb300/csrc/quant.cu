// Quantizers fused with the Huffman frequency count, plus the zero-run
// bookkeeping the Huffman coder needs.
//
// Reference: quantize (test_compress_cpu.cc:244-295) with QuantUniform
// (quant.h:189-293), QuantLog (:326-439) and QuantCodebook (:467-558);
// huffScan (test_compress_common.cc:901-921) counts every non-zero-bin value
// and splits each run of the zero bin into "dup" tokens of 2^(v+3) elements
// (v = 0..7, greedy, longest first, HuffmanDup huffman.h:13-58) plus single
// zero-bin tokens.
//
// A chunk of 4096 consecutive coefficients (reference Z-X-Y order) is one CTA.
// Runs wholly inside a chunk are decomposed there; runs that touch a chunk
// edge are joined across chunks by runs_kernel, which also records for every
// chunk where the run entering it started and where the run leaving it ends,
// so the encoder can place every dup token without another scan.
//
// Bit exactness: the uniform quantizer is evaluated with the reference's
// unfused float operations; the log quantizer compares against per-cubelet
// bin boundaries computed on the host with the host's logf (quant_host.cpp),
// because the device has no bit-identical logf; the codebook quantizer is the
// reference's lower_bound with its last-boundary special case.
#include <cfloat>

#include "wl_internal.h"

namespace wl {
namespace {

constexpr int kThreads = kChunkThreads;
constexpr int kPer = kChunk / kThreads;  // 16 consecutive elements per thread
constexpr int INF = 0x7fffffff;

__device__ __forceinline__ int find_cubelet(const long long *prefix, int n, long long c) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= c) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// greedy split of a zero-bin run (HuffmanDup::dupCount, huffman.h:46-57)
__device__ __forceinline__ void run_split(long long L, long long &singles, long long &dups) {
  dups = L / 1024;  // dupFindLongest returns 7 (1024) while L >= 1024
  int r = (int)(L % 1024);
  while (r > 8) {
    int p = 8;
    while ((p << 1) <= r) p <<= 1;
    r -= p;
    dups++;
  }
  singles = r;
}

// ---- quantizer parameters ---------------------------------------------------
__global__ void quant_params_kernel(DevBatch b) {
  const int ci = blockIdx.x * blockDim.x + threadIdx.x;
  if (ci >= b.n) return;
  const CubeletDev cd = b.cub[ci];
  CubeletState *st = b.state + ci;
  const float thr = st->threshold, maxVal = st->maxAbs;
  const int B = cd.binCount;
  if (cd.quantAlg == WL_UNIFORM) {
    // QuantUniform::init (quant.h:196-242), unfused float operations
    const int negBinCount = (B - 1) / 2, posBinCount = B / 2;
    const float range = __fsub_rn(maxVal, thr);
    st->negScale = __fdiv_rn((float)(negBinCount - 1), range);
    st->posScale = __fdiv_rn((float)(posBinCount - 1), range);
    st->negOffset = __fsub_rn(1.0f, __fmul_rn(thr, st->negScale));
    st->posOffset = __fsub_rn(1.0f, __fmul_rn(thr, st->posScale));
    st->zeroBin = (B - 1) >> 1;
  } else if (cd.quantAlg == WL_LOG) {
    st->zeroBin = (B - 1) >> 1;
    const int4 h = b.logHdr[ci];  // computed on the host (quant_host.cpp)
    st->lowBin = h.x;
    st->highNeg = h.y;
    st->nPos = h.z;
    st->nNeg = h.w;
  }
  // Lloyd: zeroBin is set by lloyd_solve
  if (cd.quantAlg != WL_LLOYD) st->dupValue = cd.compressZeros ? st->zeroBin : -1;
}

// ---- Lloyd on the |coefficient| histogram -----------------------------------
__device__ __forceinline__ void lloyd_range(const CubeletState *st, float &lo, float &hi) {
  lo = st->threshold;
  hi = st->maxAbs2;  // the reference skips the largest value (test_compress_cpu.cc:419-422)
  if (!(hi > lo)) hi = st->maxAbs;
}

__global__ void __launch_bounds__(kThreads)
lloyd_hist_kernel(DevBatch b, const float *__restrict__ coef) {
  __shared__ unsigned hist[kLloydBins];
  const long long chunk = blockIdx.x;
  const int ci = find_cubelet(b.chunkPrefix, b.n, chunk);
  const CubeletDev cd = b.cub[ci];
  if (cd.quantAlg != WL_LLOYD) return;
  const CubeletState *st = b.state + ci;
  float lo, hi;
  lloyd_range(st, lo, hi);
  if (!(hi > lo)) return;
  const float l0 = log2f(lo), scale = kLloydBins / (log2f(hi) - l0);
  for (int i = threadIdx.x; i < kLloydBins; i += kThreads) hist[i] = 0;
  __syncthreads();
  const long long start = (chunk - cd.chunkBase) * (long long)kChunk;
  const int len = (int)min((long long)kChunk, cd.n - start);
  const float *src = coef + cd.coefOff + start;
  for (int i = threadIdx.x; i < len; i += kThreads) {
    const float a = fabsf(src[i]);
    if (a > lo && a <= hi) {
      int h = (int)((log2f(a) - l0) * scale);
      h = min(max(h, 0), kLloydBins - 1);
      atomicAdd(&hist[h], 1u);
    }
  }
  __syncthreads();
  unsigned *g = reinterpret_cast<unsigned *>(b.lloydHist) + (size_t)ci * kLloydBins;
  for (int i = threadIdx.x; i < kLloydBins; i += kThreads)
    if (hist[i]) atomicAdd(&g[i], hist[i]);
}

// block-wide inclusive scan of doubles (1024 threads, 4 bins per thread)
constexpr int kLloydSmem = 2 * (kLloydBins + 1) * 8 + 3 * (kMaxBins / 2 + 1) * 4;

__global__ void __launch_bounds__(1024) lloyd_solve_kernel(DevBatch b) {
  extern __shared__ double lsm[];
  double *pw = lsm, *pwx = lsm + (kLloydBins + 1);
  float *cb = reinterpret_cast<float *>(pwx + (kLloydBins + 1));
  float *mid = cb + (kMaxBins / 2 + 1);
  float *nxt = mid + (kMaxBins / 2 + 1);
  const int ci = blockIdx.x;
  const CubeletDev cd = b.cub[ci];
  if (cd.quantAlg != WL_LLOYD) return;
  CubeletState *st = b.state + ci;
  const int B = cd.binCount, cbs = (B - 1) / 2;
  float lo, hi;
  lloyd_range(st, lo, hi);
  const unsigned *g = reinterpret_cast<const unsigned *>(b.lloydHist) + (size_t)ci * kLloydBins;
  const bool degenerate = !(hi > lo) || cbs < 1;
  const float l0 = degenerate ? 0.f : log2f(lo);
  const float w = degenerate ? 1.f : (log2f(hi) - l0) / kLloydBins;

  // prefix sums (fixed order, so the codebook is deterministic)
  if (threadIdx.x == 0) { pw[0] = 0; pwx[0] = 0; }
  for (int i = threadIdx.x; i < kLloydBins; i += 1024) {
    const double c = degenerate ? 0.0 : (double)g[i];
    const double x = exp2((double)l0 + ((double)i + 0.5) * (double)w);
    pw[i + 1] = c;
    pwx[i + 1] = c * x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i <= kLloydBins; i++) { pw[i] += pw[i - 1]; pwx[i] += pwx[i - 1]; }
  }
  // initialLloydCodebook (test_compress_common.cc:749-779)
  if (cbs >= 1) {
    const float logScale = degenerate ? 0.f : __fdiv_rn(logf(__fdiv_rn(hi, lo)), (float)cbs);
    for (int i = threadIdx.x; i < cbs; i += 1024) cb[i] = lo * expf(i * logScale);
  }
  __syncthreads();
  for (int it = 0; it < cd.lloydIters && !degenerate; it++) {
    for (int i = threadIdx.x; i + 1 < cbs; i += 1024) mid[i] = 0.5f * (cb[i] + cb[i + 1]);
    __syncthreads();
    // cell i covers histogram bins [first(i), first(i+1)): first bin whose
    // centre is >= mid[i-1]
    for (int i = threadIdx.x; i < cbs; i += 1024) {
      int a = 0, z = 0;
      if (i > 0) {
        const double m = log2((double)mid[i - 1]);
        a = (int)ceil((m - l0) / w - 0.5);
        a = min(max(a, 0), kLloydBins);
      }
      if (i + 1 < cbs) {
        const double m = log2((double)mid[i]);
        z = (int)ceil((m - l0) / w - 0.5);
        z = min(max(z, 0), kLloydBins);
      } else {
        z = kLloydBins;
      }
      if (z < a) z = a;
      const double cw = pw[z] - pw[a];
      nxt[i] = cw > 0 ? (float)((pwx[z] - pwx[a]) / cw) : cb[i];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < cbs; i += 1024) cb[i] = nxt[i];
    __syncthreads();
  }
  // setBinsFromCodebook (test_compress_common.cc:784-846), one thread, the
  // reference's float expressions
  if (threadIdx.x == 0) {
    float *bnd = b.qtable + cd.tableOff;
    float *val = b.dqtable + (size_t)ci * kMaxBins;
    const float minVal = st->minVal, maxVal = st->maxVal, thr = st->threshold;
    int nb = 0, nv = 0;
    if (cbs < 1) {
      val[nv++] = 0;
    } else {
      if ((B & 1) == 0 && fabsf(minVal) > maxVal) {
        val[nv++] = minVal;
        bnd[nb++] = __fdiv_rn(__fadd_rn(minVal, -cb[cbs - 1]), 2.0f);
      }
      val[nv++] = -cb[cbs - 1];
      for (int i = cbs - 2; i >= 0; i--) {
        bnd[nb++] = __fdiv_rn(__fadd_rn(-cb[i], -cb[i + 1]), 2.0f);
        val[nv++] = -cb[i];
      }
      bnd[nb++] = -thr;
      val[nv++] = 0;
      bnd[nb++] = thr;
      for (int i = 0; i < cbs - 1; i++) {
        val[nv++] = cb[i];
        bnd[nb++] = __fdiv_rn(__fadd_rn(cb[i], cb[i + 1]), 2.0f);
      }
      val[nv++] = cb[cbs - 1];
      if ((B & 1) == 0 && maxVal >= fabsf(minVal)) {
        val[nv++] = maxVal;
        bnd[nb++] = __fdiv_rn(__fadd_rn(maxVal, cb[cbs - 1]), 2.0f);
      }
    }
    // QuantCodebook::quant(0) (quant.h:515-526)
    int zb;
    if (nb == 0) zb = 0;
    else if (0.0f >= bnd[nb - 1]) zb = nb;
    else {
      zb = 0;
      while (zb < nb && bnd[zb] < 0.0f) zb++;
    }
    st->zeroBin = zb;
    st->dupValue = cd.compressZeros ? zb : -1;
    st->nBounds = nb;
    st->nValues = nv;
    if (nv != B) st->error = 3;
  }
}

// ---- quantize one value ------------------------------------------------------
struct QParams {
  int alg, B, zb;
  float thr, negScale, negOffset, posScale, posOffset;
  int nb;          // codebook boundaries / log: positive table length
  int lowBin, highNeg, nPos, nNeg;
};

__device__ __forceinline__ int quant_value(float x, const QParams &q, const float *tab) {
  if (q.alg == WL_UNIFORM) {
    // QuantUniform::quant (quant.h:244-276)
    if (x < 0) {
      if (x >= -q.thr) return q.zb;
      const float t = __fsub_rn(__fmul_rn(x, q.negScale), q.negOffset);
      const int bin = __float2int_rz(t) + q.zb;
      return bin < 0 ? 0 : bin;
    }
    if (x <= q.thr) return q.zb;
    const float t = __fadd_rn(__fadd_rn(__fmul_rn(x, q.posScale), q.posOffset), (float)q.zb);
    if (t > (float)(q.B - 1)) return q.B - 1;
    return __float2int_rz(t);
  }
  if (q.alg == WL_LOG) {
    // tab: [P(lowBin+1 .. B-1)] then [N(0 .. highNeg-1)], nondecreasing
    if (x < 0) {
      const float y = -x;
      if (y <= q.thr) return q.zb;
      const float *N = tab + q.nPos;
      int lo = 0, hi = q.nNeg;  // count entries <= y
      while (lo < hi) {
        int m = (lo + hi) >> 1;
        if (N[m] <= y) lo = m + 1; else hi = m;
      }
      return q.highNeg - lo;
    }
    if (x <= q.thr) return q.zb;
    int lo = 0, hi = q.nPos;
    while (lo < hi) {
      int m = (lo + hi) >> 1;
      if (tab[m] <= x) lo = m + 1; else hi = m;
    }
    return q.lowBin + lo;
  }
  // QuantCodebook::quant (quant.h:515-526)
  if (q.nb == 0) return 0;
  if (x >= tab[q.nb - 1]) return q.nb;
  int lo = 0, hi = q.nb;
  while (lo < hi) {
    int m = (lo + hi) >> 1;
    if (tab[m] < x) lo = m + 1; else hi = m;
  }
  return lo;
}

__device__ __forceinline__ QParams load_qparams(const CubeletDev &cd, const CubeletState *st) {
  QParams q;
  q.alg = cd.quantAlg;
  q.B = cd.binCount;
  q.zb = st->zeroBin;
  q.thr = st->threshold;
  q.negScale = st->negScale;
  q.negOffset = st->negOffset;
  q.posScale = st->posScale;
  q.posOffset = st->posOffset;
  q.nb = 0; q.lowBin = 0; q.highNeg = 0; q.nPos = 0; q.nNeg = 0;
  if (q.alg == WL_LLOYD) q.nb = st->nBounds;
  if (q.alg == WL_LOG) {  // table layout written by the host
    q.lowBin = st->lowBin;
    q.highNeg = st->highNeg;
    q.nPos = st->nPos;
    q.nNeg = st->nNeg;
  }
  return q;
}

// ---- quantize + count + chunk run summary ----------------------------------
__global__ void __launch_bounds__(kThreads)
quantize_kernel(DevBatch b, const float *__restrict__ coef) {
  __shared__ unsigned hist[kMaxSymbols + 1];
  __shared__ float tab[kMaxBins];
  __shared__ int wFirst[kThreads / 32], wLast[kThreads / 32];
  __shared__ unsigned long long sDup;
  const long long chunk = blockIdx.x;
  const int ci = find_cubelet(b.chunkPrefix, b.n, chunk);
  const CubeletDev cd = b.cub[ci];
  const CubeletState *st = b.state + ci;
  const QParams q = load_qparams(cd, st);
  const int dupV = st->dupValue;
  const int B = cd.binCount;
  const int nTab = q.alg == WL_LLOYD ? q.nb : (q.alg == WL_LOG ? q.nPos + q.nNeg : 0);
  for (int i = threadIdx.x; i < B + 1; i += kThreads) hist[i] = 0;
  for (int i = threadIdx.x; i < nTab; i += kThreads) tab[i] = b.qtable[cd.tableOff + i];
  if (threadIdx.x == 0) sDup = 0;
  __syncthreads();

  const long long start = (chunk - cd.chunkBase) * (long long)kChunk;
  const int len = (int)min((long long)kChunk, cd.n - start);
  const float *src = coef + cd.coefOff + start;
  uint16_t *dst = b.bins + cd.coefOff + start;
  const int p0 = threadIdx.x * kPer;

  int bins[kPer];
  if (p0 + kPer <= len) {
    const float4 *s4 = reinterpret_cast<const float4 *>(src + p0);
#pragma unroll
    for (int k = 0; k < kPer / 4; k++) {
      const float4 v = s4[k];
      bins[4 * k + 0] = quant_value(v.x, q, tab);
      bins[4 * k + 1] = quant_value(v.y, q, tab);
      bins[4 * k + 2] = quant_value(v.z, q, tab);
      bins[4 * k + 3] = quant_value(v.w, q, tab);
    }
    uint4 *d4 = reinterpret_cast<uint4 *>(dst + p0);
#pragma unroll
    for (int k = 0; k < kPer / 8; k++) {
      uint4 o;
      o.x = (unsigned)bins[8 * k + 0] | ((unsigned)bins[8 * k + 1] << 16);
      o.y = (unsigned)bins[8 * k + 2] | ((unsigned)bins[8 * k + 3] << 16);
      o.z = (unsigned)bins[8 * k + 4] | ((unsigned)bins[8 * k + 5] << 16);
      o.w = (unsigned)bins[8 * k + 6] | ((unsigned)bins[8 * k + 7] << 16);
      d4[k] = o;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kPer; k++) {
      const int p = p0 + k;
      bins[k] = p < len ? quant_value(src[p], q, tab) : dupV;
      if (p < len) dst[p] = (uint16_t)bins[k];
    }
  }

  // histogram of the values that are not part of zero runs
  int first = INF, last = -1;
#pragma unroll
  for (int k = 0; k < kPer; k++) {
    const int p = p0 + k;
    if (p >= len) break;
    if (bins[k] != dupV) {
      atomicAdd(&hist[bins[k]], 1u);
      if (first == INF) first = p;
      last = p;
    }
  }

  if (dupV >= 0) {
    // next non-zero-bin position after this thread's range, previous before it
    int sufMin = first, preMax = last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incMin = sufMin, incMax = preMax;
    for (int off = 1; off < 32; off <<= 1) {
      int vmin = __shfl_down_sync(0xffffffffu, incMin, off);
      int vmax = __shfl_up_sync(0xffffffffu, incMax, off);
      if (lane + off < 32) incMin = min(incMin, vmin);
      if (lane >= off) incMax = max(incMax, vmax);
    }
    if (lane == 0) wFirst[w] = incMin;   // min over the whole warp
    if (lane == 31) wLast[w] = incMax;   // max over the whole warp
    __syncthreads();
    int nextNZ = __shfl_down_sync(0xffffffffu, incMin, 1);
    if (lane == 31) nextNZ = INF;
    int prevNZ = __shfl_up_sync(0xffffffffu, incMax, 1);
    if (lane == 0) prevNZ = -1;
    for (int v = w + 1; v < kThreads / 32; v++) nextNZ = min(nextNZ, wFirst[v]);
    for (int v = 0; v < w; v++) prevNZ = max(prevNZ, wLast[v]);

    // runs that start inside this thread's range and end inside the chunk
    long long singles = 0, dups = 0;
    int k = 0;
    while (k < kPer && p0 + k < len) {
      if (bins[k] != dupV) { k++; continue; }
      const int s = p0 + k;
      const bool startsHere = (k > 0) ? true : (prevNZ == s - 1);
      int e = k;
      while (e < kPer && p0 + e < len && bins[e] == dupV) e++;
      int endPos;
      if (e < kPer && p0 + e < len) endPos = p0 + e;
      else endPos = (p0 + e >= len) ? INF : nextNZ;
      if (startsHere && s > 0 && endPos != INF && endPos < len) {
        long long sg, dp;
        run_split(endPos - s, sg, dp);
        singles += sg;
        dups += dp;
      }
      k = e;
    }
    if (singles) atomicAdd(&hist[dupV], (unsigned)singles);
    if (dups) atomicAdd(&sDup, (unsigned long long)dups);
    if (threadIdx.x == 0) {
      int fz = INF, lz = -1;
      for (int v = 0; v < kThreads / 32; v++) { fz = min(fz, wFirst[v]); lz = max(lz, wLast[v]); }
      const int lead = fz == INF ? len : fz;
      const int trail = lz < 0 ? len : len - 1 - lz;
      b.chunkRun[chunk] = make_int4(lead, trail, lz < 0 ? 1 : 0, len);
    }
  }
  __syncthreads();
  unsigned long long *gh = b.hist + (size_t)ci * kMaxSymbols;
  for (int i = threadIdx.x; i < B; i += kThreads)
    if (hist[i]) atomicAdd(&gh[i], (unsigned long long)hist[i]);
  if (threadIdx.x == 0 && sDup) atomicAdd(&gh[B], sDup);
}

// Join zero runs across chunk edges; one CTA per cubelet.
__device__ __forceinline__ int block_scan_max_excl(int v, int *sh, int &total) {
  // exclusive max-scan over 1024 threads (identity -1)
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = v;
  for (int off = 1; off < 32; off <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, inc, off);
    if (lane >= off) inc = max(inc, t);
  }
  if (lane == 31) sh[w] = inc;
  __syncthreads();
  if (w == 0) {
    int x = sh[lane];
    for (int off = 1; off < 32; off <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x = max(x, t);
    }
    sh[32 + lane] = x;
  }
  __syncthreads();
  int before = w > 0 ? sh[32 + w - 1] : -1;
  int ex = __shfl_up_sync(0xffffffffu, inc, 1);
  if (lane == 0) ex = -1;
  total = sh[32 + 31];
  __syncthreads();
  return max(before, ex);
}

__device__ __forceinline__ int block_scan_min_excl_rev(int v, int *sh, int &total) {
  // exclusive min-scan from the right (identity INF)
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = v;
  for (int off = 1; off < 32; off <<= 1) {
    int t = __shfl_down_sync(0xffffffffu, inc, off);
    if (lane + off < 32) inc = min(inc, t);
  }
  if (lane == 0) sh[w] = inc;
  __syncthreads();
  if (w == 0) {
    int x = sh[lane];
    for (int off = 1; off < 32; off <<= 1) {
      int t = __shfl_down_sync(0xffffffffu, x, off);
      if (lane + off < 32) x = min(x, t);
    }
    sh[32 + lane] = x;
  }
  __syncthreads();
  int after = w < 31 ? sh[32 + w + 1] : INF;
  int ex = __shfl_down_sync(0xffffffffu, inc, 1);
  if (lane == 31) ex = INF;
  total = sh[32];
  __syncthreads();
  return min(after, ex);
}

__global__ void __launch_bounds__(1024) runs_kernel(DevBatch b) {
  __shared__ int sh[64];
  __shared__ unsigned long long sSingles, sDups;
  const int ci = blockIdx.x;
  const CubeletDev cd = b.cub[ci];
  const CubeletState *st = b.state + ci;
  const int dupV = st->dupValue;
  if (dupV < 0) return;
  const int nc = cd.nChunks;
  const long long base = cd.chunkBase;
  int4 *cr = b.chunkRun + base;
  long long *ctx = b.chunkRunCtx + 2 * base;
  if (threadIdx.x == 0) { sSingles = 0; sDups = 0; }
  __syncthreads();

  // forward: previous non-all-zero chunk (exclusive)
  int carry = -1;
  for (int seg = 0; seg < nc; seg += 1024) {
    const int c = seg + threadIdx.x;
    const int v = (c < nc && !cr[c].z) ? c : -1;
    int total;
    int ex = block_scan_max_excl(v, sh, total);
    ex = max(ex, carry);
    if (c < nc) {
      long long s0 = 0;
      if (ex >= 0) {
        const int4 o = cr[ex];
        s0 = (long long)ex * kChunk + o.w - o.y;
      }
      ctx[2 * c] = s0;  // start of the run entering chunk c
    }
    carry = max(carry, total);
  }
  // backward: next non-all-zero chunk (exclusive); run ends and lengths
  int carryN = INF;
  long long singles = 0, dups = 0;
  for (int seg = ((nc - 1) / 1024) * 1024; seg >= 0; seg -= 1024) {
    const int c = seg + threadIdx.x;
    const int v = (c < nc && !cr[c].z) ? c : INF;
    int total;
    int ex = block_scan_min_excl_rev(v, sh, total);
    ex = min(ex, carryN);
    if (c < nc) {
      const long long e = ex == INF ? cd.n : (long long)ex * kChunk + cr[ex].x;
      ctx[2 * c + 1] = e;  // end of the run leaving chunk c
      const int4 me = cr[c];
      if (!me.z) {
        const long long s0 = (long long)c * kChunk + me.w - me.y;
        if (e > s0) {
          long long sg, dp;
          run_split(e - s0, sg, dp);
          singles += sg;
          dups += dp;
        }
      }
    }
    // the run starting at element 0 belongs to no chunk's tail
    if (seg == 0 && threadIdx.x == 0) {
      const int first = (v != INF) ? 0 : ex;
      const long long e = first == INF ? cd.n : (long long)first * kChunk + cr[first].x;
      if (e > 0) {
        long long sg, dp;
        run_split(e, sg, dp);
        singles += sg;
        dups += dp;
      }
    }
    carryN = min(carryN, total);
  }
  if (singles) atomicAdd(&sSingles, (unsigned long long)singles);
  if (dups) atomicAdd(&sDups, (unsigned long long)dups);
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long *gh = b.hist + (size_t)ci * kMaxSymbols;
    gh[dupV] += sSingles;
    gh[cd.binCount] += sDups;
  }
}

}  // namespace

void launch_quant_params(DevBatch &b, cudaStream_t s) {
  quant_params_kernel<<<(b.n + 127) / 128, 128, 0, s>>>(b);
}

void launch_lloyd(DevBatch &b, const float *coef, cudaStream_t s) {
  lloyd_hist_kernel<<<(unsigned)b.totalChunks, kThreads, 0, s>>>(b, coef);
  cudaFuncSetAttribute(lloyd_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kLloydSmem);
  lloyd_solve_kernel<<<b.n, 1024, kLloydSmem, s>>>(b);
}

void launch_quantize(DevBatch &b, const float *coef, cudaStream_t s) {
  quantize_kernel<<<(unsigned)b.totalChunks, kThreads, 0, s>>>(b, coef);
}

void launch_runs(DevBatch &b, cudaStream_t s) { runs_kernel<<<b.n, 1024, 0, s>>>(b); }

}  // namespace wl
