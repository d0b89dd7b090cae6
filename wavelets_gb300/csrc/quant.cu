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

#include <type_traits>

#include "wl_internal.h"

namespace wl {
namespace {

constexpr int kThreads = kChunkThreads;
constexpr int INF = 0x7fffffff;

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

// number of entries of the sorted table t[0..n) that are <= x / < x, by a
// fixed number of halving steps (no divergent loop exits)
__device__ __forceinline__ int count_le(const float *t, int n, float x) {
  int pos = 0;
  for (int step = n ? 1 << (31 - __clz(n)) : 0; step > 0; step >>= 1)
    if (step <= n - pos && t[pos + step - 1] <= x) pos += step;
  return pos;
}
__device__ __forceinline__ int count_lt(const float *t, int n, float x) {
  int pos = 0;
  for (int step = n ? 1 << (31 - __clz(n)) : 0; step > 0; step >>= 1)
    if (step <= n - pos && t[pos + step - 1] < x) pos += step;
  return pos;
}

// Lloyd bin lookup table.  Floats map to an order-preserving 32-bit key
// (sign flipped for positives, all bits for negatives); cell c holds the keys
// c << 20 .. (c+1) << 20, i.e. 1/8 octave of one sign.  lut[c] counts the
// boundaries below the smallest float of cell c, so for x in the cell the
// reference's lower_bound is lut[c] plus the boundaries of
// [lut[c], lut[c+1]) that are below x.
__device__ __forceinline__ unsigned order_key(float x) {
  const unsigned u = __float_as_uint(x);
  return u ^ ((unsigned)((int)u >> 31) | 0x80000000u);
}
__device__ __forceinline__ float cell_min(int c) {
  const unsigned k = (unsigned)c << 20;
  return __uint_as_float((k & 0x80000000u) ? (k ^ 0x80000000u) : ~k);
}

// ---- Lloyd on the |coefficient| histogram -----------------------------------
__device__ __forceinline__ void lloyd_range(const CubeletState *st, float &lo, float &hi) {
  lo = st->threshold;
  hi = st->maxAbs2;  // the reference skips the largest value (test_compress_cpu.cc:419-422)
  if (!(hi > lo)) hi = st->maxAbs;
}

// The Lloyd histogram counts threshold < |c| <= hi in bins of the |c| bit
// pattern, (bits - lloydBase) >> lloydShift: above the threshold bucket the
// compaction pass of the threshold select already counted them; the bucket's
// candidates are added here once the threshold is known.
__global__ void __launch_bounds__(kThreads)
lloyd_cand_kernel(DevBatch b, const unsigned *__restrict__ cand) {
  __shared__ unsigned hist[kLloydBins];
  const int ci = blockIdx.y;
  const CubeletDev cd = b.cub[ci];
  const CubeletState *st = b.state + ci;
  const unsigned n = st->candCount;
  if (cd.quantAlg != WL_LLOYD || st->lloydDeferred || (unsigned)blockIdx.x * kThreads >= n) return;
  const unsigned lo = __float_as_uint(st->threshold), hi = st->lloydHiBits, base = st->lloydBase;
  const int shift = st->lloydShift;
  for (int i = threadIdx.x; i < kLloydBins; i += kThreads) hist[i] = 0;
  __syncthreads();
  const unsigned *src = cand + cd.coefOff;
  for (unsigned i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const unsigned a = src[i];
    if (a > lo && a <= hi) atomicAdd(&hist[(a - base) >> shift], 1u);
  }
  __syncthreads();
  unsigned *g = reinterpret_cast<unsigned *>(b.lloydHist) + (size_t)ci * kLloydBins;
  for (int i = threadIdx.x; i < kLloydBins; i += kThreads)
    if (hist[i]) atomicAdd(&g[i], hist[i]);
}

// Cubelets whose Lloyd range the select passes could not settle early (the
// second largest |c| in the threshold bucket, or bucket 0): one pass over
// their coefficients with the final threshold.
__global__ void __launch_bounds__(kThreads)
lloyd_deferred_kernel(DevBatch b, const float *__restrict__ coef) {
  __shared__ unsigned hist[kLloydBins];
  const int ci = blockIdx.y;
  const CubeletDev cd = b.cub[ci];
  const CubeletState *st = b.state + ci;
  if (cd.quantAlg != WL_LLOYD || !st->lloydDeferred) return;
  const unsigned lo = st->lloydBase, hi = st->lloydHiBits;
  const int shift = st->lloydShift;
  for (int i = threadIdx.x; i < kLloydBins; i += kThreads) hist[i] = 0;
  __syncthreads();
  const float *src = coef + cd.coefOff;
  for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < cd.n;
       i += (long long)gridDim.x * kThreads) {
    const unsigned a = __float_as_uint(src[i]) & 0x7fffffffu;
    if (a > lo && a <= hi) atomicAdd(&hist[(a - lo) >> shift], 1u);
  }
  __syncthreads();
  unsigned *g = reinterpret_cast<unsigned *>(b.lloydHist) + (size_t)ci * kLloydBins;
  for (int i = threadIdx.x; i < kLloydBins; i += kThreads)
    if (hist[i]) atomicAdd(&g[i], hist[i]);
}

// 512 threads and shared memory sized for the batch's largest codebook:
// four CTAs per SM, so a batch of up to 4 x 152 cubelets solves in one wave.
constexpr int kSolveThreads = 512;
// prefix sums: counts (exact in 32 bits) and count * centre (double), block
// scan scratch, then two codebook buffers (cbCap each)
__host__ __device__ inline size_t lloyd_smem_bytes(int cbCap) {
  return (size_t)(kLloydBins + 1) * 8 + (size_t)(kLloydBins + 2) * 4 + 64 * 8 +
         (size_t)2 * cbCap * 4;
}

__global__ void __launch_bounds__(kSolveThreads, 4) lloyd_solve_kernel(DevBatch b, int cbCap) {
  extern __shared__ double lsm[];
  double *pwx = lsm;
  unsigned *pw = reinterpret_cast<unsigned *>(pwx + (kLloydBins + 1));
  double *scratch = reinterpret_cast<double *>(pw + (kLloydBins + 2));
  float *cb = reinterpret_cast<float *>(scratch + 64);
  float *nxt = cb + cbCap;
  const int ci = blockIdx.x;
  const CubeletDev cd = b.cub[ci];
  if (cd.quantAlg != WL_LLOYD) return;
  CubeletState *st = b.state + ci;
  const int B = cd.binCount, cbs = (B - 1) / 2;
  float lo, hi;
  lloyd_range(st, lo, hi);
  const unsigned *g = reinterpret_cast<const unsigned *>(b.lloydHist) + (size_t)ci * kLloydBins;
  const bool degenerate = !(hi > lo) || cbs < 1;
  // histogram bin i covers |c| bits [base + i 2^shift, base + (i+1) 2^shift)
  const unsigned base = st->lloydBase;
  const int shift = st->lloydShift;
  const unsigned half = (1u << shift) >> 1;
  // first bin whose centre is >= m (m > 0)
  auto first_bin = [&](float m) {
    const long long d = (long long)__float_as_uint(m) - (long long)base - (long long)half;
    const long long a = d <= 0 ? 0 : (d + (1ll << shift) - 1) >> shift;
    return (int)min(a, (long long)kLloydBins);
  };

  // prefix sums of counts and count*centre; fixed order, so the codebook is
  // deterministic: each thread sums 8 consecutive bins, then a block scan
  {
    const int per = kLloydBins / kSolveThreads;
    auto bin_at = [&](int j, double &c, double &x) {
      const int i = threadIdx.x * per + j;
      c = degenerate ? 0.0 : (double)g[i];
      x = (double)__uint_as_float(base + ((unsigned)i << shift) + half);
    };
    double sc = 0, sx = 0;
    for (int j = 0; j < per; j++) {
      double c, x;
      bin_at(j, c, x);
      sc += c;
      sx += c * x;
    }
    // inclusive warp scan of the per-thread totals
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    double ic = sc, ix = sx;
    for (int off = 1; off < 32; off <<= 1) {
      const double tc = __shfl_up_sync(0xffffffffu, ic, off);
      const double tx = __shfl_up_sync(0xffffffffu, ix, off);
      if (lane >= off) { ic += tc; ix += tx; }
    }
    double *wc = scratch;
    double *wx = wc + 32;
    if (lane == 31) { wc[wp] = ic; wx[wp] = ix; }
    __syncthreads();
    double bc = 0, bx = 0;
    for (int v = 0; v < wp; v++) { bc += wc[v]; bx += wx[v]; }
    bc += ic - sc;
    bx += ix - sx;
    if (threadIdx.x == 0) { pw[0] = 0; pwx[0] = 0; }
    // the thread's running sums again, in the same order (same values)
    double rc = 0, rx = 0;
    for (int j = 0; j < per; j++) {
      double c, x;
      bin_at(j, c, x);
      rc += c;
      rx += c * x;
      const int i = threadIdx.x * per + j;
      pw[i + 1] = (unsigned)(bc + rc);
      pwx[i + 1] = bx + rx;
    }
    __syncthreads();
  }
  // initialLloydCodebook (test_compress_common.cc:749-779)
  if (cbs >= 1) {
    const float logScale = degenerate ? 0.f : __fdiv_rn(logf(__fdiv_rn(hi, lo)), (float)cbs);
    for (int i = threadIdx.x; i < cbs; i += kSolveThreads) cb[i] = lo * expf(i * logScale);
  }
  __syncthreads();
  // one barrier per iteration: a thread forms the midpoints around its cell
  // itself, and the codebook alternates between two buffers
  float *cur = cb, *nx = nxt;
  for (int it = 0; it < cd.lloydIters && !degenerate; it++) {
    // cell i covers histogram bins [first(i), first(i+1)): first bin whose
    // centre is >= the midpoint (cb[i-1] + cb[i]) / 2
    for (int i = threadIdx.x; i < cbs; i += kSolveThreads) {
      const float c = cur[i];
      const int a = i > 0 ? first_bin(0.5f * (cur[i - 1] + c)) : 0;
      int z = i + 1 < cbs ? first_bin(0.5f * (c + cur[i + 1])) : kLloydBins;
      if (z < a) z = a;
      const double cw = (double)(pw[z] - pw[a]);
      nx[i] = cw > 0 ? (float)((pwx[z] - pwx[a]) / cw) : c;
    }
    __syncthreads();
    float *t = cur;
    cur = nx;
    nx = t;
  }
  if (cur != cb) {
    for (int i = threadIdx.x; i < cbs; i += kSolveThreads) cb[i] = cur[i];
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
  __syncthreads();
  {
    const float *bnd = b.qtable + cd.tableOff;
    const int nb = st->nBounds;
    uint16_t *lut = b.qlut + (size_t)ci * kLutStride;
    for (int c = threadIdx.x; c < kLutCells; c += kSolveThreads) {
      const float m = cell_min(c);  // NaN cells: never looked up; keep the table monotone
      lut[c] = (uint16_t)(m != m ? (c >= kLutCells / 2 ? nb : 0) : count_lt(bnd, nb, m));
    }
    if (threadIdx.x == 0) lut[kLutCells] = (uint16_t)nb;
  }
}

// ---- quantize one value ------------------------------------------------------
struct QParams {
  int alg, B, zb;
  float thr, negScale, negOffset, posScale, posOffset;
  int nb;          // codebook boundaries / log: positive table length
  int lowBin, highNeg, nPos, nNeg;
};

__device__ __forceinline__ int quant_value(float x, const QParams &q, const float *tab,
                                           const uint16_t *lut) {
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
      return q.highNeg - count_le(tab + q.nPos, q.nNeg, y);
    }
    if (x <= q.thr) return q.zb;
    return q.lowBin + count_le(tab, q.nPos, x);
  }
  // QuantCodebook::quant (quant.h:515-526): x >= last boundary -> nb, else
  // lower_bound (the number of boundaries below x; 0 for NaN)
  if (q.nb == 0 || x != x) return 0;
  if (x >= tab[q.nb - 1]) return q.nb;
  const int c = (int)(order_key(x) >> 20);
  const int lo = lut[c], hi = lut[c + 1];
  // a cell (1/8 octave) rarely holds more than two boundaries: compare with
  // them directly, search only when there are more
  if (hi - lo <= 2) {
    const int n = hi - lo;
    return lo + (n > 0 && tab[lo] < x ? 1 : 0) + (n > 1 && tab[lo + 1] < x ? 1 : 0);
  }
  return lo + count_lt(tab + lo, hi - lo, x);
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

// ---- quantize + count + tokens of the chunk ----------------------------------
// Instead of storing a bin per coefficient, a chunk stores its Huffman tokens
// in order: a token for every value that is not the zero bin, preceded by the
// tokens of the zero-bin run before it when that run starts inside the chunk.
// Runs touching a chunk edge are left to runs_kernel (counts) and the encoder
// (tokens).  A CTA codes kQuantGroup consecutive chunks of one cubelet; warp
// w owns elements [512 w, 512 w + 512) of each chunk, and everything but one
// CTA barrier per chunk is warp-local.
//
// Phase 1 (every element): -thr < x < thr is the zero bin for all three
// quantizers (uniform and log test |x| <= thr first; the codebook has the
// boundaries -thr and thr around its zero bin and none in between), so an
// element costs two compares.  The others are candidates, compacted into the
// warp's region of shared memory (in word j lane l holds element
// 512 w + 32 j + l, so loads are coalesced).
// Phase 2 (per candidate, 32 at a time): the exact bin; a candidate that is
// not the zero bin is a value.  The zero run before a value ends at the
// previous value -- the nearest lower lane with one, or the warp's last value
// of earlier rounds -- so its token count is known here, a warp scan gives
// each lane its place among the warp's tokens, and the lane stages its run
// tokens and value token in the warp's buffer (prefilled with the single
// zero-bin token, so only dup tokens and the value token are stored).
// After the CTA barrier the warp summaries (first and last value, staged
// count) give every warp the run before its first value and its place in the
// chunk, and each warp writes that run's tokens and its staged ones to the
// chunk's slot with coalesced stores.
// greedy split of a zero-bin run into dup tokens and single zero-bin tokens
// (closed form of run_split; the same counts as run_token_count)
__device__ __forceinline__ void run_split_closed(int L, int &singles, int &dups) {
  const int q = L >> 10, r = L & 1023, hi = r & ~7, lo = r & 7;
  const int big = __popc(hi >> 4);
  if (hi & 8) {
    dups = q + big + (lo > 0 ? 1 : 0);
    singles = lo > 0 ? lo : 8;
  } else {
    dups = q + big;
    singles = lo;
  }
}

// Tokens of a zero-bin run of L < 2^31 elements lying inside one chunk, in
// the order of run_tokens (whole run, no window): runs of 1024, then one dup
// token per set bit of the remainder above 8, then single zero-bin tokens.
template <class F>
__device__ __forceinline__ void run_tokens_short(int L, int dupKey, int dupV, F f) {
  for (int j = L >> 10; j > 0; j--) f(make_token(dupKey, 7));
  int r = L & 1023;
  while (r > 8) {
    const int lg = 31 - __clz(r);
    f(make_token(dupKey, lg - 3));
    r -= 1 << lg;
  }
  for (; r > 0; r--) f(make_token(dupV, 0));
}

// Token j of run_tokens_short(L, dupKey, dupV) (j below the run's count).
__device__ __forceinline__ uint16_t run_token_at(int L, int j, int dupKey, int dupV) {
  const int q = L >> 10;
  if (j < q) return make_token(dupKey, 7);
  j -= q;
  int r = L & 1023;
  while (r > 8) {
    const int lg = 31 - __clz(r);
    if (j == 0) return make_token(dupKey, lg - 3);
    j--;
    r -= 1 << lg;
  }
  return make_token(dupV, 0);
}

__global__ void __launch_bounds__(kThreads, 4)
quantize_kernel(DevBatch b, const float *__restrict__ coef, int histOff) {
  constexpr int kWords = kChunk / kThreads;  // 16 words of 32 elements per warp
  constexpr int kSpan = 32 * kWords;         // elements per warp
  constexpr int kWarps = kThreads / 32;
  constexpr unsigned kAll = 0xffffffffu;
  // sized by the launch: the quantizer table (Lloyd / log), then the counts
  // of the batch's largest alphabet
  extern __shared__ float tab[];
  unsigned *hist = reinterpret_cast<unsigned *>(tab + histOff);
  __shared__ __align__(16) uint16_t sLut[kLutStride];
  // by warp region: candidate values and positions (32 extra slots: a dump
  // for the stores of lanes without a candidate, which keeps the compaction
  // free of branches)
  __shared__ __align__(16) float sX[kChunk + 32];
  __shared__ uint16_t sPos[kChunk + 32];
  // per warp: its tokens after its first value's zero run, in order (at
  // most kSpan: each token starts at its own element of the warp's span)
  __shared__ __align__(16) uint16_t sStage[kWarps][kSpan];
  // per-warp summaries (first and last value position, staged tokens), two
  // sets used by alternate chunks
  __shared__ int wLast[2][kWarps], wFirst[2][kWarps], wTok[2][kWarps];
  const int ci = b.groupCub[blockIdx.x];
  const CubeletDev cd = b.cub[ci];
  const CubeletState *st = b.state + ci;
  const QParams q = load_qparams(cd, st);
  const int dupV = st->dupValue;
  const int B = cd.binCount;
  const int nTab = q.alg == WL_LLOYD ? q.nb : (q.alg == WL_LOG ? q.nPos + q.nNeg : 0);
  const int c0 = ((int)blockIdx.x - cd.groupBase) * kQuantGroup;  // first chunk of the cubelet
  const int nc = min(kQuantGroup, cd.nChunks - c0);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int base = w * kSpan;
  const unsigned ltMask = (1u << lane) - 1u;
  // zero-bin elements (-thr < x < thr) can be skipped only when they are
  // coded as runs; without runs every element is a candidate (|x| < 0 never)
  const float zthr = dupV >= 0 ? q.thr : 0.f;
  uint16_t *stage = sStage[w];
  const unsigned fill2 = dupV >= 0 ? (unsigned)make_token(dupV, 0) * 0x10001u : 0u;
  int singles = 0, dups = 0;  // the lane's zero-run tokens, over all chunks

  for (int i = threadIdx.x; i < B + 1; i += kThreads) hist[i] = 0;
  for (int i = threadIdx.x; i < nTab; i += kThreads) tab[i] = b.qtable[cd.tableOff + i];
  if (q.alg == WL_LLOYD) {
    const uint4 *gl = reinterpret_cast<const uint4 *>(b.qlut + (size_t)ci * kLutStride);
    uint4 *sl = reinterpret_cast<uint4 *>(sLut);
    for (int i = threadIdx.x; i < kLutStride / 8; i += kThreads) sl[i] = gl[i];
  }
  __syncthreads();

  for (int k = 0; k < nc; k++) {
    const int par = k & 1;
    const long long chunk = cd.chunkBase + c0 + k;
    const long long start = (long long)(c0 + k) * kChunk;
    const int len = (int)min((long long)kChunk, cd.n - start);
    const float *src = coef + cd.coefOff + start;

    // ---- phase 1: candidates into the warp's region; the warp's staging
    // buffer is prefilled with single zero-bin tokens
    if (dupV >= 0) {
      uint4 *s4 = reinterpret_cast<uint4 *>(stage);
      const uint4 f4 = make_uint4(fill2, fill2, fill2, fill2);
      s4[lane] = f4;
      s4[lane + 32] = f4;
    }
    int nCand = 0;  // warp-uniform
    auto phase1 = [&](auto full) {
      constexpr bool kFull = decltype(full)::value;
      float x[kWords];
#pragma unroll
      for (int j = 0; j < kWords; j++) {
        const int pos = base + 32 * j + lane;
        x[j] = (kFull || pos < len) ? src[pos] : 0.f;
      }
#pragma unroll
      for (int j = 0; j < kWords; j++) {
        const int pos = base + 32 * j + lane;
        // zero bin iff |x| < zthr (NaN is a candidate)
        const bool cand = (kFull || pos < len) && !(fabsf(x[j]) < zthr);
        const unsigned m = __ballot_sync(kAll, cand);
        const int l = cand ? base + nCand + __popc(m & ltMask) : kChunk + lane;
        sX[l] = x[j];
        sPos[l] = (uint16_t)pos;
        nCand += __popc(m);
      }
    };
    if (len == kChunk) phase1(std::true_type());
    else phase1(std::false_type());
    __syncwarp();

    // ---- phase 2 (per candidate, 32 at a time): the exact bin; a value
    // (not the zero bin) gets its token and the tokens of the zero run
    // since the warp's previous value, staged in the warp's buffer.  Single
    // zero-bin tokens are already there (prefilled), so a lane stores only
    // its dup tokens (gaps above 8) and its value token.  The warp's first
    // value stages its own token only: the run before it reaches into
    // earlier warps and is coded at the copy-out.
    // (without branches around the loads: lanes past the candidates
    // quantize whatever their slot of the warp's region holds -- every
    // quantizer reads only its bounded tables -- and are not values)
    int nStaged = 0;                  // warp-uniform
    int firstPos = -1, lastPos = -1;  // warp-uniform: the warp's values so far
    for (int r = 0; 32 * r < nCand; r++) {
      const int l = 32 * r + lane;  // < 512: inside the warp's region
      const int bin = quant_value(sX[base + l], q, tab, sLut);
      const int pos = sPos[base + l];
      const bool v = l < nCand && bin != dupV;
      const unsigned m = __ballot_sync(kAll, v);
      if (m == 0) continue;
      const unsigned lower = m & ltMask;
      const int pp = __shfl_sync(kAll, pos, lower ? 31 - __clz(lower) : 0);
      const int prev = lower ? pp : lastPos;
      const int gap = v && prev >= 0 ? pos - prev - 1 : 0;
      int sg, dp;
      run_split_closed(gap, sg, dp);  // 0, 0 for gap 0
      singles += sg;
      dups += dp;
      const int cnt = v ? 1 + sg + dp : 0;
      int inc = cnt;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(kAll, inc, d);
        if (lane >= d) inc += t;
      }
      if (v) {
        int t = nStaged + inc - cnt;
        // dup tokens in the order of run_tokens_short: runs of 1024, then
        // one per set bit of the remainder from 512 down to 16, then 8 when
        // more than 8 remain; the rest are single (prefilled) tokens
        for (int j = gap >> 10; j > 0; j--) stage[t++] = make_token(B, 7);
        const int rr = gap & 1023;
#pragma unroll
        for (int lg = 9; lg >= 4; lg--)
          if ((rr >> lg) & 1) stage[t++] = make_token(B, lg - 3);
        const bool eight = (rr & 8) && (rr & 7);
        if (eight) stage[t++] = make_token(B, 0);
        t += (rr & 8) && !eight ? 8 : (rr & 7);
        stage[t] = make_token(bin, 0);
        atomicAdd(&hist[bin], 1u);
      }
      if (firstPos < 0) firstPos = __shfl_sync(kAll, pos, __ffs(m) - 1);
      lastPos = __shfl_sync(kAll, pos, 31 - __clz(m));
      nStaged += __shfl_sync(kAll, inc, 31);
    }
    if (lane == 0) {
      wFirst[par][w] = firstPos;
      wLast[par][w] = lastPos;
      wTok[par][w] = nStaged;
    }
    __syncthreads();

    // ---- the chunk's layout from the warp summaries (lane u of every warp
    // reads warp u's; lanes >= kWarps hold an empty warp)
    int F = -1, Lu = -1, I = 0;
    if (lane < kWarps) {
      F = wFirst[par][lane];
      Lu = wLast[par][lane];
      I = wTok[par][lane];
    }
    // the value before warp u's first: positions grow with the warp index
    int pv = Lu;
#pragma unroll
    for (int d = 1; d < kWarps; d <<= 1) {
      const int t = __shfl_up_sync(kAll, pv, d);
      if (lane >= d) pv = max(pv, t);
    }
    int prevU = __shfl_up_sync(kAll, pv, 1);
    if (lane == 0) prevU = -1;
    // warp u's first run lies inside the chunk when a value precedes it
    const int g0 = F >= 0 && prevU >= 0 ? F - prevU - 1 : 0;
    int sg0, dp0;
    run_split_closed(g0, sg0, dp0);
    if (w == 0) {  // counted once per chunk
      singles += sg0;
      dups += dp0;
    }
    const int tok = sg0 + dp0 + I;
    int incT = tok;
#pragma unroll
    for (int d = 1; d < kWarps; d <<= 1) {
      const int t = __shfl_up_sync(kAll, incT, d);
      if (lane >= d) incT += t;
    }
    const int nTok = __shfl_sync(kAll, incT, kWarps - 1);
    int lead = F >= 0 ? F : len, last = Lu;
#pragma unroll
    for (int d = kWarps / 2; d > 0; d >>= 1) {
      lead = min(lead, __shfl_xor_sync(kAll, lead, d));
      last = max(last, __shfl_xor_sync(kAll, last, d));
    }
    lead = __shfl_sync(kAll, lead, 0);
    last = __shfl_sync(kAll, last, 0);

    // ---- copy-out: warp w's tokens (its first run, then the staged ones)
    // to their place in the chunk's slot, which holds the chunk's tokens from
    // the first value's position on (the lead zero run's tokens, written
    // later by runs_kernel, fit before it, since each token starts at its
    // own element)
    {
      const int o = __shfl_sync(kAll, incT - tok, w);
      const int fr = __shfl_sync(kAll, sg0 + dp0, w);
      const int gw = __shfl_sync(kAll, g0, w);
      const int nw = fr + __shfl_sync(kAll, I, w);
      uint16_t *g = b.tok + cd.coefOff + start + lead + o;
      // the first run's few tokens, then the staged ones (a plain copy)
      for (int j = lane; j < fr; j += 32) g[j] = run_token_at(gw, j, B, dupV);
      for (int j = fr + lane; j < nw; j += 32) g[j] = stage[j - fr];
    }
    __syncwarp();  // the staged tokens are read before the next prefill
    if (threadIdx.x == 0) {
      b.chunkTok[chunk] = nTok;
      b.chunkSpan[chunk] = make_int2(lead, nTok);  // runs_kernel adds the edge runs
      if (dupV >= 0) {
        const bool any = last >= 0;
        b.chunkRun[chunk] = make_int4(lead, any ? len - 1 - last : len, any ? 0 : 1, len);
      }
    }
    // one barrier per chunk: the next chunk writes the other summary set,
    // and a warp reaches this chunk's set again only after every warp has
    // passed the next chunk's barrier, i.e. has finished this chunk
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    singles += __shfl_xor_sync(kAll, singles, d);
    dups += __shfl_xor_sync(kAll, dups, d);
  }
  if (lane == 0 && dupV >= 0) {
    if (singles) atomicAdd(&hist[dupV], (unsigned)singles);
    if (dups) atomicAdd(&hist[B], (unsigned)dups);
  }
  __syncthreads();
  unsigned long long *gh = b.hist + (size_t)ci * kMaxSymbols;
  for (int i = threadIdx.x; i <= B; i += kThreads)
    if (hist[i]) atomicAdd(&gh[i], (unsigned long long)hist[i]);
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
      // Tokens of the zero runs at the chunk's edges that start inside it,
      // in stream order around the stored tokens [lead, lead + nInt): the
      // entering run's right before them, the leaving run's right after.
      const long long cstart = (long long)c * kChunk;
      uint16_t *slot = b.tok + cd.coefOff + cstart;
      const int nInt = b.chunkTok[base + c];
      const int dupKey = cd.binCount;
      int nPre = 0, nPost = 0;
      if (me.x > 0) {
        const long long runIn = ctx[2 * c];
        const long long re = me.z ? e : cstart + me.x;
        const long long w1 = cstart + (me.z ? me.w : me.x);
        run_tokens(runIn, re, cstart, w1, dupKey, dupV, [&](uint16_t) { nPre++; });
        int i = me.x - nPre;
        run_tokens(runIn, re, cstart, w1, dupKey, dupV, [&](uint16_t t) { slot[i++] = t; });
      }
      if (!me.z && me.y > 0) {
        const long long s0 = cstart + me.w - me.y;
        int i = me.x + nInt;
        run_tokens(s0, e, s0, cstart + me.w, dupKey, dupV, [&](uint16_t t) { slot[i++] = t; });
        nPost = i - (me.x + nInt);
      }
      b.chunkSpan[base + c] = make_int2(me.x - nPre, nPre + nInt + nPost);
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

void launch_lloyd(DevBatch &b, const float *coef, int maxBins, cudaStream_t s) {
  lloyd_cand_kernel<<<dim3(kCandSlices, b.n), kThreads, 0, s>>>(
      b, reinterpret_cast<const unsigned *>(b.coef2));
  lloyd_deferred_kernel<<<dim3(kCandSlices, b.n), kThreads, 0, s>>>(b, coef);
  const int cbCap = ((maxBins / 2 + 1) + 3) & ~3;
  const int smem = (int)lloyd_smem_bytes(cbCap);
  raise_smem_limit(lloyd_solve_kernel, smem);
  lloyd_solve_kernel<<<b.n, kSolveThreads, smem, s>>>(b, cbCap);
}

void launch_quantize(DevBatch &b, const float *coef, int maxTable, int maxSymbols,
                     cudaStream_t s) {
  const int histOff = (maxTable + 3) & ~3;
  const int smem = (histOff + maxSymbols + 1) * (int)sizeof(float);
  raise_smem_limit(quantize_kernel, smem);
  quantize_kernel<<<(unsigned)b.totalGroups, kThreads, smem, s>>>(b, coef, histOff);
}

void launch_runs(DevBatch &b, cudaStream_t s) { runs_kernel<<<b.n, 1024, 0, s>>>(b); }

}  // namespace wl
