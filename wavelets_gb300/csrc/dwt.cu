// Separable multi-level wavelet transform passes (forward and inverse) for
// sm_103a.
//
// One launch runs one axis pass for every cubelet of a batch.  A CTA stages a
// tile of T rows (each a full row of length L) in shared memory, runs all the
// levels of that axis on the rows in place, and writes the tile back in the
// layout the next pass reads -- the axis rotation between passes is fused
// into the store (reference: cdf97_3d dwt_cpu.cc:943-992 runs x levels,
// transpose3dFwd, y levels, transpose3dFwd, z levels; haar_3d :624-648).
//
// Levels are computed in place on a strided view of the row: level k works on
// the elements at multiples of 2^k, its low outputs land on even and its high
// outputs on odd multiples.  The final store maps every element to the
// reference's band order (low band first, then the detail bands of the last
// level down to the first, dwt_cpu.cc:703-728).
//
// CDF 9/7 runs as four lifting steps (alpha, beta, gamma, delta) with the
// scaling K folded into the store: low band * K^S, detail band of level t *
// -K^(t-1).  This reproduces the reference's sqrt(2)-normalised 9/7 filter
// bank (dwt_cpu.cc:15-43) up to float rounding; whole-sample mirroring at the
// row ends (MirroredArray dwt_cpu.h:153-184) becomes s[n/2] = s[n/2-1] and
// d[-1] = d[0] in the lifting steps.  `exact` passes instead evaluate the
// reference's filter-bank sums in its operation order with unfused float
// operations, giving bit-identical coefficients.  Haar is always the
// reference's own butterfly (a +- b) * (1/sqrt 2) (dwt_cpu.cc:159-162).
#include <cuda_runtime.h>

#include "dwt_common.cuh"
#include "wl_internal.h"

namespace wl {
namespace {
using namespace dwtc;

// reference taps (dwt_cpu.cc:15-43), double literals rounded to float
constexpr float kL0 = (float).85269867900940, kL1 = (float).377402855612650,
                kL2 = (float)-.110624404418420, kL3 = (float)-.02384946501938,
                kL4 = (float).037828455506995;
constexpr float kH0 = (float)-.788485616405660, kH1 = (float).418092273222210,
                kH2 = (float).040689417609558, kH3 = (float)-.064538882628938;
constexpr float kSL0 = (float).788485616405660, kSL1 = (float).377402855612650,
                kSL2 = (float)-.040689417609558, kSL3 = (float)-.02384946501938;
constexpr float kSH0 = (float)-.85269867900940, kSH1 = (float).418092273222210,
                kSH2 = (float).110624404418420, kSH3 = (float)-.064538882628938,
                kSH4 = (float)-.037828455506995;

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

// Shared-memory position of row element p: one pad word after every 32, so
// the power-of-two strides of the in-place levels hit distinct banks.
__host__ __device__ __forceinline__ int sw(int p) { return p + (p >> 5); }
// odd row pitch, so a warp reading one element of 32 rows is conflict-free
__host__ __device__ __forceinline__ int row_pitch(int L) { return sw(L) | 1; }

// whole-sample mirror with repeated folding (dwt_cpu.h:162-176)
__device__ __forceinline__ int mirror(int i, int n) {
  if (i < 0) i = -i;
  while (i >= n) {
    i = n * 2 - i - 2;
    if (i < 0) i = -i;
  }
  return i;
}

// band index q (reference order) -> in-place position p and level
// (level == S for the final low band)
__device__ __forceinline__ int band_to_pos(int q, int L, int S, int &lev) {
  if (q < (L >> S)) { lev = S; return q << S; }
  int t = S - 1;
  while (q >= (L >> t)) t--;
  lev = t;
  return ((q - (L >> (t + 1))) << (t + 1)) + (1 << t);
}

// ---- one level of one row --------------------------------------------------
// A level runs on the strided view row[sw(j*st)], j < n = 2*half.  The lanes of a
// warp are split into groups of G lanes (G = 32, or the power of two >= half
// when half < 32) so several short rows share a warp; `sub` is the lane's
// index in its group and `ok` whether the group has a row.  Every lane of
// the warp executes the same __syncwarp calls.

__device__ __forceinline__ void fwd_lifting_level(float *row, int half, int st, int sub,
                                                  int G, bool ok) {
  if (ok)
    for (int i = sub; i < half; i += G) {  // d += alpha (s_i + s_i+1)
      const float a = row[sw((2 * i) * st)], b = row[sw((2 * min(i + 1, half - 1)) * st)];
      row[sw((2 * i + 1) * st)] += kAlpha * (a + b);
    }
  __syncwarp();
  if (ok)
    for (int i = sub; i < half; i += G) {  // s += beta (d_i-1 + d_i)
      const float a = row[sw((2 * max(i - 1, 0) + 1) * st)], b = row[sw((2 * i + 1) * st)];
      row[sw((2 * i) * st)] += kBeta * (a + b);
    }
  __syncwarp();
  if (ok)
    for (int i = sub; i < half; i += G) {
      const float a = row[sw((2 * i) * st)], b = row[sw((2 * min(i + 1, half - 1)) * st)];
      row[sw((2 * i + 1) * st)] += kGamma * (a + b);
    }
  __syncwarp();
  if (ok)
    for (int i = sub; i < half; i += G) {
      const float a = row[sw((2 * max(i - 1, 0) + 1) * st)], b = row[sw((2 * i + 1) * st)];
      row[sw((2 * i) * st)] += kDelta * (a + b);
    }
  __syncwarp();
}

__device__ __forceinline__ void inv_lifting_level(float *row, int half, int st, int sub,
                                                  int G, bool ok) {
  if (ok)
    for (int i = sub; i < half; i += G) {
      const float a = row[sw((2 * max(i - 1, 0) + 1) * st)], b = row[sw((2 * i + 1) * st)];
      row[sw((2 * i) * st)] -= kDelta * (a + b);
    }
  __syncwarp();
  if (ok)
    for (int i = sub; i < half; i += G) {
      const float a = row[sw((2 * i) * st)], b = row[sw((2 * min(i + 1, half - 1)) * st)];
      row[sw((2 * i + 1) * st)] -= kGamma * (a + b);
    }
  __syncwarp();
  if (ok)
    for (int i = sub; i < half; i += G) {
      const float a = row[sw((2 * max(i - 1, 0) + 1) * st)], b = row[sw((2 * i + 1) * st)];
      row[sw((2 * i) * st)] -= kBeta * (a + b);
    }
  __syncwarp();
  if (ok)
    for (int i = sub; i < half; i += G) {
      const float a = row[sw((2 * i) * st)], b = row[sw((2 * min(i + 1, half - 1)) * st)];
      row[sw((2 * i + 1) * st)] -= kAlpha * (a + b);
    }
  __syncwarp();
}

// Haar butterflies (dwt_cpu.cc:159-162 forward, :193-196 inverse)
__device__ __forceinline__ void haar_level(float *row, int half, int st, int sub, int G,
                                           bool ok, bool inverse) {
  if (ok)
    for (int i = sub; i < half; i += G) {
      const float a = row[sw((2 * i) * st)], b = row[sw((2 * i + 1) * st)];
      if (!inverse) {
        row[sw((2 * i + 1) * st)] = __fmul_rn(__fsub_rn(a, b), kInvSqrt2);
        row[sw((2 * i) * st)] = __fmul_rn(__fadd_rn(a, b), kInvSqrt2);
      } else {
        row[sw((2 * i) * st)] = __fmul_rn(kInvSqrt2, __fadd_rn(a, b));
        row[sw((2 * i + 1) * st)] = __fmul_rn(kInvSqrt2, __fsub_rn(a, b));
      }
    }
  __syncwarp();
}

// reference filter bank in the reference operation order: analysis
// dwt_cpu.cc:699-725, synthesis :776-795
__device__ __forceinline__ void exact_level(float *row, float *tmp, int half, int st, int sub,
                                            int G, bool ok, bool inverse) {
  const int n = 2 * half;
  if (ok)
    for (int j = sub; j < n; j += G) tmp[j] = row[sw(j * st)];
  __syncwarp();
  if (ok)
    for (int i = sub; i < half; i += G) {
      const int j = 2 * i, k = j + 1;
      float s, d;
      if (!inverse) {
        s = __fmul_rn(kL0, tmp[j]);
        s = __fadd_rn(s, __fmul_rn(kL1, __fadd_rn(tmp[mirror(j + 1, n)], tmp[mirror(j - 1, n)])));
        s = __fadd_rn(s, __fmul_rn(kL2, __fadd_rn(tmp[mirror(j + 2, n)], tmp[mirror(j - 2, n)])));
        s = __fadd_rn(s, __fmul_rn(kL3, __fadd_rn(tmp[mirror(j + 3, n)], tmp[mirror(j - 3, n)])));
        s = __fadd_rn(s, __fmul_rn(kL4, __fadd_rn(tmp[mirror(j + 4, n)], tmp[mirror(j - 4, n)])));
        d = __fmul_rn(kH0, tmp[k]);
        d = __fadd_rn(d, __fmul_rn(kH1, __fadd_rn(tmp[mirror(k + 1, n)], tmp[mirror(k - 1, n)])));
        d = __fadd_rn(d, __fmul_rn(kH2, __fadd_rn(tmp[mirror(k + 2, n)], tmp[mirror(k - 2, n)])));
        d = __fadd_rn(d, __fmul_rn(kH3, __fadd_rn(tmp[mirror(k + 3, n)], tmp[mirror(k - 3, n)])));
      } else {
        s = __fmul_rn(tmp[j], kSL0);
        s = __fadd_rn(s, __fmul_rn(__fadd_rn(tmp[mirror(j + 1, n)], tmp[mirror(j - 1, n)]), kSL1));
        s = __fadd_rn(s, __fmul_rn(__fadd_rn(tmp[mirror(j + 2, n)], tmp[mirror(j - 2, n)]), kSL2));
        s = __fadd_rn(s, __fmul_rn(__fadd_rn(tmp[mirror(j + 3, n)], tmp[mirror(j - 3, n)]), kSL3));
        d = __fmul_rn(tmp[k], kSH0);
        d = __fadd_rn(d, __fmul_rn(__fadd_rn(tmp[mirror(k + 1, n)], tmp[mirror(k - 1, n)]), kSH1));
        d = __fadd_rn(d, __fmul_rn(__fadd_rn(tmp[mirror(k + 2, n)], tmp[mirror(k - 2, n)]), kSH2));
        d = __fadd_rn(d, __fmul_rn(__fadd_rn(tmp[mirror(k + 3, n)], tmp[mirror(k - 3, n)]), kSH3));
        d = __fadd_rn(d, __fmul_rn(__fadd_rn(tmp[mirror(k + 4, n)], tmp[mirror(k - 4, n)]), kSH4));
      }
      row[sw(j * st)] = s;
      row[sw(k * st)] = d;
    }
  __syncwarp();
}

// lane group for rows of `len` elements handled `len`-wide
__device__ __forceinline__ int group_width(int len) {
  if (len >= 32) return 32;
  int G = 1;
  while (G < len) G <<= 1;
  return G;
}

template <typename InT, typename OutT, bool INV>
__global__ void __launch_bounds__(kThreads)
dwt_pass_kernel(const PassDesc *__restrict__ passes, const int *__restrict__ tilePrefix,
                int nPasses) {
  extern __shared__ float4 smem4[];
  float *sm = reinterpret_cast<float *>(smem4);
  __shared__ long long rowIn[256], rowOut[256];
  __shared__ float scaleTab[32];

  const int bid = blockIdx.x;
  int lo = 0, hi = nPasses - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (tilePrefix[mid] <= bid) lo = mid; else hi = mid - 1;
  }
  const PassDesc &d = passes[lo];
  const int L = d.L, S = d.steps, T = d.T, pitch = row_pitch(L);
  const int r0 = (bid - tilePrefix[lo]) * T;
  const int nr = min(T, d.rows - r0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool lifting = (d.wavelet == WL_CDF97) && !d.exact;
  float *tile = sm;
  float *tmpb = sm + T * pitch;

  for (int rr = threadIdx.x; rr < nr; rr += kThreads) {
    const int r = r0 + rr, a = r / d.B, b = r - a * d.B;
    if (!INV) {
      const int as = min(a, d.clampA - 1), bs = min(b, d.clampB - 1);
      rowIn[rr] = as * d.inSA + bs * d.inSB;
    } else {
      rowIn[rr] = a * d.inSA + b * d.inSB;
    }
    rowOut[rr] = (a < d.cropA && b < d.cropB) ? a * d.outSA + b * d.outSB : -1;
  }
  if (threadIdx.x <= S && threadIdx.x < 32)
    scaleTab[threadIdx.x] = lifting ? lifting_scale(threadIdx.x, S) : 1.0f;
  __syncthreads();

  // ---- load --------------------------------------------------------------
  const InT *in = static_cast<const InT *>(d.in);
  {
    const int G = group_width(L), rpi = 32 / G, sub = lane & (G - 1), rsub = lane / G;
    for (int rb = warp * rpi; rb < nr; rb += kWarps * rpi) {
      const int rr = rb + rsub;
      if (rr >= nr) continue;
      const InT *src = in + rowIn[rr];
      float *trow = tile + rr * pitch;
      if (!INV) {
        const int cl = d.clampL - 1;
        for (int c = sub; c < L; c += G) trow[sw(c)] = load_as_float(src + min(c, cl));
      } else {
        for (int q = sub; q < L; q += G) {
          int lev;
          const int p = band_to_pos(q, L, S, lev);
          const float v = load_as_float(src + q);
          trow[sw(p)] = lifting ? v / scaleTab[lev] : v;
        }
      }
    }
  }
  __syncthreads();

  // ---- levels ------------------------------------------------------------
  for (int it = 0; it < S; it++) {
    const int lev = INV ? S - 1 - it : it;
    const int half = (L >> lev) >> 1, st = 1 << lev;
    const int G = group_width(half), rpi = 32 / G, sub = lane & (G - 1), rsub = lane / G;
    for (int rb = warp * rpi; rb < nr; rb += kWarps * rpi) {
      const int rr = rb + rsub;
      const bool ok = rr < nr;
      float *trow = tile + (ok ? rr : 0) * pitch;
      float *tmp = tmpb + (ok ? rr : 0) * L;
      if (d.wavelet == WL_HAAR) haar_level(trow, half, st, sub, G, ok, INV);
      else if (d.exact) exact_level(trow, tmp, half, st, sub, G, ok, INV);
      else if (!INV) fwd_lifting_level(trow, half, st, sub, G, ok);
      else inv_lifting_level(trow, half, st, sub, G, ok);
    }
    __syncthreads();
  }

  // ---- store -------------------------------------------------------------
  OutT *out = static_cast<OutT *>(d.out);
  const int cropL = d.cropL;
  if (d.outSB == 1 && d.outSC != 1) {
    // consecutive rows are consecutive in memory: lanes walk the rows
    const int logT = __ffs(T) - 1;
    for (int idx = threadIdx.x; idx < (L << logT); idx += kThreads) {
      const int rr = idx & (T - 1), q = idx >> logT;
      if (rr >= nr || q >= cropL) continue;
      const long long base = rowOut[rr];
      if (base < 0) continue;
      float v;
      if (!INV) {
        int lev;
        const int p = band_to_pos(q, L, S, lev);
        v = tile[rr * pitch + sw(p)] * scaleTab[lev];
      } else {
        v = tile[rr * pitch + sw(q)];
      }
      store_from_float(out + base + (long long)q * d.outSC, v);
    }
  } else {
    const int Lc = min(L, cropL);
    const int G = group_width(Lc), rpi = 32 / G, sub = lane & (G - 1), rsub = lane / G;
    for (int rb = warp * rpi; rb < nr; rb += kWarps * rpi) {
      const int rr = rb + rsub;
      if (rr >= nr) continue;
      const long long base = rowOut[rr];
      if (base < 0) continue;
      for (int q = sub; q < Lc; q += G) {
        float v;
        if (!INV) {
          int lev;
          const int p = band_to_pos(q, L, S, lev);
          v = tile[rr * pitch + sw(p)] * scaleTab[lev];
        } else {
          v = tile[rr * pitch + sw(q)];
        }
        store_from_float(out + base + (long long)q * d.outSC, v);
      }
    }
  }
}

template <typename InT, typename OutT, bool INV>
void launch_t(const PassDesc *p, const int *tp, int n, int tiles, int smem, cudaStream_t s) {
  auto k = dwt_pass_kernel<InT, OutT, INV>;
  if (smem > 32 * 1024) raise_smem_limit(k, smem);  // static + dynamic may pass 48 KB
  k<<<tiles, kThreads, smem, s>>>(p, tp, n);
}

}  // namespace

int dwt_tile_rows(int L, bool exact) {
  const int per_row = row_pitch(L) + (exact ? L : 0);
  int T = 1;
  while (T * 2 * per_row <= kTileBudget && T < 256) T *= 2;
  return T;
}

int dwt_smem_bytes(int L, int T, bool exact) {
  return (T * row_pitch(L) + (exact ? T * L : 0)) * (int)sizeof(float);
}

// inType/outType: wl_dtype codes (F32 for intermediate passes)
void launch_dwt_pass(const PassDesc *p, const int *tp, int n, int tiles, int smem,
                     int inType, int outType, bool inverse, cudaStream_t s) {
  if (!inverse) {
    switch (inType) {
      case WL_U8: launch_t<uint8_t, float, false>(p, tp, n, tiles, smem, s); break;
      case WL_U16: launch_t<uint16_t, float, false>(p, tp, n, tiles, smem, s); break;
      case WL_I32: launch_t<int32_t, float, false>(p, tp, n, tiles, smem, s); break;
      default: launch_t<float, float, false>(p, tp, n, tiles, smem, s); break;
    }
  } else {
    switch (outType) {
      case WL_U8: launch_t<float, uint8_t, true>(p, tp, n, tiles, smem, s); break;
      case WL_U16: launch_t<float, uint16_t, true>(p, tp, n, tiles, smem, s); break;
      case WL_I32: launch_t<float, int32_t, true>(p, tp, n, tiles, smem, s); break;
      default: launch_t<float, float, true>(p, tp, n, tiles, smem, s); break;
    }
  }
}

}  // namespace wl

namespace wl {
namespace {
__global__ void dequant_kernel(const int *__restrict__ bins, const float *__restrict__ table,
                               float *__restrict__ out, long long n, int nTable) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = table[min(max(bins[i], 0), nTable - 1)];
}
}  // namespace

// bins -> dequantized values through a per-bin table (dequantize,
// test_compress_common.cc:567-584; the table holds the reference's values)
namespace {
// dequantize many cubelets in one launch: blocks of 2048 elements, a block's
// cubelet found by binary search over the items' first blocks
}  // namespace

void launch_dequant(const int *bins, const float *table, float *out, long long n, int nTable,
                    cudaStream_t s) {
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  if (blocks < 1) blocks = 1;
  dequant_kernel<<<(unsigned)blocks, 256, 0, s>>>(bins, table, out, n, nTable);
}
}  // namespace wl
