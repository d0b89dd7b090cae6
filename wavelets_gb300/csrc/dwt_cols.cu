// Column-tile wavelet passes: a CTA of four or eight warps per tile of 32, 64
// or 128 rows; every lane owns one row of the tile.
//
// The row-cooperative kernel (dwt.cu) spreads a row over the lanes of a warp
// and pays index arithmetic and a warp barrier for every lifting step of
// every level.  Here a lane walks its row sequentially: a level is a
// streaming sweep that keeps a two-pair window in registers and applies all
// four lifting steps (or the Haar butterfly) on the way, so an element costs
// one shared load, one shared store and four float operations per level.
// The warps that share 32 rows split every level into segments of pairs
// (warps x 32 / rows segments: with four warps, four for a 32-row tile, two
// for a 64-row tile, none for a 128-row tile, where each warp sweeps its 32
// rows whole with no halos and no barriers between levels; eight warps
// double each).  More segments give the SM more warps per byte of shared
// memory; fewer spend less on halos and barriers.  The tile shape of each
// row-length class is chosen by measurement (the tile autotuner in the
// engine); the default is 128 rows for rows of at most 64 elements and 32
// rows above, four warps.
//
// Tile layout in shared memory: element p of tile row r at tile[p * (R+1) + r]
// for an R-row tile.  Lanes reading one position of 32 neighbouring rows hit
// 32 banks; a warp walking the positions of one row (odd stride) also hits
// 32 banks.  Each side
// of a pass picks its access pattern from the strides of the global layout:
//   - rows consecutive in memory (element stride != 1): every lane moves its
//     own row, so a warp access covers one element of 32 neighbouring rows
//     (coalesced);
//   - rows contiguous (element stride 1): a warp moves one row at a time,
//     lanes over the elements.
// Float sources are staged with cp.async (4-byte copies that need no
// registers), which keeps many loads in flight.
//
// Levels are in place on the strided view p = j * 2^k as in dwt.cu; the band
// order of the reference (low band, then detail bands of the last level down
// to the first, dwt_cpu.cc:703-728) is applied when the tile is stored
// (forward) or loaded (inverse), with the deferred lifting scale.  Every
// lifting step does the same arithmetic as in the row-cooperative kernel;
// only the order in which independent elements are visited differs.
#include <cuda_runtime.h>

#include <type_traits>

#include "dwt_common.cuh"
#include "wl_internal.h"

namespace wl {
namespace {
using namespace dwtc;

constexpr int kRows = 32;         // rows per warp (one per lane)
constexpr int kMinSegPairs = 8;   // pairs per segment below which a level is not split

__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// stage one source element into shared memory as float
template <typename T> __device__ __forceinline__ void stage(float *dst, const T *src) {
  *dst = load_as_float(src);
}
template <> __device__ __forceinline__ void stage<float>(float *dst, const float *src) {
  cp_async4(dst, src);
}

// ---- one level of one column segment -----------------------------------------
// x points at position 0 of the lane's row; consecutive elements of the level
// are P = 2^k * 33 words apart.  Pair j is (e_j, o_j) = elements (2j, 2j+1),
// j < h.  A segment [i0, i1) of pairs is written by one warp.  Its outputs
// depend on input pairs i0-2 .. i1+1: the sweep starts two pairs early
// (js = max(i0-2, 0)) -- an early start is exact from pair js+2 on -- and
// reads two pairs past the segment.  Those halo pairs belong to neighbouring
// segments, which overwrite them during the level, so they are captured into
// registers (hl: pairs js.., hr: pairs i1..) before the CTA barrier that
// starts the level.

struct Halo {
  float l[4], r[4];
};

__device__ __forceinline__ void capture_halo(const float *x, int h, int P, int i0, int i1,
                                             Halo &hb) {
  const int js = max(i0 - 2, 0);
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int jl = js + k, jr = i1 + k;
    hb.l[2 * k] = jl < i0 ? x[2 * jl * P] : 0.f;
    hb.l[2 * k + 1] = jl < i0 ? x[(2 * jl + 1) * P] : 0.f;
    hb.r[2 * k] = jr < h ? x[2 * jr * P] : 0.f;
    hb.r[2 * k + 1] = jr < h ? x[(2 * jr + 1) * P] : 0.f;
  }
}

// pair j of the sweep: halo registers outside [i0, i1), shared memory inside
__device__ __forceinline__ void pair_at(const float *x, int P, int j, int js, int i0, int i1,
                                        const Halo &hb, float &e, float &o) {
  if (j < i0) {
    const bool k = j != js;
    e = k ? hb.l[2] : hb.l[0];
    o = k ? hb.l[3] : hb.l[1];
  } else if (j < i1) {
    e = x[2 * j * P];
    o = x[(2 * j + 1) * P];
  } else {
    const bool k = j != i1;
    e = k ? hb.r[2] : hb.r[0];
    o = k ? hb.r[3] : hb.r[1];
  }
}

// Forward CDF 9/7 lifting (dwt.cu fwd_lifting_level, same operations):
//   d1_j = o_j + a (e_j + e_j+1)     e_h   = e_h-1
//   s1_j = e_j + b (d1_j-1 + d1_j)   d1_-1 = d1_0
//   d2_j = d1_j + g (s1_j + s1_j+1)  s1_h  = s1_h-1
//   s2_j = s1_j + d (d2_j-1 + d2_j)  d2_-1 = d2_0
// Iteration j reads pair j+2 and finishes pair j.
__device__ __forceinline__ void lift_fwd_seg(float *x, int h, int P, int i0, int i1,
                                             const Halo &hb) {
  const int js = max(i0 - 2, 0);
  float e0, o0, e1, o1;
  pair_at(x, P, js, js, i0, i1, hb, e0, o0);
  if (js + 1 < h) pair_at(x, P, js + 1, js, i0, i1, hb, e1, o1);
  else { e1 = e0; o1 = o0; }
  float d1 = fmaf(kAlpha, e0 + e1, o0);
  float s1 = fmaf(kBeta, d1 + d1, e0);
  float d2p = 0.f;
  // any iteration, all end rules applied
  auto generic = [&](int j) {
    float d1n = d1, s1n = s1, e2 = e1, o2 = o1;
    if (j + 1 < h) {
      if (j + 2 < h) pair_at(x, P, j + 2, js, i0, i1, hb, e2, o2);
      d1n = fmaf(kAlpha, e1 + e2, o1);
      s1n = fmaf(kBeta, d1 + d1n, e1);
    }
    const float d2 = fmaf(kGamma, s1 + s1n, d1);
    const float s2 = fmaf(kDelta, (j == 0 ? d2 : d2p) + d2, s1);
    if (j >= i0) {
      x[2 * j * P] = s2;
      x[(2 * j + 1) * P] = d2;
    }
    d2p = d2; d1 = d1n; s1 = s1n; e1 = e2; o1 = o2;
  };
  const int jm = max(i0, 1);
  for (int j = js; j < min(jm, i1); j++) generic(j);
  // 1 <= j, j+2 < i1: pair j+2 is in the segment
  const float *pr = x + 2 * (jm + 2) * P;
  float *pw = x + 2 * jm * P;
  const int jt = max(jm, i1 - 2);
#pragma unroll 4
  for (int j = jm; j < jt; j++) {
    const float e2 = pr[0], o2 = pr[P];
    pr += 2 * P;
    const float d1n = fmaf(kAlpha, e1 + e2, o1);
    const float s1n = fmaf(kBeta, d1 + d1n, e1);
    const float d2 = fmaf(kGamma, s1 + s1n, d1);
    pw[0] = fmaf(kDelta, d2p + d2, s1);
    pw[P] = d2;
    pw += 2 * P;
    d2p = d2; d1 = d1n; s1 = s1n; e1 = e2; o1 = o2;
  }
  for (int j = max(jt, min(jm, i1)); j < i1; j++) generic(j);
}

// Inverse CDF 9/7 lifting (dwt.cu inv_lifting_level, same operations):
//   s1_j = s2_j - d (d2_j-1 + d2_j)
//   d1_j = d2_j - g (s1_j + s1_j+1)
//   e_j  = s1_j - b (d1_j-1 + d1_j)
//   o_j  = d1_j - a (e_j + e_j+1)
// with the same mirrored ends.  Iteration j reads pair j+2 and finishes
// pair j.  Requires h >= 2.
__device__ __forceinline__ void lift_inv_seg(float *x, int h, int P, int i0, int i1,
                                             const Halo &hb) {
  const int js = max(i0 - 2, 0);
  float s2a, d2a, s2b, d2b;
  pair_at(x, P, js, js, i0, i1, hb, s2a, d2a);
  pair_at(x, P, js + 1, js, i0, i1, hb, s2b, d2b);
  const float s1a = fmaf(-kDelta, d2a + d2a, s2a);
  float s1c = fmaf(-kDelta, d2a + d2b, s2b);   // s1_j+1
  float d1c = fmaf(-kGamma, s1a + s1c, d2a);   // d1_j
  float ec = fmaf(-kBeta, d1c + d1c, s1a);     // e_j
  float d2c = d2b;                             // d2_j+1
  auto generic = [&](int j) {
    float s1n = s1c, d2n = d2c, d1n = d1c, en = ec;
    if (j + 2 < h) {
      float s2n;
      pair_at(x, P, j + 2, js, i0, i1, hb, s2n, d2n);
      s1n = fmaf(-kDelta, d2c + d2n, s2n);
      d1n = fmaf(-kGamma, s1c + s1n, d2c);
      en = fmaf(-kBeta, d1c + d1n, s1c);
    } else if (j + 1 < h) {
      d1n = fmaf(-kGamma, s1c + s1c, d2c);
      en = fmaf(-kBeta, d1c + d1n, s1c);
    }
    const float o = fmaf(-kAlpha, ec + en, d1c);
    if (j >= i0) {
      x[2 * j * P] = ec;
      x[(2 * j + 1) * P] = o;
    }
    s1c = s1n; d2c = d2n; d1c = d1n; ec = en;
  };
  for (int j = js; j < i0; j++) generic(j);
  // j+2 < i1: pair j+2 is in the segment
  const float *pr = x + 2 * (i0 + 2) * P;
  float *pw = x + 2 * i0 * P;
  const int jt = max(i0, i1 - 2);
#pragma unroll 4
  for (int j = i0; j < jt; j++) {
    const float s2n = pr[0], d2n = pr[P];
    pr += 2 * P;
    const float s1n = fmaf(-kDelta, d2c + d2n, s2n);
    const float d1n = fmaf(-kGamma, s1c + s1n, d2c);
    const float en = fmaf(-kBeta, d1c + d1n, s1c);
    pw[0] = ec;
    pw[P] = fmaf(-kAlpha, ec + en, d1c);
    pw += 2 * P;
    s1c = s1n; d2c = d2n; d1c = d1n; ec = en;
  }
  for (int j = jt; j < i1; j++) generic(j);
}

// one pair level (h == 1) of the inverse
__device__ __forceinline__ void lift_inv_one(float *x, int P) {
  const float s20 = x[0], d20 = x[P];
  const float s1 = fmaf(-kDelta, d20 + d20, s20);
  const float d1 = fmaf(-kGamma, s1 + s1, d20);
  const float e = fmaf(-kBeta, d1 + d1, s1);
  x[0] = e;
  x[P] = fmaf(-kAlpha, e + e, d1);
}

// Haar butterflies (dwt_cpu.cc:159-162 forward, :193-196 inverse)
__device__ __forceinline__ void haar_seg(float *x, int P, int i0, int i1, bool inverse) {
#pragma unroll 4
  for (int i = i0; i < i1; i++) {
    float *pe = x + 2 * i * P;
    const float a = pe[0], b = pe[P];
    if (!inverse) {
      pe[P] = __fmul_rn(__fsub_rn(a, b), kInvSqrt2);
      pe[0] = __fmul_rn(__fadd_rn(a, b), kInvSqrt2);
    } else {
      pe[0] = __fmul_rn(kInvSqrt2, __fadd_rn(a, b));
      pe[P] = __fmul_rn(kInvSqrt2, __fsub_rn(a, b));
    }
  }
}

// 8- and 16-bit rows read from host memory: each lane loads 16 bytes (V
// elements) of the row's first n real elements when the row is 16-byte
// aligned (few large requests suit the host link; from device memory the
// per-element loads are faster), and stores them into the transposed tile in
// V steps.  Lane l starts at element rot = l V / 32 (mod V) of its vector,
// which puts the 32 stores of a step in 32 different banks.  Returns how many
// leading elements were loaded.
template <typename InT>
__device__ __forceinline__ int load_row_vec(float *trow, const InT *src, int n, int lane,
                                            int pitch) {
  constexpr int V = 16 / (int)sizeof(InT);
  if ((reinterpret_cast<size_t>(src) & 15) != 0) return 0;
  const int nv = n / V;
  const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
  const int rot = (lane * V / 32) & (V - 1);
  for (int v = lane; v < nv; v += 32) {
    const uint4 q = s4[v];
    float *dst = trow + v * V * pitch;
#pragma unroll
    for (int k = 0; k < V; k++) {
      const int idx = (k + rot) & (V - 1);
      constexpr int perWord = 4 / (int)sizeof(InT);
      const int wi = idx / perWord, sh = (idx % perWord) * 8 * (int)sizeof(InT);
      const unsigned word = (wi & 2) ? ((wi & 1) ? q.w : q.z) : ((wi & 1) ? q.y : q.x);
      const unsigned e = (word >> sh) & (sizeof(InT) == 1 ? 0xffu : 0xffffu);
      dst[idx * pitch] = (float)e;
    }
  }
  return nv * V;
}

// lane group for rows of `len` elements moved `len`-wide
__device__ __forceinline__ int group_width(int len) {
  if (len >= 32) return 32;
  int G = 1;
  while (G < len) G <<= 1;
  return G;
}

// 8- and 16-bit rows of device memory whose starts are all 4-byte aligned:
// the lanes of a row load 32-bit words (W = 4 or 2 elements) of its first n
// real elements, U rows per lane at once so that U loads are in flight
// before the first store, and store the elements into the transposed tile
// (lane l of a row starts at element (l W / 32) mod W of its word, so a
// step's stores fall in different banks); the rest of each row (the last
// partial word and the REPEAT padding up to L) is moved element by element.
template <typename InT, int NW>
__device__ __forceinline__ void load_rows_narrow(float *tile, const InT *in,
                                                 const long long *rowIn, int nr, int L, int n,
                                                 int pitch, int warp, int lane) {
  constexpr int W = 4 / (int)sizeof(InT);
  constexpr int U = 4;
  const int nw = n / W;
  const int G = group_width(nw > 0 ? nw : 1), rpi = 32 / G;
  const int sub = lane & (G - 1), rsub = lane / G;
  const int rot = (sub * W / 32) & (W - 1);
  const int Ge = group_width(L), rpie = 32 / Ge, sube = lane & (Ge - 1), rsube = lane / Ge;
  for (int rb = warp * rpi; rb < nr; rb += U * NW * rpi) {
    for (int v0 = 0; v0 < nw; v0 += G) {
      unsigned wv[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int rr = rb + u * NW * rpi + rsub, v = v0 + sub;
        wv[u] = (rr < nr && v < nw) ? reinterpret_cast<const unsigned *>(in + rowIn[rr])[v] : 0u;
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int rr = rb + u * NW * rpi + rsub, v = v0 + sub;
        if (rr < nr && v < nw) {
          float *dst = tile + rr + v * W * pitch;
#pragma unroll
          for (int k = 0; k < W; k++) {
            const int idx = (k + rot) & (W - 1);
            const unsigned e = (wv[u] >> (idx * 8 * (int)sizeof(InT))) &
                               (sizeof(InT) == 1 ? 0xffu : 0xffffu);
            dst[idx * pitch] = (float)e;
          }
        }
      }
    }
  }
  // elements nw W .. L-1 of every row (clamped to the last real element)
  if (nw * W < L)
    for (int rb = warp * rpie; rb < nr; rb += NW * rpie) {
      const int rr = rb + rsube;
      if (rr >= nr) continue;
      const InT *src = in + rowIn[rr];
      for (int c = nw * W + sube; c < L; c += Ge)
        tile[rr + c * pitch] = load_as_float(src + min(c, n - 1));
    }
}

// ROWS = 32, 64 or 128 rows, NW = 4 or 8 warps: warp w owns rows
// 32 (w / kSegs) .. +31 of the tile and segment w % kSegs of every level of
// them, kSegs = 32 NW / ROWS.
template <typename InT, typename OutT, bool INV, bool VEC, int ROWS, int NW>
__global__ void __launch_bounds__(32 * NW)
dwt_cols_kernel(const PassDesc *__restrict__ passes, const int *__restrict__ tilePrefix,
                int nPasses) {
  static_assert(ROWS == kRows || ROWS == 2 * kRows || ROWS == 4 * kRows, "tile height");
  static_assert(NW == 4 || NW == 8, "warps per tile");
  constexpr int kThreadsC = 32 * NW;
  constexpr int kP = ROWS + 1;                 // words between positions of a row
  constexpr int kSegs = NW * kRows / ROWS;     // warps per 32 rows = segments per level
  extern __shared__ float4 smem4[];
  float *tile = reinterpret_cast<float *>(smem4);
  __shared__ long long rowIn[ROWS], rowOut[ROWS];
  __shared__ float scaleTab[32];
  // band order of rows stored / loaded contiguously: band index q holds the
  // in-place position p = bandPos[q] >> 4 of level bandPos[q] & 15, so lanes
  // walk q (coalesced global accesses) instead of p
  __shared__ uint16_t bandPos[kColsMaxL];

  const int bid = blockIdx.x;
  int lo = 0, hi = nPasses - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tilePrefix[mid] <= bid) lo = mid; else hi = mid - 1;
  }
  const PassDesc &d = passes[lo];
  const int L = d.L, S = d.steps;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int r0 = (bid - tilePrefix[lo]) * ROWS;
  const int nr = min(ROWS, d.rows - r0);
  // the row this thread moves and computes, and its share of the elements
  const int seg = warp % kSegs;
  const int me = (warp / kSegs) * kRows + lane;
  const int cFirst = seg, cStep = kSegs;
  // exact-order CDF 9/7 passes never come here (they run in dwt.cu)
  const bool lifting = d.wavelet == WL_CDF97;
  if ((int)threadIdx.x < ROWS) {
    const int r = r0 + threadIdx.x;
    long long bi = 0, bo = -1;
    if ((int)threadIdx.x < nr) {
      const int a = r / d.B, b = r - a * d.B;
      if (!INV)
        bi = (long long)min(a, d.clampA - 1) * d.inSA + (long long)min(b, d.clampB - 1) * d.inSB;
      else
        bi = (long long)a * d.inSA + (long long)b * d.inSB;
      if (a < d.cropA && b < d.cropB) bo = (long long)a * d.outSA + (long long)b * d.outSB;
    }
    rowIn[threadIdx.x] = bi;
    rowOut[threadIdx.x] = bo;
  }
  if (threadIdx.x >= kThreadsC - 32 && lane <= S)
    scaleTab[lane] = lifting ? lifting_scale(lane, S) : 1.0f;
  const bool bandRows = INV ? d.inSC == 1 : d.outSC == 1;
  if (bandRows)
    for (int q = threadIdx.x; q < L; q += kThreadsC) {
      // inverse of pos_to_band: low band q < L >> S at q << S; detail band of
      // level t (q in [L >> (t+1), L >> t)) at (1 << t) + (q - (L >> (t+1))) << (t+1)
      int t = S, pos;
      const int nLow = L >> S;
      if (q < nLow) {
        pos = q << S;
      } else {
        t = 0;
        while (q < (L >> (t + 1))) t++;
        pos = (1 << t) + ((q - (L >> (t + 1))) << (t + 1));
      }
      bandPos[q] = (uint16_t)((pos << 4) | t);
    }
  __syncthreads();

  // ---- load ----------------------------------------------------------------
  const InT *in = static_cast<const InT *>(d.in);
  const long long inSC = d.inSC;
  if (inSC != 1) {
    // own row: lanes cover one element of 32 neighbouring rows (with 32 rows
    // the warps take every fourth element)
    if (me < nr) {
      const InT *src = in + rowIn[me];
      float *col = tile + me;
      if (!INV) {
        // pointer steps over the real elements, then the REPEAT padding
        const int cl = min(L, d.clampL) - 1;
        const int cEnd = min(L, cl + 1);
        const InT *sp = src + (long long)cFirst * inSC;
        float *tp = col + cFirst * kP;
        const long long sStep = (long long)cStep * inSC;
        int c = cFirst;
#pragma unroll 4
        for (; c < cEnd; c += cStep) {
          stage(tp, sp);
          sp += sStep;
          tp += cStep * kP;
        }
        for (; c < L; c += cStep) stage(col + c * kP, src + (long long)cl * inSC);
      } else {
        // band order -> in-place positions, undoing the deferred scale
        const int nLow = L >> S;
        const float sl = scaleTab[S];
        for (int q = cFirst; q < nLow; q += cStep)
          col[(q << S) * kP] = load_as_float(src + q * inSC) / sl;
        for (int t = 0; t < S; t++) {
          const int qs = L >> (t + 1);
          const float st = scaleTab[t];
          const InT *sb = src + (long long)qs * inSC;
          float *cb = col + (1 << t) * kP;
          const int step = (2 << t) * kP;
          for (int k = cFirst; k < qs; k += cStep) cb[k * step] = load_as_float(sb + k * inSC) / st;
        }
      }
    }
  } else {
    // contiguous rows: lanes over the elements of one row (G lanes per row)
    const int G = group_width(L), rpi = 32 / G, sub = lane & (G - 1), rsub = lane / G;
    const bool narrowWords = !INV && !VEC && sizeof(InT) < 4 &&
                             (reinterpret_cast<size_t>(in) & 3) == 0 &&
                             ((d.inSA * (long long)sizeof(InT)) & 3) == 0 &&
                             ((d.inSB * (long long)sizeof(InT)) & 3) == 0;
    if (narrowWords)
      load_rows_narrow<InT, NW>(tile, in, rowIn, nr, L, min(L, d.clampL), kP, warp, lane);
    else
    for (int rb = warp * rpi; rb < nr; rb += NW * rpi) {
      const int rr = rb + rsub;
      if (rr >= nr) continue;
      const InT *src = in + rowIn[rr];
      float *trow = tile + rr;
      if (!INV) {
        const int cl = min(L, d.clampL) - 1;
        int c0 = 0;
        if (VEC && G == 32) c0 = load_row_vec(trow, src, cl + 1, lane, kP);
        for (int c = c0 + sub; c < L; c += G) stage(trow + c * kP, src + min(c, cl));
      } else {
        for (int q = sub; q < L; q += G) {
          const int e = bandPos[q];
          trow[(e >> 4) * kP] = load_as_float(src + q) / scaleTab[e & 15];
        }
      }
    }
  }
  if (std::is_same<InT, float>::value && !INV) cp_async_wait_all();
  __syncthreads();

  // ---- levels --------------------------------------------------------------
  float *x = tile + me;
  const bool rowOk = me < nr;
  for (int it = 0; it < S; it++) {
    const int lev = INV ? S - 1 - it : it;
    const int h = (L >> lev) >> 1, P = (1 << lev) * kP;
    // a level of few pairs is not split: segment 0 sweeps it whole (every
    // segment pays halo reads and a generic start and end)
    const bool split = kSegs > 1 && h >= kMinSegPairs * kSegs;
    const int i0 = split ? (seg * h) / kSegs : (seg == 0 ? 0 : h);
    const int i1 = split ? ((seg + 1) * h) / kSegs : h;
    if (!lifting) {
      if (rowOk) haar_seg(x, P, i0, i1, INV);
    } else if (h == 1) {
      if (rowOk && i0 < i1) {
        if (!INV) {
          Halo hb = {};
          lift_fwd_seg(x, 1, P, 0, 1, hb);
        } else {
          lift_inv_one(x, P);
        }
      }
    } else {
      Halo hb = {};
      if (kSegs > 1) {
        if (rowOk && i0 < i1) capture_halo(x, h, P, i0, i1, hb);
        __syncthreads();
      }
      if (rowOk && i0 < i1) {
        if (!INV) lift_fwd_seg(x, h, P, i0, i1, hb);
        else lift_inv_seg(x, h, P, i0, i1, hb);
      }
    }
    if (kSegs > 1) __syncthreads();
  }
  if (kSegs == 1) __syncthreads();

  // ---- store ---------------------------------------------------------------
  OutT *out = static_cast<OutT *>(d.out);
  const long long outSC = d.outSC;
  if (outSC != 1) {
    if (me < nr && rowOut[me] >= 0) {
      OutT *dst = out + rowOut[me];
      const float *col = tile + me;
      if (!INV) {
        const int nLow = L >> S;
        const float sl = scaleTab[S];
        for (int q = cFirst; q < nLow; q += cStep)
          store_from_float(dst + q * outSC, col[(q << S) * kP] * sl);
        for (int t = 0; t < S; t++) {
          const int qs = L >> (t + 1);
          const float st = scaleTab[t];
          OutT *db = dst + (long long)(qs + cFirst) * outSC;
          const float *cb = col + (1 << t) * kP + cFirst * ((2 << t) * kP);
          const long long dStep = (long long)cStep * outSC;
          const int cStepT = cStep * ((2 << t) * kP);
#pragma unroll 4
          for (int k = cFirst; k < qs; k += cStep) {
            store_from_float(db, *cb * st);
            db += dStep;
            cb += cStepT;
          }
        }
      } else {
        const int Lc = min(L, d.cropL);
        for (int c = cFirst; c < Lc; c += cStep) store_from_float(dst + c * outSC, col[c * kP]);
      }
    }
  } else {
    const int Lc = INV ? min(L, d.cropL) : L;
    const int G = group_width(Lc), rpi = 32 / G, sub = lane & (G - 1), rsub = lane / G;
    for (int rb = warp * rpi; rb < nr; rb += NW * rpi) {
      const int rr = rb + rsub;
      if (rr >= nr) continue;
      const long long base = rowOut[rr];
      if (base < 0) continue;
      const float *trow = tile + rr;
      if (!INV) {
        for (int q = sub; q < L; q += G) {
          const int e = bandPos[q];
          store_from_float(out + base + q, trow[(e >> 4) * kP] * scaleTab[e & 15]);
        }
      } else {
        for (int c = sub; c < Lc; c += G) store_from_float(out + base + c, trow[c * kP]);
      }
    }
  }
}

template <typename InT, typename OutT, bool INV, bool VEC, int NW>
void launch_w(const PassDesc *p, const int *tp, int n, int tiles, int smem, int rows,
              cudaStream_t s) {
  auto k = rows == kRows       ? dwt_cols_kernel<InT, OutT, INV, VEC, kRows, NW>
           : rows == 2 * kRows ? dwt_cols_kernel<InT, OutT, INV, VEC, 2 * kRows, NW>
                               : dwt_cols_kernel<InT, OutT, INV, VEC, 4 * kRows, NW>;
  if (smem > 32 * 1024) raise_smem_limit(k, smem);  // static + dynamic may pass 48 KB
  k<<<tiles, 32 * NW, smem, s>>>(p, tp, n);
}

template <typename InT, typename OutT, bool INV, bool VEC = false>
void launch_t(const PassDesc *p, const int *tp, int n, int tiles, int smem, int rows, int warps,
              cudaStream_t s) {
  if (warps == 8) launch_w<InT, OutT, INV, VEC, 8>(p, tp, n, tiles, smem, rows, s);
  else launch_w<InT, OutT, INV, VEC, 4>(p, tp, n, tiles, smem, rows, s);
}

}  // namespace

// default tile height: rows of at most 64 elements in 128-row tiles swept
// whole by each warp, longer rows in 32-row tiles of four segments
int dwt_cols_tile_rows(int L) { return L <= 64 ? 4 * kRows : kRows; }

int dwt_cols_smem_bytes(int L, int rows) { return L * (rows + 1) * (int)sizeof(float); }

// dynamic shared memory available beside the kernel's static arrays
bool dwt_cols_rows_fit(int L, int rows) {
  if (rows != kRows && rows != 2 * kRows && rows != 4 * kRows) return false;  // any warps
  // row bases, scales, band table, reserve
  const int kStatic = 2 * 4 * kRows * 8 + 32 * 4 + kColsMaxL * 2 + 1024;
  return dwt_cols_smem_bytes(L, rows) <= 227 * 1024 - kStatic;
}

void launch_dwt_cols(const PassDesc *p, const int *tp, int n, int tiles, int smem, int rows,
                     int warps, int inType, int outType, bool inverse, bool vecLoad,
                     cudaStream_t s) {
  if (!inverse) {
    switch (inType) {
      case WL_U8:
        if (vecLoad) launch_t<uint8_t, float, false, true>(p, tp, n, tiles, smem, rows, warps, s);
        else launch_t<uint8_t, float, false>(p, tp, n, tiles, smem, rows, warps, s);
        break;
      case WL_U16:
        if (vecLoad) launch_t<uint16_t, float, false, true>(p, tp, n, tiles, smem, rows, warps, s);
        else launch_t<uint16_t, float, false>(p, tp, n, tiles, smem, rows, warps, s);
        break;
      case WL_I32: launch_t<int32_t, float, false>(p, tp, n, tiles, smem, rows, warps, s); break;
      default: launch_t<float, float, false>(p, tp, n, tiles, smem, rows, warps, s); break;
    }
  } else {
    switch (outType) {
      case WL_U8: launch_t<float, uint8_t, true>(p, tp, n, tiles, smem, rows, warps, s); break;
      case WL_U16: launch_t<float, uint16_t, true>(p, tp, n, tiles, smem, rows, warps, s); break;
      case WL_I32: launch_t<float, int32_t, true>(p, tp, n, tiles, smem, rows, warps, s); break;
      default: launch_t<float, float, true>(p, tp, n, tiles, smem, rows, warps, s); break;
    }
  }
}

}  // namespace wl
