// Row-register wavelet passes: a row of L = E G elements (E = 8: L a power
// of two, 16 .. 256; E = 6: L = 48, 96, 192) is held by G lanes of a warp in
// registers, E consecutive elements per lane, read with one to three vector
// loads.  Three kernels use it:
//   - the forward z pass, in place on rows contiguous on both sides (the
//     column-tile kernel would stage every row through shared memory and
//     split its levels into segments with halos);
//   - the forward x pass, from the source rows (any element type, REPEAT
//     clamp) through a shared-memory tile to an output in which consecutive
//     rows are neighbours;
//   - the inverse z pass, in place, reading a row's band values first.
//
// A level with m pairs per lane (m = 4, 2, 1 for levels 0, 1, 2 with E = 8;
// 3, then two per lane on 3G/4 lanes, then one, with E = 6) lifts the lane's
// pairs in registers and takes the neighbouring pair values from the next and
// previous lane (four shuffles per level).  After level 2 a lane holds one
// low-pass value; each later level gathers pair j into lane j (two shuffles)
// and runs with fewer lanes.  Detail bands leave as soon as they are final,
// at their band positions (low band, then detail bands of the last level down
// to the first, dwt_cpu.cc:703-728) with the deferred lifting scale, so the
// band order costs nothing.  Every lifting step does the same arithmetic as
// dwt.cu and dwt_cols.cu (the same operands in the same order), so the
// coefficients are identical.
#include <cuda_runtime.h>

#include <type_traits>

#include "dwt_common.cuh"
#include "select_common.cuh"
#include "wl_internal.h"

namespace wl {
namespace {
using namespace dwtc;

constexpr int kRegThreads = 256;
constexpr unsigned kAll = 0xffffffffu;

// One forward level, M pairs per lane (pair k of group lane `sub` is pair
// M sub + k of the level), lanes [0, na) of the G-lane group active; the
// mirrored ends of the lifting (dwt.cu fwd_lifting_level):
//   d1_j = o_j + a (e_j + e_j+1)     e_h   = e_h-1
//   s1_j = e_j + b (d1_j-1 + d1_j)   d1_-1 = d1_0
//   d2_j = d1_j + g (s1_j + s1_j+1)  s1_h  = s1_h-1
//   s2_j = s1_j + d (d2_j-1 + d2_j)  d2_-1 = d2_0
// Returns the low-pass values in e[] and the details in o[].
template <int M, int G, bool HAAR>
__device__ __forceinline__ void fwd_level(float (&e)[M], float (&o)[M], int sub, int na) {
  if (HAAR) {  // dwt_cpu.cc:159-162
#pragma unroll
    for (int k = 0; k < M; k++) {
      const float a = e[k], b = o[k];
      o[k] = __fmul_rn(__fsub_rn(a, b), kInvSqrt2);
      e[k] = __fmul_rn(__fadd_rn(a, b), kInvSqrt2);
    }
    return;
  }
  const bool first = sub == 0, last = sub == na - 1;
  float eN = __shfl_down_sync(kAll, e[0], 1, G);
  if (last) eN = e[M - 1];
  float d1[M], s1[M];
#pragma unroll
  for (int k = 0; k < M; k++) d1[k] = fmaf(kAlpha, e[k] + (k + 1 < M ? e[k + 1] : eN), o[k]);
  float d1P = __shfl_up_sync(kAll, d1[M - 1], 1, G);
  if (first) d1P = d1[0];
#pragma unroll
  for (int k = 0; k < M; k++) s1[k] = fmaf(kBeta, (k ? d1[k - 1] : d1P) + d1[k], e[k]);
  float s1N = __shfl_down_sync(kAll, s1[0], 1, G);
  if (last) s1N = s1[M - 1];
#pragma unroll
  for (int k = 0; k < M; k++) o[k] = fmaf(kGamma, s1[k] + (k + 1 < M ? s1[k + 1] : s1N), d1[k]);
  float d2P = __shfl_up_sync(kAll, o[M - 1], 1, G);
  if (first) d2P = o[0];
#pragma unroll
  for (int k = 0; k < M; k++) e[k] = fmaf(kDelta, (k ? o[k - 1] : d2P) + o[k], s1[k]);
}

// Where the finished values of a row go: band position q of the row.
// put4 / put2 take 4 / 2 consecutive positions starting at a multiple of 4 / 2.
struct GlobalRow {  // the row itself, in place (float row, 16-byte aligned)
  float *dst;
  __device__ void put(int q, float v) const { dst[q] = v; }
  __device__ void put2(int q, float a, float b) const {
    *reinterpret_cast<float2 *>(dst + q) = make_float2(a, b);
  }
  __device__ void put4(int q, float a, float b, float c, float d) const {
    *reinterpret_cast<float4 *>(dst + q) = make_float4(a, b, c, d);
  }
};
// The last pass of a compression: the row in place, every value also counted
// into the select statistics (first radix-select digit, extremes) while it is
// still in a register.
struct GlobalRowSel {
  float *dst;
  selc::SelAcc *acc;
  __device__ void put(int q, float v) const {
    dst[q] = v;
    acc->visit(v);
  }
  __device__ void put2(int q, float a, float b) const {
    *reinterpret_cast<float2 *>(dst + q) = make_float2(a, b);
    acc->visit(a);
    acc->visit(b);
  }
  __device__ void put4(int q, float a, float b, float c, float d) const {
    *reinterpret_cast<float4 *>(dst + q) = make_float4(a, b, c, d);
    acc->visit(a);
    acc->visit(b);
    acc->visit(c);
    acc->visit(d);
  }
};
struct TileRow {  // column r of a shared-memory tile, position q at q * P + r
  float *col;
  int P;
  __device__ void put(int q, float v) const { col[q * P] = v; }
  __device__ void put2(int q, float a, float b) const { put(q, a); put(q + 1, b); }
  __device__ void put4(int q, float a, float b, float c, float d) const {
    put(q, a); put(q + 1, b); put(q + 2, c); put(q + 3, d);
  }
};

// All levels of rows of L = E G elements held E per lane (e: even, o: odd
// elements of the lane's M = E / 2 pairs), each value handed to out.put*
// (when ok) at its band position with the deferred lifting scale.
template <int G, int E, bool HAAR, class Out>
__device__ __forceinline__ void rowreg_levels(float (&e)[E / 2], float (&o)[E / 2], int sub,
                                              int S, const float *scaleTab, bool ok,
                                              const Out &out) {
  constexpr int L = E * G;
  constexpr int M = E / 2;                     // level-0 pairs per lane
  constexpr int NA1 = M == 4 ? G : 3 * G / 4;  // lanes of levels 1 and 2
  // level 0: M pairs per lane
  fwd_level<M, G, HAAR>(e, o, sub, G);
  if (ok) {
    const float sc = scaleTab[0];
    if (M == 4) out.put4(L / 2 + 4 * sub, o[0] * sc, o[1 % M] * sc, o[2 % M] * sc, o[3 % M] * sc);
    else
#pragma unroll
      for (int k = 0; k < M; k++) out.put(L / 2 + M * sub + k, o[k] * sc);
  }
  if (S == 1) {
    if (ok) {
      const float sc = scaleTab[1];
      if (M == 4) out.put4(4 * sub, e[0] * sc, e[1 % M] * sc, e[2 % M] * sc, e[3 % M] * sc);
      else
#pragma unroll
        for (int k = 0; k < M; k++) out.put(M * sub + k, e[k] * sc);
    }
    return;
  }
  // level 1: lane j of the first NA1 holds the low-pass values 4j .. 4j+3,
  // two pairs (with three per lane they are gathered from the lanes that
  // hold them)
  float q4[4];
  if (M == 4) {
#pragma unroll
    for (int r = 0; r < 4; r++) q4[r] = e[r % M];
  } else {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int v = min(4 * sub + r, L / 2 - 1);
      const int from = v / 3, reg = v - 3 * from;
      const float a = __shfl_sync(kAll, e[0], from, G);
      const float b = __shfl_sync(kAll, e[1 % M], from, G);
      const float c = __shfl_sync(kAll, e[2 % M], from, G);
      q4[r] = reg == 0 ? a : (reg == 1 ? b : c);
    }
  }
  const bool act1 = sub < NA1;
  float e1[2] = {q4[0], q4[2]}, o1[2] = {q4[1], q4[3]};
  fwd_level<2, G, HAAR>(e1, o1, sub, NA1);
  if (ok && act1) {
    const float sc = scaleTab[1];
    out.put2(L / 4 + 2 * sub, o1[0] * sc, o1[1] * sc);
  }
  if (S == 2) {
    if (ok && act1) {
      const float sc = scaleTab[2];
      out.put2(2 * sub, e1[0] * sc, e1[1] * sc);
    }
    return;
  }
  // level 2: one pair per lane
  float e2[1] = {e1[0]}, o2[1] = {e1[1]};
  fwd_level<1, G, HAAR>(e2, o2, sub, NA1);
  if (ok && act1) out.put(L / 8 + sub, o2[0] * scaleTab[2]);
  // levels 3 ..: pair j gathered into lane j of the group
  float s = e2[0];
  int na = NA1;  // lanes holding a low-pass value
  for (int lev = 3; lev < S; lev++) {
    float ge[1] = {__shfl_sync(kAll, s, (2 * sub) & (G - 1), G)};
    float go[1] = {__shfl_sync(kAll, s, (2 * sub + 1) & (G - 1), G)};
    na >>= 1;  // pairs of this level = L >> (lev + 1)
    fwd_level<1, G, HAAR>(ge, go, sub, na);
    if (ok && sub < na) out.put((L >> (lev + 1)) + sub, go[0] * scaleTab[lev]);
    s = ge[0];
  }
  if (ok && sub < (L >> S)) out.put(sub, s * scaleTab[S]);
}

// The rows [row0, row0 + kRegThreads / G) of one in-place pass of float rows;
// E = 8 or 6 elements per lane (L = E G).  scaleTab holds the deferred
// lifting scales; SEL: every value written is also visited by acc.
template <int G, int E, bool HAAR, bool SEL>
__device__ __forceinline__ void rowreg_fwd(const PassDesc &d, int row0, const float *scaleTab,
                                           selc::SelAcc &acc) {
  constexpr int M = E / 2;
  const int S = d.steps;
  const int row = row0 + (int)threadIdx.x / G;
  const int sub = threadIdx.x & (G - 1);
  const bool ok = row < d.rows;
  long long bi = 0, bo = 0;
  if (ok) {
    const int a = row / d.B, b = row - a * d.B;
    bi = (long long)a * d.inSA + (long long)b * d.inSB;
    bo = (long long)a * d.outSA + (long long)b * d.outSB;
  }
  const float *src = static_cast<const float *>(d.in) + bi;
  float e[M], o[M];
  if (ok) {
    if (M == 4) {
      const float4 *s4 = reinterpret_cast<const float4 *>(src) + 2 * sub;
      const float4 p = s4[0], q = s4[1];
      e[0] = p.x; o[0] = p.y; e[1] = p.z; o[1] = p.w;
      e[2 % M] = q.x; o[2 % M] = q.y; e[3 % M] = q.z; o[3 % M] = q.w;
    } else {
      const float2 *s2 = reinterpret_cast<const float2 *>(src) + 3 * sub;
#pragma unroll
      for (int k = 0; k < M; k++) {
        const float2 p = s2[k];
        e[k] = p.x;
        o[k] = p.y;
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < M; k++) e[k] = o[k] = 0.f;
  }
  // in place: the row (held by lanes of one warp) is read by all its lanes
  // before any of them stores
  __syncwarp();
  float *dst = static_cast<float *>(d.out) + bo;
  if (SEL) rowreg_levels<G, E, HAAR>(e, o, sub, S, scaleTab, ok, GlobalRowSel{dst, &acc});
  else rowreg_levels<G, E, HAAR>(e, o, sub, S, scaleTab, ok, GlobalRow{dst});
}

// E elements [first, first + E) of a row of n real elements as floats: one
// to three vector loads when the run is whole and aligned, else element by
// element with the REPEAT clamp to the last real element.
template <typename InT, int E>
__device__ __forceinline__ void load_run(const InT *row, int first, int n, float (&v)[E]) {
  const InT *p = row + first;
  const size_t addr = reinterpret_cast<size_t>(p);
  if (first + E <= n) {
    if (sizeof(InT) == 4 && E == 8 && (addr & 15) == 0) {
      const uint4 a = reinterpret_cast<const uint4 *>(p)[0], b = reinterpret_cast<const uint4 *>(p)[1];
      const unsigned w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
      for (int k = 0; k < E; k++)
        v[k] = sizeof(InT) == 4 && std::is_same<InT, float>::value ? __uint_as_float(w[k % 8])
                                                                     : (float)(int)w[k % 8];
      return;
    }
    if (sizeof(InT) == 4 && E == 6 && (addr & 7) == 0) {
      const uint2 *q = reinterpret_cast<const uint2 *>(p);
      const uint2 a = q[0], b = q[1], c = q[2];
      const unsigned w[6] = {a.x, a.y, b.x, b.y, c.x, c.y};
#pragma unroll
      for (int k = 0; k < E; k++)
        v[k] = std::is_same<InT, float>::value ? __uint_as_float(w[k % 6]) : (float)(int)w[k % 6];
      return;
    }
    if (sizeof(InT) == 2 && E == 8 && (addr & 15) == 0) {
      const uint4 a = reinterpret_cast<const uint4 *>(p)[0];
      const unsigned w[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
      for (int k = 0; k < E; k++) v[k] = (float)((w[(k / 2) % 4] >> (16 * (k & 1))) & 0xffffu);
      return;
    }
    if (sizeof(InT) == 2 && E == 6 && (addr & 3) == 0) {
      const unsigned *q = reinterpret_cast<const unsigned *>(p);
      const unsigned w[3] = {q[0], q[1], q[2]};
#pragma unroll
      for (int k = 0; k < E; k++) v[k] = (float)((w[(k / 2) % 3] >> (16 * (k & 1))) & 0xffffu);
      return;
    }
    if (sizeof(InT) == 1 && E == 8 && (addr & 7) == 0) {
      const uint2 a = reinterpret_cast<const uint2 *>(p)[0];
      const unsigned w[2] = {a.x, a.y};
#pragma unroll
      for (int k = 0; k < E; k++) v[k] = (float)((w[(k / 4) % 2] >> (8 * (k & 3))) & 0xffu);
      return;
    }
    if (sizeof(InT) == 1 && E == 6 && (addr & 1) == 0) {
      const unsigned short *q = reinterpret_cast<const unsigned short *>(p);
      const unsigned w[3] = {q[0], q[1], q[2]};
#pragma unroll
      for (int k = 0; k < E; k++) v[k] = (float)((w[(k / 2) % 3] >> (8 * (k & 1))) & 0xffu);
      return;
    }
  }
#pragma unroll
  for (int k = 0; k < E; k++) v[k] = load_as_float(row + min(first + k, n - 1));
}

// Rows contiguous in memory read into registers (any element type, REPEAT
// clamp to the real row length and row range), finished values written as
// columns of a shared-memory tile of R rows, then stored position by
// position: a warp writes one position of 32 consecutive rows, which are
// neighbours in the output (the forward x and y passes).
template <int G> struct TileRows {
  static constexpr int kPerRound = kRegThreads / G;  // rows one round of the block holds
  static constexpr int R = kPerRound > 32 ? kPerRound : 32;
  static constexpr int P = R + 1;  // odd stride: a position of 32 rows is conflict-free
};

template <typename InT, int G, int E, bool HAAR>
__device__ __forceinline__ void rowreg_t(const PassDesc &d, int tile, float *tileSm,
                                         float *scaleTab, long long *rowOut) {
  constexpr int L = E * G;
  constexpr int M = E / 2;
  constexpr int R = TileRows<G>::R, P = TileRows<G>::P, kPerRound = TileRows<G>::kPerRound;
  const int S = d.steps;
  const int r0 = tile * R;
  if ((int)threadIdx.x <= S) scaleTab[threadIdx.x] = HAAR ? 1.0f : lifting_scale(threadIdx.x, S);
  for (int t = threadIdx.x; t < R; t += kRegThreads) {
    const int row = r0 + t;
    long long bo = -1;
    if (row < d.rows) {
      const int a = row / d.B, b = row - a * d.B;
      bo = (long long)a * d.outSA + (long long)b * d.outSB;
    }
    rowOut[t] = bo;
  }
  __syncthreads();
  const int sub = threadIdx.x & (G - 1);
  const int n = min(L, d.clampL);  // real elements of a row
  const InT *in = static_cast<const InT *>(d.in);
  for (int rr = (int)threadIdx.x / G; rr < R; rr += kPerRound) {
    const int row = r0 + rr;
    const bool ok = row < d.rows;
    float v[E];
    if (ok) {
      const int a = row / d.B, b = row - a * d.B;
      const long long bi = (long long)min(a, d.clampA - 1) * d.inSA +
                           (long long)min(b, d.clampB - 1) * d.inSB;
      load_run<InT, E>(in + bi, E * sub, n, v);
    } else {
#pragma unroll
      for (int k = 0; k < E; k++) v[k] = 0.f;
    }
    float e[M], o[M];
#pragma unroll
    for (int k = 0; k < M; k++) {
      e[k] = v[2 * k];
      o[k] = v[2 * k + 1];
    }
    rowreg_levels<G, E, HAAR>(e, o, sub, S, scaleTab, ok, TileRow{tileSm + rr, P});
  }
  __syncthreads();
  float *out = static_cast<float *>(d.out);
  const long long outSC = d.outSC;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int rr = lane; rr < R; rr += 32) {
    const long long bo = rowOut[rr];
    if (bo < 0) continue;
    float *dst = out + bo + warp * outSC;
    const float *t = tileSm + warp * P + rr;
#pragma unroll 4
    for (int q = warp; q < L; q += kRegThreads / 32) {
      *dst = *t;
      dst += (kRegThreads / 32) * outSC;
      t += (kRegThreads / 32) * P;
    }
  }
}

template <typename InT, int G, int E>
__global__ void __launch_bounds__(kRegThreads)
dwt_rowreg_t_kernel(const PassDesc *__restrict__ passes, const int *__restrict__ tilePrefix,
                    int nPasses) {
  extern __shared__ float tileSm[];
  __shared__ float scaleTab[16];
  __shared__ long long rowOut[TileRows<G>::R];
  const int bid = blockIdx.x;
  int lo = 0, hi = nPasses - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tilePrefix[mid] <= bid) lo = mid; else hi = mid - 1;
  }
  const PassDesc &d = passes[lo];
  const int tile = bid - tilePrefix[lo];
  if (d.wavelet == WL_HAAR) rowreg_t<InT, G, E, true>(d, tile, tileSm, scaleTab, rowOut);
  else rowreg_t<InT, G, E, false>(d, tile, tileSm, scaleTab, rowOut);
}

template <typename InT, int G, int E = 8>
void launch_tg(const PassDesc *p, const int *tp, int n, int blocks, cudaStream_t s) {
  const int smem = E * G * TileRows<G>::P * (int)sizeof(float);
  auto k = dwt_rowreg_t_kernel<InT, G, E>;
  if (smem > 48 * 1024) raise_smem_limit(k, smem);
  k<<<blocks, kRegThreads, smem, s>>>(p, tp, n);
}

template <typename InT>
void launch_t_len(const PassDesc *p, const int *tp, int n, int blocks, int L, cudaStream_t s) {
  switch (L) {
    case 16: launch_tg<InT, 2>(p, tp, n, blocks, s); break;
    case 32: launch_tg<InT, 4>(p, tp, n, blocks, s); break;
    case 48: launch_tg<InT, 8, 6>(p, tp, n, blocks, s); break;
    case 64: launch_tg<InT, 8>(p, tp, n, blocks, s); break;
    case 96: launch_tg<InT, 16, 6>(p, tp, n, blocks, s); break;
    case 128: launch_tg<InT, 16>(p, tp, n, blocks, s); break;
    case 192: launch_tg<InT, 32, 6>(p, tp, n, blocks, s); break;
    default: launch_tg<InT, 32>(p, tp, n, blocks, s); break;
  }
}

// One inverse level, M pairs per lane (pair k of group lane `sub` is pair
// M sub + k), lanes [0, na) active; s: low-pass, d: detail values in, the
// even (e) and odd (o) elements out, with the mirrored ends of dwt.cu
// inv_lifting_level / dwt_cols.cu lift_inv_seg (same operands, same order):
//   s1_j = s2_j - d (d2_j-1 + d2_j)   d2_-1 = d2_0
//   d1_j = d2_j - g (s1_j + s1_j+1)   s1_h  = s1_h-1
//   e_j  = s1_j - b (d1_j-1 + d1_j)   d1_-1 = d1_0
//   o_j  = d1_j - a (e_j + e_j+1)     e_h   = e_h-1
template <int M, int G, bool HAAR>
__device__ __forceinline__ void inv_level(const float (&s2)[M], const float (&d2)[M], int sub,
                                          int na, float (&e)[M], float (&o)[M]) {
  if (HAAR) {  // dwt_cpu.cc:193-196
#pragma unroll
    for (int k = 0; k < M; k++) {
      e[k] = __fmul_rn(kInvSqrt2, __fadd_rn(s2[k], d2[k]));
      o[k] = __fmul_rn(kInvSqrt2, __fsub_rn(s2[k], d2[k]));
    }
    return;
  }
  const bool first = sub == 0, last = sub == na - 1;
  float s1[M], d1[M];
  float d2P = __shfl_up_sync(kAll, d2[M - 1], 1, G);
  if (first) d2P = d2[0];
#pragma unroll
  for (int k = 0; k < M; k++) s1[k] = fmaf(-kDelta, (k ? d2[k - 1] : d2P) + d2[k], s2[k]);
  float s1N = __shfl_down_sync(kAll, s1[0], 1, G);
  if (last) s1N = s1[M - 1];
#pragma unroll
  for (int k = 0; k < M; k++) d1[k] = fmaf(-kGamma, s1[k] + (k + 1 < M ? s1[k + 1] : s1N), d2[k]);
  float d1P = __shfl_up_sync(kAll, d1[M - 1], 1, G);
  if (first) d1P = d1[0];
#pragma unroll
  for (int k = 0; k < M; k++) e[k] = fmaf(-kBeta, (k ? d1[k - 1] : d1P) + d1[k], s1[k]);
  float eN = __shfl_down_sync(kAll, e[0], 1, G);
  if (last) eN = e[M - 1];
#pragma unroll
  for (int k = 0; k < M; k++) o[k] = fmaf(-kAlpha, e[k] + (k + 1 < M ? e[k + 1] : eN), d1[k]);
}

// Where the inverse reads a row's stored (band-order, scaled) values and
// writes its restored elements.  A lane writes elements 2 (M sub + k) and
// 2 (M sub + k) + 1 (e[k], o[k]).
struct InGlobalRow {  // the row in global memory
  const float *src;
  __device__ float get(int q) const { return src[q]; }
};
struct InTileCol {  // column r of a shared-memory tile, position q at q * P + r
  const float *col;
  int P;
  __device__ float get(int q) const { return col[q * P]; }
};
struct OutGlobalInPlace {  // the float row itself (16-byte aligned for E = 8)
  float *dst;
  template <int M>
  __device__ void put(int sub, const float (&e0)[M], const float (&o0)[M]) const {
    if (M == 4) {
      float4 *d4 = reinterpret_cast<float4 *>(dst) + 2 * sub;
      d4[0] = make_float4(e0[0], o0[0], e0[1 % M], o0[1 % M]);
      d4[1] = make_float4(e0[2 % M], o0[2 % M], e0[3 % M], o0[3 % M]);
    } else {
      float2 *d2p = reinterpret_cast<float2 *>(dst) + M * sub;
#pragma unroll
      for (int k = 0; k < M; k++) d2p[k] = make_float2(e0[k], o0[k]);
    }
  }
};
template <typename OutT> struct OutRowCrop {  // an output row of n real elements
  OutT *row;
  int n;
  template <int M>
  __device__ void put(int sub, const float (&e0)[M], const float (&o0)[M]) const {
    const int b = 2 * M * sub;
#pragma unroll
    for (int k = 0; k < M; k++) {
      if (b + 2 * k < n) store_from_float(row + b + 2 * k, e0[k]);
      if (b + 2 * k + 1 < n) store_from_float(row + b + 2 * k + 1, o0[k]);
    }
  }
};
struct OutTileCol {  // back into the tile column, natural order
  float *col;
  int P;
  template <int M>
  __device__ void put(int sub, const float (&e0)[M], const float (&o0)[M]) const {
    const int b = 2 * M * sub;
#pragma unroll
    for (int k = 0; k < M; k++) {
      col[(b + 2 * k) * P] = e0[k];
      col[(b + 2 * k + 1) * P] = o0[k];
    }
  }
};

// The inverse of rowreg_levels for one row of L = E G values in band order,
// held by G lanes: every band value the row's lanes need is read first (the
// deferred scale undone by multiplying with its reciprocal, rscale), the
// levels run from the deepest up in registers, and each lane hands its E
// restored elements to out.  ok: the row exists (else nothing is read or
// written; the lanes still take part in the shuffles).
template <int G, int E, bool HAAR, class Src, class Dst>
__device__ __forceinline__ void rowreg_inv_core(int S, const float *rscale, int sub, bool ok,
                                                const Src &in, const Dst &out) {
  constexpr int L = E * G;
  constexpr int M = E / 2;
  constexpr int NA1 = M == 4 ? G : 3 * G / 4;  // lanes of levels 1 and 2
  auto rd = [&](int q, int t) { return ok ? in.get(q) * rscale[t] : 0.f; };
  const bool act1 = sub < NA1;
  // ---- every input value, read before anything is stored
  float d0[M], d1v[2] = {0.f, 0.f}, d2v = 0.f, lowv[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int k = 0; k < M; k++) d0[k] = rd(L / 2 + M * sub + k, 0);
  if (S == 1) {
#pragma unroll
    for (int k = 0; k < M; k++) lowv[k] = rd(M * sub + k, 1);
  } else {
    if (act1) { d1v[0] = rd(L / 4 + 2 * sub, 1); d1v[1] = rd(L / 4 + 2 * sub + 1, 1); }
    if (S == 2) {
      if (act1) { lowv[0] = rd(2 * sub, 2); lowv[1] = rd(2 * sub + 1, 2); }
    } else {
      if (act1) d2v = rd(L / 8 + sub, 2);
      if (S == 3 && act1) lowv[0] = rd(sub, 3);
    }
  }
  // deeper levels (S >= 4): lane j of the first L >> (t+1) holds pair j of level t
  float dg[8];
#pragma unroll
  for (int t = 3; t < 11; t++) dg[t - 3] = 0.f;
  float sg = 0.f;
  if (S >= 4) {
#pragma unroll
    for (int t = 3; t < 11; t++)
      if (t < S && sub < (L >> (t + 1))) dg[t - 3] = rd((L >> (t + 1)) + sub, t);
    if (sub < (L >> S)) sg = rd(sub, S);
  }
  __syncwarp();  // the row is read by all its lanes before any of them stores

  // ---- levels S-1 .. 3, gathered: pair j in lane j
  float s2in = lowv[0];  // level 2's low-pass value of this lane
  if (S >= 4) {
    float s = sg;
    int na = L >> S;  // pairs of level S-1
#pragma unroll 1
    for (int t = S - 1; t >= 3; t--) {
      float sv[1] = {s}, dv[1] = {0.f}, ev[1], ov[1];
#pragma unroll
      for (int u = 3; u < 11; u++)
        if (u == t) dv[0] = dg[u - 3];
      inv_level<1, G, HAAR>(sv, dv, sub, na, ev, ov);
      // level t-1's pair j is s^{t-1}[j]: element j of level t's output
      const float a = __shfl_sync(kAll, ev[0], (sub >> 1) & (G - 1), G);
      const float b = __shfl_sync(kAll, ov[0], (sub >> 1) & (G - 1), G);
      s = (sub & 1) ? b : a;
      na <<= 1;
    }
    s2in = s;
  }
  float e1in[2], o1in[2];  // level 1's two pairs per lane: low-pass in e1in
  if (S >= 3) {
    float sv[1] = {s2in}, dv[1] = {d2v}, ev[1], ov[1];
    inv_level<1, G, HAAR>(sv, dv, sub, NA1, ev, ov);
    e1in[0] = ev[0];
    e1in[1] = ov[0];
  } else {
    e1in[0] = lowv[0];
    e1in[1] = lowv[1];
  }
  float s0[M];  // level 0's low-pass values of this lane's pairs
  if (S >= 2) {
    o1in[0] = d1v[0];
    o1in[1] = d1v[1];
    float e1[2], o1[2];
    inv_level<2, G, HAAR>(e1in, o1in, sub, NA1, e1, o1);
    // lane j of the first NA1 now holds s^0[4j .. 4j+3]
    const float q4[4] = {e1[0], o1[0], e1[1], o1[1]};
    if (M == 4) {
#pragma unroll
      for (int k = 0; k < M; k++) s0[k] = q4[k % 4];
    } else {
#pragma unroll
      for (int k = 0; k < M; k++) {
        const int v = min(M * sub + k, L / 2 - 1);
        const int from = v >> 2, reg = v & 3;
        const float a = __shfl_sync(kAll, q4[0], from, G);
        const float b = __shfl_sync(kAll, q4[1], from, G);
        const float c = __shfl_sync(kAll, q4[2], from, G);
        const float dd = __shfl_sync(kAll, q4[3], from, G);
        s0[k] = reg == 0 ? a : reg == 1 ? b : reg == 2 ? c : dd;
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < M; k++) s0[k] = lowv[k % 4];
  }
  float e0[M], o0[M];
  inv_level<M, G, HAAR>(s0, d0, sub, G, e0, o0);
  if (ok) out.put(sub, e0, o0);
}

// The inverse z pass, in place: rows [row0, row0 + kRegThreads / G) of a pass
// of float rows contiguous in memory.
template <int G, int E, bool HAAR>
__device__ __forceinline__ void rowreg_inv(const PassDesc &d, int row0, const float *rscale) {
  const int row = row0 + (int)threadIdx.x / G;
  const int sub = threadIdx.x & (G - 1);
  const bool ok = row < d.rows;
  long long bi = 0, bo = 0;
  if (ok) {
    const int a = row / d.B, b = row - a * d.B;
    bi = (long long)a * d.inSA + (long long)b * d.inSB;
    bo = (long long)a * d.outSA + (long long)b * d.outSB;
  }
  rowreg_inv_core<G, E, HAAR>(d.steps, rscale, sub, ok,
                              InGlobalRow{static_cast<const float *>(d.in) + bi},
                              OutGlobalInPlace{static_cast<float *>(d.out) + bo});
}

template <int G, int E>
__global__ void __launch_bounds__(kRegThreads)
dwt_rowreg_inv_kernel(const PassDesc *__restrict__ passes, const int *__restrict__ tilePrefix,
                      int nPasses) {
  __shared__ float rscale[16];
  const int bid = blockIdx.x;
  int lo = 0, hi = nPasses - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tilePrefix[mid] <= bid) lo = mid; else hi = mid - 1;
  }
  const PassDesc &d = passes[lo];
  const int row0 = (bid - tilePrefix[lo]) * (kRegThreads / G);
  const int S = d.steps;
  const bool haar = d.wavelet == WL_HAAR;
  if ((int)threadIdx.x <= S) rscale[threadIdx.x] = haar ? 1.0f : 1.0f / lifting_scale(threadIdx.x, S);
  __syncthreads();
  if (haar) rowreg_inv<G, E, true>(d, row0, rscale);
  else rowreg_inv<G, E, false>(d, row0, rscale);
}

// Inverse passes whose rows are strided in the input (band order along the
// row, consecutive rows neighbours in memory): the y pass (z-x-y -> z-y-x)
// and the x pass into the output type with the crop (z-y-x -> x-y-z).  A
// block takes R rows: warps load one position of 32 neighbouring rows at a
// time (coalesced) into a shared-memory tile (odd stride), the G lanes of
// each row run its levels up in registers from its tile column, and the
// restored elements leave either straight into the output row (x pass: the
// output rows are contiguous; typed, cropped) or back through the tile,
// position by position, 32 neighbouring rows per warp store (y pass).
template <typename OutT, int G, int E, bool HAAR>
__device__ __forceinline__ void rowreg_inv_t(const PassDesc &d, int tile, float *tileSm,
                                             const float *rscale, const long long *rowIn,
                                             const long long *rowOut) {
  constexpr int L = E * G;
  constexpr int R = TileRows<G>::R, P = TileRows<G>::P, kPerRound = TileRows<G>::kPerRound;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int kWarps = kRegThreads / 32;
  const float *in = static_cast<const float *>(d.in);
  const long long inSC = d.inSC;
  for (int rr = lane; rr < R; rr += 32) {
    const long long bi = rowIn[rr];
    if (bi < 0) continue;
    const float *src = in + bi + warp * inSC;
    float *t = tileSm + warp * P + rr;
#pragma unroll 4
    for (int q = warp; q < L; q += kWarps) {
      *t = *src;
      src += kWarps * inSC;
      t += kWarps * P;
    }
  }
  __syncthreads();
  OutT *out = static_cast<OutT *>(d.out);
  const bool contig = d.outSC == 1;
  const int sub = threadIdx.x & (G - 1);
  for (int rr = (int)threadIdx.x / G; rr < R; rr += kPerRound) {
    const bool ok = rowIn[rr] >= 0;
    const InTileCol src{tileSm + rr, P};
    if (contig) {
      const long long bo = rowOut[rr];
      rowreg_inv_core<G, E, HAAR>(d.steps, rscale, sub, ok && bo >= 0, src,
                                  OutRowCrop<OutT>{out + (bo < 0 ? 0 : bo), min(L, d.cropL)});
    } else {
      rowreg_inv_core<G, E, HAAR>(d.steps, rscale, sub, ok, src, OutTileCol{tileSm + rr, P});
    }
  }
  if (contig) return;
  __syncthreads();
  const long long outSC = d.outSC;
  const int n = min(L, d.cropL);
  for (int rr = lane; rr < R; rr += 32) {
    const long long bo = rowOut[rr];
    if (bo < 0) continue;
    OutT *dst = out + bo + warp * outSC;
    const float *t = tileSm + warp * P + rr;
#pragma unroll 4
    for (int q = warp; q < n; q += kWarps) {
      store_from_float(dst, *t);
      dst += kWarps * outSC;
      t += kWarps * P;
    }
  }
}

template <typename OutT, int G, int E>
__global__ void __launch_bounds__(kRegThreads)
dwt_rowreg_inv_t_kernel(const PassDesc *__restrict__ passes, const int *__restrict__ tilePrefix,
                        int nPasses) {
  extern __shared__ float tileSm[];
  __shared__ float rscale[16];
  __shared__ long long rowIn[TileRows<G>::R], rowOut[TileRows<G>::R];
  const int bid = blockIdx.x;
  int lo = 0, hi = nPasses - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tilePrefix[mid] <= bid) lo = mid; else hi = mid - 1;
  }
  const PassDesc &d = passes[lo];
  const int tile = bid - tilePrefix[lo];
  constexpr int R = TileRows<G>::R;
  const int S = d.steps;
  const bool haar = d.wavelet == WL_HAAR;
  if ((int)threadIdx.x <= S) rscale[threadIdx.x] = haar ? 1.0f : 1.0f / lifting_scale(threadIdx.x, S);
  for (int t = threadIdx.x; t < R; t += kRegThreads) {
    const int row = tile * R + t;
    long long bi = -1, bo = -1;
    if (row < d.rows) {
      const int a = row / d.B, b = row - a * d.B;
      bi = (long long)a * d.inSA + (long long)b * d.inSB;
      if (a < d.cropA && b < d.cropB) bo = (long long)a * d.outSA + (long long)b * d.outSB;
    }
    rowIn[t] = bi;
    rowOut[t] = bo;
  }
  __syncthreads();
  if (haar) rowreg_inv_t<OutT, G, E, true>(d, tile, tileSm, rscale, rowIn, rowOut);
  else rowreg_inv_t<OutT, G, E, false>(d, tile, tileSm, rscale, rowIn, rowOut);
}

template <typename OutT, int G, int E = 8>
void launch_itg(const PassDesc *p, const int *tp, int n, int blocks, cudaStream_t s) {
  const int smem = E * G * TileRows<G>::P * (int)sizeof(float);
  auto k = dwt_rowreg_inv_t_kernel<OutT, G, E>;
  if (smem > 48 * 1024) raise_smem_limit(k, smem);
  k<<<blocks, kRegThreads, smem, s>>>(p, tp, n);
}

template <typename OutT>
void launch_it_len(const PassDesc *p, const int *tp, int n, int blocks, int L, cudaStream_t s) {
  switch (L) {
    case 16: launch_itg<OutT, 2>(p, tp, n, blocks, s); break;
    case 32: launch_itg<OutT, 4>(p, tp, n, blocks, s); break;
    case 48: launch_itg<OutT, 8, 6>(p, tp, n, blocks, s); break;
    case 64: launch_itg<OutT, 8>(p, tp, n, blocks, s); break;
    case 96: launch_itg<OutT, 16, 6>(p, tp, n, blocks, s); break;
    case 128: launch_itg<OutT, 16>(p, tp, n, blocks, s); break;
    case 192: launch_itg<OutT, 32, 6>(p, tp, n, blocks, s); break;
    default: launch_itg<OutT, 32>(p, tp, n, blocks, s); break;
  }
}

template <int G, int E = 8>
void launch_ig(const PassDesc *p, const int *tp, int n, int blocks, cudaStream_t s) {
  dwt_rowreg_inv_kernel<G, E><<<blocks, kRegThreads, 0, s>>>(p, tp, n);
}

// Row rounds per block of the forward pass that also gathers the select
// statistics: about 16 K values per block, so that the block's shared digit
// histogram is flushed once per 16 K values.
__host__ __device__ constexpr int rowreg_sel_rounds(int E) { return E == 8 ? 8 : 10; }

// One block: kRegThreads / G rows of the pass found by the tile prefix (SEL:
// rowreg_sel_rounds(E) such row rounds, and the select statistics of every
// value written, merged into the cubelet's once at the end).
template <int G, int E, bool SEL>
__global__ void __launch_bounds__(kRegThreads)
dwt_rowreg_fwd_kernel(const PassDesc *__restrict__ passes, const int *__restrict__ tilePrefix,
                      int nPasses) {
  __shared__ float scaleTab[16];
  __shared__ unsigned hist[SEL ? kSelectBins : 1];
  const int bid = blockIdx.x;
  int lo = 0, hi = nPasses - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tilePrefix[mid] <= bid) lo = mid; else hi = mid - 1;
  }
  const PassDesc &d = passes[lo];
  constexpr int kRows = kRegThreads / G;
  constexpr int kRounds = SEL ? rowreg_sel_rounds(E) : 1;
  const int row0 = (bid - tilePrefix[lo]) * kRounds * kRows;
  const int S = d.steps;
  const bool haar = d.wavelet == WL_HAAR;
  if ((int)threadIdx.x <= S) scaleTab[threadIdx.x] = haar ? 1.0f : lifting_scale(threadIdx.x, S);
  if (SEL) selc::clear_hist<kRegThreads>(hist);
  selc::SelAcc acc{hist};
  __syncthreads();
  for (int r = 0; r < kRounds; r++) {
    const int rr = row0 + r * kRows;
    if (rr >= d.rows) break;  // the same for every thread of the block
    if (haar) rowreg_fwd<G, E, true, SEL>(d, rr, scaleTab, acc);
    else rowreg_fwd<G, E, false, SEL>(d, rr, scaleTab, acc);
  }
  if (SEL) selc::flush<kRegThreads>(acc, d.selHist, d.selState);
}

template <int G, int E = 8>
void launch_g(const PassDesc *p, const int *tp, int n, int blocks, bool sel, cudaStream_t s) {
  if (sel) dwt_rowreg_fwd_kernel<G, E, true><<<blocks, kRegThreads, 0, s>>>(p, tp, n);
  else dwt_rowreg_fwd_kernel<G, E, false><<<blocks, kRegThreads, 0, s>>>(p, tp, n);
}

}  // namespace

// rows of 8 G elements (G = 2 .. 32) or 6 G (G = 8, 16, 32)
static int rowreg_lanes(int L) {
  if (L >= 16 && L <= 256 && (L & (L - 1)) == 0) return L / 8;
  if (L == 48 || L == 96 || L == 192) return L / 6;
  return 0;
}

int dwt_rowreg_rows_per_block(int L, bool sel) {
  const int rows = kRegThreads / rowreg_lanes(L);
  return sel ? rows * rowreg_sel_rounds((L & (L - 1)) ? 6 : 8) : rows;
}

bool dwt_rowreg_fits(int L, int steps) {
  return rowreg_lanes(L) > 0 && steps >= 1 && L % (1 << steps) == 0 &&
         (L & (L - 1) ? (L >> steps) >= 3 : true);
}

int dwt_rowreg_t_rows_per_block(int L) {
  switch (rowreg_lanes(L)) {
    case 2: return TileRows<2>::R;
    case 4: return TileRows<4>::R;
    case 8: return TileRows<8>::R;
    case 16: return TileRows<16>::R;
    default: return TileRows<32>::R;
  }
}

void launch_dwt_rowreg_t(const PassDesc *p, const int *tp, int n, int blocks, int L, int inType,
                         cudaStream_t s) {
  switch (inType) {
    case WL_U8: launch_t_len<uint8_t>(p, tp, n, blocks, L, s); break;
    case WL_U16: launch_t_len<uint16_t>(p, tp, n, blocks, L, s); break;
    case WL_I32: launch_t_len<int32_t>(p, tp, n, blocks, L, s); break;
    default: launch_t_len<float>(p, tp, n, blocks, L, s); break;
  }
}

void launch_dwt_rowreg_inv(const PassDesc *p, const int *tp, int n, int blocks, int L,
                           cudaStream_t s) {
  switch (L) {
    case 16: launch_ig<2>(p, tp, n, blocks, s); break;
    case 32: launch_ig<4>(p, tp, n, blocks, s); break;
    case 48: launch_ig<8, 6>(p, tp, n, blocks, s); break;
    case 64: launch_ig<8>(p, tp, n, blocks, s); break;
    case 96: launch_ig<16, 6>(p, tp, n, blocks, s); break;
    case 128: launch_ig<16>(p, tp, n, blocks, s); break;
    case 192: launch_ig<32, 6>(p, tp, n, blocks, s); break;
    default: launch_ig<32>(p, tp, n, blocks, s); break;
  }
}

void launch_dwt_rowreg_inv_t(const PassDesc *p, const int *tp, int n, int blocks, int L,
                             int outType, cudaStream_t s) {
  switch (outType) {
    case WL_U8: launch_it_len<uint8_t>(p, tp, n, blocks, L, s); break;
    case WL_U16: launch_it_len<uint16_t>(p, tp, n, blocks, L, s); break;
    case WL_I32: launch_it_len<int32_t>(p, tp, n, blocks, L, s); break;
    default: launch_it_len<float>(p, tp, n, blocks, L, s); break;
  }
}

void launch_dwt_rowreg(const PassDesc *p, const int *tp, int n, int blocks, int L, bool sel,
                       cudaStream_t s) {
  switch (L) {
    case 16: launch_g<2>(p, tp, n, blocks, sel, s); break;
    case 32: launch_g<4>(p, tp, n, blocks, sel, s); break;
    case 48: launch_g<8, 6>(p, tp, n, blocks, sel, s); break;
    case 64: launch_g<8>(p, tp, n, blocks, sel, s); break;
    case 96: launch_g<16, 6>(p, tp, n, blocks, sel, s); break;
    case 128: launch_g<16>(p, tp, n, blocks, sel, s); break;
    case 192: launch_g<32, 6>(p, tp, n, blocks, sel, s); break;
    default: launch_g<32>(p, tp, n, blocks, sel, s); break;
  }
}

}  // namespace wl
