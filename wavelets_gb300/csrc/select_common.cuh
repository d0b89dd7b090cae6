// First radix-select digit and extremes of a cubelet's final coefficients,
// shared by the stand-alone first select pass (select.cu) and the last
// transform pass that produces the coefficients (dwt_rows.cu), which
// accumulates them while the values are still in registers.
//
// Reference: thresh_cpu / Traverse (thresh_cpu.cc:60-109): min starts at
// FLT_MAX and max at FLT_MIN (the smallest positive float, a reference
// quirk); the first digit is bits 31..20 of |c| (12 bits); the two largest
// |c| are kept for the Lloyd range (test_compress_cpu.cc:419-422).
#pragma once

#include <cfloat>

#include "wl_internal.h"

namespace wl {
namespace selc {

// float -> unsigned with the same order (for atomicMin/Max on signed values)
__device__ __forceinline__ unsigned ord_enc(float f) {
  unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord_dec(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// top-2 merge of multisets {a1,a2} and {b1,b2} (a1>=a2, b1>=b2)
__device__ __forceinline__ void top2_merge(unsigned &a1, unsigned &a2, unsigned b1, unsigned b2) {
  unsigned t1 = max(a1, b1);
  unsigned t2 = max(min(a1, b1), max(a2, b2));
  a1 = t1;
  a2 = t2;
}

// One thread's running statistics; hist is the CTA's shared digit histogram.
struct SelAcc {
  unsigned *hist;
  float mn = FLT_MAX, mx = FLT_MIN;  // floats: a NaN never replaces either
  unsigned a1 = 0u, a2 = 0u;         // bits of the two largest |c|
  __device__ __forceinline__ void visit(float x) {
    const unsigned a = __float_as_uint(x) & 0x7fffffffu;
    atomicAdd(&hist[a >> 20], 1u);
    mn = fminf(mn, x);
    mx = fmaxf(mx, x);
    a2 = max(a2, min(a1, a));  // top2_merge(a1, a2, a, 0)
    a1 = max(a1, a);
  }
};

// Clear the CTA's shared histogram (NT threads; a barrier must follow).
template <int NT> __device__ __forceinline__ void clear_hist(unsigned *hist) {
  for (int i = threadIdx.x; i < kSelectBins; i += NT) hist[i] = 0;
}

// Merge the CTA's statistics into the cubelet's (NT threads, all of them
// calling): histogram bins into gHist, extremes and top two into *st.
template <int NT>
__device__ __forceinline__ void flush(const SelAcc &acc, unsigned *gHist, CubeletState *st) {
  __shared__ unsigned sMin[NT / 32], sMax[NT / 32], sA1[NT / 32], sA2[NT / 32];
  unsigned mn = ord_enc(acc.mn), mx = ord_enc(acc.mx), a1 = acc.a1, a2 = acc.a2;
  for (int off = 16; off > 0; off >>= 1) {
    mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, off));
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    const unsigned b1 = __shfl_xor_sync(0xffffffffu, a1, off);
    const unsigned b2 = __shfl_xor_sync(0xffffffffu, a2, off);
    top2_merge(a1, a2, b1, b2);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { sMin[w] = mn; sMax[w] = mx; sA1[w] = a1; sA2[w] = a2; }
  __syncthreads();  // every thread's histogram counts and warp partials are in
  for (int i = threadIdx.x; i < kSelectBins; i += NT)
    if (acc.hist[i]) atomicAdd(&gHist[i], acc.hist[i]);
  if (threadIdx.x == 0) {
    for (int w2 = 1; w2 < NT / 32; w2++) {
      mn = min(mn, sMin[w2]);
      mx = max(mx, sMax[w2]);
      top2_merge(a1, a2, sA1[w2], sA2[w2]);
    }
    atomicMin(&st->minOrd, mn);
    atomicMax(&st->maxOrd, mx);
    // merge the pair into (absMax, absMax2) with a 64-bit CAS loop
    unsigned long long *pair = reinterpret_cast<unsigned long long *>(&st->absMax);
    unsigned long long old = *pair, assumed;
    do {
      assumed = old;
      unsigned n1 = (unsigned)(assumed & 0xffffffffu), n2 = (unsigned)(assumed >> 32);
      top2_merge(n1, n2, a1, a2);
      const unsigned long long nv = ((unsigned long long)n2 << 32) | n1;
      if (nv == assumed) break;
      old = atomicCAS(pair, assumed, nv);
    } while (old != assumed);
  }
}

}  // namespace selc
}  // namespace wl
