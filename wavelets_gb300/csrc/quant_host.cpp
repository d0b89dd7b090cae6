// Host-side parts of the quantizers that must use the host's libm.
// Compiled with -ffp-contract=off so every float expression below rounds
// after each operation, as the reference's x86-64 build does.
//
// QuantLog (quant.h:326-439) maps |x| through the host's logf; the device has
// no logf that agrees with it bit for bit (glibc logf is not correctly
// rounded), so the device never evaluates the log quantizer's formula.
// Instead, once a cubelet's threshold and largest |coefficient| are known,
// this file evaluates the reference's own expression with the host logf to
// find, for every bin, the smallest float at which that bin starts.  The
// quantized value is a non-decreasing function of |x| (logf is monotone), so
// counting the boundaries at or below |x| on the device reproduces the
// reference's bin exactly.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "wl_internal.h"

namespace wl {
namespace {

struct RefLog {  // QuantLog::init / quant (quant.h:337-407), host float math
  int binCount;
  float threshold, negScale, negInvScale, negOffset, posScale, posInvScale, posOffset;
  void init(int b, float t, float maxVal) {
    binCount = b;
    threshold = t;
    int negBinCount = (binCount - 1) / 2;
    negScale = (negBinCount - 1) / logf(maxVal / threshold);
    negInvScale = 1 / negScale;
    negOffset = 1 - negScale * logf(threshold);
    int posBinCount = binCount / 2;
    posScale = (posBinCount - 1) / logf(maxVal / threshold);
    posInvScale = 1 / posScale;
    posOffset = 1 - posScale * logf(threshold);
  }
  int quant(float x) const {
    int zeroBin = (binCount - 1) >> 1;
    if (x < 0) {
      x = -x;
      if (x <= threshold) return zeroBin;
      x = zeroBin - negScale * logf(x) - negOffset;
      if (x < 0) return 0;
      return (int)(x + 0.5f);
    }
    if (x <= threshold) return zeroBin;
    x = zeroBin + posScale * logf(x) + posOffset;
    if (x >= binCount) return binCount - 1;
    return (int)(x + 0.5f);
  }
  float dequant(int x) const {
    int zeroBin = (binCount - 1) >> 1;
    float sign, invScale, offset;
    if (x < zeroBin) { sign = -1; offset = negOffset; invScale = negInvScale; }
    else { sign = 1; offset = posOffset; invScale = posInvScale; }
    if (x == zeroBin) return 0;
    return sign * expf((sign * (x - zeroBin) - offset) * invScale);
  }
};

inline float bits_to_float(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
inline uint32_t float_to_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

// smallest u in [lo, hi] with pred(u) true, given pred monotone and pred(hi)
template <class P> uint32_t first_true(uint32_t lo, uint32_t hi, P pred) {
  while (lo < hi) {
    uint32_t mid = lo + (hi - lo) / 2;
    if (pred(mid)) hi = mid; else lo = mid + 1;
  }
  return lo;
}

// Same, but first narrow [lo, hi] around a guess (saves logf calls).  pred
// must be true at hi.
template <class P> uint32_t first_true_guess(uint32_t lo, uint32_t hi, double guess, P pred) {
  if (!(guess > 0) || !std::isfinite(guess)) return first_true(lo, hi, pred);
  const uint32_t ug = float_to_bits((float)guess);
  if (ug <= lo || ug >= hi) return first_true(lo, hi, pred);
  // the double-precision guess is usually within a few ulps of the answer
  uint32_t step = 4, a, b;
  for (;;) {  // a: lo or a point where pred is false
    a = ug - lo > step ? ug - step : lo;
    if (a == lo || !pred(a)) break;
    step *= 8;
  }
  step = 4;
  for (;;) {  // b: hi or a point where pred is true
    b = hi - ug > step ? ug + step : hi;
    if (b == hi || pred(b)) break;
    step *= 8;
  }
  return first_true(a, b, pred);
}

}  // namespace

// Table layout (consumed by quant_value in quant.cu):
//   lowBin  = bin of the smallest float above the threshold,
//   highNeg = bin of the negative of that float,
//   bounds[0 .. nPos)            P[m] = min x > thr with bin(x)  >= lowBin+1+m
//   bounds[nPos .. nPos+nNeg)    N[m] = min y > thr with bin(-y) <= highNeg-1-m
void log_quant_table(int binCount, float threshold, float maxVal, LogTable &t) {
  RefLog q;
  q.init(binCount, threshold, maxVal);
  t.negScale = q.negScale;
  t.negOffset = q.negOffset;
  t.posScale = q.posScale;
  t.posOffset = q.posOffset;
  const uint32_t inf = 0x7f800000u;
  const uint32_t lo = float_to_bits(threshold) + 1;  // threshold > 0
  const float above = bits_to_float(lo);
  t.lowBin = q.quant(above);
  t.highNeg = q.quant(-above);
  t.bounds.clear();
  const int zb = (binCount - 1) >> 1;
  // positive side
  uint32_t prev = lo;
  for (int j = t.lowBin + 1; j <= binCount - 1; j++) {
    // guess: bin j starts where zb + posScale*ln x + posOffset = j - 0.5
    const double guess = exp((j - 0.5 - zb - (double)q.posOffset) / (double)q.posScale);
    uint32_t u = first_true_guess(prev, inf, guess,
                                  [&](uint32_t v) { return q.quant(bits_to_float(v)) >= j; });
    t.bounds.push_back(bits_to_float(u));
    prev = u;
  }
  t.nPos = (int)t.bounds.size();
  prev = lo;
  for (int j = t.highNeg - 1; j >= 0; j--) {
    const double guess = exp((zb - (j + 0.5) - (double)q.negOffset) / (double)q.negScale);
    uint32_t u = first_true_guess(prev, inf, guess,
                                  [&](uint32_t v) { return q.quant(-bits_to_float(v)) <= j; });
    t.bounds.push_back(bits_to_float(u));
    prev = u;
  }
  t.nNeg = (int)t.bounds.size() - t.nPos;
}

// Dequantized value of every bin (QuantUniform::dequant quant.h:278-291,
// QuantLog::dequant :409-438, QuantCodebook::dequant :552-556).
void dequant_values(int quantAlg, int binCount, float threshold, float maxVal,
                    const float *codebookValues, float *out) {
  if (quantAlg == WL_LOG) {
    RefLog q;
    q.init(binCount, threshold, maxVal);
    for (int i = 0; i < binCount; i++) out[i] = q.dequant(i);
    return;
  }
  if (quantAlg == WL_UNIFORM) {
    int negBinCount = (binCount - 1) / 2, posBinCount = binCount / 2;
    float negScale = (negBinCount - 1) / (maxVal - threshold);
    float posScale = (posBinCount - 1) / (maxVal - threshold);
    float negInvScale = negScale == 0 ? 0 : 1 / negScale;
    float posInvScale = posScale == 0 ? 0 : 1 / posScale;
    float negOffset = 1 - threshold * negScale, posOffset = 1 - threshold * posScale;
    int zeroBin = (binCount - 1) >> 1;
    for (int x = 0; x < binCount; x++) {
      if (x < zeroBin) out[x] = (x - 0.5f + negOffset - zeroBin) * negInvScale;
      else if (x > zeroBin) out[x] = (x + 0.5f - posOffset - zeroBin) * posInvScale;
      else out[x] = 0;
    }
    return;
  }
  for (int i = 0; i < binCount; i++) out[i] = codebookValues ? codebookValues[i] : 0.f;
}

}  // namespace wl
