// Pieces shared by the two wavelet pass kernels (dwt.cu, dwt_cols.cu): the
// CDF 9/7 lifting constants, the deferred lifting scale, and the conversions
// between the stored data types and float.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace wl {
namespace dwtc {

// lifting factorisation of the CDF 9/7 analysis filters
constexpr float kAlpha = -1.586134342059924f;
constexpr float kBeta = -0.052980118572961f;
constexpr float kGamma = 0.882911075530934f;
constexpr float kDelta = 0.443506852043971f;
constexpr double kK = 1.149604398860241;

constexpr float kInvSqrt2 = 0.70710678118654752440f;

template <typename T> __device__ __forceinline__ float load_as_float(const T *p) {
  return (float)(*p);
}

template <typename T> __device__ __forceinline__ void store_from_float(T *p, float f);
template <> __device__ __forceinline__ void store_from_float<float>(float *p, float f) { *p = f; }
// ByteInputDataUnchanged::floatToByte (wavelet.h:155-163)
template <> __device__ __forceinline__ void store_from_float<uint8_t>(uint8_t *p, float f) {
  *p = f <= 0.f ? (uint8_t)0 : (f >= 255.f ? (uint8_t)255 : (uint8_t)f);
}
// IntInputDataUnchanged::floatToInt (wavelet.h:210-212)
template <> __device__ __forceinline__ void store_from_float<int32_t>(int32_t *p, float f) {
  *p = (int)__fadd_rn(f, 0.5f);
}
template <> __device__ __forceinline__ void store_from_float<uint16_t>(uint16_t *p, float f) {
  int v = (int)__fadd_rn(f, 0.5f);
  *p = (uint16_t)(v < 0 ? 0 : (v > 65535 ? 65535 : v));
}

// per-level store scale of the lifting form: index t < S detail, t == S low
__device__ __forceinline__ float lifting_scale(int t, int S) {
  double k = 1.0;
  if (t == S) { for (int i = 0; i < S; i++) k *= kK; return (float)k; }
  for (int i = 0; i < t; i++) k *= kK;
  return (float)(-k / kK);
}

}  // namespace dwtc
}  // namespace wl
