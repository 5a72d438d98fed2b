// rz_bits.h -- exact f64 helpers on the integer pipe, shared by the kernels
// and a host-side test (tests/test_bits.py compiles this header with g++).
// GB300 has a narrow FP64 pipe; these reproduce IEEE results bit-exactly
// with integer instructions where that is cheaper than an FP64 op.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define RZ_HD __host__ __device__ __forceinline__
#else
#define RZ_HD static inline
#endif

namespace rzb {

RZ_HD uint64_t f64_bits(double v) {
  uint64_t b;
  memcpy(&b, &v, 8);
  return b;
}

RZ_HD double bits_f64(uint64_t b) {
  double v;
  memcpy(&v, &b, 8);
  return v;
}

RZ_HD bool nan_bits(uint64_t b) { return (b & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull; }

RZ_HD int clz64(uint64_t n) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)n);
#else
  return __builtin_clzll(n);
#endif
}

// (double)y + 0.5 for 0 <= y < 2^31, exactly (the value is representable)
RZ_HD double half_int(int y) {
  const uint64_t n = 2ull * (unsigned)y + 1ull;
  const int e = 63 - clz64(n);
  return bits_f64(((uint64_t)(1022 + e) << 52) | ((n << (52 - e)) & 0x000FFFFFFFFFFFFFull));
}

// clamp(floor(t), 0, hi) as int, NaN -> 0 (0 <= hi < 2^31)
RZ_HD int floor_clamp(double t, int hi) {
  const uint64_t b = f64_bits(t);
  if (b >> 63) return 0;
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  if (e == 1024) return (b & 0x000FFFFFFFFFFFFFull) ? 0 : hi;
  if (e < 0) return 0;
  if (e >= 31) return hi;
  const uint64_t m = (b & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
  const int64_t f = (int64_t)(m >> (52 - e));
  return f > hi ? hi : (int)f;
}

// clamp(ceil(t), 0, hi) as int, NaN -> 0 (0 <= hi < 2^31)
RZ_HD int ceil_clamp(double t, int hi) {
  const uint64_t b = f64_bits(t);
  if ((b >> 63) || b == 0) return 0;
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  if (e == 1024) return (b & 0x000FFFFFFFFFFFFFull) ? 0 : hi;
  if (e < 0) return hi < 1 ? hi : 1;
  if (e >= 31) return hi;
  const int sh = 52 - e;
  const uint64_t m = (b & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
  const int64_t c = (int64_t)(m >> sh) + ((m & ((1ull << sh) - 1)) != 0);
  return c > hi ? hi : (int)c;
}

// IEEE comparisons of f64 values given as bit patterns
struct BgF64 {
  uint64_t bits;
  bool nan, zero;
};

RZ_HD BgF64 bg_f64(uint64_t bits) {
  return {bits, nan_bits(bits), (bits & 0x7FFFFFFFFFFFFFFFull) == 0};
}

RZ_HD bool eq_bg_f64(uint64_t c, const BgF64& bg) {
  return !bg.nan && (c == bg.bits || (bg.zero && (c & 0x7FFFFFFFFFFFFFFFull) == 0));
}

// IEEE a > b (false when either is NaN; -0 == +0)
RZ_HD bool gt_f64(uint64_t a, uint64_t b) {
  if (nan_bits(a) || nan_bits(b) || ((a | b) & 0x7FFFFFFFFFFFFFFFull) == 0) return false;
  const uint64_t ka = (a >> 63) ? ~a : (a | 0x8000000000000000ull);
  const uint64_t kb = (b >> 63) ? ~b : (b | 0x8000000000000000ull);
  return ka > kb;
}

}  // namespace rzb
