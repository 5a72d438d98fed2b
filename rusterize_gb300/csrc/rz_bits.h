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

// clamp(floor(fl(x + 0.5)), 0, hi) for non-NaN x, without the FP64 add:
// the exact sum is formed on the mantissa and rounded to nearest-even the
// way the add rounds it (only a carry into the next binade can round).
RZ_HD int floor_half_up(double x, int hi) {
  const uint64_t b = f64_bits(x);
  if (b >> 63) return 0;                     // x <= -0: x + 0.5 <= 0.5
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  if (e >= 31) return hi;                    // x >= 2^31 (and +inf)
  if (e <= -3) return 0;                     // x < 0.25
  if (e == -2) return b == 0x3FDFFFFFFFFFFFFFull ? (hi < 1 ? hi : 1) : 0;  // 0.5 - 2^-54 ties up to 1.0
  const uint64_t m = (b & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
  const int s = 52 - e;                      // 22..53
  const uint64_t S = m + (1ull << (s - 1));  // (x + 0.5) * 2^s, exact
  uint64_t f;
  if (S < (1ull << 53)) {
    f = S >> s;
  } else {                                   // next binade: round S/2 to even
    uint64_t h = S >> 1;
    if ((S & 1) && (h & 1)) h += 1;
    f = h >> (s - 1);
  }
  return f > (uint64_t)hi ? hi : (int)f;
}

// clamp(ceil(fl(y - 0.5)), 0, hi), NaN -> 0, without the FP64 subtract:
// for y >= 0.5 the difference is exact (Sterbenz / same-exponent cases).
RZ_HD int ceil_half_down(double y, int hi) {
  const uint64_t b = f64_bits(y);
  if (b >> 63) return 0;
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  if (e == 1024) return (b & 0x000FFFFFFFFFFFFFull) ? 0 : hi;
  if (e >= 31) return hi;
  if (e < -1) return 0;                      // y < 0.5
  if (e == -1) return b == 0x3FE0000000000000ull ? 0 : (hi < 1 ? hi : 1);  // y in [0.5, 1)
  const uint64_t m = (b & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
  const int s = 52 - e;                      // 22..52
  const uint64_t D = m - (1ull << (s - 1));  // (y - 0.5) * 2^s, exact
  const uint64_t c = (D + (1ull << s) - 1) >> s;
  return c > (uint64_t)hi ? hi : (int)c;
}

// |v| >= 1 (infinities included, NaN excluded)
RZ_HD bool abs_ge_one(double v) {
  const uint64_t b = f64_bits(v);
  return ((b >> 52) & 0x7FF) >= 1023 && !nan_bits(b);
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
