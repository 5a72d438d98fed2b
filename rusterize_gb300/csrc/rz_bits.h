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

// The bit pattern of v.  On the device it is taken by an opaque move, so
// the compiler cannot fold the integer tests below back into FP64 compare
// instructions (GB300's FP64 unit retires 2 lanes per clock per SM; the
// integer pipe 64).
RZ_HD uint64_t f64_bits(double v) {
#if defined(__CUDA_ARCH__)
  uint64_t b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(v));
  return b;
#else
  uint64_t b;
  memcpy(&b, &v, 8);
  return b;
#endif
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

// ---- filtered scanline crossings -------------------------------------------
// A polygon crossing is x = x_top + ((row + 0.5) - y_top) * dxdy in FP64 with
// dxdy = (x_bot - x_top) / (y_bot - y_top) (three correctly rounded ops per
// crossing and a division per edge), and only its pixel boundary
// clamp(floor(fl(x + 0.5)), 0, ncols) is used.  The boundary is decided here
// with FP32 arithmetic in a frame anchored at the edge's integer pixel
// origin, together with a rigorous bound E on the distance between the FP32
// value and the FP64 one; when the FP32 value lies within E of a pixel
// boundary the caller recomputes that crossing with the FP64 sequence.  This
// is a static floating-point filter (Fortune and Van Wyk, "Static analysis
// yields efficient exact integer arithmetic for computational geometry",
// ACM TOG 15(3), 1996; Shewchuk, "Adaptive precision floating-point
// arithmetic and fast robust geometric predicates", DCG 18, 1997): results
// are bit-identical to the FP64 sequence, only the work differs.

#if defined(__CUDA_ARCH__)
RZ_HD float f32_add(float a, float b) { return __fadd_rn(a, b); }
RZ_HD float f32_sub(float a, float b) { return __fsub_rn(a, b); }
RZ_HD float f32_mul(float a, float b) { return __fmul_rn(a, b); }
RZ_HD float f32_div(float a, float b) { return __fdiv_rn(a, b); }
RZ_HD float f32_floor(float a) { return floorf(a); }
RZ_HD float f32_abs(float a) { return fabsf(a); }
RZ_HD float f32_inf() { return __int_as_float(0x7F800000); }
#else
RZ_HD float f32_add(float a, float b) { return a + b; }
RZ_HD float f32_sub(float a, float b) { return a - b; }
RZ_HD float f32_mul(float a, float b) { return a * b; }
RZ_HD float f32_div(float a, float b) { return a / b; }
RZ_HD float f32_floor(float a) { return __builtin_floorf(a); }
RZ_HD float f32_abs(float a) { return __builtin_fabsf(a); }
RZ_HD float f32_inf() { return __builtin_inff(); }
#endif

// Largest pixel coordinate magnitude handled by the filter (2^22): integer
// parts and their differences stay exact in FP32 and every crossing value
// stays below 2^23, where FP32 still resolves fractions.
constexpr int CROSS_COORD_LOG2 = 22;
constexpr float CROSS_ULP = 2.384185791015625e-07f;  // 2^-22, the unit of the bound

// c ~ ci + cf with |c - (ci + cf)| < 2^-23, cf in [0, 1) and ci = floor(c)
// (or floor(c) + 1 for a negative c within 2^-40 below an integer); false
// for |c| >= 2^22, infinities and NaN.  |c| is truncated to a fixed-point
// number with 40 fraction bits (error < 2^-40) and given c's sign; its
// integer part (arithmetic shift) is ci and its top 24 fraction bits become
// cf (error < 2^-24).
RZ_HD bool split_px(double c, int& ci, float& cf) {
  const uint64_t b = f64_bits(c);
  const int E = (int)((b >> 52) & 0x7FF);
  if (E >= 1023 + CROSS_COORD_LOG2) {
    ci = 0;
    cf = 0.0f;
    return false;
  }
  const uint64_t m = (b & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = E - 1023 - 12;  // |c| * 2^40 = m * 2^sh
  uint64_t q = 0;
  if (E != 0) {
    if (sh >= 0) q = m << sh;
    else if (sh > -64) q = m >> (-sh);
  }
  const int64_t sq = (b >> 63) ? -(int64_t)q : (int64_t)q;
  ci = (int)(sq >> 40);  // arithmetic shift: floor
  const uint32_t f24 = (uint32_t)(((uint64_t)sq & ((1ull << 40) - 1)) >> 16);
  cf = (float)f24 * 5.9604644775390625e-08f;  // * 2^-24, exact
  return true;
}

// One edge in the filter's frame.  ee = +inf marks an edge whose crossings
// all take the FP64 sequence (non-finite or huge coordinates, or a nearly
// horizontal edge: those have at most one crossing).
struct CrossEdge {
  int xi, yi;   // floor of x_top, y_top
  float xf;     // x_top - xi
  float g0;     // 0.5 - (y_top - yi)
  float a;      // dxdy
  float ee;     // per-edge part of the error bound, in units of 2^-22
};

// The edge from top end (xti + xtf, yti + ytf) to bottom end (xbi + xbf,
// ybi + ybf), each given by split_px; `ok` is false when a split failed.
RZ_HD void cross_edge_frame(int xti, float xtf, int yti, float ytf, int xbi, float xbf, int ybi, float ybf, bool ok,
                            CrossEdge& e) {
  e.xi = xti;
  e.yi = yti;
  e.xf = xtf;
  // integer parts differ by < 2^23: exact in FP32
  const float dx = f32_add((float)(xbi - xti), f32_sub(xbf, xtf));
  const float dy = f32_add((float)(ybi - yti), f32_sub(ybf, ytf));
  ok = ok && dy >= 0.00390625f;  // y_bot - y_top >= 2^-8
  e.a = ok ? f32_div(dx, dy) : 0.0f;
  e.g0 = f32_sub(0.5f, ytf);
  // error of the crossing, in units of 2^-24 (u = 2^-24 is the FP32 unit
  // roundoff; the split errors are < 2u):
  //   frame offsets and the f32 crossing:   <= 7.5 + 7.5|a| + 2|d a| + |dx| + |a dy| + |p| + |s| + |t|
  //   the FP64 sequence and its +0.5:        <= 0.5 for |x| < 2^23
  // with |d| <= dy, |d a| ~ |p| and |a dy| ~ |dx| this is below
  // 8 + 8|a| + 2|dx| + 3|p| + 2|t|; the bound below uses 2^-22 units (4x).
  e.ee = ok ? f32_add(f32_add(8.0f, f32_mul(8.0f, f32_abs(e.a))), f32_mul(2.0f, f32_abs(dx))) : f32_inf();
}

RZ_HD void cross_edge_setup(double xt, double yt, double xb, double yb, CrossEdge& e) {
  int xti, yti, xbi, ybi;
  float xtf, ytf, xbf, ybf;
  bool ok = split_px(xt, xti, xtf);
  ok = split_px(yt, yti, ytf) && ok;
  ok = split_px(xb, xbi, xbf) && ok;
  ok = split_px(yb, ybi, ybf) && ok;
  cross_edge_frame(xti, xtf, yti, ytf, xbi, xbf, ybi, ybf, ok, e);
}

// Boundary clamp(floor(fl(x + 0.5)), 0, ncols) of the crossing with the
// centre of row r, or -1 when the filter cannot decide it.  r must be a
// crossing row of the edge (ceil(y_top - 0.5) <= r < ceil(y_bot - 0.5)).
RZ_HD int cross_fast(const CrossEdge& e, int r, int ncols) {
  const float d = f32_add((float)(r - e.yi), e.g0);
  const float p = f32_mul(d, e.a);
  const float s = f32_add(e.xf, p);
  const float t = f32_add(s, 0.5f);
  const float fl = f32_floor(t);
  const float fr = f32_sub(t, fl);
  const float E = f32_mul(CROSS_ULP, f32_add(e.ee, f32_add(f32_mul(3.0f, f32_abs(p)), f32_mul(2.0f, f32_abs(t)))));
  if (!(fr >= E && fr <= f32_sub(1.0f, E))) return -1;
  const int bnd = e.xi + (int)fl;
  return bnd < 0 ? 0 : (bnd > ncols ? ncols : bnd);
}

}  // namespace rzb
