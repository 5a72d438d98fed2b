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
RZ_HD float f32_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
RZ_HD float f32_floor(float a) { return floorf(a); }
RZ_HD float f32_abs(float a) { return fabsf(a); }
RZ_HD float f32_inf() { return __int_as_float(0x7F800000); }
// a / b within 2 ulp (|b| in [2^-126, 2^126])
RZ_HD float f32_div_fast(float a, float b) { return __fdividef(a, b); }
#else
RZ_HD float f32_add(float a, float b) { return a + b; }
RZ_HD float f32_sub(float a, float b) { return a - b; }
RZ_HD float f32_mul(float a, float b) { return a * b; }
RZ_HD float f32_div(float a, float b) { return a / b; }
RZ_HD float f32_fma(float a, float b, float c) { return __builtin_fmaf(a, b, c); }
RZ_HD float f32_floor(float a) { return __builtin_floorf(a); }
RZ_HD float f32_abs(float a) { return __builtin_fabsf(a); }
RZ_HD float f32_inf() { return __builtin_inff(); }
// Host stand-in for the device's 2-ulp division: the correctly rounded
// quotient moved by up to 2 ulp (chosen from the operand bits), so host tests
// exercise the error bound with the device's worst case.
RZ_HD float f32_div_fast(float a, float b) {
  float q = a / b;
  uint32_t ua, ub;
  memcpy(&ua, &a, 4);
  memcpy(&ub, &b, 4);
  const int k = (int)(((ua * 2654435761u) ^ (ub * 40503u)) >> 29) % 5 - 2;  // -2..2
  for (int i = 0; i < (k < 0 ? -k : k); ++i) q = __builtin_nextafterf(q, k < 0 ? -__builtin_inff() : __builtin_inff());
  return q;
}
#endif

// Largest pixel coordinate magnitude handled by the filter (2^22): integer
// parts and their differences stay exact in FP32 and every crossing value
// stays below 2^23, where FP32 still resolves fractions.
constexpr int CROSS_COORD_LOG2 = 22;

RZ_HD uint32_t funnel_r(uint32_t lo, uint32_t hi, int sh) {  // low word of (hi:lo) >> sh, 0 <= sh < 32
#if defined(__CUDA_ARCH__)
  return __funnelshift_r(lo, hi, (unsigned)sh);
#else
  return (uint32_t)((((uint64_t)hi << 32) | lo) >> sh);
#endif
}

// c ~ ci + cf with |c - (ci + cf)| < 2^-23, cf in [0, 1) and ci = floor(c)
// (or floor(c) + 1 for a negative c within 2^-24 below an integer); false
// for |c| >= 2^22, infinities and NaN.  The integer part of |c| and the top
// 24 bits of its fraction (truncated: error < 2^-24) come from funnel shifts
// of the significand's two 32-bit halves; a negative c becomes
// -(int part) - 1 and 1 - fraction.  *f24 (when given) receives the 24
// fraction bits of a non-negative c, before the sign is applied.
RZ_HD bool split_px(double c, int& ci, float& cf, uint32_t* f24_out = nullptr) {
  const uint64_t b = f64_bits(c);
  const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  const int E = (int)((hi >> 20) & 0x7FF);
  if (E >= 1023 + CROSS_COORD_LOG2) {
    ci = 0;
    cf = 0.0f;
    return false;
  }
  const uint32_t mh = (hi & 0xFFFFFu) | 0x100000u;  // significand bits 52..32
  uint32_t ip = 0, f24 = 0;
  if (E >= 1023) {  // 1 <= |c| < 2^22: the binary point sits s = 52 - e bits up, s in [31, 52]
    const int sh = 1075 - E;
    ip = sh >= 32 ? mh >> (sh - 32) : funnel_r(lo, mh, sh);
    f24 = funnel_r(lo, mh, sh - 24) & 0xFFFFFFu;
  } else if (E >= 1023 - 30) {  // 2^-30 <= |c| < 1: |c| * 2^24 = significand >> (28 - e)
    const int t = 1051 - E;     // in [29, 58]
    f24 = t < 32 ? funnel_r(lo, mh, t) : mh >> (t - 32);
  }                             // smaller magnitudes (and zero) split to 0 + 0
  if (f24_out) *f24_out = f24;
  if (hi >> 31) {
    ci = f24 ? -(int)ip - 1 : -(int)ip;
    f24 = f24 ? (1u << 24) - f24 : 0u;
  } else {
    ci = (int)ip;
  }
  cf = (float)f24 * 5.9604644775390625e-08f;  // * 2^-24, exact
  return true;
}

// clamp(ceil(fl(y - 0.5)), 0, hi) from y's split: for 0 <= y < 2^22 the
// subtraction is exact and the ceiling is yi or yi + 1 depending on whether
// the fraction is below or above one half; a fraction within 2^-24 of one
// half (or a negative / unsplittable y) takes the exact path.
RZ_HD int ceil_half_down_split(double y, bool ok, int yi, uint32_t f24, int hi) {
  if (ok && yi >= 0 && f24 != (1u << 23)) {
    const int r = yi + (f24 > (1u << 23) ? 1 : 0);
    return r > hi ? hi : r;
  }
  return ceil_half_down(y, hi);
}

// One edge in the filter's frame, for the crossings of rows row0, row0 + 1,
// ... of one scanline window.  e0 = +inf marks an edge whose crossings all
// take the FP64 sequence (non-finite or huge coordinates, or a nearly
// horizontal edge: those have at most one crossing).
struct CrossEdge {
  int xi;      // floor of x_top (split)
  float d0;    // (row0 + 0.5) - y_top
  float a;     // dxdy
  float c0;    // (x_top - xi) + 0.5
  float e0;    // error bound E of every crossing of the edge
  float e1;    // 1 - E
};

// Error of a crossing (row row0 + j, value t = fl(fl(d0 + j) * a + c0) with
// one FMA rounding, relative to xi), in units of u = 2^-24, the FP32 unit
// roundoff (split errors < 2u, the slope division < 4u relative, |d| <= dy
// because the row is a crossing row of the edge):
//   offset d:          2.5 + 2|d|          slope a: (5 + |dx| + 5|a| + |a dy|) / dy + 4|a|
//   |d a - D* M*| <=   5 + 7.5|a| + 2|dx| + 6|p|      c0, the split of x, t: 3 + |t|
//   the FP64 sequence and its +0.5 (|x| < 2^23):       0.5
// and since the crossing lies between the edge's end points, |p| <= |dx|
// and |t| <= |dx| + 1.5, so the total is below 28 + 7.5|a| + 15|dx|.  The
// bound used, 2^-20 (32 + 8|a| + 16|dx|) = u (512 + 128|a| + 256|dx|), is
// 16 times larger.
RZ_HD void cross_edge_frame(int xti, float xtf, int yti, float ytf, int xbi, float xbf, int ybi, float ybf, bool ok,
                            int row0, CrossEdge& e) {
  e.xi = xti;
  // integer parts differ by < 2^23: exact in FP32
  const float dx = f32_add((float)(xbi - xti), f32_sub(xbf, xtf));
  const float dy = f32_add((float)(ybi - yti), f32_sub(ybf, ytf));
  ok = ok && dy >= 0.00390625f;  // y_bot - y_top >= 2^-8
  e.a = ok ? f32_div_fast(dx, dy) : 0.0f;
  e.d0 = f32_add((float)(row0 - yti), f32_sub(0.5f, ytf));
  e.c0 = f32_add(xtf, 0.5f);
  const float E = f32_mul(9.5367431640625e-07f,  // 2^-20
                          f32_add(f32_add(32.0f, f32_mul(8.0f, f32_abs(e.a))), f32_mul(16.0f, f32_abs(dx))));
  e.e0 = ok ? E : f32_inf();
  e.e1 = ok ? f32_sub(1.0f, E) : -f32_inf();
}

RZ_HD void cross_edge_setup(double xt, double yt, double xb, double yb, int row0, CrossEdge& e) {
  int xti, yti, xbi, ybi;
  float xtf, ytf, xbf, ybf;
  bool ok = split_px(xt, xti, xtf);
  ok = split_px(yt, yti, ytf) && ok;
  ok = split_px(xb, xbi, xbf) && ok;
  ok = split_px(yb, ybi, ybf) && ok;
  cross_edge_frame(xti, xtf, yti, ytf, xbi, xbf, ybi, ybf, ok, row0, e);
}

// Boundary clamp(floor(fl(x + 0.5)), 0, ncols) of the crossing with the
// centre of row row0 + j, or -1 when the filter cannot decide it.  The row
// must be a crossing row of the edge (ceil(y_top - 0.5) <= row <
// ceil(y_bot - 0.5)) and j < 2^24.
RZ_HD int cross_fast(const CrossEdge& e, int j, int ncols) {
  const float d = f32_add(e.d0, (float)j);
  const float t = f32_fma(d, e.a, e.c0);
  const float fl = f32_floor(t);
  const float fr = f32_sub(t, fl);
  if (!(fr >= e.e0 && fr <= e.e1)) return -1;
  const int bnd = e.xi + (int)fl;
  return bnd < 0 ? 0 : (bnd > ncols ? ncols : bnd);
}

}  // namespace rzb
