"""The engine's integer-pipe replacements of f64 floor/ceil/conversions
(rusterize_gb300/csrc/rz_bits.h) against libm, on the host: the header is
compiled with g++ into a small checker and run on seeded and edge values."""

import subprocess
import tempfile
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "rusterize_gb300" / "csrc"

CHECKER = r"""
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <random>
#include "rz_bits.h"

static int ref_floor_clamp(double t, int hi) {
  double f = std::floor(t);
  if (!(f > 0.0)) return 0;           // NaN, negative, zero
  if (f >= (double)hi) return hi;
  return (int)f;
}
static int ref_ceil_clamp(double t, int hi) {
  double c = std::ceil(t);
  if (!(c > 0.0)) return 0;
  if (c >= (double)hi) return hi;
  return (int)c;
}

int main() {
  long bad = 0, n = 0;
  std::mt19937_64 rng(12345);
  const int his[] = {0, 1, 7, 1000, 20000, 40000, 2147483646};
  auto check = [&](double t) {
    for (int hi : his) {
      ++n;
      if (rzb::floor_clamp(t, hi) != ref_floor_clamp(t, hi)) { if (bad < 5) printf("floor %.17g hi=%d\n", t, hi); ++bad; }
      if (rzb::ceil_clamp(t, hi) != ref_ceil_clamp(t, hi)) { if (bad < 5) printf("ceil %.17g hi=%d\n", t, hi); ++bad; }
    }
  };
  const double specials[] = {0.0, -0.0, 0.5, -0.5, 1.0, -1.0, 0.49999999999999994, 0.5000000000000001,
                             1e-320, -1e-320, 2147483647.0, 2147483648.0, 2147483647.5, 4e9, -4e9, 1e300,
                             INFINITY, -INFINITY, NAN, -NAN, 19999.5, 19999.999999999996, 20000.0, 39999.5};
  for (double t : specials) check(t);
  for (int i = 0; i < 2000000; ++i) {
    uint64_t b = rng();
    double t;
    switch (i % 4) {
      case 0: std::memcpy(&t, &b, 8); break;                                   // any bit pattern
      case 1: t = (double)(int64_t)(b % 100000) / 7.0 - 100.0; break;           // moderate values
      case 2: t = (double)(b % 50000) + (i & 1 ? 0.5 : -0.5); break;            // exact halves
      default: t = std::nextafter((double)(b % 50000), (i & 2) ? 1e9 : -1e9);  // next to integers
    }
    check(t);
  }
  for (int y = 0; y < 5000000; ++y) {
    ++n;
    if (rzb::half_int(y) != (double)y + 0.5) { if (bad < 5) printf("half %d\n", y); ++bad; }
  }
  const int big[] = {2147483646, 2147483647, 1 << 30, (1 << 30) + 1};
  for (int y : big) { ++n; if (rzb::half_int(y) != (double)y + 0.5) ++bad; }
  // the +-0.5 roundings used by the scanline code
  auto half_check = [&](double t) {
    for (int hi : his) {
      ++n;
      if (!std::isnan(t) && rzb::floor_half_up(t, hi) != ref_floor_clamp(t + 0.5, hi)) {
        if (bad < 5) printf("floor_half_up %.17g hi=%d\n", t, hi); ++bad;
      }
      if (rzb::ceil_half_down(t, hi) != ref_ceil_clamp(t - 0.5, hi)) {
        if (bad < 5) printf("ceil_half_down %.17g hi=%d\n", t, hi); ++bad;
      }
    }
  };
  for (double t : specials) half_check(t);
  for (int k = -60; k < 40; ++k) {           // every binade edge and its neighbours
    double p = std::ldexp(1.0, k);
    for (double c : {p, p - 0.5, p + 0.5, p - 1.0}) {
      double v = c;
      for (int j = 0; j < 6; ++j) { half_check(v); half_check(-v); v = std::nextafter(v, 0.0); }
      v = c;
      for (int j = 0; j < 6; ++j) { half_check(v); v = std::nextafter(v, 1e300); }
    }
  }
  for (int i = 0; i < 2000000; ++i) {
    uint64_t b = rng();
    double t;
    switch (i % 4) {
      case 0: std::memcpy(&t, &b, 8); break;
      case 1: t = (double)(int64_t)(b % 10000000) / 4096.0 - 100.0; break;
      case 2: t = std::nextafter((double)(b % 50000) + 0.5, (i & 1) ? 1e9 : -1e9); break;
      default: t = std::ldexp((double)(b >> 11), -(int)(b % 60)); break;
    }
    half_check(t);
  }
  // f64 comparisons on bit patterns vs IEEE
  const double cmpv[] = {0.0, -0.0, 1.0, -1.0, 2.5, -2.5, 1e-310, -1e-310, INFINITY, -INFINITY, NAN, -NAN,
                         1e308, -1e308, 3.0, 0.1};
  auto cmp_check = [&](double a, double b) {
    uint64_t ab = rzb::f64_bits(a), bb = rzb::f64_bits(b);
    ++n;
    if (rzb::gt_f64(ab, bb) != (a > b)) { if (bad < 5) printf("gt %.17g %.17g\n", a, b); ++bad; }
    rzb::BgF64 bg = rzb::bg_f64(bb);
    if (rzb::eq_bg_f64(ab, bg) != (a == b)) { if (bad < 5) printf("eq %.17g %.17g\n", a, b); ++bad; }
  };
  for (double a : cmpv) for (double b : cmpv) cmp_check(a, b);
  for (double a : cmpv) { ++n; if (rzb::abs_ge_one(a) != (std::fabs(a) >= 1.0)) { if (bad < 5) printf("abs_ge_one %g\n", a); ++bad; } }
  for (int i = 0; i < 1000000; ++i) {
    uint64_t x = rng(), y = (i & 1) ? rng() : x ^ (rng() & 0xF);
    double a, b;
    std::memcpy(&a, &x, 8);
    std::memcpy(&b, &y, 8);
    cmp_check(a, b);
  }
  printf("%ld %ld\n", n, bad);
  return bad != 0;
}
"""


def test_integer_pipe_f64_helpers_match_libm():
    with tempfile.TemporaryDirectory() as d:
        src = Path(d) / "check.cpp"
        exe = Path(d) / "check"
        src.write_text(CHECKER)
        res = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}", str(src), "-o", str(exe)],
                             capture_output=True, text=True)
        if res.returncode != 0:
            pytest.fail("checker did not compile:\n" + res.stderr)
        run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
        assert run.returncode == 0, run.stdout
