"""Host-side checks of the record-scratch sizing (rusterize_gb300/csrc/rz_layout.h)
at its boundary sizes: the arrays of one pass never overlap, stay inside the
buffer, start on the alignment of their element type (8 bytes for the
sorted uint2 records), and every record index
and bucket offset fits in 32 bits.  The header is compiled with g++ into a
small checker that prints one line per case."""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "rusterize_gb300" / "csrc"

CHECKER = r"""
#include <cstdio>
#include <cstdint>
#include <initializer_list>
#include "rz_layout.h"
using namespace rzl;

static int bad = 0;
#define CHECK(c, ...) do { if (!(c)) { ++bad; std::printf("FAIL " __VA_ARGS__); std::printf("\n"); } } while (0)

static void check_layout(uint64_t bytes) {
  const RecordLayout L = record_layout(bytes);
  CHECK(L.cap % 2 == 0, "cap odd for %llu", (unsigned long long)bytes);
  CHECK(L.cap <= RECORD_CAP_MAX, "cap above 32-bit limit for %llu", (unsigned long long)bytes);
  CHECK(L.end <= bytes || L.cap == 0, "layout end %llu beyond buffer %llu", (unsigned long long)L.end,
        (unsigned long long)bytes);
  CHECK(L.end + RECORD_PAD <= bytes || L.cap == 0, "no pad for %llu", (unsigned long long)bytes);
  // arrays in order, each cap elements long
  CHECK(L.off_part == L.off_wid + 4 * L.cap && L.off_mask == L.off_part + 4 * L.cap, "u32 arrays overlap");
  CHECK(L.off_sorted == L.off_mask + 4 * L.cap && L.end == L.off_sorted + 8 * L.cap, "sorted overlaps");
  CHECK(L.off_sorted % 8 == 0, "alignment for %llu", (unsigned long long)bytes);
  // the largest record index and a bucket offset one past it fit in 32 bits
  CHECK(L.cap == 0 || L.cap - 1 <= 0xFFFFFFFFull, "index width");
  CHECK(L.cap <= 0xFFFFFFFFull, "offset width");
  // the full buffer is used: one more record would not fit or pass the limit
  const uint64_t next = L.cap + 2;
  CHECK(record_bytes_for(next) > bytes || next > RECORD_CAP_MAX, "buffer %llu underused (cap %llu)",
        (unsigned long long)bytes, (unsigned long long)L.cap);
}

int main() {
  const uint64_t base[] = {0, 1, 15, 16, 17, 28, 44, 71, 72, 73, 1000, 1ull << 20, 64ull << 20, 1ull << 32,
                           RECORD_BYTES * 0xFFFFFFF0ull + 15, RECORD_BYTES * 0xFFFFFFF0ull + 16,
                           RECORD_BYTES * 0xFFFFFFF0ull + 17, RECORD_BYTES * 0xFFFFFFF2ull + 16,
                           RECORD_BYTES * 0x100000000ull + 16, 1ull << 40, 1ull << 44};
  for (uint64_t b : base)
    for (int d = -40; d <= 40; ++d) {
      if ((int64_t)b + d < 0) continue;
      check_layout(b + d);
    }
  // requests and regrowth
  for (uint64_t want : {0ull, 1ull, 2ull, 3ull, 1ull << 31, 0xFFFFFFEFull, 0xFFFFFFF0ull, 0xFFFFFFF1ull,
                        0xFFFFFFFFull, 1ull << 33}) {
    const uint64_t c = record_cap_request(want);
    CHECK(c % 2 == 0 && c <= RECORD_CAP_MAX, "request %llu", (unsigned long long)want);
    CHECK(c >= (want < RECORD_CAP_MAX ? want - (want & 1) : RECORD_CAP_MAX), "request shrank %llu",
          (unsigned long long)want);
  }
  for (uint64_t count : {1ull, 1000ull, 1ull << 31, 0xFFFFFC00ull, 0xFFFFFFEFull, 0xFFFFFFF0ull}) {
    const uint64_t c = record_cap_regrow(count);
    CHECK(c >= count && c <= RECORD_CAP_MAX && c % 2 == 0, "regrow %llu -> %llu", (unsigned long long)count,
          (unsigned long long)c);
  }
  for (uint64_t count : {0xFFFFFFF1ull, 0x100000000ull, 1ull << 40})
    CHECK(record_cap_regrow(count) == 0, "regrow beyond the limit %llu", (unsigned long long)count);
  std::printf("checked, %d failures\n", bad);
  return bad != 0;
}
"""


def test_record_layout_boundaries(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "check_layout.cpp"
    src.write_text(CHECKER)
    exe = tmp_path / "check_layout"
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", str(CSRC), str(src), "-o", str(exe)], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout[-4000:]
    assert "0 failures" in res.stdout
