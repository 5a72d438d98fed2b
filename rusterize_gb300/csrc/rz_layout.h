// rz_layout.h -- host-side sizing of the engine's record scratch.  Plain
// C++ (no CUDA), so tests/test_layout.py compiles it with g++ and checks the
// arithmetic at its boundary sizes.
//
// One pass of span generation writes coverage records into one buffer cut
// into four arrays of `cap` entries each:
//   wid[cap]     u32  word id of the record
//   part[cap]    u32  part | flags
//   mask[cap]    u32  covered pixels of the word
//   sorted[cap]  u64  {part | word << 27 | flags, mask} grouped by bucket (uint2)
// 20 bytes per record (RECORD_BYTES).  Record counts and bucket offsets are
// 32-bit on the device, so cap never exceeds RECORD_CAP_MAX, and cap is even
// so that `sorted` starts on an 8-byte boundary.
#pragma once

#include <cstddef>
#include <cstdint>

namespace rzl {

constexpr uint64_t RECORD_BYTES = 20;
constexpr uint64_t RECORD_CAP_MAX = 0xFFFFFFF0ull;  // < 2^32: every record index and bucket offset fits in 32 bits
constexpr uint64_t RECORD_PAD = 16;                 // slack after the last array

struct RecordLayout {
  uint64_t cap = 0;  // records per array (even, <= RECORD_CAP_MAX)
  uint64_t off_wid = 0, off_part = 0, off_mask = 0, off_sorted = 0;
  uint64_t end = 0;  // bytes used (<= the buffer size)
};

// Bytes of buffer that hold `cap` records.
inline uint64_t record_bytes_for(uint64_t cap) { return RECORD_BYTES * cap + RECORD_PAD; }

// The capacity to ask for: at least `want`, clamped to the 32-bit limit, even.
inline uint64_t record_cap_request(uint64_t want) {
  if (want > RECORD_CAP_MAX) want = RECORD_CAP_MAX;
  return want & ~1ull;
}

// The carve-up of a buffer of `buffer_bytes`: as many records as fit, at most
// RECORD_CAP_MAX (even).  A buffer below record_bytes_for(2) gives cap 0.
inline RecordLayout record_layout(uint64_t buffer_bytes) {
  RecordLayout L;
  uint64_t cap = buffer_bytes > RECORD_PAD ? (buffer_bytes - RECORD_PAD) / RECORD_BYTES : 0;
  L.cap = record_cap_request(cap);
  L.off_wid = 0;
  L.off_part = 4 * L.cap;
  L.off_mask = 8 * L.cap;
  L.off_sorted = 12 * L.cap;  // cap even: a multiple of 8
  L.end = 20 * L.cap;
  return L;
}

// The growth step after a pass that counted `count` records into a buffer of
// `cap`: a quarter more plus slack, clamped.  Returns 0 when `count` itself
// is beyond the 32-bit limit (the call must fail).
inline uint64_t record_cap_regrow(uint64_t count) {
  if (count > RECORD_CAP_MAX) return 0;
  const uint64_t want = count + count / 4 + 1024;
  return record_cap_request(want < count ? RECORD_CAP_MAX : want);
}

}  // namespace rzl
