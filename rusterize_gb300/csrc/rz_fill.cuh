// rz_fill.cuh -- bucket fill: every (band, row, column-tile) bucket is staged
// as `background`, its coverage records are applied in part order (= the
// reference's per-geometry write order, rasterize.rs:162-196) with the pixel
// function, and the tile is written to the raster once.
//
// Pixel functions restate rust/src/rasterization/pixel_functions.rs:56-122
// (integer `+=` wraps, as in a release build of the crate).
#pragma once

#include <cstdint>
#include <type_traits>

#include "rz_device.cuh"

namespace rzd {

// One job of a batch call, as the fill sees it: where its buckets start and
// where its raster goes.
struct FillJob {
  unsigned long long bucket0;  // first bucket of the job (in the call's numbering)
  void* out;                   // (nrows, ncols) raster of the job
  int nrows, ncols;
  unsigned ntx, pad;
};

struct FillArgs {
  const unsigned* offsets;  // [nbuckets + 1]
  const uint2* recs;        // {part | word << REC_W_SHIFT | DEDUP_BIT, mask} grouped by bucket
  uint2* brecs;             // scratch of the records' size: the deep buckets' records grouped by word, at
                            // the records' own positions (nullptr: the per-word kernel scans whole buckets)
  const void* pvals;        // burn value of each part (T), or nullptr: every record burns `scalar`
  unsigned long long nbuckets;
  unsigned long long scalar;  // raw bits of the single value when pvals == nullptr
  void* out;                // (bands, nrows, ncols)
  unsigned long long bg;    // raw bits of the background
  uint4 bg16;               // background replicated over 16 bytes
  int nrows, ncols;
  unsigned ntx;
  unsigned* big;            // buckets left to the per-word kernel
  Ctrl* ctrl;
  unsigned long long rec_cap;
  int sort_max;              // tiles of up to this many records are sorted by one warp (<= FILL_WARP_SORT)
  int sort_cap;              // k_fill_warp: sort entries per warp (a power of two >= sort_max)
  int warp_bytes;            // k_fill_warp: shared memory per warp
  unsigned long long* work;  // chunk counter of this fill (zero before the launch)
  unsigned* nbig;            // entries of `big` (zero before the launch)
  // bucket b of this fill is bucket bucket0 + b of the call (a fill may run
  // over a sub-range of the buckets); batch calls: its raster is that of the
  // job owning it; jobs == nullptr: out / ncols / ntx
  const FillJob* jobs;
  unsigned n_jobs;
  unsigned long long bucket0;
};

__device__ __forceinline__ unsigned long long gb_of(const FillArgs& a, unsigned long long b) {
  return a.bucket0 + b;
}

// The raster tile of bucket b: its first pixel and its width (the last tile
// of a row is cut at ncols).
template <typename T>
__device__ __forceinline__ T* bucket_tile(const FillArgs& a, unsigned long long b, int& len) {
  T* out;
  int nrows, ncols;
  unsigned ntx, lb;
  if (a.jobs) {
    const unsigned long long gb = a.bucket0 + b;
    unsigned lo = 0, hi = a.n_jobs;  // jobs[lo].bucket0 <= gb < jobs[hi].bucket0
    while (hi - lo > 1) {
      const unsigned mid = (lo + hi) >> 1;
      if (a.jobs[mid].bucket0 <= gb) lo = mid; else hi = mid;
    }
    const FillJob j = a.jobs[lo];
    out = static_cast<T*>(j.out);
    nrows = j.nrows;
    ncols = j.ncols;
    ntx = j.ntx;
    lb = (unsigned)(gb - j.bucket0);
  } else {
    out = static_cast<T*>(a.out);
    nrows = a.nrows;  // all bands: rows of the (bands * nrows) stack
    ncols = a.ncols;
    ntx = a.ntx;
    lb = (unsigned)(a.bucket0 + b);  // a fill of a sub-range starts at bucket bucket0
  }
  const unsigned rowid = lb / ntx;  // 32-bit: a 64-bit divide runs on the FP64 pipe
  const int c0 = (int)(lb - rowid * ntx) << TW_SHIFT;
  len = min(TW, ncols - c0);
  if (rowid >= (unsigned)nrows) {  // never taken: the buckets of a fill are its rasters' tiles
    if ((threadIdx.x & 31) == 0) set_error(a.ctrl, ERR_RANGE, gb_of(a, b));
    len = 0;
    return out;
  }
  return out + (unsigned long long)rowid * (unsigned long long)ncols + c0;
}

template <typename T> __device__ __forceinline__ bool is_nan_v(T v) { return false; }
template <> __device__ __forceinline__ bool is_nan_v<float>(float v) { return isnan(v); }
template <> __device__ __forceinline__ bool is_nan_v<double>(double v) { return isnan(v); }

template <typename T> __device__ __forceinline__ T add_wrap(T a, T b) {
  if constexpr (std::is_integral<T>::value) {
    using U = typename std::make_unsigned<T>::type;
    return (T)(U)((U)a + (U)b);
  } else {
    return a + b;
  }
}

template <typename T> __device__ __forceinline__ T from_bits(unsigned long long b) {
  T v;
  memcpy(&v, &b, sizeof(T));
  return v;
}

template <typename T> inline T from_bits_host(unsigned long long b) {
  T v;
  memcpy(&v, &b, sizeof(T));
  return v;
}

enum { F_SUM = 0, F_FIRST = 1, F_LAST = 2, F_MIN = 3, F_MAX = 4, F_COUNT = 5, F_ANY = 6 };

template <typename T, int FN>
__device__ __forceinline__ void apply_px(T& cur, T v, T bg) {
  if constexpr (FN == F_SUM) {
    if (cur == bg || is_nan_v(cur) || is_nan_v(v)) cur = v; else cur = add_wrap(cur, v);
  } else if constexpr (FN == F_FIRST) {
    if (cur == bg || is_nan_v(cur)) cur = v;
  } else if constexpr (FN == F_LAST) {
    cur = v;
  } else if constexpr (FN == F_MIN) {
    if (cur == bg || is_nan_v(cur) || cur > v) cur = v;
  } else if constexpr (FN == F_MAX) {
    if (cur == bg || is_nan_v(cur) || cur < v) cur = v;
  } else if constexpr (FN == F_COUNT) {
    if (cur == bg || is_nan_v(cur)) cur = T(1); else cur = add_wrap(cur, T(1));
  } else {
    cur = T(1);
  }
}

// float64 fold with the comparisons on the integer pipe: `cur == bg`, NaN
// tests and `<`/`>` are decided on the bit patterns (IEEE: -0 == +0, NaN
// compares false), only the accumulating add of sum/count issues FP64.
using rzb::BgF64;
using rzb::bg_f64;
using rzb::eq_bg_f64;
using rzb::gt_f64;

template <int FN>
__device__ __forceinline__ void apply_px_f64(double& cur, double v, const BgF64& bg) {
  const unsigned long long c = f64_bits(cur);
  if constexpr (FN == F_SUM) {
    if (eq_bg_f64(c, bg) || nan_bits(c) || nan_bits(f64_bits(v))) cur = v; else cur = __dadd_rn(cur, v);
  } else if constexpr (FN == F_FIRST) {
    if (eq_bg_f64(c, bg) || nan_bits(c)) cur = v;
  } else if constexpr (FN == F_LAST) {
    cur = v;
  } else if constexpr (FN == F_MIN) {
    if (eq_bg_f64(c, bg) || nan_bits(c) || gt_f64(c, f64_bits(v))) cur = v;
  } else if constexpr (FN == F_MAX) {
    if (eq_bg_f64(c, bg) || nan_bits(c) || gt_f64(f64_bits(v), c)) cur = v;
  } else if constexpr (FN == F_COUNT) {
    if (eq_bg_f64(c, bg) || nan_bits(c)) cur = 1.0; else cur = __dadd_rn(cur, 1.0);
  } else {
    cur = 1.0;
  }
}

// one pixel-function step; for float64 the background is pre-classified
template <typename T, int FN>
__device__ __forceinline__ void apply_one(T& cur, T v, T bg, const BgF64& bgc) {
  if constexpr (std::is_same<T, double>::value) apply_px_f64<FN>(cur, v, bgc);
  else apply_px<T, FN>(cur, v, bg);
}

// The first write onto the background always takes the reset branch of
// every pixel function (cur == bg, or cur is NaN when bg is NaN): its result
// is the value itself, or 1 for count / any.  No arithmetic is issued, so
// the compiler cannot speculate an FP64 add for it.
template <typename T, int FN>
__device__ __forceinline__ T first_write(T v) {
  if constexpr (FN == F_COUNT || FN == F_ANY) return T(1);
  else return v;
}

// The burn value of a record: its part's value (values[geometry of the part],
// gathered once per part by the prep), or the call's single value.
template <typename T>
__device__ __forceinline__ T rec_value(const FillArgs& a, unsigned rec_x) {
  if (a.pvals) return static_cast<const T*>(a.pvals)[rec_x & REC_PART_MASK];
  return from_bits<T>(a.scalar);
}

// ---- order-free first / last ---------------------------------------------
// `last` leaves a pixel at the value of the largest part that writes it.
// `first` takes the first write and keeps it unless it is the background or
// NaN (pixel_functions.rs:56-122), and every part writes one value: so the
// pixel ends at the value of the smallest part whose value is neither
// ("sticky"), or -- when no written value is sticky -- at the value of the
// largest part (every write replaced the one before).  Both are reductions
// over the parts that write the pixel, and need no sort: one pass over the
// records in any order keeps, per pixel, the largest part (+1, 0 = none) and,
// for `first`, the smallest sticky part (~0u = none).
constexpr int OF_WARP_MAX = 1024;  // deeper buckets go to the per-word kernel

template <typename T>
__device__ __forceinline__ T part_value(const FillArgs& a, unsigned p) {
  if (a.pvals) return static_cast<const T*>(a.pvals)[p];
  return from_bits<T>(a.scalar);
}

template <typename T>
__device__ __forceinline__ bool first_resets(T v, T bg, const BgF64& bgc) {
  if constexpr (std::is_same<T, double>::value) {
    const unsigned long long b = f64_bits(v);
    return eq_bg_f64(b, bgc) || nan_bits(b);
  } else {
    return v == bg || is_nan_v(v);
  }
}

// A record for the order-free pass: the part, bit 31 set when its value is
// sticky for `first` (the DEDUP flag plays no role for first / last: a part
// writes one value, so repeated writes of a part change nothing).
template <typename T, int FN>
__device__ __forceinline__ unsigned of_key(const FillArgs& a, unsigned rx, T bg, const BgF64& bgc) {
  unsigned k = rx & REC_PART_MASK;
  if constexpr (FN == F_FIRST) {
    if (!first_resets<T>(rec_value<T>(a, rx), bg, bgc)) k |= DEDUP_BIT;
  }
  return k;
}

template <int FN>
__device__ __forceinline__ void of_update(unsigned& maxp1, unsigned& ming, unsigned k) {
  const unsigned p = k & REC_PART_MASK;
  maxp1 = max(maxp1, p + 1u);
  if (FN == F_FIRST && (k & DEDUP_BIT)) ming = min(ming, p);
}

template <typename T, int FN>
__device__ __forceinline__ T of_result(const FillArgs& a, unsigned maxp1, unsigned ming, T bg) {
  if (FN == F_FIRST && ming != 0xFFFFFFFFu) return part_value<T>(a, ming);
  if (maxp1 == 0u) return bg;
  return part_value<T>(a, maxp1 - 1u);
}

// `min` / `max` (cur == bg || NaN || cur > v, resp. < v) are order-free
// too when no written value is the background or NaN: after the first write
// every step keeps the running minimum (maximum) and an equal value does not
// replace it, so the pixel ends at the value of the smallest part among those
// whose value equals the extreme (only -0.0 and +0.0 are equal with other
// bits).  A pass that meets such a value falls back to the sorted fold.
template <typename T, int FN>
__device__ __forceinline__ bool of_better(T v, unsigned p, T bv, unsigned bp) {
  if (bp == 0xFFFFFFFFu) return true;
  bool ahead, eq;
  if constexpr (std::is_same<T, double>::value) {
    const unsigned long long x = f64_bits(v), y = f64_bits(bv);
    ahead = FN == F_MIN ? gt_f64(y, x) : gt_f64(x, y);
    eq = x == y || ((x | y) & 0x7FFFFFFFFFFFFFFFull) == 0;
  } else {
    ahead = FN == F_MIN ? v < bv : v > bv;
    eq = v == bv;
  }
  return ahead || (eq && p < bp);
}

template <typename T>
__device__ __forceinline__ T shfl_val(T v, int src) {
  if constexpr (sizeof(T) == 8) {
    unsigned long long b;
    memcpy(&b, &v, 8);
    b = __shfl_sync(0xFFFFFFFFu, b, src);
    T r;
    memcpy(&r, &b, 8);
    return r;
  } else {
    unsigned b = 0;
    memcpy(&b, &v, sizeof(T));
    b = __shfl_sync(0xFFFFFFFFu, b, src);
    T r;
    memcpy(&r, &b, sizeof(T));
    return r;
  }
}



// copy a staged tile to the raster (16-byte stores when aligned)
template <typename T>
__device__ __forceinline__ void store_tile(T* dst, const T* seg, int len, int lane, int nthr) {
  if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
    const int nv = (int)((len * sizeof(T)) >> 4);
    const uint4* s4 = reinterpret_cast<const uint4*>(seg);
    uint4* d4 = reinterpret_cast<uint4*>(dst);
    for (int i = lane; i < nv; i += nthr) __stcs(d4 + i, s4[i]);
    for (int i = (int)((nv * 16) / sizeof(T)) + lane; i < len; i += nthr) dst[i] = seg[i];
  } else {
    for (int i = lane; i < len; i += nthr) dst[i] = seg[i];
  }
}

template <typename T>
__device__ __forceinline__ void store_bg(T* dst, int len, const uint4& bg16, T bg, int lane, int nthr) {
  if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
    const int nv = (int)((len * sizeof(T)) >> 4);
    uint4* d4 = reinterpret_cast<uint4*>(dst);
    for (int i = lane; i < nv; i += nthr) __stcs(d4 + i, bg16);
    for (int i = (int)((nv * 16) / sizeof(T)) + lane; i < len; i += nthr) dst[i] = bg;
  } else {
    for (int i = lane; i < len; i += nthr) dst[i] = bg;
  }
}

template <typename T>
constexpr int seg_bytes() {
  return (int)((TW * sizeof(T) + 15) / 16 * 16);
}

// Sorted record in shared memory: key = part << 4 | word, the mask, the
// DEDUP flag and the value's bits.
struct __align__(16) SRec {
  unsigned key;
  unsigned mask;
  unsigned long long vbits;
};

__device__ __forceinline__ unsigned rec_key(unsigned x) {
  return ((x & REC_PART_MASK) << 4) | ((x >> REC_W_SHIFT) & 15u);
}

template <typename T>
__device__ __forceinline__ unsigned long long to_bits(T v) {
  unsigned long long b = 0;
  memcpy(&b, &v, sizeof(T));
  return b;
}

// One pixel-function step, with the FP64 add of a float64 sum issued only
// when some lane of the warp needs it (a write onto the background takes the
// reset branch of every pixel function and needs no arithmetic).
template <typename T, int FN>
__device__ __forceinline__ void apply_step(T& c, T v, bool on, T bg, const BgF64& bgc) {
  if constexpr (std::is_same<T, double>::value && (FN == F_SUM || FN == F_COUNT)) {
    const unsigned long long cb = f64_bits(c);
    const bool reset = eq_bg_f64(cb, bgc) || nan_bits(cb) || (FN == F_SUM && nan_bits(f64_bits(v)));
    if (on && reset) c = FN == F_SUM ? v : 1.0;
    const bool add = on && !reset;
    if (__any_sync(0xFFFFFFFFu, add)) {
      if (add) c = __dadd_rn(c, FN == F_SUM ? v : 1.0);
    }
  } else {
    if (on) apply_one<T, FN>(c, v, bg, bgc);
  }
}

// ---- warp fill -------------------------------------------------------------
// One warp per bucket.  A warp takes FILL_CHUNK consecutive buckets (one coalesced
// load of their offsets) and loads the next bucket's records and values
// while it works on the current one.
//
// Records of different words touch different pixels, so only the part
// order within a word matters.  Up to FILL_WARP_MAX records are sorted by
// (word, part) with a bitonic network in registers (two records per lane),
// up to the schedule's sort_max in shared memory, and then walked once:
// lane l keeps pixel l of the current word in a register, applies each
// record whose mask covers it, and stores the word when the walk moves on
// (words without records are background).  A pixel-function step that needs
// a float64 add issues it only when some lane of the warp needs it.  Records
// of one deduplicating part and word are adjacent in the order and write a
// pixel once (PixelCache).  Deeper buckets go to the per-word kernel.
//
// first / last (buckets of up to OF_WARP_MAX records), and min / max when no
// written value is the background or NaN, take the order-free pass instead.
constexpr int FILL_WARPS_PER_BLOCK = 8;
constexpr int FILL_CHUNK = 4;

// Shared memory of one k_fill_warp warp: the sort's records and keys (a
// power of two of entries, at least sort_max, so that the bitonic network's
// padding stays inside), or the order-free pass's per-pixel state, whichever
// is larger.  A smaller sort_max lets more warps share an SM.
inline int fill_sort_cap(int sort_max) {
  int e = FILL_WARP_MAX;
  while (e < sort_max) e <<= 1;
  return e;
}

template <typename T>
inline int fill_warp_bytes(int fn, int sort_cap) {
  int b = sort_cap * ((int)sizeof(SRec) + 8);
  if (fn == F_FIRST || fn == F_LAST) b = b > 2 * WPT * 32 * 4 ? b : 2 * WPT * 32 * 4;
  if (fn == F_MIN || fn == F_MAX) {
    const int m = WPT * 32 * ((int)sizeof(T) + 4);
    b = b > m ? b : m;
  }
  return (b + 15) & ~15;
}

// the two records (positions lane and lane + 32) of a bucket held by a lane
template <typename T>
struct LanePair {
  uint2 r0, r1;
  T v0, v1;
};

template <typename T>
__device__ __forceinline__ LanePair<T> load_pair(const FillArgs& a, unsigned o0, int n) {
  const int lane = threadIdx.x & 31;
  LanePair<T> p;
  p.r0 = p.r1 = make_uint2(0u, 0u);
  p.v0 = p.v1 = T(0);
  if (n <= FILL_WARP_MAX) {
    if (lane < n) {
      p.r0 = a.recs[o0 + lane];
      p.v0 = rec_value<T>(a, p.r0.x);
    }
    if (lane + 32 < n) {
      p.r1 = a.recs[o0 + lane + 32];
      p.v1 = rec_value<T>(a, p.r1.x);
    }
  }
  return p;
}

// One compare-exchange step of a bitonic network over elements held one per
// lane (partner lane ^ j); `up` is the direction of this element's block.
__device__ __forceinline__ void bitonic_step(unsigned& key, unsigned& idx, int j, bool up) {
  const int lane = threadIdx.x & 31;
  const unsigned pk = __shfl_xor_sync(0xFFFFFFFFu, key, j), pi = __shfl_xor_sync(0xFFFFFFFFu, idx, j);
  const bool lower = (lane & j) == 0;
  // keep the smaller element in the lower slot of an ascending block
  const bool pless = pk < key || (pk == key && pi < idx);
  if (lower == up ? pless : !pless) {
    key = pk;
    idx = pi;
  }
}

// Sort (key, idx) pairs held at positions lane and lane + 32 ascending.
__device__ __forceinline__ void warp_sort64(unsigned& k0, unsigned& i0, unsigned& k1, unsigned& i1, bool two) {
  const int lane = threadIdx.x & 31;
  // bitonic sort of each half (32 elements, one per lane); the second half
  // descending when two halves are merged
  for (int kk = 2; kk <= 32; kk <<= 1) {
    for (int j = kk >> 1; j > 0; j >>= 1) {
      const bool up0 = (lane & kk) == 0 || kk == 32;
      bitonic_step(k0, i0, j, kk == 32 ? true : up0);
      if (two) bitonic_step(k1, i1, j, kk == 32 ? false : ((lane & kk) == 0));
    }
  }
  if (!two) return;
  // merge: half 0 ascending, half 1 descending -> bitonic sequence of 64
  {
    const bool sw = k1 < k0 || (k1 == k0 && i1 < i0);
    if (sw) {
      const unsigned tk = k0, ti = i0;
      k0 = k1;
      i0 = i1;
      k1 = tk;
      i1 = ti;
    }
  }
  for (int j = 16; j > 0; j >>= 1) {
    bitonic_step(k0, i0, j, true);
    bitonic_step(k1, i1, j, true);
  }
}

// ascending bitonic sort of k[0..np) (np = next power of two >= n, padded
// with ~0) by one warp in shared memory
__device__ __forceinline__ void warp_sort_u64(unsigned long long* k, int n) {
  int np = 1;
  while (np < n) np <<= 1;
  const int lane = threadIdx.x & 31;
  for (int i = n + lane; i < np; i += 32) k[i] = ~0ull;
  __syncwarp();
  for (int kk = 2; kk <= np; kk <<= 1) {
    for (int j = kk >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < np; i += 32) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const unsigned long long x = k[i], y = k[ixj];
          const bool up = (i & kk) == 0;
          if ((x > y) == up) {
            k[i] = y;
            k[ixj] = x;
          }
        }
      }
      __syncwarp();
    }
  }
}

// Walk n records in (word, part) order -- srec itself, or srec[skey[p] & 0xFF]
// when a sorted key array is given -- and write the tile: lane l folds pixel
// l of the current word and stores the word when the walk moves on; words
// without records are background.
template <typename T, int FN, bool DEDUP>
__device__ __forceinline__ void fold_words(const SRec* srec, const unsigned long long* skey, int n, T* dst, int len,
                                           T bg, const BgF64& bgc) {
  const int lane = threadIdx.x & 31;
  int cw = -1;
  T c = bg;
  unsigned prev_key = 0xFFFFFFFFu, seen = 0u;
  for (int p = 0; p < n; ++p) {
    const SRec e = skey ? srec[(unsigned)skey[p] & 0xFFu] : srec[p];
    const int w = (int)((e.key >> REC_W_SHIFT) & 15u);
    if (w != cw) {
      if (cw >= 0 && cw * 32 + lane < len) dst[cw * 32 + lane] = c;
      for (int ww = cw + 1; ww < w; ++ww)
        if (ww * 32 + lane < len) dst[ww * 32 + lane] = bg;
      cw = w;
      c = bg;
      prev_key = 0xFFFFFFFFu;
    }
    unsigned mask = e.mask;
    if (DEDUP && (e.key & DEDUP_BIT)) {
      const unsigned key = e.key & ~DEDUP_BIT;
      if (key != prev_key) seen = 0u;
      mask &= ~seen;
      seen |= e.mask;
      prev_key = key;
    }
    apply_step<T, FN>(c, from_bits<T>(e.vbits), (mask >> lane) & 1u, bg, bgc);
  }
  if (cw * 32 + lane < len) dst[cw * 32 + lane] = c;
  for (int ww = cw + 1; ww < WPT; ++ww)
    if (ww * 32 + lane < len) dst[ww * 32 + lane] = bg;
}

template <typename T, int FN, bool DEDUP>
__global__ void __launch_bounds__(FILL_WARPS_PER_BLOCK * 32) k_fill_warp(FillArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  Ctrl* ctrl = a.ctrl;
  if (ctrl->err || ctrl->span_count > a.rec_cap) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  SRec* srec = reinterpret_cast<SRec*>(smem + warp * a.warp_bytes);
  const T bg = from_bits<T>(a.bg);
  const BgF64 bgc = bg_f64(a.bg);
  const unsigned long long nchunks = (a.nbuckets + FILL_CHUNK - 1) / FILL_CHUNK;
  while (true) {
    unsigned long long ch = 0;
    if (lane == 0) ch = atomicAdd(a.work, 1ull);
    ch = __shfl_sync(0xFFFFFFFFu, ch, 0);
    if (ch >= nchunks) break;
    const unsigned long long b0 = ch * FILL_CHUNK;
    const int nb = (int)min((unsigned long long)FILL_CHUNK, a.nbuckets - b0);
    const unsigned off = a.offsets[b0 + (lane < nb ? lane : nb)];
    const unsigned off_end = a.offsets[b0 + nb];
    unsigned o_next = __shfl_sync(0xFFFFFFFFu, off, 0);
    int n_next = (int)((nb > 1 ? __shfl_sync(0xFFFFFFFFu, off, 1) : off_end) - o_next);
    LanePair<T> nxt = load_pair<T>(a, o_next, n_next);
    for (int k = 0; k < nb; ++k) {
      const unsigned long long b = b0 + k;
      const int n = n_next;
      const unsigned o_cur = o_next;
      const LanePair<T> pr = nxt;
      if (k + 1 < nb) {  // prefetch the next bucket
        o_next = __shfl_sync(0xFFFFFFFFu, off, k + 1);
        n_next = (int)((k + 2 < nb ? __shfl_sync(0xFFFFFFFFu, off, (k + 2) & 31) : off_end) - o_next);
        nxt = load_pair<T>(a, o_next, n_next);
      }
      int len;
      T* dst = bucket_tile<T>(a, b, len);
      if (n == 0) {
        store_bg<T>(dst, len, a.bg16, bg, lane, 32);
        continue;
      }
      if constexpr (FN == F_FIRST || FN == F_LAST) {
        if (n > OF_WARP_MAX) {
          if (lane == 0) a.big[atomicAdd(a.nbig, 1u)] = (unsigned)b;
          continue;
        }
        // per pixel (word w, lane l) at w * 32 + l: each lane owns its
        // column, so the pass needs no synchronisation
        unsigned* smax = reinterpret_cast<unsigned*>(srec);
        unsigned* smin = smax + WPT * 32;
#pragma unroll
        for (int w = 0; w < WPT; ++w) {
          smax[w * 32 + lane] = 0u;
          if (FN == F_FIRST) smin[w * 32 + lane] = 0xFFFFFFFFu;
        }
        for (int i0 = 0; i0 < n; i0 += 32) {
          const int i = i0 + lane;
          unsigned kx = 0u, km = 0u, kw = 0u;
          if (i < n) {
            const uint2 r = a.recs[o_cur + i];
            kx = of_key<T, FN>(a, r.x, bg, bgc);
            km = r.y;
            kw = (r.x >> REC_W_SHIFT) & 15u;
          }
          const int cnt = min(32, n - i0);
          for (int j = 0; j < cnt; ++j) {
            const unsigned xj = __shfl_sync(0xFFFFFFFFu, kx, j), mj = __shfl_sync(0xFFFFFFFFu, km, j);
            const unsigned wj = __shfl_sync(0xFFFFFFFFu, kw, j);
            if ((mj >> lane) & 1u) {
              const unsigned ix = wj * 32u + (unsigned)lane;
              unsigned mx = smax[ix], mn = FN == F_FIRST ? smin[ix] : 0u;
              of_update<FN>(mx, mn, xj);
              smax[ix] = mx;
              if (FN == F_FIRST) smin[ix] = mn;
            }
          }
        }
#pragma unroll
        for (int w = 0; w < WPT; ++w) {
          const int x = w * 32 + lane;
          if (x < len) dst[x] = of_result<T, FN>(a, smax[x], FN == F_FIRST ? smin[x] : 0xFFFFFFFFu, bg);
        }
        continue;
      }
      if constexpr (FN == F_MIN || FN == F_MAX) {
        if (n <= OF_WARP_MAX) {
          // per pixel (word w, lane l) at w * 32 + l: its extreme and part
          T* sval = reinterpret_cast<T*>(srec);
          unsigned* spart = reinterpret_cast<unsigned*>(sval + WPT * 32);
#pragma unroll
          for (int w = 0; w < WPT; ++w) spart[w * 32 + lane] = 0xFFFFFFFFu;
          bool bad = false;
          for (int i0 = 0; i0 < n; i0 += 32) {
            const int i = i0 + lane;
            unsigned kx = 0u, km = 0u;
            T kv = T(0);
            if (i < n) {
              const uint2 r = a.recs[o_cur + i];
              kv = rec_value<T>(a, r.x);
              kx = r.x;
              km = r.y;
              bad = bad || first_resets<T>(kv, bg, bgc);
            }
            if (__any_sync(0xFFFFFFFFu, bad)) break;
            const int cnt = min(32, n - i0);
            for (int j = 0; j < cnt; ++j) {
              const unsigned xj = __shfl_sync(0xFFFFFFFFu, kx, j), mj = __shfl_sync(0xFFFFFFFFu, km, j);
              const T vj = shfl_val<T>(kv, j);
              if ((mj >> lane) & 1u) {
                const unsigned ix = ((xj >> REC_W_SHIFT) & 15u) * 32u + (unsigned)lane;
                const unsigned pj = xj & REC_PART_MASK;
                if (of_better<T, FN>(vj, pj, sval[ix], spart[ix])) {
                  sval[ix] = vj;
                  spart[ix] = pj;
                }
              }
            }
          }
          if (!__any_sync(0xFFFFFFFFu, bad)) {
#pragma unroll
            for (int w = 0; w < WPT; ++w) {
              const int x = w * 32 + lane;
              if (x < len) dst[x] = spart[x] == 0xFFFFFFFFu ? bg : sval[x];
            }
            continue;
          }
          __syncwarp();  // the sorted fold below reuses the shared memory
        }
      }
      if (n > FILL_WARP_MAX) {
        if (n > a.sort_max) {
          if (lane == 0) a.big[atomicAdd(a.nbig, 1u)] = (unsigned)b;
          continue;
        }
        // up to sort_max records: staged and sorted in shared memory,
        // key = (word, part) << 8 | position
        const unsigned o0 = o_cur;
        unsigned long long* skey = reinterpret_cast<unsigned long long*>(srec + a.sort_cap);
        for (int i = lane; i < n; i += 32) {
          const uint2 r = a.recs[o0 + i];
          SRec e;
          e.key = r.x;
          e.mask = r.y;
          e.vbits = to_bits<T>(rec_value<T>(a, r.x));
          srec[i] = e;
          skey[i] = ((unsigned long long)(r.x & ~DEDUP_BIT) << 8) | (unsigned)i;
        }
        warp_sort_u64(skey, n);
        fold_words<T, FN, DEDUP>(srec, skey, n, dst, len, bg, bgc);
        __syncwarp();
        continue;
      }
      // (word, part) keys; invalid positions sort last
      unsigned k0 = lane < n ? pr.r0.x & ~DEDUP_BIT : 0xFFFFFFFFu, i0 = (unsigned)lane;
      unsigned k1 = lane + 32 < n ? pr.r1.x & ~DEDUP_BIT : 0xFFFFFFFFu, i1 = (unsigned)lane + 32u;
      const bool two = n > 32;
      {
        const unsigned nk0 = __shfl_down_sync(0xFFFFFFFFu, k0, 1), nk1 = __shfl_down_sync(0xFFFFFFFFu, k1, 1);
        const unsigned k1_first = __shfl_sync(0xFFFFFFFFu, k1, 0);
        const bool ord = k0 <= (lane == 31 ? k1_first : nk0) && (lane == 31 || k1 <= nk1);
        if (!__all_sync(0xFFFFFFFFu, ord)) warp_sort64(k0, i0, k1, i1, two);
      }
      // sorted position p (lane p, then lane p - 32) holds original record i:
      // fetch it from the lane that loaded it and store it at p
      {
        const int s0 = (int)(i0 & 31u), s1 = (int)(i1 & 31u);
        const unsigned ax = __shfl_sync(0xFFFFFFFFu, pr.r0.x, s0), am = __shfl_sync(0xFFFFFFFFu, pr.r0.y, s0);
        const T av = shfl_val<T>(pr.v0, s0);
        SRec e;
        if (two) {
          const unsigned bx = __shfl_sync(0xFFFFFFFFu, pr.r1.x, s0), bm = __shfl_sync(0xFFFFFFFFu, pr.r1.y, s0);
          const T bv = shfl_val<T>(pr.v1, s0);
          const bool hi0 = i0 >= 32u;
          e.key = hi0 ? bx : ax;
          e.mask = hi0 ? bm : am;
          e.vbits = to_bits<T>(hi0 ? bv : av);
          if (lane < n) srec[lane] = e;
          const unsigned cx = __shfl_sync(0xFFFFFFFFu, pr.r0.x, s1), cm = __shfl_sync(0xFFFFFFFFu, pr.r0.y, s1);
          const T cv = shfl_val<T>(pr.v0, s1);
          const unsigned dx = __shfl_sync(0xFFFFFFFFu, pr.r1.x, s1), dm = __shfl_sync(0xFFFFFFFFu, pr.r1.y, s1);
          const T dv = shfl_val<T>(pr.v1, s1);
          const bool hi1 = i1 >= 32u;
          e.key = hi1 ? dx : cx;
          e.mask = hi1 ? dm : cm;
          e.vbits = to_bits<T>(hi1 ? dv : cv);
          if (lane + 32 < n) srec[lane + 32] = e;
        } else {
          e.key = ax;
          e.mask = am;
          e.vbits = to_bits<T>(av);
          if (lane < n) srec[lane] = e;
        }
      }
      __syncwarp();
      fold_words<T, FN, DEDUP>(srec, (const unsigned long long*)nullptr, n, dst, len, bg, bgc);
      __syncwarp();
    }
  }
}

// ---- deep buckets: records grouped by word ------------------------------
// One warp per deep bucket (the `big` list k_fill_warp leaves) counts the
// bucket's records per word and copies them, grouped by word in word order,
// to the same positions of `brecs`.  The per-(bucket, word) warps then find
// their word's records by a binary search and read only those, instead of
// scanning the whole bucket (sixteen words, twice each).  The order within
// a word is not kept; the per-word kernel orders by part itself.
constexpr int BIN_WARPS = 8;

static __global__ void __launch_bounds__(BIN_WARPS * 32) k_big_bin(FillArgs a) {
  __shared__ unsigned s_pos[BIN_WARPS][WPT];
  const Ctrl* ctrl = a.ctrl;
  if (ctrl->err || ctrl->span_count > a.rec_cap) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned* pos = s_pos[warp];
  const unsigned nbig = *a.nbig;
  const unsigned nwarps = gridDim.x * BIN_WARPS;
  for (unsigned it = blockIdx.x * BIN_WARPS + warp; it < nbig; it += nwarps) {
    const unsigned b = a.big[it];
    const unsigned o0 = a.offsets[b];
    const unsigned n = a.offsets[b + 1] - o0;
    unsigned cnt = 0;  // lane w < WPT: records of word w
    for (unsigned i0 = 0; i0 < n; i0 += 32) {
      const unsigned i = i0 + lane;
      const unsigned w = i < n ? (a.recs[o0 + i].x >> REC_W_SHIFT) & 15u : 0xFFu;
#pragma unroll
      for (int k = 0; k < WPT; ++k) {
        const unsigned c = __popc(__ballot_sync(0xFFFFFFFFu, w == (unsigned)k));
        if (lane == k) cnt += c;
      }
    }
    unsigned incl = cnt;  // inclusive scan over lanes 0..WPT-1
#pragma unroll
    for (int o = 1; o < WPT; o <<= 1) {
      const unsigned t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane < WPT) pos[lane] = incl - cnt;
    __syncwarp();
    for (unsigned i0 = 0; i0 < n; i0 += 32) {
      const unsigned i = i0 + lane;
      uint2 r = make_uint2(0u, 0u);
      unsigned w = 0xFFu;
      if (i < n) {
        r = a.recs[o0 + i];
        w = (r.x >> REC_W_SHIFT) & 15u;
      }
      const unsigned peers = __match_any_sync(0xFFFFFFFFu, w);
      const int leader = __ffs(peers) - 1;
      const unsigned rank = __popc(peers & ((1u << lane) - 1u));
      unsigned base = 0;
      if (lane == leader && w < (unsigned)WPT) base = atomicAdd(&pos[w], (unsigned)__popc(peers));
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
      if (w < (unsigned)WPT) a.brecs[o0 + base + rank] = r;
    }
    __syncwarp();
  }
}

// The records of word `wsel` in a deep bucket grouped by k_big_bin: the
// range [lo, hi) of [0, n) whose word is wsel (binary searches on the word).
__device__ __forceinline__ void word_range(const uint2* r, unsigned n, unsigned wsel, unsigned& lo, unsigned& hi) {
  unsigned l = 0, h = n;  // first index whose word is >= wsel
  while (l < h) {
    const unsigned m = (l + h) >> 1;
    if (((r[m].x >> REC_W_SHIFT) & 15u) < wsel) l = m + 1; else h = m;
  }
  lo = l;
  h = n;  // first index whose word is > wsel
  while (l < h) {
    const unsigned m = (l + h) >> 1;
    if (((r[m].x >> REC_W_SHIFT) & 15u) <= wsel) l = m + 1; else h = m;
  }
  hi = l;
}

// ---- deep buckets: one warp per (bucket, word) --------------------------
// The word's records are taken in part order, at most BIG_CAP at a time: a
// histogram over the pending part ids picks the largest prefix range that
// fits, the range is gathered, sorted (bitonic, shared memory) and folded:
// lane l keeps pixel l of the word in a register and walks the sorted
// records to the next one covering its pixel, so every step applies one
// record per lane.  A single part with more than BIG_CAP records in the word
// is applied in chunks (its records share one value and their order does
// not change the result).  first / last, and min / max without a background
// or NaN value among the word's records, take one order-free pass instead.
constexpr int BIG_WARPS = 4;
constexpr int BIG_HIST = 256;

template <typename T>
constexpr int big_warp_bytes() { return BIG_CAP * 8 + BIG_CAP * (int)sizeof(T) + BIG_HIST * 4; }

// ascending bitonic sort of k[0..np) with np = next power of two >= n
// (padded with ~0), carrying v along
template <typename T>
__device__ __forceinline__ void warp_sort_keys(unsigned long long* k, T* v, int n) {
  int np = 1;
  while (np < n) np <<= 1;
  const int lane = threadIdx.x & 31;
  for (int i = n + lane; i < np; i += 32) k[i] = ~0ull;
  __syncwarp();
  for (int kk = 2; kk <= np; kk <<= 1) {
    for (int j = kk >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < np; i += 32) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const unsigned long long x = k[i], y = k[ixj];
          const bool up = (i & kk) == 0;
          if ((x > y) == up) {
            k[i] = y;
            k[ixj] = x;
            const T t = v[i];
            v[i] = v[ixj];
            v[ixj] = t;
          }
        }
      }
      __syncwarp();
    }
  }
}

// Fold keys[0..m) (part << 33 | dedup << 32 | mask, part order) into this
// lane's pixel: each step every lane advances to the next record covering
// its pixel (skipping repeats of a deduplicating part) and applies it.
template <typename T, int FN, bool DEDUP>
__device__ __forceinline__ void fold_sorted(const unsigned long long* keys, const T* vals, int m, T& c,
                                            unsigned& last_part, T bg, const BgF64& bgc) {
  const unsigned bit = 1u << (threadIdx.x & 31);
  int j = 0;
  bool active = true;
  while (__any_sync(0xFFFFFFFFu, active)) {
    T v = T(0);
    bool on = false;
    if (active) {
      while (j < m) {
        const unsigned long long kj = keys[j];
        const unsigned part = (unsigned)(kj >> 33);
        if (((unsigned)kj & bit) && !(DEDUP && ((kj >> 32) & 1u) && part == last_part)) break;
        ++j;
      }
      if (j < m) {
        on = true;
        v = vals[j];
        last_part = (unsigned)(keys[j] >> 33);
        ++j;
      } else {
        active = false;
      }
    }
    apply_step<T, FN>(c, v, on, bg, bgc);
  }
}

template <typename T, int FN, bool DEDUP>
__global__ void __launch_bounds__(BIG_WARPS * 32) k_fill_big(FillArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Ctrl* ctrl = a.ctrl;
  if (ctrl->err || ctrl->span_count > a.rec_cap) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char* wbase = smem + warp * big_warp_bytes<T>();
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(wbase);
  T* vals = reinterpret_cast<T*>(wbase + BIG_CAP * 8);
  unsigned* hist = reinterpret_cast<unsigned*>(wbase + BIG_CAP * 8 + BIG_CAP * sizeof(T));
  const T bg = from_bits<T>(a.bg);
  const BgF64 bgc = bg_f64(a.bg);
  const unsigned long long items = (unsigned long long)*a.nbig * WPT;
  const unsigned long long nwarps = (unsigned long long)gridDim.x * BIG_WARPS;
  for (unsigned long long it = (unsigned long long)blockIdx.x * BIG_WARPS + warp; it < items; it += nwarps) {
    const unsigned long long b = a.big[it / WPT];
    const unsigned wsel = (unsigned)(it % WPT);
    unsigned o0 = a.offsets[b];
    int n = (int)(a.offsets[b + 1] - o0);
    const uint2* recs = a.recs;
    if (a.brecs) {  // only this word's records, from the grouped copy
      unsigned lo, hi;
      word_range(a.brecs + o0, (unsigned)n, wsel, lo, hi);
      recs = a.brecs;
      o0 += lo;
      n = (int)(hi - lo);
    }
    int len;
    T* dst = bucket_tile<T>(a, b, len);
    const int x = (int)wsel * 32 + lane;
    if constexpr (FN == F_FIRST || FN == F_LAST) {  // order-free: one pass, no sort
      unsigned maxp1 = 0u, ming = 0xFFFFFFFFu;
      for (int i0 = 0; i0 < n; i0 += 32) {
        const int i = i0 + lane;
        unsigned kx = 0u, km = 0u;
        if (i < n) {
          const uint2 r = recs[o0 + i];
          kx = of_key<T, FN>(a, r.x, bg, bgc);
          km = ((r.x >> REC_W_SHIFT) & 15u) == wsel ? r.y : 0u;
        }
        const int cnt = min(32, n - i0);
        for (int j = 0; j < cnt; ++j) {
          const unsigned xj = __shfl_sync(0xFFFFFFFFu, kx, j), mj = __shfl_sync(0xFFFFFFFFu, km, j);
          if ((mj >> lane) & 1u) of_update<FN>(maxp1, ming, xj);
        }
      }
      if (x < len) dst[x] = of_result<T, FN>(a, maxp1, ming, bg);
      continue;
    }
    if constexpr (FN == F_MIN || FN == F_MAX) {  // order-free unless a value resets the pixel
      T bv = bg;
      unsigned bp = 0xFFFFFFFFu;
      bool bad = false;
      for (int i0 = 0; i0 < n; i0 += 32) {
        const int i = i0 + lane;
        unsigned kx = 0u, km = 0u;
        T kv = T(0);
        if (i < n) {
          const uint2 r = recs[o0 + i];
          if (((r.x >> REC_W_SHIFT) & 15u) == wsel) {
            kv = rec_value<T>(a, r.x);
            kx = r.x;
            km = r.y;
            bad = bad || first_resets<T>(kv, bg, bgc);
          }
        }
        if (__any_sync(0xFFFFFFFFu, bad)) break;
        const int cnt = min(32, n - i0);
        for (int j = 0; j < cnt; ++j) {
          const unsigned xj = __shfl_sync(0xFFFFFFFFu, kx, j), mj = __shfl_sync(0xFFFFFFFFu, km, j);
          const T vj = shfl_val<T>(kv, j);
          if ((mj >> lane) & 1u) {
            const unsigned pj = xj & REC_PART_MASK;
            if (of_better<T, FN>(vj, pj, bv, bp)) {
              bv = vj;
              bp = pj;
            }
          }
        }
      }
      if (!__any_sync(0xFFFFFFFFu, bad)) {
        if (x < len) dst[x] = bv;
        continue;
      }
    }
    T c = bg;
    unsigned last_part = 0xFFFFFFFFu;
    unsigned lo_part = 0;  // parts < lo_part are done
    while (true) {
      unsigned cnt = 0, pmin = 0xFFFFFFFFu, pmax = 0;
      for (int i = lane; i < n; i += 32) {
        const unsigned rx = recs[o0 + i].x;
        const unsigned part = rx & REC_PART_MASK;
        if (((rx >> REC_W_SHIFT) & 15u) == wsel && part >= lo_part) {
          ++cnt;
          pmin = min(pmin, part);
          pmax = max(pmax, part);
        }
      }
      cnt = __reduce_add_sync(0xFFFFFFFFu, cnt);
      if (cnt == 0) break;
      pmin = __reduce_min_sync(0xFFFFFFFFu, pmin);
      pmax = __reduce_max_sync(0xFFFFFFFFu, pmax);
      unsigned hi = pmax + 1;  // parts [lo_part, hi) this round
      bool single = false;
      if (cnt > (unsigned)BIG_CAP) {
        unsigned span_lo = pmin, span_hi = pmax;  // inclusive
        while (true) {
          int shift = 0;
          while (((span_hi - span_lo) >> shift) >= (unsigned)BIG_HIST) ++shift;
          for (int h = lane; h < BIG_HIST; h += 32) hist[h] = 0u;
          __syncwarp();
          for (int i = lane; i < n; i += 32) {
            const unsigned rx = recs[o0 + i].x;
            const unsigned part = rx & REC_PART_MASK;
            if (((rx >> REC_W_SHIFT) & 15u) == wsel && part >= span_lo && part <= span_hi)
              atomicAdd(&hist[(part - span_lo) >> shift], 1u);
          }
          __syncwarp();
          // largest prefix of bins with at most BIG_CAP records (lane 0)
          int jsel = -1;
          if (lane == 0) {
            unsigned cum = 0;
            for (int h = 0; h < BIG_HIST; ++h) {
              if (cum + hist[h] > (unsigned)BIG_CAP) break;
              cum += hist[h];
              jsel = h;
            }
          }
          jsel = __shfl_sync(0xFFFFFFFFu, jsel, 0);
          __syncwarp();
          if (jsel >= 0) {
            hi = span_lo + ((unsigned)(jsel + 1) << shift);
            break;
          }
          if (shift == 0) {  // one part alone exceeds BIG_CAP
            hi = span_lo + 1;
            single = true;
            break;
          }
          span_hi = span_lo + (1u << shift) - 1u;  // zoom into the first bin
        }
      }
      // gather [lo_part, hi) of this word (chunks of BIG_CAP for a single part)
      int m = 0;
      for (int i0 = 0; i0 < n; i0 += 32) {
        const int i = i0 + lane;
        uint2 r = make_uint2(0u, 0u);
        bool take = false;
        if (i < n) {
          r = recs[o0 + i];
          const unsigned part = r.x & REC_PART_MASK;
          take = ((r.x >> REC_W_SHIFT) & 15u) == wsel && part >= lo_part && part < hi;
        }
        const unsigned mk = __ballot_sync(0xFFFFFFFFu, take);
        if (take) {
          const int pos = m + __popc(mk & ((1u << lane) - 1u));
          // part (order), then the DEDUP flag, then the mask
          keys[pos] = ((unsigned long long)(r.x & REC_PART_MASK) << 33) | ((unsigned long long)(r.x >> 31) << 32) |
                      r.y;
          vals[pos] = rec_value<T>(a, r.x);
        }
        m += __popc(mk);
        if (single && m > BIG_CAP - 32) {  // fold a chunk of the single part
          __syncwarp();
          fold_sorted<T, FN, DEDUP>(keys, vals, m, c, last_part, bg, bgc);
          m = 0;
          __syncwarp();
        }
      }
      __syncwarp();
      if (!single) warp_sort_keys(keys, vals, m);
      __syncwarp();
      fold_sorted<T, FN, DEDUP>(keys, vals, m, c, last_part, bg, bgc);
      __syncwarp();
      lo_part = hi;
    }
    if (x < len) dst[x] = c;
  }
}

// ---- order-free fill: count / any --------------------------------------
// Integer `count` with background 0 (and float count with background 0 or
// NaN) equals the pixel's coverage depth: every write after the first adds
// one and no intermediate count can equal the background.  `any` is 1
// wherever the depth is non-zero.  Neither needs values or order.  One warp
// per bucket (FILL_CHUNK consecutive buckets per task, the next bucket's records
// loaded while the current one is counted); every record is broadcast to the
// warp and lane l adds its bit l to the counter of the record's word.
constexpr int DEPTH_WARPS = 8;

// 32 x 32 bit transpose across a warp: lane i holds row i on entry and
// column l (bit i = bit l of row i) in lane l on return.  Five butterfly
// stages, each swapping the off-diagonal j x j blocks of every 2j x 2j block.
__device__ __forceinline__ unsigned warp_transpose32(unsigned x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int j = 16 >> s;
    const unsigned m = s == 0 ? 0x0000FFFFu : s == 1 ? 0x00FF00FFu : s == 2 ? 0x0F0F0F0Fu : s == 3 ? 0x33333333u
                                                                                                    : 0x55555555u;
    const unsigned y = __shfl_xor_sync(0xFFFFFFFFu, x, j);
    x = (lane & j) ? ((x & ~m) | ((y >> j) & m)) : ((x & m) | ((y << j) & ~m));
  }
  return x;
}

template <typename T, int FN>
__global__ void __launch_bounds__(DEPTH_WARPS * 32) k_fill_depth(FillArgs a) {
  Ctrl* ctrl = a.ctrl;
  if (ctrl->err || ctrl->span_count > a.rec_cap) return;
  const int lane = threadIdx.x & 31;
  const T bg = from_bits<T>(a.bg);
  const unsigned long long nchunks = (a.nbuckets + FILL_CHUNK - 1) / FILL_CHUNK;
  while (true) {
    unsigned long long ch = 0;
    if (lane == 0) ch = atomicAdd(a.work, 1ull);
    ch = __shfl_sync(0xFFFFFFFFu, ch, 0);
    if (ch >= nchunks) break;
    const unsigned long long b0 = ch * FILL_CHUNK;
    const int nb = (int)min((unsigned long long)FILL_CHUNK, a.nbuckets - b0);
    const unsigned off = a.offsets[b0 + (lane < nb ? lane : nb)];
    const unsigned off_end = a.offsets[b0 + nb];
    unsigned o_next = __shfl_sync(0xFFFFFFFFu, off, 0);
    unsigned e_next = nb > 1 ? __shfl_sync(0xFFFFFFFFu, off, 1) : off_end;
    uint2 nxt = lane < (int)(e_next - o_next) ? a.recs[o_next + lane] : make_uint2(0u, 0u);
    for (int k = 0; k < nb; ++k) {
      const unsigned long long b = b0 + k;
      const unsigned o0 = o_next, o1 = e_next;
      const int n = (int)(o1 - o0);
      uint2 r = nxt;
      if (k + 1 < nb) {
        o_next = __shfl_sync(0xFFFFFFFFu, off, k + 1);
        e_next = k + 2 < nb ? __shfl_sync(0xFFFFFFFFu, off, (k + 2) & 31) : off_end;
        nxt = lane < (int)(e_next - o_next) ? a.recs[o_next + lane] : make_uint2(0u, 0u);
      }
      int len;
      T* dst = bucket_tile<T>(a, b, len);
      if (n == 0) {
        store_bg<T>(dst, len, a.bg16, bg, lane, 32);
        continue;
      }
      // 32 records at a time, bit-sliced: after the transpose lane l holds
      // bit l of every record's mask, so the depth of pixel (w, l) grows by
      // the records of word w among those bits (lanes past the end hold an
      // empty mask and add nothing)
      unsigned c[WPT];
#pragma unroll
      for (int w = 0; w < WPT; ++w) c[w] = 0u;
      for (int i0 = 0; i0 < n; i0 += 32) {
        if (i0 > 0) r = i0 + lane < n ? a.recs[o0 + i0 + lane] : make_uint2(0u, 0u);
        const unsigned wd = (r.x >> REC_W_SHIFT) & 15u;
        const unsigned t = warp_transpose32(r.y);
#pragma unroll
        for (int w = 0; w < WPT; ++w) c[w] += (unsigned)__popc(t & __ballot_sync(0xFFFFFFFFu, wd == (unsigned)w));
      }
#pragma unroll
      for (int w = 0; w < WPT; ++w) {
        const unsigned d = c[w];
        T v = bg;
        if (d) {
          if constexpr (FN == F_ANY) v = T(1);
          else if constexpr (std::is_integral<T>::value) v = (T)(typename std::make_unsigned<T>::type)d;
          else v = (T)d;
        }
        if (w * 32 + lane < len) dst[w * 32 + lane] = v;
      }
    }
  }
}

// Host launcher shared by the per-dtype translation units.
template <typename T>
bool depth_exact(const FillArgs& a, int fn, bool dedup) {
  if (fn == F_ANY) return true;
  if (fn != F_COUNT || dedup) return false;
  const T bg = from_bits_host<T>(a.bg);
  if constexpr (std::is_integral<T>::value) return bg == T(0);
  else return bg == T(0) || bg != bg;
}

template <typename T>
int launch_fill_t(const FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  // persistent grids: as many blocks as fit on the GPU at once, chunks of
  // buckets handed out by an atomic counter
  const unsigned long long nchunks = (a.nbuckets + FILL_CHUNK - 1) / FILL_CHUNK;
  auto persistent = [&](const void* kern, int threads, int smem_bytes, int per_block_units) {
    int bps = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, threads, smem_bytes);
    if (bps < 1) bps = 1;
    unsigned long long want = (nchunks + per_block_units - 1) / per_block_units;
    unsigned long long g = (unsigned long long)num_sms * bps;
    if (want < g) g = want;
    return (unsigned)(g ? g : 1);
  };
  if (depth_exact<T>(a, fn, dedup)) {
    if (fn == F_ANY) {
      const unsigned grid = persistent((const void*)k_fill_depth<T, F_ANY>, DEPTH_WARPS * 32, 0, DEPTH_WARPS);
      k_fill_depth<T, F_ANY><<<grid, DEPTH_WARPS * 32, 0, s>>>(a);
    } else {
      const unsigned grid = persistent((const void*)k_fill_depth<T, F_COUNT>, DEPTH_WARPS * 32, 0, DEPTH_WARPS);
      k_fill_depth<T, F_COUNT><<<grid, DEPTH_WARPS * 32, 0, s>>>(a);
    }
    return 1;
  }
  int launches = 0;
#define RZ_FILL_CASE(FNV, DD)                                                                             \
  {                                                                                                       \
    FillArgs aw = a;                                                                                      \
    aw.sort_cap = fill_sort_cap(a.sort_max);                                                              \
    aw.warp_bytes = fill_warp_bytes<T>(FNV, aw.sort_cap);                                                 \
    const int ws = FILL_WARPS_PER_BLOCK * aw.warp_bytes;                                                  \
    constexpr int bs = BIG_WARPS * big_warp_bytes<T>();                                                   \
    cudaFuncSetAttribute(k_fill_warp<T, FNV, DD>, cudaFuncAttributeMaxDynamicSharedMemorySize, ws);       \
    cudaFuncSetAttribute(k_fill_big<T, FNV, DD>, cudaFuncAttributeMaxDynamicSharedMemorySize, bs);        \
    const unsigned grid =                                                                                 \
        persistent((const void*)k_fill_warp<T, FNV, DD>, FILL_WARPS_PER_BLOCK * 32, ws, FILL_WARPS_PER_BLOCK); \
    k_fill_warp<T, FNV, DD><<<grid, FILL_WARPS_PER_BLOCK * 32, ws, s>>>(aw);                              \
    if (a.brecs) {                                                                                        \
      k_big_bin<<<num_sms * 2, BIN_WARPS * 32, 0, s>>>(a);                                                \
      ++launches;                                                                                         \
    }                                                                                                     \
    k_fill_big<T, FNV, DD><<<num_sms * 4, BIG_WARPS * 32, bs, s>>>(a);                                    \
    launches += 2;                                                                                        \
  }
  switch (fn) {
    case F_SUM:
      if (dedup) RZ_FILL_CASE(F_SUM, true) else RZ_FILL_CASE(F_SUM, false)
      break;
    case F_FIRST: RZ_FILL_CASE(F_FIRST, false) break;
    case F_LAST: RZ_FILL_CASE(F_LAST, false) break;
    case F_MIN: RZ_FILL_CASE(F_MIN, false) break;
    case F_MAX: RZ_FILL_CASE(F_MAX, false) break;
    case F_COUNT:
      if (dedup) RZ_FILL_CASE(F_COUNT, true) else RZ_FILL_CASE(F_COUNT, false)
      break;
    default: RZ_FILL_CASE(F_ANY, false) break;
  }
#undef RZ_FILL_CASE
  return launches;
}

}  // namespace rzd

#define RZ_DECLARE_FILL(NAME) \
  int NAME(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s);
RZ_DECLARE_FILL(rz_fill_u8)
RZ_DECLARE_FILL(rz_fill_u16)
RZ_DECLARE_FILL(rz_fill_u32)
RZ_DECLARE_FILL(rz_fill_u64)
RZ_DECLARE_FILL(rz_fill_i8)
RZ_DECLARE_FILL(rz_fill_i16)
RZ_DECLARE_FILL(rz_fill_i32)
RZ_DECLARE_FILL(rz_fill_i64)
RZ_DECLARE_FILL(rz_fill_f32)
RZ_DECLARE_FILL(rz_fill_f64)
