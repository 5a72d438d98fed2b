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

struct FillArgs {
  const unsigned* offsets;  // [nbuckets + 1]
  const uint2* recs;        // {part | word << REC_W_SHIFT | DEDUP_BIT, mask} grouped by bucket
  unsigned long long nbuckets;
  const void* values;       // per-geometry values, or nullptr
  unsigned long long scalar;  // raw bits of the single value when values == nullptr
  const unsigned* part_geom;
  void* out;                // (bands, nrows, ncols)
  unsigned long long bg;    // raw bits of the background
  uint4 bg16;               // background replicated over 16 bytes
  int nrows, ncols;
  unsigned ntx;
  unsigned* big;            // buckets left to the per-word kernel
  Ctrl* ctrl;
  unsigned long long rec_cap;
};

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

template <typename T>
__device__ __forceinline__ T value_of(const FillArgs& a, unsigned part) {
  if (a.values) return static_cast<const T*>(a.values)[a.part_geom[part]];
  return from_bits<T>(a.scalar);
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
// One warp per bucket of at most FILL_WARP_MAX records.  Each record gets
// its rank in (part, word) order by counting the smaller keys (ties broken
// by position), is written to that slot with its value, and the records are
// then applied in order: lane l owns pixel l of every word of the tile, so a
// record is one broadcast load, a bit test and the pixel function.  Records
// of one deduplicating part and word are adjacent in that order and write a
// pixel once (PixelCache).
constexpr int FILL_WARPS_PER_BLOCK = 8;

template <typename T>
constexpr int fill_warp_bytes() {
  return TW * (int)sizeof(T) + FILL_WARP_MAX * (int)sizeof(SRec) + FILL_WARP_MAX * 4;
}

template <typename T, int FN, bool DEDUP>
__global__ void __launch_bounds__(FILL_WARPS_PER_BLOCK * 32) k_fill_warp(FillArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Ctrl* ctrl = a.ctrl;
  if (ctrl->err || ctrl->span_count > a.rec_cap) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char* base = smem + warp * fill_warp_bytes<T>();
  T* cur = reinterpret_cast<T*>(base);
  SRec* srec = reinterpret_cast<SRec*>(base + TW * sizeof(T));
  unsigned* keys = reinterpret_cast<unsigned*>(srec + FILL_WARP_MAX);
  const T bg = from_bits<T>(a.bg);
  const BgF64 bgc = bg_f64(a.bg);
  T* out = static_cast<T*>(a.out);
  const unsigned long long nwarps = (unsigned long long)gridDim.x * FILL_WARPS_PER_BLOCK;
  for (unsigned long long b = (unsigned long long)blockIdx.x * FILL_WARPS_PER_BLOCK + warp; b < a.nbuckets;
       b += nwarps) {
    const unsigned o0 = a.offsets[b];
    const int n = (int)(a.offsets[b + 1] - o0);
    const unsigned rowid = (unsigned)b / a.ntx;  // 32-bit: a 64-bit divide runs on the FP64 pipe
    const int c0 = (int)((unsigned)b - rowid * a.ntx) << TW_SHIFT;
    const int len = min(TW, a.ncols - c0);
    T* dst = out + (unsigned long long)rowid * (unsigned long long)a.ncols + c0;
    if (n == 0) {
      store_bg<T>(dst, len, a.bg16, bg, lane, 32);
      continue;
    }
    if (n > FILL_WARP_MAX) {
      if (lane == 0) a.big[atomicAdd(&a.ctrl->big_count, 1u)] = (unsigned)b;
      continue;
    }
    // this lane's records: positions lane and lane + 32
    uint2 r0 = make_uint2(0u, 0u), r1 = make_uint2(0u, 0u);
    unsigned k0 = 0xFFFFFFFFu, k1 = 0xFFFFFFFFu;
    if (lane < n) { r0 = a.recs[o0 + lane]; k0 = rec_key(r0.x); }
    if (lane + 32 < n) { r1 = a.recs[o0 + lane + 32]; k1 = rec_key(r1.x); }
    T v0 = T(0), v1 = T(0);
    if (lane < n) v0 = value_of<T>(a, r0.x & REC_PART_MASK);
    if (lane + 32 < n) v1 = value_of<T>(a, r1.x & REC_PART_MASK);
    if (lane < n) keys[lane] = k0;
    if (lane + 32 < n) keys[lane + 32] = k1;
    // background tile
    {
      uint4* c4 = reinterpret_cast<uint4*>(cur);
      for (int i = lane; i < (int)(TW * sizeof(T) / 16); i += 32) c4[i] = a.bg16;
    }
    __syncwarp();
    // rank = smaller keys + equal keys at smaller positions
    int rk0 = 0, rk1 = 0;
    for (int j = 0; j < n; ++j) {
      const unsigned kj = keys[j];
      rk0 += (kj < k0) || (kj == k0 && j < lane);
      rk1 += (kj < k1) || (kj == k1 && j < lane + 32);
    }
    if (lane < n) {
      SRec e;
      e.key = k0 | (r0.x & DEDUP_BIT);
      e.mask = r0.y;
      e.vbits = to_bits<T>(v0);
      srec[rk0] = e;
    }
    if (lane + 32 < n) {
      SRec e;
      e.key = k1 | (r1.x & DEDUP_BIT);
      e.mask = r1.y;
      e.vbits = to_bits<T>(v1);
      srec[rk1] = e;
    }
    __syncwarp();
    unsigned prev_key = 0xFFFFFFFFu, seen = 0u;
    for (int j = 0; j < n; ++j) {
      const SRec e = srec[j];
      const unsigned key = e.key & ~DEDUP_BIT;
      unsigned mask = e.mask;
      if (DEDUP && (e.key & DEDUP_BIT)) {
        if (key != prev_key) seen = 0u;
        mask &= ~seen;
        seen |= e.mask;
      }
      prev_key = key;
      const int w = (int)(key & 15u);
      const bool on = (mask >> lane) & 1u;
      T c = cur[w * 32 + lane];
      apply_step<T, FN>(c, from_bits<T>(e.vbits), on, bg, bgc);
      if (on) cur[w * 32 + lane] = c;
    }
    __syncwarp();
    store_tile<T>(dst, cur, len, lane, 32);
    __syncwarp();
  }
}

// ---- deep buckets: one warp per (bucket, word) --------------------------
// The word's records are taken in part order, at most BIG_CAP at a time: a
// histogram over the pending part ids picks the largest prefix range that
// fits, the range is gathered, sorted (bitonic, shared memory) and applied;
// lane l keeps pixel l of the word in a register throughout.  A single part
// with more than BIG_CAP records in the word is applied in chunks (its
// records share one value and their order does not change the result).
constexpr int BIG_WARPS = 4;
constexpr int BIG_HIST = 256;

constexpr int big_warp_bytes() { return BIG_CAP * 8 + BIG_HIST * 4; }

__device__ __forceinline__ void warp_sort_keys(unsigned long long* k, int n) {
  // ascending bitonic sort of k[0..np) with np = next power of two >= n (padded with ~0)
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
          if ((x > y) == up) { k[i] = y; k[ixj] = x; }
        }
      }
      __syncwarp();
    }
  }
}

template <typename T, int FN, bool DEDUP>
__global__ void __launch_bounds__(BIG_WARPS * 32) k_fill_big(FillArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Ctrl* ctrl = a.ctrl;
  if (ctrl->err || ctrl->span_count > a.rec_cap) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem + warp * big_warp_bytes());
  unsigned* hist = reinterpret_cast<unsigned*>(keys + BIG_CAP);
  const T bg = from_bits<T>(a.bg);
  const BgF64 bgc = bg_f64(a.bg);
  T* out = static_cast<T*>(a.out);
  const unsigned long long items = (unsigned long long)ctrl->big_count * WPT;
  const unsigned long long nwarps = (unsigned long long)gridDim.x * BIG_WARPS;
  for (unsigned long long it = (unsigned long long)blockIdx.x * BIG_WARPS + warp; it < items; it += nwarps) {
    const unsigned long long b = a.big[it / WPT];
    const unsigned wsel = (unsigned)(it % WPT);
    const unsigned o0 = a.offsets[b];
    const int n = (int)(a.offsets[b + 1] - o0);
    const unsigned rowid = (unsigned)b / a.ntx;
    const int c0 = (int)((unsigned)b - rowid * a.ntx) << TW_SHIFT;
    const int x = c0 + (int)wsel * 32 + lane;
    T c = bg;
    unsigned lo_part = 0;  // parts < lo_part are done
    unsigned prev_key = 0xFFFFFFFFu, seen = 0u;
    while (true) {
      unsigned cnt = 0, pmin = 0xFFFFFFFFu, pmax = 0;
      for (int i = lane; i < n; i += 32) {
        const unsigned rx = a.recs[o0 + i].x;
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
      unsigned hi = pmax + 1;  // parts [pmin, hi) this round
      bool single = false;
      if (cnt > (unsigned)BIG_CAP) {
        unsigned span_lo = pmin, span_hi = pmax;  // inclusive
        while (true) {
          int shift = 0;
          while (((span_hi - span_lo) >> shift) >= (unsigned)BIG_HIST) ++shift;
          for (int h = lane; h < BIG_HIST; h += 32) hist[h] = 0u;
          __syncwarp();
          for (int i = lane; i < n; i += 32) {
            const unsigned rx = a.recs[o0 + i].x;
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
      // gather [lo_part, hi) of this word, in chunks of BIG_CAP when single
      int m = 0;
      for (int i0 = 0; i0 < n; i0 += 32) {
        const int i = i0 + lane;
        uint2 r = make_uint2(0u, 0u);
        bool take = false;
        if (i < n) {
          r = a.recs[o0 + i];
          const unsigned part = r.x & REC_PART_MASK;
          take = ((r.x >> REC_W_SHIFT) & 15u) == wsel && part >= lo_part && part < hi;
        }
        const unsigned mk = __ballot_sync(0xFFFFFFFFu, take);
        if (take) {
          const int pos = m + __popc(mk & ((1u << lane) - 1u));
          // part (order), then the DEDUP flag, then the mask
          keys[pos] = ((unsigned long long)(r.x & REC_PART_MASK) << 33) |
                      ((unsigned long long)(r.x >> 31) << 32) | r.y;
        }
        m += __popc(mk);
        if (single && m > BIG_CAP - 32) {  // flush a chunk of the single part
          __syncwarp();
          const T v = value_of<T>(a, hi - 1);
          for (int j = 0; j < m; ++j) {
            const unsigned long long kj = keys[j];
            unsigned mask = (unsigned)kj;
            const unsigned part = (unsigned)(kj >> 33);
            if (DEDUP && ((kj >> 32) & 1u)) {
              if (part != prev_key) seen = 0u;
              mask &= ~seen;
              seen |= (unsigned)kj;
            }
            prev_key = part;
            apply_step<T, FN>(c, v, (mask >> lane) & 1u, bg, bgc);
          }
          m = 0;
          __syncwarp();
        }
      }
      __syncwarp();
      if (!single) warp_sort_keys(keys, m);
      for (int j0 = 0; j0 < m; j0 += 32) {  // values of this chunk, 32 at a time
        T vj = T(0);
        if (j0 + lane < m) vj = value_of<T>(a, (unsigned)(keys[j0 + lane] >> 33));
        const int jn = min(32, m - j0);
        for (int jj = 0; jj < jn; ++jj) {
          const unsigned long long kj = keys[j0 + jj];
          const T v = shfl_val<T>(vj, jj);
          unsigned mask = (unsigned)kj;
          const unsigned part = (unsigned)(kj >> 33);
          if (DEDUP && ((kj >> 32) & 1u)) {
            if (part != prev_key) seen = 0u;
            mask &= ~seen;
            seen |= (unsigned)kj;
          }
          prev_key = part;
          apply_step<T, FN>(c, v, (mask >> lane) & 1u, bg, bgc);
        }
      }
      __syncwarp();
      lo_part = hi;
    }
    if (x < a.ncols) out[(unsigned long long)rowid * (unsigned long long)a.ncols + x] = c;
  }
}

// ---- order-free fill: count / any --------------------------------------
// Integer `count` with background 0 (and float count with background 0 or
// NaN) equals the pixel's coverage depth: every write after the first adds
// one and no intermediate count can equal the background.  `any` is 1
// wherever the depth is non-zero.  Neither needs values or order: one warp
// per bucket adds every record's mask bits into per-pixel depths (lane l
// owns pixel l of every word).
constexpr int DEPTH_WARPS = 8;

template <typename T, int FN>
__global__ void __launch_bounds__(DEPTH_WARPS * 32) k_fill_depth(FillArgs a) {
  __shared__ unsigned s_depth[DEPTH_WARPS][TW];
  const Ctrl* ctrl = a.ctrl;
  if (ctrl->err || ctrl->span_count > a.rec_cap) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned* depth = s_depth[warp];
  const T bg = from_bits<T>(a.bg);
  T* out = static_cast<T*>(a.out);
  const unsigned long long nwarps = (unsigned long long)gridDim.x * DEPTH_WARPS;
  for (unsigned long long b = (unsigned long long)blockIdx.x * DEPTH_WARPS + warp; b < a.nbuckets; b += nwarps) {
    const unsigned o0 = a.offsets[b];
    const int n = (int)(a.offsets[b + 1] - o0);
    const unsigned rowid = (unsigned)b / a.ntx;
    const int c0 = (int)((unsigned)b - rowid * a.ntx) << TW_SHIFT;
    const int len = min(TW, a.ncols - c0);
    T* dst = out + (unsigned long long)rowid * (unsigned long long)a.ncols + c0;
    if (n == 0) {
      store_bg<T>(dst, len, a.bg16, bg, lane, 32);
      continue;
    }
#pragma unroll
    for (int w = 0; w < WPT; ++w) depth[w * 32 + lane] = 0u;
    for (int i0 = 0; i0 < n; i0 += 32) {
      uint2 r = make_uint2(0u, 0u);
      if (i0 + lane < n) r = a.recs[o0 + i0 + lane];
      const int jn = min(32, n - i0);
      for (int j = 0; j < jn; ++j) {
        const unsigned rx = __shfl_sync(0xFFFFFFFFu, r.x, j), ry = __shfl_sync(0xFFFFFFFFu, r.y, j);
        const int w = (int)((rx >> REC_W_SHIFT) & 15u);
        depth[w * 32 + lane] += (ry >> lane) & 1u;
      }
    }
#pragma unroll
    for (int w = 0; w < WPT; ++w) {
      const unsigned d = depth[w * 32 + lane];
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
  if (depth_exact<T>(a, fn, dedup)) {
    unsigned long long want = (a.nbuckets + DEPTH_WARPS - 1) / DEPTH_WARPS;
    unsigned grid = (unsigned)(want < (unsigned long long)num_sms * 16 ? want : num_sms * 16ull);
    if (grid == 0) grid = 1;
    if (fn == F_ANY) k_fill_depth<T, F_ANY><<<grid, DEPTH_WARPS * 32, 0, s>>>(a);
    else k_fill_depth<T, F_COUNT><<<grid, DEPTH_WARPS * 32, 0, s>>>(a);
    return 1;
  }
  int launches = 0;
#define RZ_FILL_CASE(FNV, DD)                                                                             \
  {                                                                                                       \
    constexpr int ws = FILL_WARPS_PER_BLOCK * fill_warp_bytes<T>();                                       \
    constexpr int bs = BIG_WARPS * big_warp_bytes();                                                      \
    cudaFuncSetAttribute(k_fill_warp<T, FNV, DD>, cudaFuncAttributeMaxDynamicSharedMemorySize, ws);       \
    cudaFuncSetAttribute(k_fill_big<T, FNV, DD>, cudaFuncAttributeMaxDynamicSharedMemorySize, bs);        \
    unsigned long long want = (a.nbuckets + FILL_WARPS_PER_BLOCK - 1) / FILL_WARPS_PER_BLOCK;             \
    unsigned grid = (unsigned)(want < (unsigned long long)num_sms * 16 ? want : num_sms * 16ull);         \
    if (grid == 0) grid = 1;                                                                              \
    k_fill_warp<T, FNV, DD><<<grid, FILL_WARPS_PER_BLOCK * 32, ws, s>>>(a);                               \
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
