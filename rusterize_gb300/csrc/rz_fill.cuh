// rz_fill.cuh -- bucket fill: every (band, row, column-tile) bucket is staged
// in shared memory as `background`, its spans are applied in part order
// (= the reference's per-geometry write order, rasterize.rs:162-196) with
// the pixel function, and the tile is written to the raster once.
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
  const uint2* spans;       // {part, xs} grouped by bucket
  unsigned long long nbuckets;
  const void* values;       // per-geometry values, or nullptr
  unsigned long long scalar;  // raw bits of the single value when values == nullptr
  const unsigned* part_geom;
  void* out;                // (bands, nrows, ncols)
  unsigned long long bg;    // raw bits of the background
  uint4 bg16;               // background replicated over 16 bytes
  int nrows, ncols;
  unsigned ntx;
  unsigned* big;            // buckets left to the block-level kernel
  Ctrl* ctrl;
  unsigned long long span_cap;
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



// ascending bitonic sort of keys[0..n) (n a power of two) by the block
__device__ __forceinline__ void block_sort_smem(unsigned long long* keys, int n) {
  for (int k = 2; k <= n; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const unsigned long long a = keys[i], b = keys[ixj];
          const bool up = (i & k) == 0;
          if ((a > b) == up) { keys[i] = b; keys[ixj] = a; }
        }
      }
      __syncthreads();
    }
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

// ---- per-pixel fill ------------------------------------------------------
// One warp per bucket.  Each pixel of the tile keeps the indices of up to
// PX_K spans covering it; every lane then folds its own pixels, applying
// those spans in part order -- exactly the reference's per-pixel write order,
// with no per-bucket sort.  Spans longer than PX_LONG are spread over the
// warp.  Buckets with more than SMALL_MAX spans, or with a pixel covered more
// than PX_K times, are left to the block-level kernel.
constexpr int PX_K = 8;
constexpr int PX_LONG = 64;
constexpr int PX_WARPS = 4;

template <typename T>
constexpr int px_warp_bytes() {
  return SMALL_MAX * 8 + ((SMALL_MAX * (int)sizeof(T) + 15) / 16) * 16 + TW * 2 + TW * PX_K + SMALL_MAX + TW * 4;
}

template <typename T>
constexpr int small_smem_bytes() {
  return PX_WARPS * px_warp_bytes<T>();
}

// register pixel x for span i; true when the pixel list overflows
__device__ __forceinline__ bool px_add(unsigned* depth, unsigned char* lists, int x, int i) {
  const unsigned sh = (x & 1) * 16;
  const unsigned d = (atomicAdd(&depth[x >> 1], 1u << sh) >> sh) & 0xFFFFu;
  if (d < PX_K) {
    lists[x * PX_K + d] = (unsigned char)i;
    return false;
  }
  return true;
}

__device__ __forceinline__ void cswap(unsigned long long& a, unsigned long long& b) {
  const unsigned long long lo = a < b ? a : b, hi = a < b ? b : a;
  a = lo;
  b = hi;
}

template <typename T, int FN, bool DEDUP>
__global__ void __launch_bounds__(PX_WARPS * 32) k_fill_small(FillArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Ctrl* ctrl = a.ctrl;
  if (ctrl->err || ctrl->span_count > a.span_cap) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char* base = smem + warp * px_warp_bytes<T>();
  uint2* sp = reinterpret_cast<uint2*>(base);
  T* vals = reinterpret_cast<T*>(base + SMALL_MAX * 8);
  unsigned* depth = reinterpret_cast<unsigned*>(base + SMALL_MAX * 8 + ((SMALL_MAX * (int)sizeof(T) + 15) / 16) * 16);
  unsigned char* lists = reinterpret_cast<unsigned char*>(depth + TW / 2);
  unsigned char* longs = lists + TW * PX_K;
  unsigned short* deep = reinterpret_cast<unsigned short*>(longs + SMALL_MAX);
  const T bg = from_bits<T>(a.bg);
  const BgF64 bgc = bg_f64(a.bg);
  T* out = static_cast<T*>(a.out);
  const unsigned long long nwarps = (unsigned long long)gridDim.x * PX_WARPS;
  for (unsigned long long b = (unsigned long long)blockIdx.x * PX_WARPS + warp; b < a.nbuckets; b += nwarps) {
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
    if (n > SMALL_MAX) {
      if (lane == 0) a.big[atomicAdd(&a.ctrl->big_count, 1u)] = (unsigned)b;
      continue;
    }
    for (int i = lane; i < n; i += 32) {
      const uint2 s = a.spans[o0 + i];
      sp[i] = s;
      vals[i] = value_of<T>(a, s.x);
    }
    for (int i = lane; i < TW / 2; i += 32) depth[i] = 0u;
    __syncwarp();
    // coverage: pixel writes are dealt to lanes with a warp prefix sum over
    // the span lengths (every lane registers one pixel per step)
    bool over = false;
    for (int i0 = 0; i0 < n; i0 += 32) {
      const int i = i0 + lane;
      int x0 = 0, ln = 0;
      if (i < n) {
        const unsigned xs = sp[i].y;
        x0 = (int)(xs & X_MASK);
        ln = (int)((xs >> 12) & X_MASK) - x0;
      }
      int incl = ln;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += t;
      }
      const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
      const int excl = incl - ln;
      for (int m0 = 0; m0 < total; m0 += 32) {
        const int m = m0 + lane;
        int s = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
          const int e = __shfl_sync(0xFFFFFFFFu, excl, s + step);
          if (e <= m) s += step;
        }
        const int es = __shfl_sync(0xFFFFFFFFu, excl, s);
        const int xs0 = __shfl_sync(0xFFFFFFFFu, x0, s);
        if (m < total) over |= px_add(depth, lists, xs0 + (m - es), i0 + s);
      }
    }
    if (__any_sync(0xFFFFFFFFu, over)) {
      if (lane == 0) a.big[atomicAdd(&a.ctrl->big_count, 1u)] = (unsigned)b;
      __syncwarp();
      continue;
    }
    __syncwarp();
    // pixels covered at most once are resolved in place; deeper ones are
    // queued: depth-2 pixels (most of them) are folded in one dense pass,
    // deeper ones go through a second queue and the general sorted fold, so
    // the FP64 adds of a float sum run with dense lanes
    int ndeep = 0;
    for (int x0 = 0; x0 < len; x0 += 32) {
      const int x = x0 + lane;
      unsigned d = 0;
      if (x < len) d = (depth[x >> 1] >> ((x & 1) * 16)) & 0xFFFFu;
      const bool dp = d >= 2;
      const unsigned m = __ballot_sync(0xFFFFFFFFu, dp);
      if (dp) deep[ndeep + __popc(m & ((1u << lane) - 1u))] = (unsigned short)x;
      ndeep += __popc(m);
      if (x < len && !dp) dst[x] = d == 1 ? first_write<T, FN>(vals[lists[x * PX_K]]) : bg;
    }
    __syncwarp();
    int nd3 = 0;
    unsigned short* deep3 = deep + TW;  // second queue, after the first
    for (int q0 = 0; q0 < ndeep; q0 += 32) {
      const int q = q0 + lane;
      int x = 0;
      unsigned d = 0;
      if (q < ndeep) {
        x = deep[q];
        d = (depth[x >> 1] >> ((x & 1) * 16)) & 0xFFFFu;
      }
      const bool d3 = d >= 3;
      const unsigned m = __ballot_sync(0xFFFFFFFFu, d3);
      if (d3) deep3[nd3 + __popc(m & ((1u << lane) - 1u))] = (unsigned short)x;
      nd3 += __popc(m);
      if (d == 2) {
        // two spans in part order (the same part twice is a line; with the
        // PixelCache it counts once)
        unsigned i0 = lists[x * PX_K], i1 = lists[x * PX_K + 1];
        unsigned p0 = sp[i0].x, p1 = sp[i1].x;
        if (p1 < p0 || (p1 == p0 && i1 < i0)) {
          const unsigned ti = i0; i0 = i1; i1 = ti;
          const unsigned tp = p0; p0 = p1; p1 = tp;
        }
        T cur = first_write<T, FN>(vals[i0]);
        if (!(DEDUP && p1 == p0 && (sp[i1].y & DEDUP_BIT))) apply_one<T, FN>(cur, vals[i1], bg, bgc);
        dst[x] = cur;
      }
    }
    __syncwarp();
    for (int q = lane; q < nd3; q += 32) {
      const int x = deep3[q];
      const unsigned d = (depth[x >> 1] >> ((x & 1) * 16)) & 0xFFFFu;
      const uint2 pk = *reinterpret_cast<const uint2*>(lists + x * PX_K);
      unsigned long long k[PX_K];
#pragma unroll
      for (int j = 0; j < PX_K; ++j) {
        const unsigned idx = ((j < 4 ? pk.x : pk.y) >> (8 * (j & 3))) & 0xFFu;
        k[j] = (unsigned)j < d ? (((unsigned long long)sp[idx].x << 32) | idx) : ~0ull;
      }
      // sort by (part, span index): 4-key network, or Batcher's 8-key
      // odd-even merge network when more than 4 spans cover the pixel
      if (d <= 4) {
        cswap(k[0], k[1]); cswap(k[2], k[3]); cswap(k[0], k[2]); cswap(k[1], k[3]); cswap(k[1], k[2]);
      } else {
        cswap(k[0], k[1]); cswap(k[2], k[3]); cswap(k[4], k[5]); cswap(k[6], k[7]);
        cswap(k[0], k[2]); cswap(k[1], k[3]); cswap(k[4], k[6]); cswap(k[5], k[7]);
        cswap(k[1], k[2]); cswap(k[5], k[6]);
        cswap(k[0], k[4]); cswap(k[1], k[5]); cswap(k[2], k[6]); cswap(k[3], k[7]);
        cswap(k[2], k[4]); cswap(k[3], k[5]);
        cswap(k[1], k[2]); cswap(k[3], k[4]); cswap(k[5], k[6]);
      }
      unsigned prev = (unsigned)(k[0] >> 32);
      T cur = first_write<T, FN>(vals[(unsigned)k[0] & 0xFFu]);
      for (unsigned j = 1; j < d; ++j) {
        const unsigned long long kj = j < 4 ? (j < 2 ? k[1] : (j == 2 ? k[2] : k[3]))
                                           : (j < 6 ? (j == 4 ? k[4] : k[5]) : (j == 6 ? k[6] : k[7]));
        const unsigned idx = (unsigned)kj & 0xFFu, part = (unsigned)(kj >> 32);
        if (DEDUP && (sp[idx].y & DEDUP_BIT) && part == prev) continue;  // PixelCache
        prev = part;
        apply_one<T, FN>(cur, vals[idx], bg, bgc);
      }
      dst[x] = cur;
    }
    __syncwarp();
  }
}

// ---- order-free fill: count / any --------------------------------------
// Integer `count` with background 0 (and float count with background 0 or
// NaN) equals the pixel's coverage depth: every write after the first adds
// one and no intermediate count can equal the background.  `any` is 1
// wherever the depth is non-zero.  Neither needs values, lists or order.
constexpr int DEPTH_WARPS = 8;
constexpr int DEPTH_MAX_SPANS = 65535;  // 16-bit depth counters

template <typename T, int FN>
__global__ void __launch_bounds__(DEPTH_WARPS * 32) k_fill_depth(FillArgs a) {
  __shared__ unsigned s_depth[DEPTH_WARPS][TW / 2];
  const Ctrl* ctrl = a.ctrl;
  if (ctrl->err || ctrl->span_count > a.span_cap) return;
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
    if (n > DEPTH_MAX_SPANS) {
      if (lane == 0) a.big[atomicAdd(&a.ctrl->big_count, 1u)] = (unsigned)b;
      continue;
    }
    for (int i = lane; i < TW / 2; i += 32) depth[i] = 0u;
    __syncwarp();
    for (int i0 = 0; i0 < n; i0 += 32) {
      const int i = i0 + lane;
      int x0 = 0, ln = 0;
      if (i < n) {
        const unsigned xs = a.spans[o0 + i].y;
        x0 = (int)(xs & X_MASK);
        ln = (int)((xs >> 12) & X_MASK) - x0;
      }
      int incl = ln;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += t;
      }
      const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
      const int excl = incl - ln;
      for (int m0 = 0; m0 < total; m0 += 32) {
        const int m = m0 + lane;
        int s = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
          const int e = __shfl_sync(0xFFFFFFFFu, excl, s + step);
          if (e <= m) s += step;
        }
        const int es = __shfl_sync(0xFFFFFFFFu, excl, s);
        const int xs0 = __shfl_sync(0xFFFFFFFFu, x0, s);
        if (m < total) {
          const int x = xs0 + (m - es);
          atomicAdd(&depth[x >> 1], 1u << ((x & 1) * 16));
        }
      }
    }
    __syncwarp();
    for (int x = lane; x < len; x += 32) {
      const unsigned d = (depth[x >> 1] >> ((x & 1) * 16)) & 0xFFFFu;
      T v = bg;
      if (d) {
        if constexpr (FN == F_ANY) v = T(1);
        else if constexpr (std::is_integral<T>::value) v = (T)(typename std::make_unsigned<T>::type)d;
        else v = (T)d;
      }
      dst[x] = v;
    }
    __syncwarp();
  }
}

constexpr int BIG_THREADS = 256;
constexpr int BIG_HIST = 1024;

template <typename T, bool DEDUP>
constexpr int big_smem_bytes() {
  return seg_bytes<T>() + BIG_CAP * 8 + BIG_CAP * (int)sizeof(T) + (DEDUP ? TW * 4 : 0) + BIG_HIST * 4;
}

// apply keys[0..m) in order: thread t owns tile columns [4t, 4t+4)
template <typename T, int FN, bool DEDUP>
__device__ __forceinline__ void block_apply(T* seg, unsigned* mark, const unsigned long long* keys, const T* vals,
                                            int m, T bg, const BgF64& bgc) {
  constexpr int PPT = TW / BIG_THREADS;
  const int lo = threadIdx.x * PPT, hi = lo + PPT;
  for (int k = 0; k < m; ++k) {
    const unsigned long long kk = keys[k];
    const unsigned xs = (unsigned)kk;
    const int x0 = (int)(xs & X_MASK), x1 = (int)((xs >> 12) & X_MASK);
    if (x1 <= lo || x0 >= hi) continue;
    const T v = vals[k];
    const int e = min(x1, hi);
    if (DEDUP && (xs & DEDUP_BIT)) {
      const unsigned part = (unsigned)(kk >> 32);
      for (int x = max(x0, lo); x < e; ++x)
        if (mark[x] != part) { mark[x] = part; apply_one<T, FN>(seg[x], v, bg, bgc); }
    } else {
      for (int x = max(x0, lo); x < e; ++x) apply_one<T, FN>(seg[x], v, bg, bgc);
    }
  }
}

// One block per deferred bucket.  Spans are taken in part order, at most
// BIG_CAP at a time: a 1024-bin histogram over the part ids still pending
// picks the largest prefix range that fits; a single part with more than
// BIG_CAP spans is applied in chunks (its spans share one value and their
// relative order does not change the result).
template <typename T, int FN, bool DEDUP>
__global__ void __launch_bounds__(BIG_THREADS) k_fill_big(FillArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Ctrl* ctrl = a.ctrl;
  if (ctrl->err || ctrl->span_count > a.span_cap) return;
  T* seg = reinterpret_cast<T*>(smem);
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem + seg_bytes<T>());
  T* vals = reinterpret_cast<T*>(smem + seg_bytes<T>() + BIG_CAP * 8);
  unsigned* mark = reinterpret_cast<unsigned*>(smem + seg_bytes<T>() + BIG_CAP * 8 + BIG_CAP * sizeof(T));
  unsigned* hist = reinterpret_cast<unsigned*>(smem + seg_bytes<T>() + BIG_CAP * 8 + BIG_CAP * sizeof(T) +
                                               (DEDUP ? TW * 4 : 0));
  __shared__ unsigned s_cnt, s_min, s_max;
  __shared__ unsigned long long s_hi;
  __shared__ int s_single;
  const T bg = from_bits<T>(a.bg);
  const BgF64 bgc = bg_f64(a.bg);
  T* out = static_cast<T*>(a.out);
  const unsigned nbig = ctrl->big_count;
  for (unsigned bi = blockIdx.x; bi < nbig; bi += gridDim.x) {
    const unsigned long long b = a.big[bi];
    const unsigned o0 = a.offsets[b];
    const int n = (int)(a.offsets[b + 1] - o0);
    const unsigned long long rowid = (unsigned)b / a.ntx;
    const int c0 = (int)(b - rowid * a.ntx) << TW_SHIFT;
    const int len = min(TW, a.ncols - c0);
    T* dst = out + rowid * (unsigned long long)a.ncols + c0;
    for (int i = threadIdx.x; i < TW; i += BIG_THREADS) {
      seg[i] = bg;
      if (DEDUP) mark[i] = 0xFFFFFFFFu;
    }
    __syncthreads();
    unsigned long long lo_part = 0;  // parts < lo_part are done
    while (true) {
      // pending part range
      if (threadIdx.x == 0) { s_cnt = 0; s_min = 0xFFFFFFFFu; s_max = 0; }
      __syncthreads();
      unsigned lmin = 0xFFFFFFFFu, lmax = 0, lcnt = 0;
      for (int i = threadIdx.x; i < n; i += BIG_THREADS) {
        const unsigned part = a.spans[o0 + i].x;
        if (part >= lo_part) { lmin = min(lmin, part); lmax = max(lmax, part); ++lcnt; }
      }
      if (lcnt) { atomicMin(&s_min, lmin); atomicMax(&s_max, lmax); atomicAdd(&s_cnt, lcnt); }
      __syncthreads();
      const unsigned cnt = s_cnt;
      if (cnt == 0) break;
      const unsigned pmin = s_min;
      unsigned long long pmax = s_max;
      if (cnt <= (unsigned)BIG_CAP) {
        if (threadIdx.x == 0) { s_hi = pmax + 1; s_single = 0; }
      } else {
        while (true) {
          int shift = 0;
          while (((pmax - pmin) >> shift) >= (unsigned long long)BIG_HIST) ++shift;
          for (int i = threadIdx.x; i < BIG_HIST; i += BIG_THREADS) hist[i] = 0;
          __syncthreads();
          for (int i = threadIdx.x; i < n; i += BIG_THREADS) {
            const unsigned part = a.spans[o0 + i].x;
            if (part >= pmin && part <= pmax) atomicAdd(&hist[(part - pmin) >> shift], 1u);
          }
          __syncthreads();
          if (threadIdx.x == 0) {
            unsigned cum = 0;
            int j = -1;
            for (int h = 0; h < BIG_HIST; ++h) {
              if (cum + hist[h] > (unsigned)BIG_CAP) break;
              cum += hist[h];
              j = h;
            }
            s_single = 0;
            if (j >= 0) s_hi = (unsigned long long)pmin + ((unsigned long long)(j + 1) << shift);
            else if (shift == 0) { s_hi = (unsigned long long)pmin + 1; s_single = 1; }
            else s_hi = 0;  // zoom into the first bin
          }
          __syncthreads();
          if (s_hi != 0) break;
          pmax = (unsigned long long)pmin + (1ull << shift) - 1;
          __syncthreads();
        }
      }
      __syncthreads();  // s_hi / s_single are written by thread 0 above
      const unsigned long long hi = s_hi;
      const bool single = s_single != 0;
      __syncthreads();
      if (!single) {
        if (threadIdx.x == 0) s_cnt = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += BIG_THREADS) {
          const uint2 sp = a.spans[o0 + i];
          if (sp.x >= pmin && (unsigned long long)sp.x < hi) {
            const unsigned slot = atomicAdd(&s_cnt, 1u);
            keys[slot] = ((unsigned long long)sp.x << 32) | sp.y;
          }
        }
        __syncthreads();
        const int m = (int)s_cnt;
        int np = 1;
        while (np < m) np <<= 1;
        for (int i = m + threadIdx.x; i < np; i += BIG_THREADS) keys[i] = ~0ull;
        __syncthreads();
        block_sort_smem(keys, np);
        for (int i = threadIdx.x; i < m; i += BIG_THREADS) vals[i] = value_of<T>(a, (unsigned)(keys[i] >> 32));
        __syncthreads();
        block_apply<T, FN, DEDUP>(seg, mark, keys, vals, m, bg, bgc);
        __syncthreads();
      } else {
        // one part with more than BIG_CAP spans: any order, in chunks
        const T v = value_of<T>(a, pmin);
        for (int base = 0; base < n; base += BIG_CAP) {
          if (threadIdx.x == 0) s_cnt = 0;
          __syncthreads();
          for (int i = base + threadIdx.x; i < min(n, base + BIG_CAP); i += BIG_THREADS) {
            const uint2 sp = a.spans[o0 + i];
            if (sp.x == pmin) {
              const unsigned slot = atomicAdd(&s_cnt, 1u);
              keys[slot] = ((unsigned long long)sp.x << 32) | sp.y;
              vals[slot] = v;
            }
          }
          __syncthreads();
          block_apply<T, FN, DEDUP>(seg, mark, keys, vals, (int)s_cnt, bg, bgc);
          __syncthreads();
        }
      }
      lo_part = hi;
      __syncthreads();
    }
    store_tile<T>(dst, seg, len, threadIdx.x, BIG_THREADS);
    __syncthreads();
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
  int launches = 0;
  if (depth_exact<T>(a, fn, dedup)) {
    unsigned long long want = (a.nbuckets + DEPTH_WARPS - 1) / DEPTH_WARPS;
    unsigned grid = (unsigned)(want < (unsigned long long)num_sms * 16 ? want : num_sms * 16ull);
    if (grid == 0) grid = 1;
    if (fn == F_ANY) {
      k_fill_depth<T, F_ANY><<<grid, DEPTH_WARPS * 32, 0, s>>>(a);
      cudaFuncSetAttribute(k_fill_big<T, F_ANY, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           big_smem_bytes<T, false>());
      k_fill_big<T, F_ANY, false><<<num_sms * 2, BIG_THREADS, big_smem_bytes<T, false>(), s>>>(a);
    } else {
      k_fill_depth<T, F_COUNT><<<grid, DEPTH_WARPS * 32, 0, s>>>(a);
      cudaFuncSetAttribute(k_fill_big<T, F_COUNT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           big_smem_bytes<T, false>());
      k_fill_big<T, F_COUNT, false><<<num_sms * 2, BIG_THREADS, big_smem_bytes<T, false>(), s>>>(a);
    }
    return 2;
  }
#define RZ_FILL_CASE(FNV, DD)                                                                        \
  {                                                                                                  \
    constexpr int ss = small_smem_bytes<T>();                                                        \
    constexpr int bs = big_smem_bytes<T, DD>();                                                      \
    cudaFuncSetAttribute(k_fill_small<T, FNV, DD>, cudaFuncAttributeMaxDynamicSharedMemorySize, ss); \
    cudaFuncSetAttribute(k_fill_big<T, FNV, DD>, cudaFuncAttributeMaxDynamicSharedMemorySize, bs);   \
    unsigned long long want = (a.nbuckets + PX_WARPS - 1) / PX_WARPS;                                \
    unsigned grid = (unsigned)(want < (unsigned long long)num_sms * 32 ? want : num_sms * 32ull);    \
    if (grid == 0) grid = 1;                                                                         \
    k_fill_small<T, FNV, DD><<<grid, PX_WARPS * 32, ss, s>>>(a);                                     \
    k_fill_big<T, FNV, DD><<<num_sms * 2, BIG_THREADS, bs, s>>>(a);                                  \
    launches += 2;                                                                                   \
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
