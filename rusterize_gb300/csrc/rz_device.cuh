// rz_device.cuh -- device-side types and helpers shared by the engine's
// kernels (span generation, bucketing, fill).  sm_103a only.
#pragma once

#include <cooperative_groups.h>
#include <cstdint>
#include <cuda_runtime.h>

#include "rz_bits.h"

namespace rzd {

namespace cg = cooperative_groups;

// ---- tiling --------------------------------------------------------------
// The output is cut into buckets of (band, row, column tile).  A tile is TW
// pixels (WPT 32-pixel words) of one row; the fill kernels own one bucket at
// a time and write each output pixel exactly once.
constexpr int TW_SHIFT = 9;
constexpr int TW = 1 << TW_SHIFT;
constexpr int WPT = TW / 32;

// Coverage records.  Span generation emits one record per (part, raster
// row, 32-pixel word) that the part covers: the word id
// ((band * nrows + row) * ntx * WPT + word of the row), the part and the
// 32-bit mask of covered pixels.  After the scatter a record is
// {part | word-in-tile << REC_W_SHIFT | DEDUP_BIT, mask}, grouped by bucket.
constexpr uint32_t REC_W_SHIFT = 27;
constexpr uint32_t REC_PART_MASK = (1u << REC_W_SHIFT) - 1u;  // parts are < 2^27
// the part deduplicates its writes (PixelCache semantics): a pixel covered
// by several records of the part is written once
constexpr uint32_t DEDUP_BIT = 1u << 31;

// Polygon scanline windows: per (part, row window) a parity bitmap of
// BITMAP_WORDS 32-bit words lives in shared memory.
// Narrow parts (bitmap row <= SMALL_BW words) take one warp per window with
// a small bitmap; wider parts take one block per window.
constexpr int BITMAP_WORDS = 8192;
// Parts wider than BITMAP_WORDS words take column windows of COLWIN_WORDS
// words and COLWIN_ROWS rows; a crossing left of a column window only flips
// its row's parity, one right of it is only counted.
constexpr int COLWIN_WORDS = 1024;
constexpr int COLWIN_ROWS = BITMAP_WORDS / COLWIN_WORDS;
constexpr int WR_MAX = 128;                 // rows per window
constexpr int POLY_THREADS = 256;
constexpr int POLY_QENT = 32;               // bytes of one queued edge
constexpr int POLY_WARP_QCAP = 64;          // queued edges per warp
constexpr int POLY_SMEM = BITMAP_WORDS * 4 + (POLY_THREADS / 32) * POLY_WARP_QCAP * POLY_QENT;
constexpr int SMALL_BW = 32;
constexpr int SMALL_BITMAP_WORDS = 1024;
constexpr int SMALL_WARPS = 4;  // warps (independent windows) per block
constexpr int SMALL_WARP_SMEM = POLY_WARP_QCAP * POLY_QENT + SMALL_BITMAP_WORDS * 4 + 3 * WR_MAX * 4 + 16;
constexpr int SMALL_SMEM = SMALL_WARPS * SMALL_WARP_SMEM;

// Launch shapes and thresholds that change only the schedule, never a
// result: every setting burns the same records in the same order per pixel.
// The context holds one set (rz_tuning in the C ABI); the autotuner picks it.
struct Tune {
  int narrow_chunk;      // narrow polygon windows taken per work grab (1..64)
  int rows_per_window;   // polygon window height cap (8..WR_MAX)
  int narrow_max_words;  // windows at most this many 32-pixel words wide take the narrow kernel (1..SMALL_BW)
  int fill_sort_max;     // the warp fill sorts up to this many records of a tile (FILL_WARP_MAX..FILL_WARP_SORT)
};

// Fill: buckets with at most the schedule's sort threshold (<= FILL_WARP_SORT)
// records are sorted and applied by one warp; larger ones go to the per-word
// path, which takes at most BIG_CAP records of one word at a time.  The
// order-free functions (first, last, and min / max without background or NaN
// values) skip the sort.
constexpr int FILL_WARP_MAX = 64;    // records held in registers (two per lane)
constexpr int FILL_WARP_SORT = 256;  // records sorted in shared memory by one warp
constexpr int BIG_CAP = 1024;

// Longest Bresenham walk one thread performs for a single segment.
constexpr long long LINE_MAX_STEPS = 1ll << 26;

enum : unsigned {
  ERR_NONE = 0,
  ERR_BAD_TABLE = 1,   // offsets not monotone / out of range
  ERR_BAD_KIND = 2,
  ERR_BAD_BAND = 3,
  ERR_BITMAP = 4,      // crossing outside its part's bitmap (non-finite geometry)
  ERR_TOO_WIDE = 5,    // polygon part wider than the bitmap
  ERR_LINE_LONG = 6,   // segment needs more than LINE_MAX_STEPS steps
  ERR_BAD_JOB = 7,     // a batch job's table does not start at 0 / end at its counts
  ERR_RANGE = 8,       // a record or a raster tile outside the call's buckets (an engine defect)
  ERR_TRIPLET = 9,     // a sparse triplet outside the raster it is replayed onto
};

// Device control block, reset at the start of every pass.
struct Ctrl {
  unsigned long long span_count;
  unsigned long long pixel_writes;
  unsigned long long crossings;
  unsigned long long edges;
  unsigned long long work;       // wide-part polygon window work counter
  unsigned long long err_index;
  unsigned int err;
  unsigned int big_count;
  unsigned long long work_small;  // narrow-part polygon window work counter
  unsigned long long fill_work;    // fill kernels: chunk / item counter
  unsigned long long pad[8];
};

// The world -> pixel map of the call (edges.rs:94-97).  A batch of jobs
// maps every job's vertices to pixels first (k_batch_vertices) and then runs
// with the identity map: xmin = +0, ymax = -0, resolution 1 and the pixel y
// stored negated, which gives back every pixel coordinate bit for bit.
struct Grid {
  double xmin, ymax, xres, yres, inv_xres, inv_yres;
  int pow2_x, pow2_y;  // resolution a power of two: multiply by the exact reciprocal
  int unit_x, unit_y;  // resolution 1: the division is the identity
  int touched;         // all_touched: lines and polygon rings take the AllTouched walk
};

// The raster a part burns into, per job of a call (one entry for a single
// call): its size, where its record words start, and the record flags of its
// line and polygon parts.  A call may burn only a window of its raster: the
// rows [row_lo, row_hi) of the bands [band_lo, band_hi).  Every pixel
// decision is still taken on the whole raster's grid (clipping, line
// filters, walks), and only writes inside the window are kept, so the window
// equals the same slice of a whole burn.
struct JobDims {
  int nrows, ncols;
  unsigned ntx;        // 512-pixel column tiles per row
  unsigned wid_base;   // first record word id of the job's window
  unsigned line_flag;  // DEDUP_BIT: line parts write each pixel once (PixelCache)
  unsigned poly_flag;  // DEDUP_BIT: polygon parts write each pixel once (all_touched sum / count)
  unsigned long long geom0;  // first geometry of the job
  int row_lo, row_hi;        // window rows (whole raster: 0, nrows)
  unsigned band_lo, band_hi; // window bands (whole raster: 0, bands)
};

struct Geo {
  const unsigned long long* part_offsets;
  const unsigned char* part_kind;
  const unsigned long long* ring_offsets;
  const unsigned long long* vertex_offsets;
  const double2* xy;
  const unsigned* bands;  // per geometry, or nullptr
  const unsigned char* ring_closed = nullptr;  // per ring: LineString::is_closed of the world coordinates, or nullptr (taken from xy)
  unsigned long long n_geoms, n_parts, n_rings, n_vertices;
};

// Per-part plan written by the prep kernel.
struct PartPlan {
  int row0, row1;  // polygon rows [row0, row1)
  int col0;        // bitmap column origin
  int bw;          // bitmap words per row
  int wr;          // rows per window
  unsigned band;   // output band of the part
  int nrows, ncols;  // the part's raster
  unsigned wid0;     // record word id of (band, row 0) of the part's raster, modulo 2^32
                     // (a window that starts at row r puts row r at wid0 + r * wpr)
  unsigned wpr;      // record words per raster row (ntx * WPT)
  unsigned flags;    // flags of the part's records (DEDUP_BIT)
  int rlo, rhi;      // rows of the window: pixels outside are not written
  unsigned ncw;      // column windows (0: one window spans the part's columns)
};

// Part-level counters, scanned (exclusive) into offsets: polygon windows of
// wide parts and of narrow parts, line / point vertices, line / point parts.
enum { PC_WINDOWS = 0, PC_WIN_SMALL, PC_LINE_V, PC_POINT_V, PC_LINE_P, PC_POINT_P, PC_N };

// Coverage records before the scatter (structure of arrays).
struct RecBuf {
  unsigned* wid;   // word id
  unsigned* part;  // part | DEDUP_BIT
  unsigned* mask;  // covered pixels of the word
  unsigned long long cap;
  unsigned long long nbuckets;  // buckets of the call: every record's bucket is below
};

__device__ __forceinline__ void set_error(Ctrl* c, unsigned code, unsigned long long idx) {
  if (atomicCAS(&c->err, 0u, code) == 0u) c->err_index = idx;
}

// world -> pixel, edges.rs:94-97 (no FMA).  A power-of-two resolution divides
// exactly like a multiplication by its reciprocal, so that path is identical.
__device__ __forceinline__ double to_px(const Grid& g, double wx) {
  double d = __dsub_rn(wx, g.xmin);
  if (g.unit_x) return d;
  return g.pow2_x ? __dmul_rn(d, g.inv_xres) : __ddiv_rn(d, g.xres);
}
__device__ __forceinline__ double to_py(const Grid& g, double wy) {
  double d = __dsub_rn(g.ymax, wy);
  if (g.unit_y) return d;
  return g.pow2_y ? __dmul_rn(d, g.inv_yres) : __ddiv_rn(d, g.yres);
}

using rzb::abs_ge_one;
using rzb::ceil_clamp;
using rzb::ceil_half_down;
using rzb::f64_bits;
using rzb::floor_half_up;
using rzb::floor_clamp;
using rzb::half_int;
using rzb::nan_bits;
using rzb::CrossEdge;
using rzb::cross_edge_setup;
using rzb::cross_fast;

// `(y - 0.5).ceil() as usize`, clamped to [0, nrows] (edges.rs:32-33).
__device__ __forceinline__ int row_ceil(double py, int nrows) { return ceil_half_down(py, nrows); }

// Rust f64::min / f64::max (NaN-ignoring)
__device__ __forceinline__ double min_rs(double a, double b) {
  return isnan(a) ? b : (isnan(b) ? a : (a < b ? a : b));
}
__device__ __forceinline__ double max_rs(double a, double b) {
  return isnan(a) ? b : (isnan(b) ? a : (a > b ? a : b));
}

// Rust `f64 as isize` (saturating; NaN -> 0)
__device__ __forceinline__ long long as_isize(double v) {
  if (isnan(v)) return 0;
  if (v <= -9223372036854775808.0) return (long long)0x8000000000000000ull;
  if (v >= 9223372036854775808.0) return 0x7FFFFFFFFFFFFFFFll;
  return (long long)v;
}

// The job of geometry `gi`: the last job whose first geometry is <= gi.
__device__ __forceinline__ unsigned job_of(const JobDims* jobs, unsigned n_jobs, unsigned long long gi) {
  unsigned lo = 0, hi = n_jobs;  // jobs[lo].geom0 <= gi < jobs[hi].geom0
  while (hi - lo > 1) {
    const unsigned mid = (lo + hi) >> 1;
    if (jobs[mid].geom0 <= gi) lo = mid; else hi = mid;
  }
  return lo;
}

// Emit the run [xs, xe) of row `y` of the part planned in `pl` as coverage
// records, one per 32-pixel word.  Slots are taken with warp-aggregated
// atomics.
__device__ __forceinline__ void emit_run(const RecBuf& rb, unsigned* bucket_count, Ctrl* ctrl, const PartPlan& pl,
                                         int y, int xs, int xe, unsigned part_flags) {
  const unsigned row_wid = pl.wid0 + (unsigned)y * pl.wpr;
  for (int wd = xs >> 5; (wd << 5) < xe; ++wd) {
    const int lo = max(xs, wd << 5) - (wd << 5), hi = min(xe, (wd << 5) + 32) - (wd << 5);
    const unsigned mask = (hi == 32 ? 0xFFFFFFFFu : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
    const unsigned wid = row_wid + (unsigned)wd;
    if (wid / WPT >= rb.nbuckets) {  // never taken: parts are clipped to their raster
      set_error(ctrl, ERR_RANGE, wid);
      return;
    }
    cg::coalesced_group grp = cg::coalesced_threads();
    unsigned long long slot0 = 0;
    if (grp.thread_rank() == 0) slot0 = atomicAdd(&ctrl->span_count, (unsigned long long)grp.size());
    slot0 = grp.shfl(slot0, 0);
    const unsigned long long slot = slot0 + grp.thread_rank();
    if (slot < rb.cap) {
      rb.wid[slot] = wid;
      rb.part[slot] = part_flags;
      rb.mask[slot] = mask;
    }
    atomicAdd(&bucket_count[wid / WPT], 1u);
  }
}

}  // namespace rzd
