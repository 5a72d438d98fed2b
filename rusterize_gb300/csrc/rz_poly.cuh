// rz_poly.cuh -- polygon scanline crossings -> spans (burn_polygon,
// rust/src/rasterization/burners.rs:261-320, with PolyEdge from
// rust/src/geo/edges.rs:17-56 and extract_ring's filters, edges.rs:90-110).
//
// Work item: one (polygon part, row window).  Every crossing of an edge with
// a scanline centre is evaluated in FP64 exactly as PolyEdge::intersect_at
// and rounded to its pixel boundary r = clamp(floor(x + 0.5), 0, ncols).
// That rounding is monotone, so pairing the x-sorted crossings two by two
// (burners.rs:302-316) covers exactly the pixels whose count of boundaries
// r <= x is odd: each crossing toggles bit r of a per-row parity bitmap and
// spans are read back as consecutive pairs of set bits -- no sort is needed.
// chunks_exact(2) drops the largest crossing of an odd row; such rows are
// fixed up by toggling their maximum r once more.  Positive-NaN crossings
// sort after every number (total_cmp) and only pair into empty spans, so they
// are skipped; negative NaNs round to 0 and sort first.
//
// FP64 is the narrow pipe on GB300, so the work is staged to keep every lane
// busy when it issues FP64:
//   1. one lane per vertex: y -> pixel and its first scanline (3 FP64 ops);
//      edges that reach a scanline of the window are queued (ballot+popc)
//   2. one lane per queued edge: horizontal filter, x -> pixel, slope
//   3. crossings are dealt to lanes with a warp-shuffle prefix sum over the
//      queued edges' row counts, so edges with very uneven row spans still
//      keep all 32 lanes busy (4 FP64 ops per crossing)
// Narrow parts run one window per warp (warp-level sync only, small bitmap);
// wide parts run one window per block of POLY_THREADS.
#pragma once

#include "rz_device.cuh"

namespace rzd {

struct PolyQueue {
  double* a;       // py0 -> y_top
  double* b;       // py1 -> dxdy
  double* c;       // x_top
  unsigned* v;     // vertex index relative to the part | top flag (bit 31)
  unsigned* rows;  // first row - r0 (bits 0-7) | row count (bits 8-15)
};

struct PolyWin {
  int r0, r1, col0, nbits, bw;
};

template <int NT>  // cooperating threads: one warp (32) or the block
__device__ __forceinline__ void scope_sync() {
  if constexpr (NT == 32) __syncwarp(); else __syncthreads();
}

template <int NT>
__device__ __forceinline__ int scope_tid() {
  if constexpr (NT == 32) return threadIdx.x & 31; else return threadIdx.x;
}

// stage 2 + 3 over the queued edges; MODE 0 toggles crossings, MODE 1
// records the largest boundary of rows flagged odd.
template <int MODE, int NT>
__device__ __forceinline__ void poly_flush(const Geo& geo, const Grid& g, const PolyQueue& q, int nq,
                                           unsigned long long vs, const PolyWin& w, unsigned* bm,
                                           const int* rowslot, int* oddmax, Ctrl* ctrl, unsigned long long part,
                                           unsigned long long& ncross) {
  for (int i = scope_tid<NT>(); i < nq; i += NT) {
    const double py0 = q.a[i], py1 = q.b[i];
    const unsigned vv = q.v[i];
    const bool top0 = vv >> 31;
    const unsigned long long v = vs + (vv & 0x7FFFFFFFu);
    // extract_ring's horizontal filter (edges.rs:100): |y0 - y1| >= EPSILON.
    // Queued end points differ; two distinct doubles of magnitude >= 1 are
    // at least 2^-52 apart, so only smaller ones need the subtraction.
    if (!(abs_ge_one(py0) && abs_ge_one(py1))) {
      const unsigned long long dbits = f64_bits(__dsub_rn(py0, py1)) & 0x7FFFFFFFFFFFFFFFull;
      if (!(dbits >= 0x3CB0000000000000ull && dbits <= 0x7FF0000000000000ull)) {
        q.rows[i] &= 0xFFu;  // no crossings
        continue;
      }
    }
    const double px0 = to_px(g, geo.xy[v].x), px1 = to_px(g, geo.xy[v + 1].x);
    const double xt = top0 ? px0 : px1, yt = top0 ? py0 : py1;
    const double xb = top0 ? px1 : px0, yb = top0 ? py1 : py0;
    q.a[i] = yt;
    q.b[i] = __ddiv_rn(__dsub_rn(xb, xt), __dsub_rn(yb, yt));  // edges.rs:36
    q.c[i] = xt;
  }
  scope_sync<NT>();
  const int lane = threadIdx.x & 31;
  const int first = NT == 32 ? 0 : (threadIdx.x >> 5) * 32;
  for (int base = first; base < nq; base += NT) {
    const int i = base + lane;
    const unsigned rw = i < nq ? q.rows[i] : 0u;
    const int n = (int)(rw >> 8);
    int incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    const int excl = incl - n;
    for (int m0 = 0; m0 < total; m0 += 32) {
      const int m = m0 + lane;
      // largest source lane s with excl(s) <= m
      int s = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int e = __shfl_sync(0xFFFFFFFFu, excl, s + step);
        if (e <= m) s += step;
      }
      const int es = __shfl_sync(0xFFFFFFFFu, excl, s);
      if (m >= total) continue;
      const int k = base + s;
      const int rowrel = (int)(q.rows[k] & 0xFFu) + (m - es);
      const double yt = q.a[k], dxdy = q.b[k], xt = q.c[k];
      // PolyEdge::intersect_at (edges.rs:50-55), no FMA
      const double cy = half_int(w.r0 + rowrel);
      const double x = __dadd_rn(xt, __dmul_rn(__dsub_rn(cy, yt), dxdy));
      const unsigned long long xb = f64_bits(x);
      int r;
      if (nan_bits(xb)) {
        if (!(xb >> 63)) continue;  // +NaN: after every number, pairs into an empty span
        r = 0;
      } else {
        r = floor_half_up(x, g.ncols);  // floor(x + 0.5) clamped, burners.rs:310-311
      }
      const int loc = r - w.col0;
      if (loc < 0 || loc >= w.nbits) {
        set_error(ctrl, ERR_BITMAP, part);
        continue;
      }
      if (MODE == 0) {
        atomicXor(&bm[rowrel * w.bw + (loc >> 5)], 1u << (loc & 31));
        ++ncross;
      } else if (rowslot[rowrel] >= 0) {
        atomicMax(&oddmax[rowslot[rowrel]], loc);
      }
    }
  }
  scope_sync<NT>();
}

// Walk the part's edges once (stage 1), flushing the queue when it fills.
template <int MODE, int NT, int QCAP>
__device__ __forceinline__ void poly_pass(const Geo& geo, const Grid& g, unsigned long long rb, unsigned long long re,
                                          const PolyWin& w, unsigned* bm, const PolyQueue& q, int* s_q,
                                          const int* rowslot, int* oddmax, Ctrl* ctrl, unsigned long long part,
                                          unsigned long long& ncross) {
  const int lane = threadIdx.x & 31, tid = scope_tid<NT>();
  const unsigned long long vs = geo.vertex_offsets[rb], ve = geo.vertex_offsets[re];
  unsigned long long ring = rb;
  for (unsigned long long base = vs; base < ve; base += NT) {
    const unsigned long long v = base + tid;
    const bool has = v < ve;
    double py0 = 0.0;
    int ys0 = 0;
    if (has) {
      py0 = to_py(g, geo.xy[v].y);
      ys0 = row_ceil(py0, g.nrows);
    }
    double py1 = __shfl_down_sync(0xFFFFFFFFu, py0, 1);
    int ys1 = __shfl_down_sync(0xFFFFFFFFu, ys0, 1);
    bool push = false;
    unsigned rows = 0, vrel = 0;
    if (has) {
      if (geo.vertex_offsets[ring + 1] <= v) {
        int steps = 0;
        while (steps < 4 && geo.vertex_offsets[ring + 1] <= v) { ++ring; ++steps; }
        if (geo.vertex_offsets[ring + 1] <= v) {
          unsigned long long lo = ring, hi = re;  // vo[lo] <= v < vo[hi]
          while (hi - lo > 1) {
            const unsigned long long mid = (lo + hi) >> 1;
            if (geo.vertex_offsets[mid] <= v) lo = mid; else hi = mid;
          }
          ring = lo;
        }
      }
      if (v + 1 < geo.vertex_offsets[ring + 1]) {
        if (lane == 31) {
          py1 = to_py(g, geo.xy[v + 1].y);
          ys1 = row_ceil(py1, g.nrows);
        }
        // a scanline centre lies in [y_top, y_bot) iff the first scanlines
        // of the end points differ; the raster-row filter (edges.rs:105)
        // only removes edges without rows in [0, nrows)
        if (ys0 != ys1) {
          const bool top0 = ys0 < ys1;
          const int a = max(top0 ? ys0 : ys1, w.r0), b = min(top0 ? ys1 : ys0, w.r1);
          if (a < b) {
            push = true;
            rows = (unsigned)(a - w.r0) | ((unsigned)(b - a) << 8);
            vrel = (unsigned)(v - vs) | (top0 ? 0x80000000u : 0u);
          }
        }
      }
    }
    const unsigned mask = __ballot_sync(0xFFFFFFFFu, push);
    if (mask) {
      int pos0 = 0;
      if (lane == 0) pos0 = atomicAdd(s_q, __popc(mask));
      pos0 = __shfl_sync(0xFFFFFFFFu, pos0, 0);
      if (push) {
        const int pos = pos0 + __popc(mask & ((1u << lane) - 1u));
        q.a[pos] = py0;
        q.b[pos] = py1;
        q.v[pos] = vrel;
        q.rows[pos] = rows;
      }
    }
    scope_sync<NT>();
    const int nq = *s_q;
    if (nq > QCAP - NT || base + NT >= ve) {
      if (nq > 0) poly_flush<MODE, NT>(geo, g, q, nq, vs, w, bm, rowslot, oddmax, ctrl, part, ncross);
      if (tid == 0) *s_q = 0;
      scope_sync<NT>();
    }
  }
}

// window index -> part: the largest p with off[p] <= w, found by one warp
// with a 32-ary search (about four dependent loads for 10^6 parts)
__device__ __forceinline__ unsigned long long window_part(const unsigned long long* poff, int col,
                                                          unsigned long long n_parts, unsigned long long w) {
  const int lane = threadIdx.x & 31;
  unsigned long long lo = 0, hi = n_parts;  // off[lo] <= w < off[hi]
  while (hi - lo > 1) {
    const unsigned long long span = hi - lo;
    const unsigned long long step = (span + 31) / 32;
    const unsigned long long idx = lo + (unsigned long long)lane * step;
    const bool le = idx < hi && (idx == lo || poff[idx * PC_N + col] <= w);
    const unsigned m = __ballot_sync(0xFFFFFFFFu, le);
    const int last = 31 - __clz(m);  // lanes 0..last satisfy (prefix property)
    const unsigned long long nlo = lo + (unsigned long long)last * step;
    const unsigned long long nhi = min(hi, nlo + step);
    lo = nlo;
    hi = nhi;
  }
  return lo;
}

// rows with an odd number of crossings; NT threads, rows dealt to warps
template <int NT>
__device__ __forceinline__ void find_odd_rows(const unsigned* bm, int nr, int bw, int* rowslot, int* oddrow,
                                              int* oddmax, int* s_nodd) {
  const int lane = threadIdx.x & 31;
  const int warp = NT == 32 ? 0 : (threadIdx.x >> 5);
  for (int i = warp; i < nr; i += NT / 32) {
    unsigned par = 0;
    for (int wd = lane; wd < bw; wd += 32) par ^= (unsigned)__popc(bm[i * bw + wd]) & 1u;
    par = __reduce_xor_sync(0xFFFFFFFFu, par);
    if (lane == 0 && par) {
      const int slot = atomicAdd(s_nodd, 1);
      rowslot[i] = slot;
      oddrow[slot] = i;
      oddmax[slot] = -1;
    }
  }
}

// Spans of one bitmap row = pairs of consecutive set bits.  One warp walks
// the row 32 words at a time; every lane hands each span whose end bit lies
// in its word to `f(xs, xe, lane_rank)`, where lane_rank numbers the pieces
// (tile-cut parts) of the row in x order.  Returns the row's piece count.
template <typename F>
__device__ __forceinline__ unsigned row_spans(const unsigned* row, int bw, int col0, F&& f) {
  const int lane = threadIdx.x & 31;
  unsigned carry_cnt = 0, carry_pieces = 0;
  int carry_last = -1;
  for (int wb = 0; wb < bw; wb += 32) {
    const int wd = wb + lane;
    const unsigned bits0 = wd < bw ? row[wd] : 0u;
    const int cnt = __popc(bits0);
    int incl = cnt;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += t;
    }
    int mx = bits0 ? wd * 32 + 31 - __clz(bits0) : -1;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xFFFFFFFFu, mx, o);
      if (lane >= o) mx = max(mx, t);
    }
    int prev0 = __shfl_up_sync(0xFFFFFFFFu, mx, 1);
    if (lane == 0) prev0 = -1;
    prev0 = max(prev0, carry_last);
    const unsigned g0 = carry_cnt + (unsigned)(incl - cnt);
    // pass a: this lane's piece count
    unsigned bits = bits0, gidx = g0, mine = 0;
    int prev = prev0;
    while (bits) {
      const int pos = wd * 32 + __ffs(bits) - 1;
      bits &= bits - 1;
      if (gidx & 1u) {
        const int xs = col0 + prev, xe = col0 + pos;
        mine += (unsigned)(((xe - 1) >> TW_SHIFT) - (xs >> TW_SHIFT) + 1);
      }
      prev = pos;
      ++gidx;
    }
    unsigned pin = mine;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned t = __shfl_up_sync(0xFFFFFFFFu, pin, o);
      if (lane >= o) pin += t;
    }
    // pass b: hand the spans out with their rank
    unsigned rank = carry_pieces + pin - mine;
    bits = bits0;
    gidx = g0;
    prev = prev0;
    while (bits) {
      const int pos = wd * 32 + __ffs(bits) - 1;
      bits &= bits - 1;
      if (gidx & 1u) {
        const int xs = col0 + prev, xe = col0 + pos;
        f(xs, xe, rank);
        rank += (unsigned)(((xe - 1) >> TW_SHIFT) - (xs >> TW_SHIFT) + 1);
      }
      prev = pos;
      ++gidx;
    }
    carry_cnt += (unsigned)__shfl_sync(0xFFFFFFFFu, incl, 31);
    carry_pieces += __shfl_sync(0xFFFFFFFFu, pin, 31);
    carry_last = max(carry_last, __shfl_sync(0xFFFFFFFFu, mx, 31));
  }
  return carry_pieces;
}

// Emit the window's spans: count pieces per row, reserve all output slots
// with ONE atomic, then write every piece at its rank (no per-span
// round trip; bucket counts are fire-and-forget reductions).
template <int NT>
__device__ __forceinline__ void extract_spans(const unsigned* bm, const PolyWin& w, const PartPlan& pl,
                                              unsigned long long p, const Grid& g, const SpanBuf& sb,
                                              unsigned* bucket_count, Ctrl* ctrl, unsigned long long& npix,
                                              unsigned* row_off, unsigned long long* s_base) {
  const int lane = threadIdx.x & 31;
  const int warp = NT == 32 ? 0 : (threadIdx.x >> 5);
  const int nr = w.r1 - w.r0, bw = w.bw;
  for (int i = warp; i < nr; i += NT / 32) {
    const unsigned n = row_spans(bm + i * bw, bw, pl.col0, [](int, int, unsigned) {});
    if (lane == 0) row_off[i] = n;
  }
  scope_sync<NT>();
  if (warp == 0) {  // exclusive scan over <= 64 rows, reserve the window's slots
    const unsigned a0 = lane < nr ? row_off[lane] : 0u, a1 = lane + 32 < nr ? row_off[lane + 32] : 0u;
    unsigned i0 = a0, i1 = a1;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned t0 = __shfl_up_sync(0xFFFFFFFFu, i0, o), t1 = __shfl_up_sync(0xFFFFFFFFu, i1, o);
      if (lane >= o) { i0 += t0; i1 += t1; }
    }
    const unsigned tot0 = __shfl_sync(0xFFFFFFFFu, i0, 31);
    const unsigned tot = tot0 + __shfl_sync(0xFFFFFFFFu, i1, 31);
    __syncwarp();
    if (lane < nr) row_off[lane] = i0 - a0;
    if (lane + 32 < nr) row_off[lane + 32] = tot0 + i1 - a1;
    if (lane == 0) *s_base = tot ? atomicAdd(&ctrl->span_count, (unsigned long long)tot) : 0ull;
  }
  scope_sync<NT>();
  const unsigned long long base = *s_base;
  const unsigned long long rowband = (unsigned long long)pl.band * (unsigned)g.nrows;
  for (int i = warp; i < nr; i += NT / 32) {
    const int y = w.r0 + i;
    const unsigned long long rowid = rowband + (unsigned)y;
    const unsigned long long rbase = base + row_off[i];
    row_spans(bm + i * bw, bw, pl.col0, [&](int xs, int xe, unsigned rank) {
      npix += (unsigned long long)(xe - xs);
      for (int t = xs >> TW_SHIFT; (t << TW_SHIFT) < xe; ++t, ++rank) {
        const int tb = t << TW_SHIFT;
        const unsigned a = (unsigned)(max(xs, tb) - tb), b = (unsigned)(min(xe, tb + TW) - tb);
        const unsigned bucket = (unsigned)(rowid * g.ntx + (unsigned)t);
        const unsigned long long slot = rbase + rank;
        if (slot < sb.cap) {
          sb.bucket[slot] = bucket;
          sb.part[slot] = (unsigned)p;
          sb.xs[slot] = a | (b << 12);
        }
        atomicAdd(&bucket_count[bucket], 1u);
      }
    });
  }
}

// Narrow parts (one warp per window): a row has at most SMALL_BW words, so
// one LANE walks a whole row; the per-row piece offsets come from one warp
// scan per 32 rows.
__device__ __forceinline__ unsigned lane_row_pieces(const unsigned* row, int bw, int col0) {
  unsigned par = 0, pieces = 0;
  int start = 0;
  for (int wd = 0; wd < bw; ++wd) {
    unsigned bits = row[wd];
    while (bits) {
      const int pos = wd * 32 + __ffs(bits) - 1;
      bits &= bits - 1;
      if (par) {
        const int xs = col0 + start, xe = col0 + pos;
        pieces += (unsigned)(((xe - 1) >> TW_SHIFT) - (xs >> TW_SHIFT) + 1);
      } else {
        start = pos;
      }
      par ^= 1u;
    }
  }
  return pieces;
}

__device__ __forceinline__ void find_odd_rows_lane(const unsigned* bm, int nr, int bw, int* rowslot, int* oddrow,
                                                   int* oddmax, int* s_nodd) {
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < nr; i += 32) {
    unsigned par = 0;
    for (int wd = 0; wd < bw; ++wd) par ^= (unsigned)__popc(bm[i * bw + wd]);
    if (par & 1u) {
      const int slot = atomicAdd(s_nodd, 1);
      rowslot[i] = slot;
      oddrow[slot] = i;
      oddmax[slot] = -1;
    }
  }
}

__device__ __forceinline__ void extract_spans_lane(const unsigned* bm, const PolyWin& w, const PartPlan& pl,
                                                   unsigned long long p, const Grid& g, const SpanBuf& sb,
                                                   unsigned* bucket_count, Ctrl* ctrl, unsigned long long& npix) {
  const int lane = threadIdx.x & 31;
  const int nr = w.r1 - w.r0, bw = w.bw;
  // pieces of rows lane and lane + 32, their exclusive offsets, one reservation
  const unsigned c0 = lane < nr ? lane_row_pieces(bm + lane * bw, bw, pl.col0) : 0u;
  const unsigned c1 = lane + 32 < nr ? lane_row_pieces(bm + (lane + 32) * bw, bw, pl.col0) : 0u;
  unsigned i0 = c0, i1 = c1;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned t0 = __shfl_up_sync(0xFFFFFFFFu, i0, o), t1 = __shfl_up_sync(0xFFFFFFFFu, i1, o);
    if (lane >= o) { i0 += t0; i1 += t1; }
  }
  const unsigned tot0 = __shfl_sync(0xFFFFFFFFu, i0, 31);
  const unsigned tot = tot0 + __shfl_sync(0xFFFFFFFFu, i1, 31);
  unsigned long long base = 0;
  if (lane == 0 && tot) base = atomicAdd(&ctrl->span_count, (unsigned long long)tot);
  base = __shfl_sync(0xFFFFFFFFu, base, 0);
  const unsigned long long rowband = (unsigned long long)pl.band * (unsigned)g.nrows;
  for (int h = 0; h < 2; ++h) {
    const int i = lane + 32 * h;
    if (i >= nr) continue;
    unsigned long long slot = base + (h == 0 ? i0 - c0 : tot0 + i1 - c1);
    const unsigned long long rowid = rowband + (unsigned)(w.r0 + i);
    const unsigned* row = bm + i * bw;
    unsigned par = 0;
    int start = 0;
    for (int wd = 0; wd < bw; ++wd) {
      unsigned bits = row[wd];
      while (bits) {
        const int pos = wd * 32 + __ffs(bits) - 1;
        bits &= bits - 1;
        if (par) {
          const int xs = pl.col0 + start, xe = pl.col0 + pos;
          npix += (unsigned long long)(xe - xs);
          for (int t = xs >> TW_SHIFT; (t << TW_SHIFT) < xe; ++t, ++slot) {
            const int tb = t << TW_SHIFT;
            const unsigned a = (unsigned)(max(xs, tb) - tb), b = (unsigned)(min(xe, tb + TW) - tb);
            const unsigned bucket = (unsigned)(rowid * g.ntx + (unsigned)t);
            if (slot < sb.cap) {
              sb.bucket[slot] = bucket;
              sb.part[slot] = (unsigned)p;
              sb.xs[slot] = a | (b << 12);
            }
            atomicAdd(&bucket_count[bucket], 1u);
          }
        } else {
          start = pos;
        }
        par ^= 1u;
      }
    }
  }
}

// one (part, window): zero the bitmap, toggle crossings, fix odd rows, emit
template <int NT, int QCAP>
__device__ __forceinline__ void poly_window(const Geo& geo, const Grid& g, const PartPlan& pl, unsigned long long p,
                                            int k, unsigned* bm, const PolyQueue& q, int* s_q, int* rowslot,
                                            int* oddmax, int* oddrow, int* s_nodd, unsigned long long* s_base,
                                            const SpanBuf& sb, unsigned* bucket_count, Ctrl* ctrl,
                                            unsigned long long& ncross, unsigned long long& npix) {
  const int tid = scope_tid<NT>();
  PolyWin win;
  win.r0 = pl.row0 + k * pl.wr;
  win.r1 = min(win.r0 + pl.wr, pl.row1);
  win.col0 = pl.col0;
  win.bw = pl.bw;
  win.nbits = pl.bw * 32;
  const int nr = win.r1 - win.r0, bw = pl.bw;
  for (int i = tid; i < nr * bw; i += NT) bm[i] = 0u;
  for (int i = tid; i < WR_MAX; i += NT) rowslot[i] = -1;
  if (tid == 0) { *s_q = 0; *s_nodd = 0; }
  scope_sync<NT>();
  const unsigned long long rb = geo.ring_offsets[p], re = geo.ring_offsets[p + 1];
  poly_pass<0, NT, QCAP>(geo, g, rb, re, win, bm, q, s_q, rowslot, oddmax, ctrl, p, ncross);
  if constexpr (NT == 32) find_odd_rows_lane(bm, nr, bw, rowslot, oddrow, oddmax, s_nodd);
  else find_odd_rows<NT>(bm, nr, bw, rowslot, oddrow, oddmax, s_nodd);
  scope_sync<NT>();
  if (*s_nodd > 0) {
    unsigned long long dummy = 0;
    poly_pass<1, NT, QCAP>(geo, g, rb, re, win, bm, q, s_q, rowslot, oddmax, ctrl, p, dummy);
    for (int t = tid; t < *s_nodd; t += NT) {
      const int i = oddrow[t], loc = oddmax[t];
      if (loc >= 0) bm[i * bw + (loc >> 5)] ^= 1u << (loc & 31);
    }
    scope_sync<NT>();
  }
  // oddrow is free again: it holds the per-row piece offsets
  if constexpr (NT == 32) extract_spans_lane(bm, win, pl, p, g, sb, bucket_count, ctrl, npix);
  else extract_spans<NT>(bm, win, pl, p, g, sb, bucket_count, ctrl, npix, reinterpret_cast<unsigned*>(oddrow), s_base);
  scope_sync<NT>();
}

__device__ __forceinline__ void flush_counters(unsigned long long ncross, unsigned long long npix, Ctrl* ctrl) {
  for (int o = 16; o > 0; o >>= 1) {
    ncross += __shfl_xor_sync(0xFFFFFFFFu, ncross, o);
    npix += __shfl_xor_sync(0xFFFFFFFFu, npix, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (ncross) atomicAdd(&ctrl->crossings, ncross);
    if (npix) atomicAdd(&ctrl->pixel_writes, npix);
  }
}

// wide parts: one block per window
__global__ void __launch_bounds__(POLY_THREADS) k_poly_spans(Geo geo, Grid g, const PartPlan* __restrict__ plan,
                                                              const unsigned long long* __restrict__ poff,
                                                              SpanBuf sb, unsigned* bucket_count, Ctrl* ctrl) {
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned* bm = reinterpret_cast<unsigned*>(smem);
  PolyQueue q;
  q.a = reinterpret_cast<double*>(smem + BITMAP_WORDS * 4);
  q.b = q.a + POLY_QCAP;
  q.c = q.b + POLY_QCAP;
  q.v = reinterpret_cast<unsigned*>(q.c + POLY_QCAP);
  q.rows = q.v + POLY_QCAP;
  __shared__ int rowslot[WR_MAX];
  __shared__ int oddmax[WR_MAX];
  __shared__ int oddrow[WR_MAX];
  __shared__ int s_nodd, s_q;
  __shared__ unsigned long long s_part, s_w, s_base;
  if (ctrl->err) return;
  const unsigned long long total = poff[geo.n_parts * PC_N + PC_WINDOWS];
  unsigned long long ncross = 0, npix = 0;
  while (true) {
    if (threadIdx.x == 0) s_w = atomicAdd(&ctrl->work, 1ull);
    __syncthreads();
    const unsigned long long wi = s_w;
    if (wi >= total) break;
    if (threadIdx.x < 32) {
      const unsigned long long p = window_part(poff, PC_WINDOWS, geo.n_parts, wi);
      if (threadIdx.x == 0) s_part = p;
    }
    __syncthreads();
    const unsigned long long p = s_part;
    const PartPlan pl = plan[p];
    const int k = (int)(wi - poff[p * PC_N + PC_WINDOWS]);
    poly_window<POLY_THREADS, POLY_QCAP>(geo, g, pl, p, k, bm, q, &s_q, rowslot, oddmax, oddrow, &s_nodd, &s_base,
                                         sb, bucket_count, ctrl, ncross, npix);
  }
  flush_counters(ncross, npix, ctrl);
}

// narrow parts: one warp per window, SMALL_WARPS independent warps per block
__global__ void __launch_bounds__(SMALL_WARPS * 32, 4) k_poly_spans_narrow(Geo geo, Grid g,
                                                                        const PartPlan* __restrict__ plan,
                                                                        const unsigned long long* __restrict__ poff,
                                                                        SpanBuf sb, unsigned* bucket_count,
                                                                        Ctrl* ctrl) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char* base = smem + warp * SMALL_WARP_SMEM;
  PolyQueue q;
  q.a = reinterpret_cast<double*>(base);
  q.b = q.a + SMALL_QCAP;
  q.c = q.b + SMALL_QCAP;
  q.v = reinterpret_cast<unsigned*>(q.c + SMALL_QCAP);
  q.rows = q.v + SMALL_QCAP;
  unsigned* bm = q.rows + SMALL_QCAP;
  int* rowslot = reinterpret_cast<int*>(bm + SMALL_BITMAP_WORDS);
  int* oddmax = rowslot + WR_MAX;
  int* oddrow = oddmax + WR_MAX;
  unsigned long long* s_base = reinterpret_cast<unsigned long long*>(oddrow + WR_MAX);
  int* s_q = reinterpret_cast<int*>(s_base + 1);
  int* s_nodd = s_q + 1;
  if (ctrl->err) return;
  const unsigned long long total = poff[geo.n_parts * PC_N + PC_WIN_SMALL];
  unsigned long long ncross = 0, npix = 0;
  while (true) {
    unsigned long long wi = 0;
    if (lane == 0) wi = atomicAdd(&ctrl->work_small, 1ull);
    wi = __shfl_sync(0xFFFFFFFFu, wi, 0);
    if (wi >= total) break;
    const unsigned long long p = window_part(poff, PC_WIN_SMALL, geo.n_parts, wi);
    const PartPlan pl = plan[p];
    const int k = (int)(wi - poff[p * PC_N + PC_WIN_SMALL]);
    poly_window<32, SMALL_QCAP>(geo, g, pl, p, k, bm, q, s_q, rowslot, oddmax, oddrow, s_nodd, s_base, sb,
                                bucket_count, ctrl, ncross, npix);
  }
  flush_counters(ncross, npix, ctrl);
}

}  // namespace rzd
