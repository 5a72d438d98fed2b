// rz_poly.cuh -- polygon scanline crossings -> spans (burn_polygon,
// rust/src/rasterization/burners.rs:261-320, with PolyEdge from
// rust/src/geo/edges.rs:17-56 and extract_ring's filters, edges.rs:90-110).
//
// Work item: one (polygon part, row window).  Every crossing of an edge with
// a scanline centre is rounded to its pixel boundary
// r = clamp(floor(x + 0.5), 0, ncols) with the value of
// PolyEdge::intersect_at.  That rounding is monotone, so pairing the
// x-sorted crossings two by two (burners.rs:302-316) covers exactly the
// pixels whose count of boundaries r <= x is odd: each crossing toggles bit r
// of a per-row parity bitmap and spans are read back as consecutive pairs of
// set bits -- no sort is needed.  chunks_exact(2) drops the largest crossing
// of an odd row; such rows are fixed up by toggling their maximum r once
// more.  Positive-NaN crossings sort after every number (total_cmp) and only
// pair into empty spans, so they are skipped; negative NaNs round to 0 and
// sort first.
//
// FP64 is the narrow pipe on GB300.  The pixel coordinates of the vertices
// are the reference's FP64 values, but the crossings are decided by the FP32
// filter of rz_bits.h (cross_edge_setup's arithmetic / cross_fast), which
// returns the FP64 boundary whenever it can prove it and otherwise hands the
// crossing to the reference's FP64 sequence (cross_exact).
//
// Everything runs warp by warp, without block barriers inside a pass:
//   1. vertex pass: one lane per vertex computes its pixel coordinates, first
//      scanline and filter frame once; the lane owns the edge that ENDS at its
//      vertex and gets the previous vertex by one register rotation (the
//      chunk's first lane keeps the previous chunk's last vertex).  Edges with
//      a scanline of the window are queued in shared memory.
//   2. crossings: dealt to lanes in order over the queued edges' row counts,
//      so edges with very uneven row spans keep all 32 lanes busy; each one
//      toggles its bit in the window's bitmap (shared-memory atomics).
//   3. extraction: the bitmap is read 32 words per round.  A pixel is
//      covered when the number of boundaries at or left of it in its row is
//      odd, so a word's coverage mask is the inclusive prefix XOR of its bits,
//      inverted when the row's set bits before the word are odd in number
//      (a row-segmented warp scan plus the previous round's carry).  Every
//      non-zero mask becomes a coverage record, staged in shared memory and
//      written out in coalesced runs with one slot reservation per flush.
// Narrow parts run one window per warp; wide parts run one window per block
// whose warps take contiguous vertex ranges and row ranges of the window.
#pragma once

#include <climits>

#include "rz_device.cuh"

namespace rzd {

// One queued edge in the crossing filter's frame (CrossEdge, rz_bits.h).
struct __align__(16) QEnt {
  int xi;
  float d0, a, c0, e0, e1;
  unsigned v;     // first vertex of the edge, relative to the part | top flag (bit 31)
  unsigned rows;  // first row - r0 (bits 0-7) | row count (bits 8-15)
};
static_assert(sizeof(QEnt) == 32, "queue entry layout");

constexpr int QCAP = POLY_WARP_QCAP;
constexpr int STAGE_CAP = (QCAP * 32) / 12 / 8 * 8;  // staged records per warp (aliases the queue)

struct PolyWin {
  int r0, r1, col0, nbits, bw;
  int nrows, ncols;  // the part's raster
  bool colwin;       // a column window: crossings may fall left or right of it
};

// Per-warp shared-memory scratch: the edge queue, which doubles as the
// record staging area between passes.
struct WarpScratch {
  QEnt* q;
  unsigned* st_wid;
  unsigned* st_part;
  unsigned* st_mask;
  __device__ __forceinline__ void init(void* base) {
    q = reinterpret_cast<QEnt*>(base);
    st_wid = reinterpret_cast<unsigned*>(base);
    st_part = st_wid + STAGE_CAP;
    st_mask = st_part + STAGE_CAP;
  }
};

// The crossing of edge v (top end first when `top0`) with the centre of row
// `row`, by the reference's FP64 sequence: PolyEdge::new's slope and
// intersect_at (edges.rs:27-55), no FMA.  Used for the crossings the FP32
// filter leaves undecided.  Returns the boundary, or -1 for a +NaN crossing.
__device__ __noinline__ int cross_exact(const Geo& geo, const Grid& g, unsigned long long v, bool top0, int row,
                                        int ncols) {
  const double2 w0 = geo.xy[v], w1 = geo.xy[v + 1];
  const double px0 = to_px(g, w0.x), py0 = to_py(g, w0.y), px1 = to_px(g, w1.x), py1 = to_py(g, w1.y);
  const double xt = top0 ? px0 : px1, yt = top0 ? py0 : py1;
  const double xb = top0 ? px1 : px0, yb = top0 ? py1 : py0;
  const double dxdy = __ddiv_rn(__dsub_rn(xb, xt), __dsub_rn(yb, yt));
  const double x = __dadd_rn(xt, __dmul_rn(__dsub_rn(half_int(row), yt), dxdy));
  const unsigned long long xbits = f64_bits(x);
  if (nan_bits(xbits)) return (xbits >> 63) ? 0 : -1;  // -NaN sorts first; +NaN pairs into an empty span
  return floor_half_up(x, ncols);                      // floor(x + 0.5) clamped, burners.rs:310-311
}

// The queued edge of crossing m0 + lane: the last edge starting at or before
// it.  Every queued edge has at least one row, so edge starts are distinct
// and one OR-reduction of "start" bits plus a popcount finds it (edge `lane`
// has row count n and exclusive row prefix excl).  Returns the edge index in
// the queue's 32-edge group and sets j to the crossing's row within the edge.
__device__ __forceinline__ int cross_edge_of(int m0, int n, int excl, int& j) {
  const int lane = threadIdx.x & 31;
  const unsigned bit = (n > 0 && excl >= m0 && excl < m0 + 32) ? (1u << (excl - m0)) : 0u;
  const unsigned starts = __reduce_or_sync(0xFFFFFFFFu, bit);
  const int before = __popc(__ballot_sync(0xFFFFFFFFu, n > 0 && excl < m0));
  const int s = before + __popc(starts & ((2u << lane) - 1u)) - 1;
  const int es = __shfl_sync(0xFFFFFFFFu, excl, s & 31);
  j = m0 + lane - es;
  return s;
}

// The boundary of a crossing (FP32 filter, FP64 fallback), relative to the
// window's first column, or INT_MIN for a crossing that burns nothing
// (+NaN); ERR_BITMAP outside the window's bitmap.
template <bool COLW>
__device__ __forceinline__ int cross_loc(const Geo& geo, const Grid& g, const QEnt& qe, int j, int rowrel,
                                         unsigned long long vs, const PolyWin& w, Ctrl* ctrl,
                                         unsigned long long part) {
  CrossEdge ce;
  ce.xi = qe.xi;
  ce.d0 = qe.d0;
  ce.a = qe.a;
  ce.c0 = qe.c0;
  ce.e0 = qe.e0;
  ce.e1 = qe.e1;
  int r = cross_fast(ce, j, w.ncols);
  if (r < 0) {
    r = cross_exact(geo, g, vs + (qe.v & 0x7FFFFFFFu), qe.v >> 31, w.r0 + rowrel, w.ncols);
    if (r < 0) return INT_MIN;
  }
  const int loc = r - w.col0;
  if (!(COLW && w.colwin) && (loc < 0 || loc >= w.nbits)) {
    set_error(ctrl, ERR_BITMAP, part);
    return INT_MIN;
  }
  return loc;
}

// A column window's crossings left of it flip its row's carry (bit 0 of
// `side`), those right of it flip bit 1: only the parity of each matters.
template <int MODE, bool COLW>
__device__ __forceinline__ void cross_apply(int loc, int rowrel, const PolyWin& w, unsigned* bm, const int* rowslot,
                                            int* oddmax, unsigned* side, unsigned long long& ncross) {
  if (loc == INT_MIN) return;
  if (MODE == 0) {
    if (COLW && loc < 0) atomicXor(&side[rowrel], 1u);
    else if (COLW && loc >= w.nbits) atomicXor(&side[rowrel], 2u);
    else atomicXor(&bm[rowrel * w.bw + (loc >> 5)], 1u << (loc & 31));
    ++ncross;
  } else if (rowslot[rowrel] >= 0) {
    atomicMax(&oddmax[rowslot[rowrel]], loc);
  }
}

// Crossings of the nq queued edges, dealt to lanes in order over the edges'
// row counts so that edges with very uneven row spans keep all 32 lanes busy.
// Two rounds of 32 crossings are taken per iteration, their steps
// interleaved, so that their latencies overlap.  MODE 0 toggles every
// boundary in the bitmap; MODE 1 records the largest boundary of rows flagged
// odd.
template <int MODE, bool COLW>
__device__ __forceinline__ void warp_cross(const Geo& geo, const Grid& g, const QEnt* q, int nq,
                                           unsigned long long vs, const PolyWin& w, unsigned* bm,
                                           const int* rowslot, int* oddmax, unsigned* side, Ctrl* ctrl,
                                           unsigned long long part, unsigned long long& ncross) {
  const int lane = threadIdx.x & 31;
  for (int base = 0; base < nq; base += 32) {
    const int i = base + lane;
    const int n = i < nq ? (int)(q[i].rows >> 8) : 0;
    int incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    const int excl = incl - n;
    for (int m0 = 0; m0 < total; m0 += 64) {
      int ja, jb;
      const int sa = cross_edge_of(m0, n, excl, ja);
      const int sb = cross_edge_of(m0 + 32, n, excl, jb);  // past the end: every lane's crossing is >= total
      const bool ha = m0 + lane < total, hb = m0 + 32 + lane < total;
      const QEnt qa = q[base + (ha ? sa : 0)];
      const QEnt qb = q[base + (hb ? sb : 0)];
      const int ra = (int)(qa.rows & 0xFFu) + ja, rbw = (int)(qb.rows & 0xFFu) + jb;
      const int la = ha ? cross_loc<COLW>(geo, g, qa, ja, ra, vs, w, ctrl, part) : INT_MIN;
      const int lb = hb ? cross_loc<COLW>(geo, g, qb, jb, rbw, vs, w, ctrl, part) : INT_MIN;
      cross_apply<MODE, COLW>(la, ra, w, bm, rowslot, oddmax, side, ncross);
      cross_apply<MODE, COLW>(lb, rbw, w, bm, rowslot, oddmax, side, ncross);
    }
  }
}

// Per-vertex values the vertex pass carries: pixel y (for the horizontal
// filter), first scanline, and the filter frame of the vertex.
struct VtxState {
  double py;
  int ys, xi, yi;
  float xf, yf;
  bool ok;
};

__device__ __forceinline__ VtxState vtx_state(const Grid& g, double2 w, int nrows) {
  VtxState s;
  s.py = to_py(g, w.y);
  uint32_t yf24 = 0;
  const bool oky = rzb::split_px(s.py, s.yi, s.yf, &yf24);
  s.ys = rzb::ceil_half_down_split(s.py, oky, s.yi, yf24, nrows);  // edges.rs:32-33
  const double px = to_px(g, w.x);
  const bool okx = rzb::split_px(px, s.xi, s.xf);
  s.ok = okx && oky;
  return s;
}

__device__ __forceinline__ VtxState rotate_prev(const VtxState& s, VtxState& carry, int lane) {
  const int src = (lane + 31) & 31;
  VtxState r;
  r.py = __shfl_sync(0xFFFFFFFFu, s.py, src);
  r.ys = __shfl_sync(0xFFFFFFFFu, s.ys, src);
  r.xi = __shfl_sync(0xFFFFFFFFu, s.xi, src);
  r.yi = __shfl_sync(0xFFFFFFFFu, s.yi, src);
  r.xf = __shfl_sync(0xFFFFFFFFu, s.xf, src);
  r.yf = __shfl_sync(0xFFFFFFFFu, s.yf, src);
  r.ok = __shfl_sync(0xFFFFFFFFu, (int)s.ok, src) != 0;
  if (lane == 0) {  // lane 0 receives this chunk's last vertex: the next chunk's predecessor
    const VtxState prev = carry;
    carry = r;
    return prev;
  }
  return r;
}

// One warp walks vertices [vb, ve) of the part (indices relative to the
// part's first vertex vs) and burns the crossings of the edges ending at
// them into the window's bitmap.  Ring starts (no edge ends there) are the
// part's first vertex and the ring ends of earlier rings; parts with at most
// 32 rings keep those in registers.
template <int MODE, bool COLW>
__device__ __forceinline__ void warp_pass(const Geo& geo, const Grid& g, unsigned long long rb,
                                          unsigned long long re, unsigned long long vs, unsigned vb, unsigned ve,
                                          const PolyWin& w, unsigned* bm, QEnt* q, const int* rowslot, int* oddmax,
                                          unsigned* side, Ctrl* ctrl, unsigned long long part,
                                          unsigned long long& ncross) {
  const int lane = threadIdx.x & 31;
  if (vb >= ve) return;
  const double2* xy = geo.xy + vs;
  // pull the warp's vertex range into L2 (one 128-byte line per lane and
  // instruction), so that the one-chunk-ahead loads below hit L2
  for (unsigned off = vb * 16u + (unsigned)lane * 128u; off < ve * 16u; off += 32u * 128u)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(reinterpret_cast<const char*>(xy) + off));
  const unsigned nring = (unsigned)(re - rb);
  const bool few = nring <= 32;
  unsigned rend = 0xFFFFFFFFu;  // lane j: end (exclusive) of ring rb + j = start of the next ring
  if (few && (unsigned)lane < nring) rend = (unsigned)(geo.vertex_offsets[rb + 1 + lane] - vs);
  unsigned long long ring = rb;  // parts with many rings: ring of this lane's vertex
  VtxState carry;
  carry.py = 0.0;
  carry.ys = carry.xi = carry.yi = 0;
  carry.xf = carry.yf = 0.0f;
  carry.ok = false;
  if (vb > 0 && lane == 0) carry = vtx_state(g, xy[vb - 1], w.nrows);
  double2 wc = make_double2(0.0, 0.0);
  if (vb + lane < ve) wc = xy[vb + lane];
  int nq = 0;
  for (unsigned base = vb; base < ve; base += 32) {
    const unsigned v = base + lane;
    const bool has = v < ve;
    double2 wn = make_double2(0.0, 0.0);
    if (v + 32 < ve) wn = xy[v + 32];
    bool start = v == 0;
    if (few) {
      for (unsigned j = 0; j < nring; ++j) start |= (v == __shfl_sync(0xFFFFFFFFu, rend, (int)j));
    } else if (has) {
      const unsigned long long va = vs + v;
      if (geo.vertex_offsets[ring + 1] <= va) {
        unsigned long long lo = ring, hi = re;  // vo[lo] <= va < vo[hi]
        while (hi - lo > 1) {
          const unsigned long long mid = (lo + hi) >> 1;
          if (geo.vertex_offsets[mid] <= va) lo = mid; else hi = mid;
        }
        ring = lo;
      }
      start = start || va == geo.vertex_offsets[ring];
    }
    const VtxState cur = vtx_state(g, wc, w.nrows);
    const VtxState prv = rotate_prev(cur, carry, lane);
    bool push = false;
    QEnt e;
    if (has && !start && prv.ys != cur.ys) {
      // a scanline centre lies in [y_top, y_bot) iff the first scanlines of
      // the end points differ; the raster-row filter (edges.rs:105) only
      // removes edges without rows in [0, nrows).  The edge runs from the
      // previous vertex (v - 1) to v.
      const bool top0 = prv.ys < cur.ys;
      const int a = max(top0 ? prv.ys : cur.ys, w.r0), b = min(top0 ? cur.ys : prv.ys, w.r1);
      if (a < b) {
        // horizontal filter |y0 - y1| >= EPSILON: two distinct doubles of
        // magnitude >= 1 are at least 2^-52 apart, so only smaller end
        // points need the subtraction
        bool keep = true;
        if (!(abs_ge_one(prv.py) && abs_ge_one(cur.py))) {
          const unsigned long long dbits = f64_bits(__dsub_rn(prv.py, cur.py)) & 0x7FFFFFFFFFFFFFFFull;
          keep = dbits >= 0x3CB0000000000000ull && dbits <= 0x7FF0000000000000ull;
        }
        if (keep) {
          const VtxState& t = top0 ? prv : cur;
          const VtxState& bt = top0 ? cur : prv;
          CrossEdge ce;
          rzb::cross_edge_frame(t.xi, t.xf, t.yi, t.yf, bt.xi, bt.xf, bt.yi, bt.yf, t.ok && bt.ok, a, ce);
          e.xi = ce.xi;
          e.d0 = ce.d0;
          e.a = ce.a;
          e.c0 = ce.c0;
          e.e0 = ce.e0;
          e.e1 = ce.e1;
          e.v = (v - 1) | (top0 ? 0x80000000u : 0u);
          e.rows = (unsigned)(a - w.r0) | ((unsigned)(b - a) << 8);
          push = true;
        }
      }
    }
    const unsigned mask = __ballot_sync(0xFFFFFFFFu, push);
    if (push) q[nq + __popc(mask & ((1u << lane) - 1u))] = e;
    nq += __popc(mask);
    if (nq > QCAP - 32 || base + 32 >= ve) {
      __syncwarp();
      if (nq > 0) warp_cross<MODE, COLW>(geo, g, q, nq, vs, w, bm, rowslot, oddmax, side, ctrl, part, ncross);
      nq = 0;
      __syncwarp();
    }
    wc = wn;
  }
}

// ---- coverage extraction ----------------------------------------------------

// Write the warp's staged records: one slot reservation, coalesced stores,
// and one bucket-count update per run of equal buckets.
__device__ __forceinline__ void stage_flush(WarpScratch& ws, int& st_n, const RecBuf& rb, unsigned* bucket_count,
                                            Ctrl* ctrl) {
  const int lane = threadIdx.x & 31;
  if (st_n == 0) return;
  __syncwarp();
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(&ctrl->span_count, (unsigned long long)st_n);
  base = __shfl_sync(0xFFFFFFFFu, base, 0);
  for (int j0 = 0; j0 < st_n; j0 += 32) {
    const int j = j0 + lane;
    const bool valid = j < st_n;
    const unsigned wid = valid ? ws.st_wid[j] : 0xFFFFFFFFu;
    if (valid) {
      const unsigned long long slot = base + (unsigned)j;
      if (slot < rb.cap) {
        rb.wid[slot] = wid;
        rb.part[slot] = ws.st_part[j];
        rb.mask[slot] = ws.st_mask[j];
      }
    }
    const unsigned bucket = valid ? wid / WPT : 0xFFFFFFFFu;
    const unsigned same = __match_any_sync(0xFFFFFFFFu, bucket);
    if (valid && (__ffs(same) - 1) == lane) {
      if (bucket < rb.nbuckets) atomicAdd(&bucket_count[bucket], (unsigned)__popc(same));
      else set_error(ctrl, ERR_RANGE, wid);  // never taken: windows are clipped to their raster
    }
  }
  st_n = 0;
  __syncwarp();
}

// Coverage records of rows [0, nr) of a bitmap of bw words per row (row i is
// raster row r0 + i, bit b of word wd is column col0 + 32 wd + b; col0 is a
// multiple of 32, so bitmap words are raster words).  Words are taken 32 per
// round; rows are contiguous runs of lanes, so the parity of the set bits
// before each word comes from a row-segmented XOR scan plus the carry of the
// previous round.
// `side` (column windows, else nullptr): bit 0 of side[row] is the parity of
// the row's crossings left of the window, which every word of the row takes.
__device__ __forceinline__ void warp_extract(const unsigned* bm, int nr, int bw, int r0, int col0,
                                             const PartPlan& pl, unsigned part, WarpScratch& ws, int& st_n,
                                             const RecBuf& rb, unsigned* bucket_count, Ctrl* ctrl,
                                             unsigned long long& npix, const unsigned* side) {
  const int lane = threadIdx.x & 31;
  const int nw = nr * bw;
  const float inv_bw = 1.0f / (float)bw;
  const unsigned wpr = pl.wpr;  // record words per raster row
  const unsigned w0 = pl.wid0 + ((unsigned)col0 >> 5);
  const unsigned flags = part | pl.flags;
  int c_row = -1;
  unsigned c_par = 0;
  for (int i0 = 0; i0 < nw; i0 += 32) {
    const int i = i0 + lane;
    const bool valid = i < nw;
    // i / bw exactly: (i + 0.5) / bw is at least 0.5 / bw away from an integer
    const int row = valid ? (int)__fmul_rn(__fadd_rn((float)i, 0.5f), inv_bw) : 0x7FFFFFFF;
    const int wd = i - row * bw;
    const unsigned bits = valid ? bm[i] : 0u;
    unsigned par = (unsigned)__popc(bits) & 1u;
    const unsigned own = par;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned tp = __shfl_up_sync(0xFFFFFFFFu, par, o);
      const int tr = __shfl_up_sync(0xFFFFFFFFu, row, o);
      if (lane >= o && tr == row) par ^= tp;
    }
    unsigned before = par ^ own;  // set bits of the row before this word (parity)
    if (row == c_row) before ^= c_par;
    {
      const int lrow = __shfl_sync(0xFFFFFFFFu, row, 31);
      unsigned lpar = __shfl_sync(0xFFFFFFFFu, par, 31);
      if (lrow == c_row) lpar ^= c_par;
      c_row = lrow;
      c_par = lpar;
    }
    if (side && valid) before ^= side[row] & 1u;  // crossings left of a column window
    unsigned cov = bits;  // inclusive prefix XOR of the word's bits
    cov ^= cov << 1;
    cov ^= cov << 2;
    cov ^= cov << 4;
    cov ^= cov << 8;
    cov ^= cov << 16;
    if (before) cov = ~cov;
    const bool emit = valid && cov != 0u;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, emit);
    if (m == 0u) continue;
    const int cnt = __popc(m);
    if (cnt > STAGE_CAP - st_n) stage_flush(ws, st_n, rb, bucket_count, ctrl);
    if (emit) {
      const int k = st_n + __popc(m & ((1u << lane) - 1u));
      ws.st_wid[k] = (unsigned)(r0 + row) * wpr + w0 + (unsigned)wd;
      ws.st_part[k] = flags;
      ws.st_mask[k] = cov;
      npix += (unsigned long long)__popc(cov);
    }
    st_n += cnt;
  }
}

// rows of the window with an odd number of crossings (one lane per row);
// a column window adds the crossings left and right of it (`side`)
__device__ __forceinline__ void warp_find_odd_rows(const unsigned* bm, int rb, int re, int bw, int* rowslot,
                                                   int* oddrow, int* oddmax, int* s_nodd, const unsigned* side) {
  for (int i = rb + (threadIdx.x & 31); i < re; i += 32) {
    unsigned par = side ? (side[i] ^ (side[i] >> 1)) : 0u;
    for (int wd = 0; wd < bw; ++wd) par ^= (unsigned)__popc(bm[i * bw + wd]);
    if (par & 1u) {
      const int slot = atomicAdd(s_nodd, 1);
      rowslot[i] = slot;
      oddrow[slot] = i;
      oddmax[slot] = INT_MIN;
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

// Row window k of a part whose columns fit one bitmap.
__device__ __forceinline__ PolyWin make_row_window(const PartPlan& pl, int k) {
  PolyWin win;
  win.r0 = pl.row0 + k * pl.wr;
  win.r1 = min(win.r0 + pl.wr, pl.row1);
  win.colwin = false;
  win.col0 = pl.col0;
  win.bw = pl.bw;
  win.nbits = pl.bw * 32;
  win.nrows = pl.nrows;
  win.ncols = pl.ncols;
  return win;
}

// Window k of a part: row windows, or (parts wider than one bitmap) row
// windows times column windows, column window fastest.
__device__ __forceinline__ PolyWin make_window(const PartPlan& pl, unsigned long long k) {
  PolyWin win;
  const unsigned long long ncw = pl.ncw > 1 ? pl.ncw : 1;
  const int kr = (int)(k / ncw), kc = (int)(k % ncw);
  win.r0 = pl.row0 + kr * pl.wr;
  win.r1 = min(win.r0 + pl.wr, pl.row1);
  win.colwin = pl.ncw > 1;
  win.col0 = pl.col0 + (win.colwin ? kc * COLWIN_WORDS * 32 : 0);
  win.bw = win.colwin ? min(COLWIN_WORDS, pl.bw - kc * COLWIN_WORDS) : pl.bw;
  win.nbits = win.bw * 32;
  win.nrows = pl.nrows;
  win.ncols = pl.ncols;
  return win;
}

// ---- narrow parts: one window per warp ------------------------------------
__global__ void __launch_bounds__(SMALL_WARPS * 32, 5) k_poly_spans_narrow(Geo geo, Grid g,
                                                                        const PartPlan* __restrict__ plan,
                                                                        const unsigned long long* __restrict__ poff,
                                                                        RecBuf sb, unsigned* bucket_count,
                                                                        int narrow_chunk, Ctrl* ctrl) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char* base = smem + warp * SMALL_WARP_SMEM;
  WarpScratch ws;
  ws.init(base);
  unsigned* bm = reinterpret_cast<unsigned*>(base + QCAP * sizeof(QEnt));
  int* rowslot = reinterpret_cast<int*>(bm + SMALL_BITMAP_WORDS);
  int* oddmax = rowslot + WR_MAX;
  int* oddrow = oddmax + WR_MAX;
  int* s_nodd = oddrow + WR_MAX;
  if (ctrl->err) return;
  const unsigned long long total = poff[geo.n_parts * PC_N + PC_WIN_SMALL];
  unsigned long long ncross = 0, npix = 0;
  int st_n = 0;
  unsigned long long wi = 0, wend = 0, p = 0;
  while (true) {
    // windows are taken narrow_chunk at a time: the part of the first is
    // searched, the following ones walk forward from it
    if (wi >= wend) {
      unsigned long long c0 = 0;
      if (lane == 0) c0 = atomicAdd(&ctrl->work_small, (unsigned long long)narrow_chunk);
      c0 = __shfl_sync(0xFFFFFFFFu, c0, 0);
      if (c0 >= total) break;
      wi = c0;
      wend = min(total, c0 + (unsigned long long)narrow_chunk);
      p = window_part(poff, PC_WIN_SMALL, geo.n_parts, wi);
    } else {
      while (poff[(p + 1) * PC_N + PC_WIN_SMALL] <= wi) ++p;
    }
    const PartPlan pl = plan[p];
    const unsigned long long k = wi - poff[p * PC_N + PC_WIN_SMALL];
    const PolyWin win = make_row_window(pl, (int)k);  // narrow parts never take column windows
    const int nr = win.r1 - win.r0, bw = win.bw;
    for (int i = lane; i < nr * bw; i += 32) bm[i] = 0u;
    for (int i = lane; i < WR_MAX; i += 32) rowslot[i] = -1;
    if (lane == 0) *s_nodd = 0;
    const unsigned long long rb = geo.ring_offsets[p], re = geo.ring_offsets[p + 1];
    const unsigned long long vs = geo.vertex_offsets[rb];
    const unsigned nv = (unsigned)(geo.vertex_offsets[re] - vs);
    __syncwarp();
    warp_pass<0, false>(geo, g, rb, re, vs, 0, nv, win, bm, ws.q, rowslot, oddmax, nullptr, ctrl, p, ncross);
    __syncwarp();
    warp_find_odd_rows(bm, 0, nr, bw, rowslot, oddrow, oddmax, s_nodd, nullptr);
    __syncwarp();
    const int nodd = *s_nodd;
    if (nodd > 0) {
      unsigned long long dummy = 0;
      warp_pass<1, false>(geo, g, rb, re, vs, 0, nv, win, bm, ws.q, rowslot, oddmax, nullptr, ctrl, p, dummy);
      __syncwarp();
      for (int t = lane; t < nodd; t += 32) {
        const int i = oddrow[t], loc = oddmax[t];
        if (loc != INT_MIN) bm[i * bw + (loc >> 5)] ^= 1u << (loc & 31);
      }
      __syncwarp();
    }
    warp_extract(bm, nr, bw, win.r0, win.col0, pl, (unsigned)p, ws, st_n, sb, bucket_count, ctrl, npix, nullptr);
    stage_flush(ws, st_n, sb, bucket_count, ctrl);  // the stage aliases the queue of the next window
    ++wi;
  }
  flush_counters(ncross, npix, ctrl);
}

// ---- wide parts: one window per block ---------------------------------------
// Warp w walks vertices [w nv / W, (w + 1) nv / W) with its own queue and
// extracts rows [w nr / W, (w + 1) nr / W); the bitmap is shared.
__global__ void __launch_bounds__(POLY_THREADS) k_poly_spans(Geo geo, Grid g, const PartPlan* __restrict__ plan,
                                                              const unsigned long long* __restrict__ poff,
                                                              RecBuf sb, unsigned* bucket_count, Ctrl* ctrl) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int W = POLY_THREADS / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned* bm = reinterpret_cast<unsigned*>(smem);
  WarpScratch ws;
  ws.init(smem + BITMAP_WORDS * 4 + warp * QCAP * sizeof(QEnt));
  __shared__ int rowslot[WR_MAX];
  __shared__ int oddmax[WR_MAX];
  __shared__ int oddrow[WR_MAX];
  __shared__ int s_nodd;
  __shared__ unsigned s_side[WR_MAX];  // column windows: parity of crossings left (bit 0) / right (bit 1)
  __shared__ unsigned long long s_part, s_w;
  if (ctrl->err) return;
  const unsigned long long total = poff[geo.n_parts * PC_N + PC_WINDOWS];
  unsigned long long ncross = 0, npix = 0;
  int st_n = 0;
  while (true) {
    if (threadIdx.x == 0) s_w = atomicAdd(&ctrl->work, 1ull);
    __syncthreads();
    const unsigned long long wi = s_w;
    if (wi >= total) break;
    if (warp == 0) {
      const unsigned long long p = window_part(poff, PC_WINDOWS, geo.n_parts, wi);
      if (lane == 0) s_part = p;
    }
    __syncthreads();
    const unsigned long long p = s_part;
    const PartPlan pl = plan[p];
    const unsigned long long k = wi - poff[p * PC_N + PC_WINDOWS];
    const PolyWin win = make_window(pl, k);
    const int nr = win.r1 - win.r0, bw = win.bw;
    unsigned* side = win.colwin ? s_side : nullptr;
    for (int i = threadIdx.x; i < nr * bw; i += POLY_THREADS) bm[i] = 0u;
    for (int i = threadIdx.x; i < WR_MAX; i += POLY_THREADS) {
      rowslot[i] = -1;
      s_side[i] = 0u;
    }
    if (threadIdx.x == 0) s_nodd = 0;
    const unsigned long long rb = geo.ring_offsets[p], re = geo.ring_offsets[p + 1];
    const unsigned long long vs = geo.vertex_offsets[rb];
    const unsigned nv = (unsigned)(geo.vertex_offsets[re] - vs);
    const unsigned vb = (unsigned)((unsigned long long)nv * warp / W);
    const unsigned ve = (unsigned)((unsigned long long)nv * (warp + 1) / W);
    __syncthreads();
    warp_pass<0, true>(geo, g, rb, re, vs, vb, ve, win, bm, ws.q, rowslot, oddmax, side, ctrl, p, ncross);
    __syncthreads();
    const int rlo = nr * warp / W, rhi = nr * (warp + 1) / W;
    warp_find_odd_rows(bm, rlo, rhi, bw, rowslot, oddrow, oddmax, &s_nodd, side);
    __syncthreads();
    const int nodd = s_nodd;
    if (nodd > 0) {
      unsigned long long dummy = 0;
      warp_pass<1, true>(geo, g, rb, re, vs, vb, ve, win, bm, ws.q, rowslot, oddmax, side, ctrl, p, dummy);
      __syncthreads();
      // drop the largest crossing of each odd row again: in the bitmap, or in
      // the carry when it lies left of a column window (right of it: no effect)
      for (int t = threadIdx.x; t < nodd; t += POLY_THREADS) {
        const int i = oddrow[t], loc = oddmax[t];
        if (loc == INT_MIN) continue;
        if (loc < 0) s_side[i] ^= 1u;
        else if (loc < win.nbits) bm[i * bw + (loc >> 5)] ^= 1u << (loc & 31);
      }
      __syncthreads();
    }
    warp_extract(bm + rlo * bw, rhi - rlo, bw, win.r0 + rlo, win.col0, pl, (unsigned)p, ws, st_n, sb,
                 bucket_count, ctrl, npix, side ? side + rlo : nullptr);
    stage_flush(ws, st_n, sb, bucket_count, ctrl);
    __syncthreads();
  }
  flush_counters(ncross, npix, ctrl);
}

}  // namespace rzd
