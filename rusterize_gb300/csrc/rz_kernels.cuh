// rz_kernels.cuh -- validation, per-part planning, span generation
// (polygon scanlines, Bresenham lines, points) and the bucket scatter.
//
// Reference semantics restated here (ttrotto/rusterize, rust/src/):
//   geo/edges.rs:79-134              world->pixel, extract_point/ring/line filters
//   rasterization/burners.rs:40-91   Standard::burn_line (Bresenham)
//   rasterization/burners.rs:250-258 burn_point
//   rasterization/burners.rs:261-320 burn_polygon (active-edge scanline, even-odd)
//   rasterization/burn_geometry.rs   part semantics (pooled rings / edges)
#pragma once

#include "rz_device.cuh"

namespace rzd {

// ---------------------------------------------------------------- tables ----
// Reject tables that would make any later kernel read out of bounds.
__global__ void k_validate(Geo geo, Ctrl* ctrl) {
  const unsigned long long tid = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = tid; i <= geo.n_geoms; i += stride) {
    unsigned long long a = geo.part_offsets[i];
    if ((i == 0 && a != 0) || (i == geo.n_geoms && a != geo.n_parts) ||
        (i > 0 && a < geo.part_offsets[i - 1]) || a > geo.n_parts)
      set_error(ctrl, ERR_BAD_TABLE, i);
  }
  for (unsigned long long i = tid; i <= geo.n_parts; i += stride) {
    unsigned long long a = geo.ring_offsets[i];
    if ((i == 0 && a != 0) || (i == geo.n_parts && a != geo.n_rings) ||
        (i > 0 && a < geo.ring_offsets[i - 1]) || a > geo.n_rings)
      set_error(ctrl, ERR_BAD_TABLE, (1ull << 62) | i);
    if (i < geo.n_parts && geo.part_kind[i] > 2) set_error(ctrl, ERR_BAD_KIND, i);
  }
  for (unsigned long long i = tid; i <= geo.n_rings; i += stride) {
    unsigned long long a = geo.vertex_offsets[i];
    if ((i == 0 && a != 0) || (i == geo.n_rings && a != geo.n_vertices) ||
        (i > 0 && a < geo.vertex_offsets[i - 1]) || a > geo.n_vertices)
      set_error(ctrl, ERR_BAD_TABLE, (2ull << 62) | i);
  }
}

__global__ void k_check_bands(Geo geo, unsigned n_bands, Ctrl* ctrl) {
  if (ctrl->err) return;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < geo.n_geoms;
       i += stride)
    if (geo.bands[i] >= n_bands) set_error(ctrl, ERR_BAD_BAND, i);
}

// part -> owning geometry index
__global__ void k_part_geom(Geo geo, unsigned* part_geom, Ctrl* ctrl) {
  if (ctrl->err) return;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long gi = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; gi < geo.n_geoms;
       gi += stride) {
    for (unsigned long long p = geo.part_offsets[gi]; p < geo.part_offsets[gi + 1]; ++p)
      part_geom[p] = (unsigned)gi;
  }
}

// ------------------------------------------------------------ part plans ----
// One warp per part.  Polygon parts get their row range and bitmap window
// geometry from the min/max of their world coordinates (the world->pixel
// map is monotone, so transforming the extremes gives the pixel extremes);
// line and point parts just report their vertex counts.
__global__ void k_part_prep(Geo geo, Grid g, const unsigned* part_geom, PartPlan* plan,
                            unsigned long long* counts /*[P][PC_N]*/, Ctrl* ctrl) {
  if (ctrl->err) return;
  const int lane = threadIdx.x & 31;
  const unsigned long long warp0 = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
  const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
  unsigned long long edges = 0;
  for (unsigned long long p = warp0; p < geo.n_parts; p += nwarps) {
    const unsigned kind = geo.part_kind[p];
    const unsigned long long rb = geo.ring_offsets[p], re = geo.ring_offsets[p + 1];
    const unsigned long long vs = geo.vertex_offsets[rb], ve = geo.vertex_offsets[re];
    const unsigned band = geo.bands ? geo.bands[part_geom[p]] : 0u;
    unsigned long long c[PC_N] = {0, 0, 0, 0, 0};
    PartPlan pl = {0, 0, 0, 0, 0, band};
    if (kind != 0) {
      // segments = vertices - non-empty rings
      unsigned long long nonempty = 0;
      for (unsigned long long r = rb + lane; r < re; r += 32)
        nonempty += geo.vertex_offsets[r + 1] > geo.vertex_offsets[r];
      for (int o = 16; o > 0; o >>= 1) nonempty += __shfl_xor_sync(0xFFFFFFFFu, nonempty, o);
      edges += (lane == 0) ? (ve - vs) - nonempty : 0;
    }
    if (kind == 1) {
      c[PC_LINE_V] = ve - vs;
      c[PC_LINE_P] = 1;
    } else if (kind == 0) {
      c[PC_POINT_V] = ve - vs;
      c[PC_POINT_P] = 1;
    } else {
      double ylo = INFINITY, yhi = -INFINITY, xlo = INFINITY, xhi = -INFINITY;
      int nan_x = 0;
      for (unsigned long long v = vs + lane; v < ve; v += 32) {
        double2 w = geo.xy[v];
        if (!isnan(w.y)) { ylo = fmin(ylo, w.y); yhi = fmax(yhi, w.y); }
        if (!isnan(w.x)) { xlo = fmin(xlo, w.x); xhi = fmax(xhi, w.x); }
        else nan_x = 1;
      }
      for (int o = 16; o > 0; o >>= 1) {
        ylo = fmin(ylo, __shfl_xor_sync(0xFFFFFFFFu, ylo, o));
        yhi = fmax(yhi, __shfl_xor_sync(0xFFFFFFFFu, yhi, o));
        xlo = fmin(xlo, __shfl_xor_sync(0xFFFFFFFFu, xlo, o));
        xhi = fmax(xhi, __shfl_xor_sync(0xFFFFFFFFu, xhi, o));
      }
      nan_x = __any_sync(0xFFFFFFFFu, nan_x);
      if (ylo <= yhi) {
        // pixel y decreases with world y
        const int row0 = row_ceil(to_py(g, yhi), g.nrows);
        const int row1 = row_ceil(to_py(g, ylo), g.nrows);
        if (row1 > row0) {
          double c_lo = 0.0, c_hi = (double)g.ncols;
          if (xlo <= xhi && !nan_x) {
            const double pxl = to_px(g, xlo), pxh = to_px(g, xhi);
            // crossings are interpolations between edge end points; allow a
            // rounding margin that grows with the coordinate magnitude
            const double mag = fmax(fabs(pxl), fabs(pxh));
            const double margin = 2.0 + ldexp(mag, -40);
            c_lo = floor(pxl - margin);
            c_hi = ceil(pxh + margin);
          }
          const int col0 = c_lo <= 0.0 ? 0 : (c_lo >= g.ncols ? g.ncols : (int)c_lo);
          const int colmax = c_hi <= 0.0 ? 0 : (c_hi >= g.ncols ? g.ncols : (int)c_hi);
          const int bw = (colmax - col0 + 1 + 31) >> 5;
          int wr = BITMAP_WORDS / bw;
          if (wr > WR_MAX) wr = WR_MAX;
          if (wr < 1) {
            if (lane == 0) set_error(ctrl, ERR_TOO_WIDE, p);
          } else {
            pl.row0 = row0;
            pl.row1 = row1;
            pl.col0 = col0;
            pl.bw = bw;
            pl.wr = wr;
            c[PC_WINDOWS] = (unsigned long long)((row1 - row0 + wr - 1) / wr);
          }
        }
      }
    }
    if (lane == 0) {
      plan[p] = pl;
#pragma unroll
      for (int k = 0; k < PC_N; ++k) counts[p * PC_N + k] = c[k];
    }
  }
  for (int o = 16; o > 0; o >>= 1) edges += __shfl_xor_sync(0xFFFFFFFFu, edges, o);
  if (lane == 0 && edges) atomicAdd(&ctrl->edges, edges);
}

// compact lists of line and point parts
__global__ void k_part_lists(Geo geo, const unsigned long long* off /*[P+1][PC_N]*/, unsigned* line_parts,
                             unsigned* point_parts, Ctrl* ctrl) {
  if (ctrl->err) return;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long p = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; p < geo.n_parts;
       p += stride) {
    const unsigned kind = geo.part_kind[p];
    if (kind == 1) line_parts[off[p * PC_N + PC_LINE_P]] = (unsigned)p;
    else if (kind == 0) point_parts[off[p * PC_N + PC_POINT_P]] = (unsigned)p;
  }
}

// -------------------------------------------------------------- polygons ----
// One CTA per (part, row window).  Every edge crossing of a scanline centre
// is evaluated in FP64 exactly as PolyEdge::intersect_at (edges.rs:50-55) and
// rounded to its pixel boundary r = clamp(floor(x + 0.5), 0, ncols)
// (burners.rs:310-311).  Because that rounding is monotone, pairing the
// x-sorted crossings (burners.rs:302-316) covers exactly the pixels whose
// count of boundaries r <= x is odd, so each crossing toggles bit r of a
// per-row parity bitmap and spans are read back as consecutive set bits.
// chunks_exact(2) drops the largest crossing of an odd row: such rows are
// fixed up by toggling their maximum r once more.  Positive-NaN crossings
// sort after every number (total_cmp) and pair into empty spans, so they
// are skipped; negative NaNs round to 0 and sort first.
template <int MODE>  // 0: toggle crossings, 1: max crossing of odd rows
__device__ __forceinline__ void poly_edges(const Geo& geo, const Grid& g, unsigned long long rb,
                                           unsigned long long re, int r0, int r1, int col0, int bw,
                                           unsigned* bm, const int* rowslot, int* oddmax, Ctrl* ctrl,
                                           unsigned long long p, unsigned long long& ncross) {
  const int lane = threadIdx.x & 31;
  const unsigned long long vs = geo.vertex_offsets[rb], ve = geo.vertex_offsets[re];
  unsigned long long ring = rb;
  const int nbits = bw * 32;
  for (unsigned long long base = vs; base < ve; base += POLY_THREADS) {
    const unsigned long long v = base + threadIdx.x;
    const bool has = v < ve;
    double2 w0 = make_double2(0.0, 0.0);
    double py0 = 0.0;
    int ys0 = 0;
    if (has) {
      w0 = geo.xy[v];
      py0 = to_py(g, w0.y);
      ys0 = row_ceil(py0, g.nrows);
    }
    // vertex v+1 from the next lane (lane 31 loads it)
    double py1 = __shfl_down_sync(0xFFFFFFFFu, py0, 1);
    int ys1 = __shfl_down_sync(0xFFFFFFFFu, ys0, 1);
    if (!has) continue;
    // ring containing v
    if (geo.vertex_offsets[ring + 1] <= v) {
      int steps = 0;
      while (steps < 4 && geo.vertex_offsets[ring + 1] <= v) { ++ring; ++steps; }
      if (geo.vertex_offsets[ring + 1] <= v) {
        unsigned long long lo = ring, hi = re;  // vo[lo] <= v < vo[hi]
        while (hi - lo > 1) {
          unsigned long long mid = (lo + hi) >> 1;
          if (geo.vertex_offsets[mid] <= v) lo = mid; else hi = mid;
        }
        ring = lo;
      }
    }
    if (v + 1 >= geo.vertex_offsets[ring + 1]) continue;  // last vertex of its ring
    double2 w1;
    if (lane == 31 || v + 1 >= base + POLY_THREADS) {
      w1 = geo.xy[v + 1];
      py1 = to_py(g, w1.y);
      ys1 = row_ceil(py1, g.nrows);
    }
    if (ys0 == ys1) continue;  // no scanline centre in [y_top, y_bot)
    // extract_ring's horizontal filter (edges.rs:100); the raster-row filter
    // (:105) only removes edges without rows in [0, nrows), already empty here
    if (!(fabs(__dsub_rn(py0, py1)) >= 2.220446049250313e-16)) continue;
    const bool top0 = ys0 < ys1;  // y0 < y1 (ceil is monotone, values differ)
    const int ystart = top0 ? ys0 : ys1, yend = top0 ? ys1 : ys0;
    const int a = max(ystart, r0), b = min(yend, r1);
    if (a >= b) continue;
    if (lane != 31 && v + 1 < base + POLY_THREADS) w1 = geo.xy[v + 1];
    const double px0 = to_px(g, w0.x), px1 = to_px(g, w1.x);
    const double xt = top0 ? px0 : px1, yt = top0 ? py0 : py1;
    const double xb = top0 ? px1 : px0, yb = top0 ? py1 : py0;
    const double dxdy = __ddiv_rn(__dsub_rn(xb, xt), __dsub_rn(yb, yt));  // edges.rs:36
    for (int y = a; y < b; ++y) {
      if (MODE == 1 && rowslot[y - r0] < 0) continue;
      const double cy = __dadd_rn((double)y, 0.5);
      const double x = __dadd_rn(xt, __dmul_rn(__dsub_rn(cy, yt), dxdy));
      int r;
      if (isnan(x)) {
        if (!signbit(x)) continue;
        r = 0;
      } else {
        const double f = floor(__dadd_rn(x, 0.5));
        r = f <= 0.0 ? 0 : (f >= (double)g.ncols ? g.ncols : (int)f);
      }
      const int loc = r - col0;
      if (loc < 0 || loc >= nbits) {
        set_error(ctrl, ERR_BITMAP, p);
        continue;
      }
      if (MODE == 0) {
        atomicXor(&bm[(y - r0) * bw + (loc >> 5)], 1u << (loc & 31));
        ++ncross;
      } else {
        atomicMax(&oddmax[rowslot[y - r0]], loc);
      }
    }
  }
}

__global__ void __launch_bounds__(POLY_THREADS) k_poly_spans(Geo geo, Grid g, const PartPlan* __restrict__ plan,
                                                              const unsigned long long* __restrict__ poff,
                                                              SpanBuf sb, unsigned* bucket_count, Ctrl* ctrl) {
  __shared__ unsigned bm[BITMAP_WORDS];
  __shared__ int rowslot[WR_MAX];
  __shared__ int oddmax[WR_MAX];
  __shared__ int oddrow[WR_MAX];
  __shared__ int s_nodd;
  __shared__ unsigned long long s_part, s_w;
  if (ctrl->err) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned long long total = poff[geo.n_parts * PC_N + PC_WINDOWS];
  unsigned long long ncross = 0, npix = 0;
  while (true) {
    if (threadIdx.x == 0) {
      const unsigned long long w = atomicAdd(&ctrl->work, 1ull);
      s_w = w;
      if (w < total) {
        unsigned long long lo = 0, hi = geo.n_parts;  // off[lo] <= w < off[hi]
        while (hi - lo > 1) {
          const unsigned long long mid = (lo + hi) >> 1;
          if (poff[mid * PC_N + PC_WINDOWS] <= w) lo = mid; else hi = mid;
        }
        s_part = lo;
      }
      s_nodd = 0;
    }
    __syncthreads();
    const unsigned long long w = s_w;
    if (w >= total) break;
    const unsigned long long p = s_part;
    const PartPlan pl = plan[p];
    const int k = (int)(w - poff[p * PC_N + PC_WINDOWS]);
    const int r0 = pl.row0 + k * pl.wr;
    const int r1 = min(r0 + pl.wr, pl.row1);
    const int nr = r1 - r0, bw = pl.bw;
    for (int i = threadIdx.x; i < nr * bw; i += POLY_THREADS) bm[i] = 0u;
    if (threadIdx.x < WR_MAX) rowslot[threadIdx.x] = -1;
    __syncthreads();
    const unsigned long long rb = geo.ring_offsets[p], re = geo.ring_offsets[p + 1];
    poly_edges<0>(geo, g, rb, re, r0, r1, pl.col0, bw, bm, rowslot, oddmax, ctrl, p, ncross);
    __syncthreads();
    // rows with an odd number of crossings
    for (int i = warp; i < nr; i += POLY_THREADS / 32) {
      unsigned par = 0;
      for (int wd = lane; wd < bw; wd += 32) par ^= (unsigned)__popc(bm[i * bw + wd]) & 1u;
      par = __reduce_xor_sync(0xFFFFFFFFu, par);
      if (lane == 0 && par) {
        const int slot = atomicAdd(&s_nodd, 1);
        rowslot[i] = slot;
        oddrow[slot] = i;
        oddmax[slot] = -1;
      }
    }
    __syncthreads();
    if (s_nodd > 0) {
      unsigned long long dummy = 0;
      poly_edges<1>(geo, g, rb, re, r0, r1, pl.col0, bw, bm, rowslot, oddmax, ctrl, p, dummy);
      __syncthreads();
      if (threadIdx.x < s_nodd) {
        const int i = oddrow[threadIdx.x], loc = oddmax[threadIdx.x];
        if (loc >= 0) bm[i * bw + (loc >> 5)] ^= 1u << (loc & 31);
      }
      __syncthreads();
    }
    // spans = pairs of consecutive set bits, one warp per row
    for (int i = warp; i < nr; i += POLY_THREADS / 32) {
      const int y = r0 + i;
      unsigned carry_cnt = 0;
      int carry_last = -1;
      for (int wb = 0; wb < bw; wb += 32) {
        const int wd = wb + lane;
        unsigned bits = wd < bw ? bm[i * bw + wd] : 0u;
        const int cnt = __popc(bits);
        int incl = cnt;
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
          if (lane >= o) incl += t;
        }
        const int mylast = bits ? wd * 32 + 31 - __clz(bits) : -1;
        int mx = mylast;
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xFFFFFFFFu, mx, o);
          if (lane >= o) mx = max(mx, t);
        }
        int prev = __shfl_up_sync(0xFFFFFFFFu, mx, 1);
        if (lane == 0) prev = -1;
        prev = max(prev, carry_last);
        unsigned gidx = carry_cnt + (unsigned)(incl - cnt);
        while (bits) {
          const int b = __ffs(bits) - 1;
          bits &= bits - 1;
          const int pos = wd * 32 + b;
          if (gidx & 1u) {
            const int xs = pl.col0 + prev, xe = pl.col0 + pos;
            npix += (unsigned long long)(xe - xs);
            emit_span(sb, bucket_count, ctrl, g, pl.band, y, xs, xe, (unsigned)p, 0u);
          }
          prev = pos;
          ++gidx;
        }
        carry_cnt += (unsigned)__shfl_sync(0xFFFFFFFFu, incl, 31);
        carry_last = max(carry_last, __shfl_sync(0xFFFFFFFFu, mx, 31));
      }
    }
    __syncthreads();
  }
  for (int o = 16; o > 0; o >>= 1) {
    ncross += __shfl_xor_sync(0xFFFFFFFFu, ncross, o);
    npix += __shfl_xor_sync(0xFFFFFFFFu, npix, o);
  }
  if (lane == 0) {
    if (ncross) atomicAdd(&ctrl->crossings, ncross);
    if (npix) atomicAdd(&ctrl->pixel_writes, npix);
  }
}

// ------------------------------------------------------------- lines -------
// Locate, for compacted index t, the list slot q with cum(q) <= t < cum(q+1)
// where cum(q) = off[list[q]*PC_N + col].  Lane 0 binary-searches the warp's
// first index, the others walk forward from it.
__device__ __forceinline__ unsigned long long locate(const unsigned* list, unsigned long long nlist,
                                                     const unsigned long long* off, int col,
                                                     unsigned long long t, unsigned long long t_first) {
  unsigned long long q0 = 0;
  if ((threadIdx.x & 31) == 0) {
    unsigned long long lo = 0, hi = nlist;  // cum(lo) <= t_first < cum(hi) (cum(nlist) = total)
    while (hi - lo > 1) {
      const unsigned long long mid = (lo + hi) >> 1;
      if (off[(unsigned long long)list[mid] * PC_N + col] <= t_first) lo = mid; else hi = mid;
    }
    q0 = lo;
  }
  q0 = __shfl_sync(0xFFFFFFFFu, q0, 0);
  unsigned long long q = q0;
  while (q + 1 < nlist && off[(unsigned long long)list[q + 1] * PC_N + col] <= t) ++q;
  return q;
}

__device__ __forceinline__ unsigned long long ring_of(const Geo& geo, unsigned long long rb,
                                                      unsigned long long re, unsigned long long v) {
  unsigned long long lo = rb, hi = re;  // vo[lo] <= v < vo[hi]
  while (hi - lo > 1) {
    const unsigned long long mid = (lo + hi) >> 1;
    if (geo.vertex_offsets[mid] <= v) lo = mid; else hi = mid;
  }
  return lo;
}

struct RunEmitter {
  int y = -1, xa = 0, xb = 0;  // current run [xa, xb) in row y
  unsigned long long npix = 0;
};

__device__ __forceinline__ void run_flush(RunEmitter& re, const SpanBuf& sb, unsigned* bucket_count,
                                          Ctrl* ctrl, const Grid& g, unsigned band, unsigned part,
                                          unsigned flags) {
  if (re.y >= 0) {
    re.npix += (unsigned long long)(re.xb - re.xa);
    emit_span(sb, bucket_count, ctrl, g, band, re.y, re.xa, re.xb, part, flags);
  }
  re.y = -1;
}

__device__ __forceinline__ void run_add(RunEmitter& re, const SpanBuf& sb, unsigned* bucket_count, Ctrl* ctrl,
                                        const Grid& g, unsigned band, unsigned part, unsigned flags, int y,
                                        int x) {
  if (re.y == y && x == re.xb) { re.xb = x + 1; return; }
  if (re.y == y && x == re.xa - 1) { re.xa = x; return; }
  run_flush(re, sb, bucket_count, ctrl, g, band, part, flags);
  re.y = y;
  re.xa = x;
  re.xb = x + 1;
}

// One thread per line vertex v: segment (v, v+1) of its linestring, burned
// with Standard::burn_line's integer Bresenham (burners.rs:40-91) after
// extract_line's bbox filter (edges.rs:112-134).  The end pixel of the
// part's last kept segment is written by k_line_endpix.
__global__ void k_line_spans(Geo geo, Grid g, const PartPlan* __restrict__ plan,
                             const unsigned long long* __restrict__ poff, const unsigned* __restrict__ line_parts,
                             unsigned long long* last_kept, unsigned dedup_flag, SpanBuf sb,
                             unsigned* bucket_count, Ctrl* ctrl) {
  if (ctrl->err) return;
  const unsigned long long nlist = poff[geo.n_parts * PC_N + PC_LINE_P];
  const unsigned long long total = poff[geo.n_parts * PC_N + PC_LINE_V];
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  RunEmitter run;
  for (unsigned long long t0 = blockIdx.x * (unsigned long long)blockDim.x + (threadIdx.x & ~31u); t0 < total;
       t0 += stride) {
    const unsigned long long t = t0 + (threadIdx.x & 31);
    const unsigned long long q = locate(line_parts, nlist, poff, PC_LINE_V, t < total ? t : total - 1, t0);
    if (t >= total) continue;
    const unsigned p = line_parts[q];
    const unsigned long long rb = geo.ring_offsets[p], re = geo.ring_offsets[p + 1];
    const unsigned long long v = geo.vertex_offsets[rb] + (t - poff[(unsigned long long)p * PC_N + PC_LINE_V]);
    const unsigned long long r = ring_of(geo, rb, re, v);
    if (v + 1 >= geo.vertex_offsets[r + 1]) continue;
    const double2 w0 = geo.xy[v], w1 = geo.xy[v + 1];
    const double x0 = to_px(g, w0.x), y0 = to_py(g, w0.y);
    const double x1 = to_px(g, w1.x), y1 = to_py(g, w1.y);
    const double min_x = min_rs(x0, x1), max_x = max_rs(x0, x1);
    const double min_y = min_rs(y0, y1), max_y = max_rs(y0, y1);
    if (!(min_x < (double)g.ncols && max_x >= 0.0 && min_y < (double)g.nrows && max_y >= 0.0)) continue;
    atomicMax(&last_kept[p], v + 1);  // 0 = no kept segment
    long long ix0 = as_isize(floor(x0)), iy0 = as_isize(floor(y0));
    const long long ix1 = as_isize(floor(x1)), iy1 = as_isize(floor(y1));
    // step counts checked in f64 first: saturated end points (+-inf) would
    // overflow the integer differences
    if (fabs((double)ix1 - (double)ix0) > (double)LINE_MAX_STEPS ||
        fabs((double)iy1 - (double)iy0) > (double)LINE_MAX_STEPS) {
      set_error(ctrl, ERR_LINE_LONG, v);
      continue;
    }
    const long long dx = ix1 > ix0 ? ix1 - ix0 : ix0 - ix1;
    const long long dy = -(iy1 > iy0 ? iy1 - iy0 : iy0 - iy1);
    const long long sx = ix0 < ix1 ? 1 : -1, sy = iy0 < iy1 ? 1 : -1;
    long long err = dx + dy;
    const unsigned band = plan[p].band;
    while (ix0 != ix1 || iy0 != iy1) {
      if (ix0 >= 0 && ix0 < g.ncols && iy0 >= 0 && iy0 < g.nrows)
        run_add(run, sb, bucket_count, ctrl, g, band, p, dedup_flag, (int)iy0, (int)ix0);
      const long long e2 = 2 * err;
      if (e2 >= dy) { err += dy; ix0 += sx; }
      if (e2 <= dx) { err += dx; iy0 += sy; }
    }
    run_flush(run, sb, bucket_count, ctrl, g, band, p, dedup_flag);
  }
  unsigned long long npix = run.npix;
  for (int o = 16; o > 0; o >>= 1) npix += __shfl_xor_sync(0xFFFFFFFFu, npix, o);
  if ((threadIdx.x & 31) == 0 && npix) atomicAdd(&ctrl->pixel_writes, npix);
}

// burners.rs:87-89: after the last kept segment of the part, its end pixel
// is written unless that segment's linestring is closed.
__global__ void k_line_endpix(Geo geo, Grid g, const PartPlan* __restrict__ plan,
                              const unsigned long long* __restrict__ poff, const unsigned* __restrict__ line_parts,
                              const unsigned long long* __restrict__ last_kept, unsigned dedup_flag, SpanBuf sb,
                              unsigned* bucket_count, Ctrl* ctrl) {
  if (ctrl->err) return;
  const unsigned long long nlist = poff[geo.n_parts * PC_N + PC_LINE_P];
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  unsigned long long npix = 0;
  for (unsigned long long q = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; q < nlist; q += stride) {
    const unsigned p = line_parts[q];
    if (last_kept[p] == 0) continue;
    const unsigned long long v = last_kept[p] - 1;
    const unsigned long long rb = geo.ring_offsets[p], re = geo.ring_offsets[p + 1];
    const unsigned long long r = ring_of(geo, rb, re, v);
    const double2 first = geo.xy[geo.vertex_offsets[r]];
    const double2 last = geo.xy[geo.vertex_offsets[r + 1] - 1];
    if (first.x == last.x && first.y == last.y) continue;  // LineString::is_closed
    const double2 w1 = geo.xy[v + 1];
    const long long ix = as_isize(floor(to_px(g, w1.x))), iy = as_isize(floor(to_py(g, w1.y)));
    if (ix >= 0 && ix < g.ncols && iy >= 0 && iy < g.nrows) {
      ++npix;
      emit_span(sb, bucket_count, ctrl, g, plan[p].band, (int)iy, (int)ix, (int)ix + 1, p, dedup_flag);
    }
  }
  if (npix) atomicAdd(&ctrl->pixel_writes, npix);
}

// ------------------------------------------------------------- points ------
// extract_point (edges.rs:79-88) + burn_point (burners.rs:250-258)
__global__ void k_point_spans(Geo geo, Grid g, const PartPlan* __restrict__ plan,
                              const unsigned long long* __restrict__ poff, const unsigned* __restrict__ point_parts,
                              SpanBuf sb, unsigned* bucket_count, Ctrl* ctrl) {
  if (ctrl->err) return;
  const unsigned long long nlist = poff[geo.n_parts * PC_N + PC_POINT_P];
  const unsigned long long total = poff[geo.n_parts * PC_N + PC_POINT_V];
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  unsigned long long npix = 0;
  for (unsigned long long t0 = blockIdx.x * (unsigned long long)blockDim.x + (threadIdx.x & ~31u); t0 < total;
       t0 += stride) {
    const unsigned long long t = t0 + (threadIdx.x & 31);
    const unsigned long long q = locate(point_parts, nlist, poff, PC_POINT_V, t < total ? t : total - 1, t0);
    if (t >= total) continue;
    const unsigned p = point_parts[q];
    const unsigned long long v =
        geo.vertex_offsets[geo.ring_offsets[p]] + (t - poff[(unsigned long long)p * PC_N + PC_POINT_V]);
    const double2 w = geo.xy[v];
    const double x = to_px(g, w.x), y = to_py(g, w.y);
    if (x >= 0.0 && x < (double)g.ncols && y >= 0.0 && y < (double)g.nrows) {
      ++npix;
      emit_span(sb, bucket_count, ctrl, g, plan[p].band, (int)y, (int)x, (int)x + 1, p, 0u);
    }
  }
  for (int o = 16; o > 0; o >>= 1) npix += __shfl_xor_sync(0xFFFFFFFFu, npix, o);
  if ((threadIdx.x & 31) == 0 && npix) atomicAdd(&ctrl->pixel_writes, npix);
}

// ------------------------------------------------------------- scatter -----
// Move each span into its bucket's range.  Order inside a bucket is
// arbitrary here; the fill kernels restore part order.
__global__ void k_scatter(SpanBuf sb, const unsigned* __restrict__ offsets, unsigned* counts, uint2* sorted,
                          Ctrl* ctrl) {
  if (ctrl->err || ctrl->span_count > sb.cap) return;
  const unsigned long long n = ctrl->span_count;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n; i += stride) {
    const unsigned b = sb.bucket[i];
    const unsigned pos = offsets[b] + atomicSub(&counts[b], 1u) - 1u;
    sorted[pos] = make_uint2(sb.part[i], sb.xs[i]);
  }
}

}  // namespace rzd
