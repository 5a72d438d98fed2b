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

#include <type_traits>

#include "rz_device.cuh"
#include "rz_poly.cuh"

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
// line and point parts just report their vertex counts.  The kernel waits
// on dependent loads, so it is held to six blocks per SM (at most 42
// registers) for more loads in flight.
__global__ void __launch_bounds__(256, 6) k_part_prep(Geo geo, Grid g, JobDims one, const JobDims* __restrict__ jobs,
                                                     unsigned n_jobs, const unsigned* part_geom, PartPlan* plan,
                                                     unsigned long long* counts /*[P][PC_N]*/, Tune tn, Ctrl* ctrl) {
  if (ctrl->err) return;
  const int lane = threadIdx.x & 31;
  const unsigned long long warp0 = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
  const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
  unsigned long long edges = 0;
  for (unsigned long long p = warp0; p < geo.n_parts; p += nwarps) {
    const unsigned kind = geo.part_kind[p];
    const unsigned long long rb = geo.ring_offsets[p], re = geo.ring_offsets[p + 1];
    const unsigned long long vs = geo.vertex_offsets[rb], ve = geo.vertex_offsets[re];
    const unsigned gi = part_geom[p];
    const unsigned band = geo.bands ? geo.bands[gi] : 0u;
    const JobDims jd = jobs ? jobs[job_of(jobs, n_jobs, gi)] : one;
    unsigned long long c[PC_N] = {0, 0, 0, 0, 0, 0};
    PartPlan pl;
    pl.row0 = pl.row1 = pl.col0 = pl.bw = pl.wr = 0;
    pl.band = band;
    pl.nrows = jd.nrows;
    pl.ncols = jd.ncols;
    pl.wpr = jd.ntx * WPT;
    // unsigned arithmetic wraps: row r of the window lands on wid0 + r * wpr
    pl.wid0 = jd.wid_base + (band - jd.band_lo) * (unsigned)(jd.row_hi - jd.row_lo) * pl.wpr -
              (unsigned)jd.row_lo * pl.wpr;
    pl.flags = kind == 1 ? jd.line_flag : (kind == 2 ? jd.poly_flag : 0u);
    pl.rlo = jd.row_lo;
    pl.rhi = jd.row_hi;
    pl.ncw = 0;
    // parts of bands outside the window burn nothing in this call
    const bool in_window = band >= jd.band_lo && band < jd.band_hi && jd.row_lo < jd.row_hi;
    if (!in_window) {
      if (lane == 0) {
        plan[p] = pl;
#pragma unroll
        for (int k = 0; k < PC_N; ++k) counts[p * PC_N + k] = 0;
      }
      continue;
    }
    if (kind != 0) {
      // segments = vertices - non-empty rings
      unsigned long long nonempty = 0;
      for (unsigned long long r = rb + lane; r < re; r += 32)
        nonempty += geo.vertex_offsets[r + 1] > geo.vertex_offsets[r];
      for (int o = 16; o > 0; o >>= 1) nonempty += __shfl_xor_sync(0xFFFFFFFFu, nonempty, o);
      edges += (lane == 0) ? (ve - vs) - nonempty : 0;
    }
    if (kind == 1 || (kind == 2 && g.touched)) {  // all_touched also walks polygon rings
      c[PC_LINE_V] = ve - vs;
      c[PC_LINE_P] = 1;
    }
    if (kind == 1) {
    } else if (kind == 0) {
      c[PC_POINT_V] = ve - vs;
      c[PC_POINT_P] = 1;
    } else {
      // min / max of the world coordinates on the integer pipe: monotone
      // keys of the bit patterns, NaN excluded (edges with NaN never burn)
      long long ylo = 0x7FFFFFFFFFFFFFFFll, yhi = (long long)0x8000000000000000ull;
      long long xlo = 0x7FFFFFFFFFFFFFFFll, xhi = (long long)0x8000000000000000ull;
      int nan_x = 0;
      auto fold = [&](double2 w) {
        const unsigned long long by = f64_bits(w.y), bx = f64_bits(w.x);
        if (!nan_bits(by)) {
          const long long k = (long long)(by ^ ((unsigned long long)((long long)by >> 63) >> 1));
          ylo = min(ylo, k);
          yhi = max(yhi, k);
        }
        if (!nan_bits(bx)) {
          const long long k = (long long)(bx ^ ((unsigned long long)((long long)bx >> 63) >> 1));
          xlo = min(xlo, k);
          xhi = max(xhi, k);
        } else {
          nan_x = 1;
        }
      };
      // four loads in flight per lane; min / max are idempotent, so a
      // missing vertex folds the first one again
      for (unsigned long long v = vs + lane; v < ve; v += 128) {
        const double2 w = geo.xy[v];
        const double2 w2 = v + 32 < ve ? geo.xy[v + 32] : w;
        const double2 w3 = v + 64 < ve ? geo.xy[v + 64] : w;
        const double2 w4 = v + 96 < ve ? geo.xy[v + 96] : w;
        fold(w);
        fold(w2);
        fold(w3);
        fold(w4);
      }
      for (int o = 16; o > 0; o >>= 1) {
        ylo = min(ylo, (long long)__shfl_xor_sync(0xFFFFFFFFu, (unsigned long long)ylo, o));
        yhi = max(yhi, (long long)__shfl_xor_sync(0xFFFFFFFFu, (unsigned long long)yhi, o));
        xlo = min(xlo, (long long)__shfl_xor_sync(0xFFFFFFFFu, (unsigned long long)xlo, o));
        xhi = max(xhi, (long long)__shfl_xor_sync(0xFFFFFFFFu, (unsigned long long)xhi, o));
      }
      nan_x = __any_sync(0xFFFFFFFFu, nan_x);
      auto unkey = [](long long k) {
        const unsigned long long b = (unsigned long long)k ^ ((unsigned long long)(k >> 63) >> 1);
        return __longlong_as_double((long long)b);
      };
      if (ylo <= yhi) {
        // pixel y decreases with world y
        const int row0 = max(row_ceil(to_py(g, unkey(yhi)), jd.nrows), jd.row_lo);
        const int row1 = min(row_ceil(to_py(g, unkey(ylo)), jd.nrows), jd.row_hi);
        if (row1 > row0) {
          double c_lo = 0.0, c_hi = (double)jd.ncols;
          if (xlo <= xhi && !nan_x) {
            const double pxl = to_px(g, unkey(xlo)), pxh = to_px(g, unkey(xhi));
            // crossings are interpolations between edge end points; allow a
            // rounding margin that grows with the coordinate magnitude
            const double mag = fmax(fabs(pxl), fabs(pxh));
            const double margin = 2.0 + ldexp(mag, -40);
            c_lo = floor(pxl - margin);
            c_hi = ceil(pxh + margin);
          }
          // the bitmap starts on a 32-pixel word so that its words are raster words
          const int col0 = (c_lo <= 0.0 ? 0 : (c_lo >= jd.ncols ? jd.ncols : (int)c_lo)) & ~31;
          const int colmax = c_hi <= 0.0 ? 0 : (c_hi >= jd.ncols ? jd.ncols : (int)c_hi);
          const int bw = (colmax - col0 + 1 + 31) >> 5;
          const bool narrow = bw <= tn.narrow_max_words;
          pl.row0 = row0;
          pl.row1 = row1;
          pl.col0 = col0;
          pl.bw = bw;
          if (bw > BITMAP_WORDS) {  // wider than one bitmap: windows of columns too
            const int wr = min(COLWIN_ROWS, tn.rows_per_window);
            pl.wr = wr;
            pl.ncw = (unsigned)((bw + COLWIN_WORDS - 1) / COLWIN_WORDS);
            c[PC_WINDOWS] = (unsigned long long)((row1 - row0 + wr - 1) / wr) * pl.ncw;
          } else {
            int wr = (narrow ? SMALL_BITMAP_WORDS : BITMAP_WORDS) / bw;
            if (wr > tn.rows_per_window) wr = tn.rows_per_window;
            pl.wr = wr;
            c[narrow ? PC_WIN_SMALL : PC_WINDOWS] = (unsigned long long)((row1 - row0 + wr - 1) / wr);
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
    // a part is listed when it was counted (parts outside the call's window are not)
    if (off[(p + 1) * PC_N + PC_LINE_P] > off[p * PC_N + PC_LINE_P])
      line_parts[off[p * PC_N + PC_LINE_P]] = (unsigned)p;
    else if (off[(p + 1) * PC_N + PC_POINT_P] > off[p * PC_N + PC_POINT_P])
      point_parts[off[p * PC_N + PC_POINT_P]] = (unsigned)p;
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

__device__ __forceinline__ void run_flush(RunEmitter& re, const RecBuf& sb, unsigned* bucket_count,
                                          Ctrl* ctrl, const PartPlan& pl, unsigned part) {
  if (re.y >= 0) {
    re.npix += (unsigned long long)(re.xb - re.xa);
    emit_run(sb, bucket_count, ctrl, pl, re.y, re.xa, re.xb, part | pl.flags);
  }
  re.y = -1;
}

__device__ __forceinline__ void run_add(RunEmitter& re, const RecBuf& sb, unsigned* bucket_count, Ctrl* ctrl,
                                        const PartPlan& pl, unsigned part, int y, int x) {
  if (re.y == y && x == re.xb) { re.xb = x + 1; return; }
  if (re.y == y && x == re.xa - 1) { re.xa = x; return; }
  run_flush(re, sb, bucket_count, ctrl, pl, part);
  re.y = y;
  re.xa = x;
  re.xb = x + 1;
}

// AllTouched::burn_line for one segment (burners.rs:94-247, adapted there
// from GDAL's llrasterize.cpp): every pixel the segment touches, visited
// left to right, calling emit(y, x) for those inside the raster.  The FP64
// steps are the reference's, without FMA.  Returns false when the walk takes
// more steps than a segment of its extent can need (pathological input),
// after which the caller reports an error.
template <typename Emit>
__device__ __forceinline__ bool all_touched_walk(double df_x, double df_y, double df_x_end, double df_y_end,
                                                 int nrows_i, int ncols_i, Emit&& emit) {
  const double EPSILON_INTERSECT = 1e-4, TOLERANCE = 1e-9;
  const long long nrows = nrows_i, ncols = ncols_i;
  const double nrows_f = (double)nrows_i, ncols_f = (double)ncols_i;
  if (df_x > df_x_end) {  // proceed left to right
    double t = df_x; df_x = df_x_end; df_x_end = t;
    t = df_y; df_y = df_y_end; df_y_end = t;
  }
  if (fabs(__dsub_rn(df_x, df_x_end)) < 0.01) {  // vertical
    if (df_y_end < df_y) { const double t = df_y; df_y = df_y_end; df_y_end = t; }
    const long long ix = as_isize(floor(df_x_end));
    long long iy = as_isize(floor(df_y));
    long long iy_end = as_isize(floor(__dsub_rn(df_y_end, EPSILON_INTERSECT)));
    if (ix < 0 || ix >= ncols) return true;
    iy = iy > 0 ? iy : 0;
    iy_end = iy_end < nrows - 1 ? iy_end : nrows - 1;
    if (iy_end - iy > LINE_MAX_STEPS) return false;
    for (long long y = iy; y <= iy_end; ++y) emit((int)y, (int)ix);
    return true;
  }
  if (fabs(__dsub_rn(df_y, df_y_end)) < 0.01) {  // horizontal
    if (df_x_end < df_x) { const double t = df_x; df_x = df_x_end; df_x_end = t; }
    long long ix = as_isize(floor(df_x));
    const long long iy = as_isize(floor(df_y));
    long long ix_end = as_isize(floor(__dsub_rn(df_x_end, EPSILON_INTERSECT)));
    if (iy < 0 || iy >= nrows) return true;
    ix = ix > 0 ? ix : 0;
    ix_end = ix_end < ncols - 1 ? ix_end : ncols - 1;
    if (ix_end - ix > LINE_MAX_STEPS) return false;
    for (long long x = ix; x <= ix_end; ++x) emit((int)iy, (int)x);
    return true;
  }
  // sloped
  const double slope = __ddiv_rn(__dsub_rn(df_y_end, df_y), __dsub_rn(df_x_end, df_x));
  const double inv_slope = __ddiv_rn(1.0, slope);
  if (df_x < 0.0) { df_y = __dadd_rn(df_y, __dmul_rn(__dsub_rn(0.0, df_x), slope)); df_x = 0.0; }
  if (df_x_end > ncols_f) {
    df_y_end = __dadd_rn(df_y_end, __dmul_rn(__dsub_rn(ncols_f, df_x_end), slope));
    df_x_end = ncols_f;
  }
  if (df_y < 0.0) { df_x = __dadd_rn(df_x, __dmul_rn(__dsub_rn(0.0, df_y), inv_slope)); df_y = 0.0; }
  else if (df_y > nrows_f) { df_x = __dadd_rn(df_x, __dmul_rn(__dsub_rn(nrows_f, df_y), inv_slope)); df_y = nrows_f; }
  if (df_y_end < 0.0) df_x_end = __dadd_rn(df_x_end, __dmul_rn(__dsub_rn(0.0, df_y_end), inv_slope));
  else if (df_y_end > nrows_f) df_x_end = __dadd_rn(df_x_end, __dmul_rn(__dsub_rn(nrows_f, df_y_end), inv_slope));
  // clamp to the raster (f64::clamp)
  df_x = df_x < 0.0 ? 0.0 : (df_x > ncols_f ? ncols_f : df_x);
  df_x_end = df_x_end < 0.0 ? 0.0 : (df_x_end > ncols_f ? ncols_f : df_x_end);
  // every step crosses a pixel boundary in x or y (or nudges y by TOLERANCE
  // across one) and the clipped walk stays within the raster, so it needs
  // fewer steps than this
  long long budget = 4 * (ncols + nrows + 4) + 1024;
  while (df_x >= 0.0 && df_x < df_x_end) {
    if (--budget < 0) return false;
    const long long ix = as_isize(floor(df_x));
    const long long iy = as_isize(floor(df_y));
    if (ix >= 0 && ix < ncols && iy >= 0 && iy < nrows) emit((int)iy, (int)ix);
    double sx = __dsub_rn(floor(__dadd_rn(df_x, 1.0)), df_x);
    double sy = __dmul_rn(sx, slope);
    if (as_isize(floor(__dadd_rn(df_y, sy))) == iy) {
      df_x = __dadd_rn(df_x, sx);
      df_y = __dadd_rn(df_y, sy);
    } else if (slope < 0.0) {
      sy = __dsub_rn((double)iy, df_y);
      if (sy > -TOLERANCE) sy = -TOLERANCE;
      sx = __ddiv_rn(sy, slope);
      df_x = __dadd_rn(df_x, sx);
      df_y = __dadd_rn(df_y, sy);
    } else {
      sy = __dsub_rn((double)(iy + 1), df_y);
      if (sy < TOLERANCE) sy = TOLERANCE;
      sx = __ddiv_rn(sy, slope);
      df_x = __dadd_rn(df_x, sx);
      df_y = __dadd_rn(df_y, sy);
    }
  }
  return true;
}

// One thread per line vertex v: segment (v, v+1) of its linestring, burned
// with Standard::burn_line's integer Bresenham (burners.rs:40-91) after
// extract_line's bbox filter (edges.rs:112-134).  The end pixel of the
// part's last kept segment is written by k_line_endpix.
__global__ void k_line_spans(Geo geo, Grid g, const PartPlan* __restrict__ plan,
                             const unsigned long long* __restrict__ poff, const unsigned* __restrict__ line_parts,
                             unsigned long long* last_kept, RecBuf sb, unsigned* bucket_count, Ctrl* ctrl) {
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
    const PartPlan pl = plan[p];
    if (!(min_x < (double)pl.ncols && max_x >= 0.0 && min_y < (double)pl.nrows && max_y >= 0.0)) continue;
    if (g.touched) {  // AllTouched::burn_line; polygon rings too (burn_geometry.rs:88-100, 226-238)
      // a polygon's ring walk carries the polygon's flags: it shares the
      // polygon's PixelCache (sum / count only), not the non-square-pixel
      // cache of LineString::burn
      const bool ok = all_touched_walk(x0, y0, x1, y1, pl.nrows, pl.ncols, [&](int yy, int xx) {
        if (yy >= pl.rlo && yy < pl.rhi) run_add(run, sb, bucket_count, ctrl, pl, p, yy, xx);
      });
      run_flush(run, sb, bucket_count, ctrl, pl, p);
      if (!ok) set_error(ctrl, ERR_LINE_LONG, v);
      continue;
    }
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
    while (ix0 != ix1 || iy0 != iy1) {
      if (ix0 >= 0 && ix0 < pl.ncols && iy0 >= pl.rlo && iy0 < pl.rhi)
        run_add(run, sb, bucket_count, ctrl, pl, p, (int)iy0, (int)ix0);
      const long long e2 = 2 * err;
      if (e2 >= dy) { err += dy; ix0 += sx; }
      if (e2 <= dx) { err += dx; iy0 += sy; }
    }
    run_flush(run, sb, bucket_count, ctrl, pl, p);
  }
  unsigned long long npix = run.npix;
  for (int o = 16; o > 0; o >>= 1) npix += __shfl_xor_sync(0xFFFFFFFFu, npix, o);
  if ((threadIdx.x & 31) == 0 && npix) atomicAdd(&ctrl->pixel_writes, npix);
}

// burners.rs:87-89: after the last kept segment of the part, its end pixel
// is written unless that segment's linestring is closed.
__global__ void k_line_endpix(Geo geo, Grid g, const PartPlan* __restrict__ plan,
                              const unsigned long long* __restrict__ poff, const unsigned* __restrict__ line_parts,
                              const unsigned long long* __restrict__ last_kept, RecBuf sb,
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
    if (geo.ring_closed) {
      if (geo.ring_closed[r]) continue;
    } else {
      const double2 first = geo.xy[geo.vertex_offsets[r]];
      const double2 last = geo.xy[geo.vertex_offsets[r + 1] - 1];
      if (first.x == last.x && first.y == last.y) continue;  // LineString::is_closed
    }
    const double2 w1 = geo.xy[v + 1];
    const long long ix = as_isize(floor(to_px(g, w1.x))), iy = as_isize(floor(to_py(g, w1.y)));
    const PartPlan pl = plan[p];
    if (ix >= 0 && ix < pl.ncols && iy >= pl.rlo && iy < pl.rhi) {
      ++npix;
      emit_run(sb, bucket_count, ctrl, pl, (int)iy, (int)ix, (int)ix + 1, p | pl.flags);
    }
  }
  if (npix) atomicAdd(&ctrl->pixel_writes, npix);
}

// ------------------------------------------------------------- points ------
// extract_point (edges.rs:79-88) + burn_point (burners.rs:250-258)
__global__ void k_point_spans(Geo geo, Grid g, const PartPlan* __restrict__ plan,
                              const unsigned long long* __restrict__ poff, const unsigned* __restrict__ point_parts,
                              RecBuf sb, unsigned* bucket_count, Ctrl* ctrl) {
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
    const PartPlan pl = plan[p];
    // extract_point keeps 0 <= y < nrows; the window keeps rows [rlo, rhi) of those
    if (x >= 0.0 && x < (double)pl.ncols && y >= (double)pl.rlo && y < (double)pl.rhi) {
      ++npix;
      emit_run(sb, bucket_count, ctrl, pl, (int)y, (int)x, (int)x + 1, p);
    }
  }
  for (int o = 16; o > 0; o >>= 1) npix += __shfl_xor_sync(0xFFFFFFFFu, npix, o);
  if ((threadIdx.x & 31) == 0 && npix) atomicAdd(&ctrl->pixel_writes, npix);
}

// ------------------------------------------------------------- scatter -----
// Move each coverage record into its bucket's range as {part | word-in-tile
// << REC_W_SHIFT | DEDUP_BIT, mask}.  Order inside a bucket is arbitrary
// here; the fill kernels restore part order (and look up each part's burn
// value).  Records of one bucket that sit in one warp (neighbouring words of
// a row) take their slots with one atomic.
__global__ void k_scatter(RecBuf sb, const unsigned* __restrict__ offsets, unsigned* counts, uint2* sorted,
                          Ctrl* ctrl) {
  if (ctrl->err || ctrl->span_count > sb.cap) return;
  const unsigned long long n = ctrl->span_count;
  const int lane = threadIdx.x & 31;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i0 = blockIdx.x * (unsigned long long)blockDim.x + (threadIdx.x & ~31u); i0 < n;
       i0 += stride) {
    const unsigned long long i = i0 + lane;
    const bool valid = i < n;
    const unsigned wid = valid ? sb.wid[i] : 0xFFFFFFFFu;
    const unsigned b = valid ? wid / WPT : 0xFFFFFFFFu;
    const unsigned same = __match_any_sync(0xFFFFFFFFu, b);
    const int leader = __ffs(same) - 1;
    unsigned left = 0;  // records of the bucket not placed yet, before this group
    if (valid && lane == leader) left = atomicSub(&counts[b], (unsigned)__popc(same));
    left = __shfl_sync(0xFFFFFFFFu, left, leader);
    if (valid) {
      const unsigned rank = (unsigned)__popc(same & ((1u << lane) - 1u));
      const unsigned pos = offsets[b + 1] - left + rank;  // arrival order
      sorted[pos] = make_uint2(sb.part[i] | ((wid % WPT) << REC_W_SHIFT), sb.mask[i]);
    }
  }
}

// The burn value of every part (VB bytes): values[part_geom[p]].
template <int VB>
__global__ void k_part_values(const unsigned* __restrict__ part_geom, const void* __restrict__ values,
                              unsigned long long n_parts, void* pvals, Ctrl* ctrl) {
  using V = typename std::conditional<VB == 1, unsigned char,
            typename std::conditional<VB == 2, unsigned short,
            typename std::conditional<VB == 4, unsigned, unsigned long long>::type>::type>::type;
  if (ctrl->err) return;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long p = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; p < n_parts; p += stride)
    static_cast<V*>(pvals)[p] = static_cast<const V*>(values)[part_geom[p]];
}

}  // namespace rzd
