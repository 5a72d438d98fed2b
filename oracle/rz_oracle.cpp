// rz_oracle.cpp -- CPU restatement of rusterize's burn path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU engine is
// checked against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline legs may load it; the product (rusterize_gb300/) never does.
//
// It restates, function by function, the Rust crate `rusterize` (rust/src/)
// as published in ttrotto/rusterize.  The reference cannot be compiled here
// (no cargo/rustc), so parity is pinned instead against the reference's own
// golden rasters (python/test/data/*.tif) and known-answer tests
// (R/rusterize/tests/testthat/*.R, rust/src/rasterization/burn_geometry.rs
// tests); see tests/test_oracle_golden.py.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fPIC -shared (no fast-math):
// every f64 expression below must round exactly like the Rust code, so no
// FMA contraction is allowed.
//
// Geometry input is the flat "parts" layout shared with the engine:
//   part_offsets[G+1]   geometry g owns parts [part_offsets[g], part_offsets[g+1])
//   part_kind[P]        0 = point set, 1 = line set, 2 = polygon (pooled rings)
//   ring_offsets[P+1]   part p owns rings [ring_offsets[p], ring_offsets[p+1])
//   vertex_offsets[R+1] ring r owns vertices [vertex_offsets[r], vertex_offsets[r+1])
//   ring_flags[R]       bit0 = hole (only used to infer the extent)
//   xy[2V]              world x,y interleaved, f64
// A GeometryCollection is the concatenation of its members' parts, which is
// exactly how `Burn for GeometryCollection` recurses (burn_geometry.rs:64-74).

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <limits>
#include <vector>

namespace {

enum PartKind : uint8_t { KIND_POINT = 0, KIND_LINE = 1, KIND_POLYGON = 2 };
enum PixelFn : int { FN_SUM = 0, FN_FIRST, FN_LAST, FN_MIN, FN_MAX, FN_COUNT, FN_ANY };
enum Dtype : int {
  DT_U8 = 0, DT_U16, DT_U32, DT_U64, DT_I8, DT_I16, DT_I32, DT_I64, DT_F32, DT_F64
};

// rust/src/geo/raster.rs:8-20
struct RasterInfo {
  uint64_t ncols, nrows;
  double xmin, xmax, ymin, ymax, xres, yres;
};

struct Geoms {
  uint64_t n_geoms;
  const uint64_t* part_offsets;
  const uint8_t* part_kind;
  const uint64_t* ring_offsets;
  const uint64_t* vertex_offsets;
  const uint8_t* ring_flags;
  const double* xy;
};

// Rust `f64 as usize`: saturating, NaN -> 0.
inline uint64_t as_usize(double v) {
  if (!(v > 0.0)) return 0;
  if (v >= 18446744073709551616.0) return UINT64_MAX;
  return (uint64_t)v;
}
// Rust `f64 as isize`: saturating, NaN -> 0.
inline int64_t as_isize(double v) {
  if (v != v) return 0;
  if (v <= -9223372036854775808.0) return INT64_MIN;
  if (v >= 9223372036854775808.0) return INT64_MAX;
  return (int64_t)v;
}
// Rust `f64::clamp` (NaN stays NaN).
inline double clampf(double v, double lo, double hi) {
  if (v < lo) return lo;
  if (v > hi) return hi;
  return v;
}
// Rust `f64::total_cmp` key.
inline int64_t total_key(double v) {
  int64_t b;
  std::memcpy(&b, &v, 8);
  return b ^ (int64_t)(((uint64_t)(b >> 63)) >> 1);
}
// Rust `f64::min` / `f64::max` (NaN-ignoring).
inline double fmin_rs(double a, double b) { return (a != a) ? b : ((b != b) ? a : (a < b ? a : b)); }
inline double fmax_rs(double a, double b) { return (a != a) ? b : ((b != b) ? a : (a > b ? a : b)); }

// ---------------------------------------------------------------- edges ----
// rust/src/geo/edges.rs:5-14
struct PointEdge { uint64_t x, y; };

// rust/src/geo/edges.rs:17-56
struct PolyEdge {
  uint64_t ystart, yend;
  double x0, y0, dxdy, x_at_yline;
};

PolyEdge make_poly_edge(double x0, double y0, double x1, double y1) {
  double xt, yt, xb, yb;
  if (y0 < y1) { xt = x0; yt = y0; xb = x1; yb = y1; }
  else         { xt = x1; yt = y1; xb = x0; yb = y0; }
  PolyEdge e;
  e.ystart = as_usize(std::ceil(yt - 0.5));
  e.yend = as_usize(std::ceil(yb - 0.5));
  e.dxdy = (xb - xt) / (yb - yt);
  e.x0 = xt;
  e.y0 = yt;
  e.x_at_yline = std::numeric_limits<double>::infinity();
  return e;
}

inline double intersect_at(const PolyEdge& e, uint64_t yline) {
  double center_y = (double)yline + 0.5;
  return e.x0 + (center_y - e.y0) * e.dxdy;
}

// rust/src/geo/edges.rs:59-77
struct LineEdge { double x0, y0, x1, y1; bool is_closed; };

// rust/src/geo/edges.rs:79-88
void extract_point(std::vector<PointEdge>& edges, double px, double py, const RasterInfo& ri) {
  double x = (px - ri.xmin) / ri.xres;
  double y = (ri.ymax - py) / ri.yres;
  if (x >= 0.0 && x < (double)ri.ncols && y >= 0.0 && y < (double)ri.nrows)
    edges.push_back({as_usize(x), as_usize(y)});
}

// rust/src/geo/edges.rs:90-110
void extract_ring(std::vector<PolyEdge>& edges, const double* xy, uint64_t n, const RasterInfo& ri) {
  double rows = (double)ri.nrows;
  for (uint64_t i = 0; i + 1 < n; ++i) {
    double x0 = (xy[2 * i] - ri.xmin) / ri.xres;
    double y0 = (ri.ymax - xy[2 * i + 1]) / ri.yres;
    double x1 = (xy[2 * i + 2] - ri.xmin) / ri.xres;
    double y1 = (ri.ymax - xy[2 * i + 3]) / ri.yres;
    if (std::fabs(y0 - y1) >= DBL_EPSILON) {
      double min_y = fmin_rs(y0, y1);
      double max_y = fmax_rs(y0, y1);
      if (min_y < rows && max_y >= 0.0) edges.push_back(make_poly_edge(x0, y0, x1, y1));
    }
  }
}

// geo-types LineString::is_closed: first coord == last coord (empty => true)
bool ring_is_closed(const double* xy, uint64_t n) {
  if (n == 0) return true;
  return xy[0] == xy[2 * (n - 1)] && xy[1] == xy[2 * (n - 1) + 1];
}

// rust/src/geo/edges.rs:112-134
void extract_line(std::vector<LineEdge>& edges, const double* xy, uint64_t n, const RasterInfo& ri) {
  double rows = (double)ri.nrows;
  double cols = (double)ri.ncols;
  bool is_closed = ring_is_closed(xy, n);
  for (uint64_t i = 0; i + 1 < n; ++i) {
    double x0 = (xy[2 * i] - ri.xmin) / ri.xres;
    double y0 = (ri.ymax - xy[2 * i + 1]) / ri.yres;
    double x1 = (xy[2 * i + 2] - ri.xmin) / ri.xres;
    double y1 = (ri.ymax - xy[2 * i + 3]) / ri.yres;
    double min_x = fmin_rs(x0, x1), max_x = fmax_rs(x0, x1);
    double min_y = fmin_rs(y0, y1), max_y = fmax_rs(y0, y1);
    if (min_x < cols && max_x >= 0.0 && min_y < rows && max_y >= 0.0)
      edges.push_back({x0, y0, x1, y1, is_closed});
  }
}

// ---------------------------------------------------------- pixel cache ----
// rust/src/rasterization/pixel_cache.rs:7-58
struct PixelCache {
  std::vector<uint8_t> bits;
  uint64_t width;
  int64_t xmin, ymin;

  explicit PixelCache(const std::vector<LineEdge>& le) {
    double xmn = DBL_MAX, ymn = DBL_MAX, xmx = -DBL_MAX, ymx = -DBL_MAX;
    for (const auto& e : le) {
      xmn = fmin_rs(fmin_rs(xmn, e.x0), e.x1);
      ymn = fmin_rs(fmin_rs(ymn, e.y0), e.y1);
      xmx = fmax_rs(fmax_rs(xmx, e.x0), e.x1);
      ymx = fmax_rs(fmax_rs(ymx, e.y0), e.y1);
    }
    width = as_usize(std::floor(xmx) - std::floor(xmn)) + 1;
    uint64_t length = as_usize(std::floor(ymx) - std::floor(ymn)) + 1;
    bits.assign(width * length, 0);
    xmin = as_isize(xmn);
    ymin = as_isize(ymn);
  }
  uint64_t idx(uint64_t x, uint64_t y) const {
    uint64_t lx = (uint64_t)((int64_t)x - xmin);
    uint64_t ly = (uint64_t)((int64_t)y - ymin);
    return ly * width + lx;
  }
  bool insert(uint64_t x, uint64_t y) {
    uint64_t i = idx(x, y);
    if (bits.at(i)) return false;  // .at(): fixedbitset panics out of range too
    bits[i] = 1;
    return true;
  }
  bool contains(uint64_t x, uint64_t y) const {
    uint64_t i = idx(x, y);
    return i < bits.size() && bits[i];
  }
};

// -------------------------------------------------------- pixel functions ----
// rust/src/rasterization/pixel_functions.rs:56-122.  Integer `+=` wraps, as
// in a release build of the crate.
template <typename T> inline bool is_nan(T v) { return v != v; }

template <typename T> inline T wrap_add(T a, T b) {
  if constexpr (std::is_integral<T>::value) {
    using U = typename std::make_unsigned<T>::type;
    return (T)(U)((U)a + (U)b);
  } else {
    return a + b;
  }
}

template <typename T>
inline void apply_fn(int fn, T& cur, T value, T bg) {
  switch (fn) {
    case FN_SUM:
      if (cur == bg || is_nan(cur) || is_nan(value)) cur = value; else cur = wrap_add(cur, value);
      break;
    case FN_FIRST:
      if (cur == bg || is_nan(cur)) cur = value;
      break;
    case FN_LAST:
      cur = value;
      break;
    case FN_MIN:
      if (cur == bg || is_nan(cur) || cur > value) cur = value;
      break;
    case FN_MAX:
      if (cur == bg || is_nan(cur) || cur < value) cur = value;
      break;
    case FN_COUNT:
      if (cur == bg || is_nan(cur)) cur = (T)1; else cur = wrap_add(cur, (T)1);
      break;
    case FN_ANY:
      cur = (T)1;
      break;
  }
}

// ------------------------------------------------------------- writers ----
// rust/src/encoding/writers.rs:10-78.  A writer is the dense band plus an
// optional dedup cache in "line" (insert) or "fill" (skip-if-present) mode.
template <typename T>
struct Writer {
  T* band;
  uint64_t ncols;
  int fn;
  T bg;
  PixelCache* cache = nullptr;
  int mode = 0;  // 0 direct, 1 LineWriter, 2 FillWriter
  uint64_t* nwrites = nullptr;
  // SparseArrayWriter (writers.rs:86-131): record the triplet instead
  std::vector<uint64_t>* srows = nullptr;
  std::vector<uint64_t>* scols = nullptr;
  std::vector<T>* svals = nullptr;

  void write(uint64_t y, uint64_t x, T value) {
    if (mode == 1) { if (!cache->insert(x, y)) return; }
    else if (mode == 2) { if (cache->contains(x, y)) return; }
    if (nwrites) ++*nwrites;
    if (srows) {
      srows->push_back(y);
      scols->push_back(x);
      svals->push_back(value);
      return;
    }
    apply_fn(fn, band[y * ncols + x], value, bg);
  }
};

// ------------------------------------------------------------- burners ----
// rust/src/rasterization/burners.rs:40-91  (Standard)
template <typename T>
void burn_line_standard(const std::vector<LineEdge>& le, const RasterInfo& ri, T value, Writer<T>& w) {
  if (le.empty()) return;
  int64_t nrows = (int64_t)ri.nrows, ncols = (int64_t)ri.ncols;
  size_t last_idx = le.size() - 1;
  for (size_t idx = 0; idx < le.size(); ++idx) {
    const LineEdge& e = le[idx];
    int64_t ix0 = as_isize(std::floor(e.x0));
    int64_t ix1 = as_isize(std::floor(e.x1));
    int64_t iy0 = as_isize(std::floor(e.y0));
    int64_t iy1 = as_isize(std::floor(e.y1));
    int64_t dx = std::llabs(ix1 - ix0);
    int64_t dy = -std::llabs(iy1 - iy0);
    int64_t sx = ix0 < ix1 ? 1 : -1;
    int64_t sy = iy0 < iy1 ? 1 : -1;
    int64_t err = dx + dy;
    while (ix0 != ix1 || iy0 != iy1) {
      if (ix0 >= 0 && ix0 < ncols && iy0 >= 0 && iy0 < nrows) w.write((uint64_t)iy0, (uint64_t)ix0, value);
      int64_t e2 = 2 * err;
      if (e2 >= dy) { err += dy; ix0 += sx; }
      if (e2 <= dx) { err += dx; iy0 += sy; }
    }
    if (idx == last_idx && !e.is_closed && ix0 >= 0 && ix0 < ncols && iy0 >= 0 && iy0 < nrows)
      w.write((uint64_t)iy0, (uint64_t)ix0, value);
  }
}

// rust/src/rasterization/burners.rs:99-246  (AllTouched, GDAL-derived)
template <typename T>
void burn_line_all_touched(const std::vector<LineEdge>& le, const RasterInfo& ri, T value, Writer<T>& w) {
  const double EPSILON_INTERSECT = 1e-4;
  const double TOLERANCE = 1e-9;
  if (le.empty()) return;
  int64_t nrows = (int64_t)ri.nrows, ncols = (int64_t)ri.ncols;
  double nrows_f = (double)ri.nrows, ncols_f = (double)ri.ncols;
  for (const LineEdge& e : le) {
    double df_x = e.x0, df_y = e.y0, df_x_end = e.x1, df_y_end = e.y1;
    if (df_x > df_x_end) { std::swap(df_x, df_x_end); std::swap(df_y, df_y_end); }
    // vertical
    if (std::fabs(df_x - df_x_end) < 0.01) {
      if (df_y_end < df_y) std::swap(df_y, df_y_end);
      int64_t ix = as_isize(std::floor(df_x_end));
      int64_t iy = as_isize(std::floor(df_y));
      int64_t iy_end = as_isize(std::floor(df_y_end - EPSILON_INTERSECT));
      if (ix < 0 || ix >= ncols) continue;
      iy = std::max<int64_t>(iy, 0);
      iy_end = std::min<int64_t>(iy_end, nrows - 1);
      for (int64_t y = iy; y <= iy_end; ++y) w.write((uint64_t)y, (uint64_t)ix, value);
      continue;
    }
    // horizontal
    if (std::fabs(df_y - df_y_end) < 0.01) {
      if (df_x_end < df_x) std::swap(df_x, df_x_end);
      int64_t ix = as_isize(std::floor(df_x));
      int64_t iy = as_isize(std::floor(df_y));
      int64_t ix_end = as_isize(std::floor(df_x_end - EPSILON_INTERSECT));
      if (iy < 0 || iy >= nrows) continue;
      ix = std::max<int64_t>(ix, 0);
      ix_end = std::min<int64_t>(ix_end, ncols - 1);
      for (int64_t x = ix; x <= ix_end; ++x) w.write((uint64_t)iy, (uint64_t)x, value);
      continue;
    }
    // sloped
    double slope = (df_y_end - df_y) / (df_x_end - df_x);
    double inv_slope = 1.0 / slope;
    if (df_x < 0.0) { df_y += (0.0 - df_x) * slope; df_x = 0.0; }
    if (df_x_end > ncols_f) { df_y_end += (ncols_f - df_x_end) * slope; df_x_end = ncols_f; }
    if (df_y < 0.0) { df_x += (0.0 - df_y) * inv_slope; df_y = 0.0; }
    else if (df_y > nrows_f) { df_x += (nrows_f - df_y) * inv_slope; df_y = nrows_f; }
    if (df_y_end < 0.0) { df_x_end += (0.0 - df_y_end) * inv_slope; }
    else if (df_y_end > nrows_f) { df_x_end += (nrows_f - df_y_end) * inv_slope; }
    df_x = clampf(df_x, 0.0, ncols_f);
    df_x_end = clampf(df_x_end, 0.0, ncols_f);
    while (df_x >= 0.0 && df_x < df_x_end) {
      int64_t ix = as_isize(std::floor(df_x));
      int64_t iy = as_isize(std::floor(df_y));
      if (ix >= 0 && ix < ncols && iy >= 0 && iy < nrows) w.write((uint64_t)iy, (uint64_t)ix, value);
      double sx = std::floor(df_x + 1.0) - df_x;
      double sy = sx * slope;
      if (as_isize(std::floor(df_y + sy)) == iy) {
        df_x += sx; df_y += sy;
      } else if (slope < 0.0) {
        sy = (double)iy - df_y;
        if (sy > -TOLERANCE) sy = -TOLERANCE;
        sx = sy / slope;
        df_x += sx; df_y += sy;
      } else {
        sy = (double)(iy + 1) - df_y;
        if (sy < TOLERANCE) sy = TOLERANCE;
        sx = sy / slope;
        df_x += sx; df_y += sy;
      }
    }
  }
}

// rust/src/rasterization/burners.rs:250-258
template <typename T>
void burn_point(const std::vector<PointEdge>& pe, T value, Writer<T>& w) {
  for (const auto& p : pe) w.write(p.y, p.x, value);
}

// rust/src/rasterization/burners.rs:261-320
template <typename T>
void burn_polygon(std::vector<PolyEdge>& polyedges, const RasterInfo& ri, T value, Writer<T>& w) {
  if (polyedges.empty()) return;
  std::sort(polyedges.begin(), polyedges.end(),
            [](const PolyEdge& a, const PolyEdge& b) { return a.ystart < b.ystart; });
  uint64_t yline = polyedges[0].ystart;
  std::vector<PolyEdge> active;
  size_t head = 0;  // polyedges[head..] not yet transferred
  double ncols = (double)ri.ncols;
  while (yline < ri.nrows && (!active.empty() || head < polyedges.size())) {
    while (head < polyedges.size() && polyedges[head].ystart <= yline) active.push_back(polyedges[head++]);
    active.erase(std::remove_if(active.begin(), active.end(),
                                [yline](const PolyEdge& e) { return !(e.yend > yline); }),
                 active.end());
    if (active.empty()) { ++yline; continue; }
    for (auto& e : active) e.x_at_yline = intersect_at(e, yline);
    std::sort(active.begin(), active.end(), [](const PolyEdge& a, const PolyEdge& b) {
      return total_key(a.x_at_yline) < total_key(b.x_at_yline);
    });
    for (size_t k = 0; k + 1 < active.size(); k += 2) {
      double x1 = active[k].x_at_yline;
      double x2 = active[k + 1].x_at_yline;
      uint64_t xstart = as_usize(clampf(std::floor(x1 + 0.5), 0.0, ncols));
      uint64_t xend = as_usize(clampf(std::floor(x2 + 0.5), 0.0, ncols));
      for (uint64_t xpix = xstart; xpix < xend; ++xpix) w.write(yline, xpix, value);
    }
    ++yline;
  }
}

// ------------------------------------------------------- burn dispatch ----
// rust/src/rasterization/burn_geometry.rs:24-243, one "part" at a time.
template <typename T>
void burn_part(const Geoms& g, uint64_t p, const RasterInfo& ri, T value, Writer<T> w,
               bool all_touched, bool dedup, uint64_t* nedges) {
  uint8_t kind = g.part_kind[p];
  uint64_t r0 = g.ring_offsets[p], r1 = g.ring_offsets[p + 1];
  auto ring_ptr = [&](uint64_t r) { return g.xy + 2 * g.vertex_offsets[r]; };
  auto ring_len = [&](uint64_t r) { return g.vertex_offsets[r + 1] - g.vertex_offsets[r]; };

  if (kind == KIND_POINT) {
    std::vector<PointEdge> pe;
    for (uint64_t r = r0; r < r1; ++r) {
      const double* v = ring_ptr(r);
      for (uint64_t i = 0; i < ring_len(r); ++i) extract_point(pe, v[2 * i], v[2 * i + 1], ri);
    }
    if (nedges) *nedges += pe.size();
    burn_point(pe, value, w);
  } else if (kind == KIND_LINE) {
    std::vector<LineEdge> le;
    for (uint64_t r = r0; r < r1; ++r) extract_line(le, ring_ptr(r), ring_len(r), ri);
    if (nedges) *nedges += le.size();
    auto burn = [&](Writer<T>& ww) {
      if (all_touched) burn_line_all_touched(le, ri, value, ww);
      else burn_line_standard(le, ri, value, ww);
    };
    // burn_geometry.rs:179-185
    if (ri.xres != ri.yres || dedup) {
      PixelCache cache(le);
      Writer<T> lw = w;
      lw.cache = &cache;
      lw.mode = 1;
      burn(lw);
    } else {
      burn(w);
    }
  } else {
    std::vector<PolyEdge> pe;
    for (uint64_t r = r0; r < r1; ++r) extract_ring(pe, ring_ptr(r), ring_len(r), ri);
    if (nedges) *nedges += pe.size();
    if (!all_touched) {
      burn_polygon(pe, ri, value, w);
      return;
    }
    std::vector<LineEdge> le;
    for (uint64_t r = r0; r < r1; ++r) extract_line(le, ring_ptr(r), ring_len(r), ri);
    if (dedup) {  // handle_polygon, burn_geometry.rs:226-234
      PixelCache cache(le);
      Writer<T> lw = w;
      lw.cache = &cache;
      lw.mode = 1;
      burn_line_all_touched(le, ri, value, lw);
      Writer<T> fw = w;
      fw.cache = &cache;
      fw.mode = 2;
      burn_polygon(pe, ri, value, fw);
    } else {
      burn_line_all_touched(le, ri, value, w);
      burn_polygon(pe, ri, value, w);
    }
  }
}

template <typename T>
int rasterize_t(const Geoms& g, const T* values, const uint32_t* band_of_geom, uint32_t n_bands,
                const RasterInfo& ri, int fn, T bg, bool all_touched, T* out,
                uint64_t* nwrites, uint64_t* nedges) {
  uint64_t band_px = ri.nrows * ri.ncols;
  uint64_t nb = band_of_geom ? n_bands : 1;
  for (uint64_t i = 0; i < nb * band_px; ++i) out[i] = bg;  // raster.rs:23-28
  bool dedup = all_touched && (fn == FN_SUM || fn == FN_COUNT);  // prelude.rs:116-118
  // rasterize.rs:162-196: geometries in index order, each band independently
  for (uint64_t i = 0; i < g.n_geoms; ++i) {
    uint64_t b = band_of_geom ? band_of_geom[i] : 0;
    if (b >= nb) return -1;
    Writer<T> w;
    w.band = out + b * band_px;
    w.ncols = ri.ncols;
    w.fn = fn;
    w.bg = bg;
    w.nwrites = nwrites;
    T v = values ? values[i] : (T)1;
    for (uint64_t p = g.part_offsets[i]; p < g.part_offsets[i + 1]; ++p)
      burn_part<T>(g, p, ri, v, w, all_touched, dedup, nedges);
  }
  return 0;
}

// SparseArray::build (rasterize.rs:118-152): per band (in band order) the
// triplets of its geometries in index order; bands concatenated.
template <typename T>
int rasterize_sparse_t(const Geoms& g, const T* values, const uint32_t* band_of_geom, uint32_t n_bands,
                       const RasterInfo& ri, int fn, bool all_touched, std::vector<uint64_t>& rows,
                       std::vector<uint64_t>& cols, std::vector<T>& vals, uint64_t* band_counts) {
  uint64_t nb = band_of_geom ? n_bands : 1;
  bool dedup = all_touched && (fn == FN_SUM || fn == FN_COUNT);
  std::vector<std::vector<uint64_t>> br(nb), bc(nb);
  std::vector<std::vector<T>> bv(nb);
  for (uint64_t i = 0; i < g.n_geoms; ++i) {
    uint64_t b = band_of_geom ? band_of_geom[i] : 0;
    if (b >= nb) return -1;
    Writer<T> w;
    w.band = nullptr;
    w.ncols = ri.ncols;
    w.fn = fn;
    w.bg = (T)0;
    w.srows = &br[b];
    w.scols = &bc[b];
    w.svals = &bv[b];
    T v = values ? values[i] : (T)1;
    for (uint64_t p = g.part_offsets[i]; p < g.part_offsets[i + 1]; ++p)
      burn_part<T>(g, p, ri, v, w, all_touched, dedup, nullptr);
  }
  for (uint64_t b = 0; b < nb; ++b) {
    band_counts[b] = br[b].size();
    rows.insert(rows.end(), br[b].begin(), br[b].end());
    cols.insert(cols.end(), bc[b].begin(), bc[b].end());
    vals.insert(vals.end(), bv[b].begin(), bv[b].end());
  }
  return 0;
}

// --------------------------------------------------------- raster info ----
// geo BoundingRect as used by RasterInfoBuilder::build_with (raster.rs:75-86):
// points/lines use every coordinate, polygons only exterior rings.
struct BBox { bool some = false; double xmin, ymin, xmax, ymax; };

void bbox_add_point(BBox& b, double x, double y) {
  // geo get_bounding_rect / get_min_max
  if (!b.some) { b.some = true; b.xmin = b.xmax = x; b.ymin = b.ymax = y; return; }
  if (x > b.xmax) b.xmax = x; else if (x < b.xmin) b.xmin = x;
  if (y > b.ymax) b.ymax = y; else if (y < b.ymin) b.ymin = y;
}

// SparseArray::build_array (rust/src/encoding/arrays.rs:103-141): the raster
// starts at the background, and each band's triplets, in order, apply the
// pixel function to their pixel.  -3 for a triplet outside the raster, where
// the reference's array indexing panics.
template <typename T>
int sparse_build_t(const uint64_t* band_counts, uint32_t n_bands, const uint64_t* rows, const uint64_t* cols,
                   const T* vals, uint64_t nrows, uint64_t ncols, int fn, T bg, T* out) {
  const uint64_t plane = nrows * ncols;
  std::fill(out, out + (uint64_t)n_bands * plane, bg);
  uint64_t off = 0;
  for (uint32_t b = 0; b < n_bands; ++b) {
    T* band = out + (uint64_t)b * plane;
    for (uint64_t i = off; i < off + band_counts[b]; ++i) {
      if (rows[i] >= nrows || cols[i] >= ncols) return -3;
      apply_fn(fn, band[rows[i] * ncols + cols[i]], vals[i], bg);
    }
    off += band_counts[b];
  }
  return 0;
}

}  // namespace

extern "C" {

// Burn `n_geoms` geometries; out is (bands, nrows, ncols) C-order of `dtype`.
// raster = {xmin, xmax, ymin, ymax, xres, yres}.  Returns 0 or -1 (bad band).
int rzo_rasterize(uint64_t n_geoms, const uint64_t* part_offsets, const uint8_t* part_kind,
                  const uint64_t* ring_offsets, const uint64_t* vertex_offsets, const double* xy,
                  const void* values, int dtype, const uint32_t* band_of_geom, uint32_t n_bands,
                  const double* raster, uint64_t nrows, uint64_t ncols, int pixel_fn,
                  const void* bg, int all_touched, void* out, uint64_t* nwrites, uint64_t* nedges) {
  Geoms g{n_geoms, part_offsets, part_kind, ring_offsets, vertex_offsets, nullptr, xy};
  RasterInfo ri{ncols, nrows, raster[0], raster[1], raster[2], raster[3], raster[4], raster[5]};
  bool at = all_touched != 0;
#define RZO_CASE(CODE, T)                                                                   \
  case CODE:                                                                                \
    return rasterize_t<T>(g, (const T*)values, band_of_geom, n_bands, ri, pixel_fn,         \
                          *(const T*)bg, at, (T*)out, nwrites, nedges);
  switch (dtype) {
    RZO_CASE(DT_U8, uint8_t)
    RZO_CASE(DT_U16, uint16_t)
    RZO_CASE(DT_U32, uint32_t)
    RZO_CASE(DT_U64, uint64_t)
    RZO_CASE(DT_I8, int8_t)
    RZO_CASE(DT_I16, int16_t)
    RZO_CASE(DT_I32, int32_t)
    RZO_CASE(DT_I64, int64_t)
    RZO_CASE(DT_F32, float)
    RZO_CASE(DT_F64, double)
    default: return -2;
  }
#undef RZO_CASE
}

// Sparse (COO) burn: triplets in the reference's write order, in buffers
// allocated with malloc (free them with rzo_free).  band_counts has n_bands
// entries (1 without bands).
int rzo_rasterize_sparse(uint64_t n_geoms, const uint64_t* part_offsets, const uint8_t* part_kind,
                         const uint64_t* ring_offsets, const uint64_t* vertex_offsets, const double* xy,
                         const void* values, int dtype, const uint32_t* band_of_geom, uint32_t n_bands,
                         const double* raster, uint64_t nrows, uint64_t ncols, int pixel_fn, int all_touched,
                         uint64_t* count, uint64_t** rows_out, uint64_t** cols_out, void** vals_out,
                         uint64_t* band_counts) {
  Geoms g{n_geoms, part_offsets, part_kind, ring_offsets, vertex_offsets, nullptr, xy};
  RasterInfo ri{ncols, nrows, raster[0], raster[1], raster[2], raster[3], raster[4], raster[5]};
  bool at = all_touched != 0;
  std::vector<uint64_t> rows, cols;
  int st = -2;
  size_t tsize = 0;
  void* vbuf = nullptr;
#define RZO_SCASE(CODE, T)                                                                                 \
  case CODE: {                                                                                             \
    std::vector<T> vals;                                                                                   \
    st = rasterize_sparse_t<T>(g, (const T*)values, band_of_geom, n_bands, ri, pixel_fn, at, rows, cols,  \
                               vals, band_counts);                                                         \
    tsize = sizeof(T);                                                                                     \
    vbuf = std::malloc(vals.size() * tsize + 1);                                                           \
    if (vbuf && !vals.empty()) std::memcpy(vbuf, vals.data(), vals.size() * tsize);                       \
    break;                                                                                                 \
  }
  switch (dtype) {
    RZO_SCASE(DT_U8, uint8_t)
    RZO_SCASE(DT_U16, uint16_t)
    RZO_SCASE(DT_U32, uint32_t)
    RZO_SCASE(DT_U64, uint64_t)
    RZO_SCASE(DT_I8, int8_t)
    RZO_SCASE(DT_I16, int16_t)
    RZO_SCASE(DT_I32, int32_t)
    RZO_SCASE(DT_I64, int64_t)
    RZO_SCASE(DT_F32, float)
    RZO_SCASE(DT_F64, double)
    default: return -2;
  }
#undef RZO_SCASE
  if (st != 0) {
    std::free(vbuf);
    return st;
  }
  *count = rows.size();
  *rows_out = (uint64_t*)std::malloc(rows.size() * 8 + 8);
  *cols_out = (uint64_t*)std::malloc(cols.size() * 8 + 8);
  if (!rows.empty()) {
    std::memcpy(*rows_out, rows.data(), rows.size() * 8);
    std::memcpy(*cols_out, cols.data(), cols.size() * 8);
  }
  *vals_out = vbuf;
  return 0;
}

void rzo_free(void* p) { std::free(p); }

// Restatement of RasterInfoBuilder (rust/src/geo/raster.rs:50-156) as driven
// by RawRasterInfo::build (python/src/geo/raster.rs:17-41).
// flags bit0 has_shape, bit1 has_res, bit2 has_extent, bit3 tap.
// out_info = {xmin, xmax, ymin, ymax, xres, yres}; out_shape = {nrows, ncols}.
// Returns 0, or an error code: 1 unspecified extent, 2 no bbox, 3 neither
// shape nor res, 4 both, 5 shape <= 0, 6 res <= 0.
int rzo_raster_info(uint64_t n_geoms, const uint64_t* part_offsets, const uint8_t* part_kind,
                    const uint64_t* ring_offsets, const uint64_t* vertex_offsets,
                    const uint8_t* ring_flags, const double* xy, uint32_t flags,
                    const uint64_t* shape, const double* res, const double* extent,
                    double* out_info, uint64_t* out_shape) {
  bool has_shape = flags & 1, has_res = flags & 2, has_extent = flags & 4, tap = flags & 8;
  double xmin, ymin, xmax, ymax;
  bool inferred;
  if (has_extent) {
    if (extent[0] == 0.0 && extent[1] == 0.0 && extent[2] == 0.0 && extent[3] == 0.0) {
      // total_cmp(&0.0) == Equal only for +0.0
      bool all_pos_zero = true;
      for (int i = 0; i < 4; ++i) all_pos_zero &= !std::signbit(extent[i]);
      if (all_pos_zero) return 1;
    }
    xmin = extent[0]; ymin = extent[1]; xmax = extent[2]; ymax = extent[3];
    inferred = false;
  } else {
    BBox acc;
    for (uint64_t gi = 0; gi < n_geoms; ++gi) {
      BBox gb;  // per-geometry rect, folded member by member
      for (uint64_t p = part_offsets[gi]; p < part_offsets[gi + 1]; ++p) {
        BBox pb;
        for (uint64_t r = ring_offsets[p]; r < ring_offsets[p + 1]; ++r) {
          if (part_kind[p] == KIND_POLYGON && ring_flags && (ring_flags[r] & 1)) continue;
          for (uint64_t v = vertex_offsets[r]; v < vertex_offsets[r + 1]; ++v)
            bbox_add_point(pb, xy[2 * v], xy[2 * v + 1]);
        }
        if (!pb.some) continue;
        if (!gb.some) gb = pb;
        else {
          gb.xmin = fmin_rs(gb.xmin, pb.xmin); gb.ymin = fmin_rs(gb.ymin, pb.ymin);
          gb.xmax = fmax_rs(gb.xmax, pb.xmax); gb.ymax = fmax_rs(gb.ymax, pb.ymax);
        }
      }
      if (!gb.some) continue;
      if (!acc.some) acc = gb;
      else {
        acc.xmin = fmin_rs(acc.xmin, gb.xmin); acc.ymin = fmin_rs(acc.ymin, gb.ymin);
        acc.xmax = fmax_rs(acc.xmax, gb.xmax); acc.ymax = fmax_rs(acc.ymax, gb.ymax);
      }
    }
    if (!acc.some) return 2;
    xmin = acc.xmin; ymin = acc.ymin; xmax = acc.xmax; ymax = acc.ymax;
    inferred = true;
  }
  if (!has_shape && !has_res) return 3;
  if (has_shape && has_res) return 4;
  uint64_t nrows = has_shape ? shape[0] : 0, ncols = has_shape ? shape[1] : 0;
  double xres = has_res ? res[0] : 0.0, yres = has_res ? res[1] : 0.0;
  if (has_shape && (nrows == 0 || ncols == 0)) return 5;
  if (has_res && (xres <= 0.0 || yres <= 0.0)) return 6;
  if (inferred && !tap && has_res) {
    xmin -= xres / 2.0; xmax += xres / 2.0;
    ymin -= yres / 2.0; ymax += yres / 2.0;
  }
  if (!has_res) {
    xres = (xmax - xmin) / (double)ncols;
    yres = (ymax - ymin) / (double)nrows;
  } else if (tap) {
    xmin = std::floor(xmin / xres) * xres;
    xmax = std::ceil(xmax / xres) * xres;
    ymin = std::floor(ymin / yres) * yres;
    ymax = std::ceil(ymax / yres) * yres;
  }
  if (!has_shape) {
    nrows = as_usize(0.5 + (ymax - ymin) / yres);
    ncols = as_usize(0.5 + (xmax - xmin) / xres);
  }
  out_info[0] = xmin; out_info[1] = xmax; out_info[2] = ymin; out_info[3] = ymax;
  out_info[4] = xres; out_info[5] = yres;
  out_shape[0] = nrows; out_shape[1] = ncols;
  return 0;
}

// Replay of a triplet stream onto a background raster (n_bands x nrows x
// ncols of `dtype`); bg points at one value of `dtype`.
int rzo_sparse_build(const uint64_t* band_counts, uint32_t n_bands, const uint64_t* rows, const uint64_t* cols,
                     const void* vals, int dtype, uint64_t nrows, uint64_t ncols, int pixel_fn, const void* bg,
                     void* out) {
#define RZO_BCASE(CODE, T)                                                                              \
  case CODE:                                                                                           \
    return sparse_build_t<T>(band_counts, n_bands, rows, cols, (const T*)vals, nrows, ncols, pixel_fn, \
                             *(const T*)bg, (T*)out);
  switch (dtype) {
    RZO_BCASE(DT_U8, uint8_t)
    RZO_BCASE(DT_U16, uint16_t)
    RZO_BCASE(DT_U32, uint32_t)
    RZO_BCASE(DT_U64, uint64_t)
    RZO_BCASE(DT_I8, int8_t)
    RZO_BCASE(DT_I16, int16_t)
    RZO_BCASE(DT_I32, int32_t)
    RZO_BCASE(DT_I64, int64_t)
    RZO_BCASE(DT_F32, float)
    RZO_BCASE(DT_F64, double)
    default: return -2;
  }
#undef RZO_BCASE
}

}  // extern "C"
