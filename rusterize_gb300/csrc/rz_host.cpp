// rz_host.cpp -- host side of the boundary: geometry readers (WKT/WKB ->
// parts table), the raster-grid builder and small enum helpers.  No CUDA here.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "rz_internal.h"

using rz::fail;
using rz::GeomTable;

extern "C" int rz_abi_version(void) { return RZ_ABI_VERSION; }

extern "C" size_t rz_dtype_size(rz_dtype dt) {
  switch (dt) {
    case RZ_U8: case RZ_I8: return 1;
    case RZ_U16: case RZ_I16: return 2;
    case RZ_U32: case RZ_I32: case RZ_F32: return 4;
    case RZ_U64: case RZ_I64: case RZ_F64: return 8;
  }
  return 0;
}

// PixelFunction::from_str, rust/src/rasterization/pixel_functions.rs:18-33.
extern "C" rz_status rz_pixel_fn_from_str(const char* name, rz_pixel_fn* out, char* err,
                                          size_t errlen) {
  rz::clear_err(err, errlen);
  static const char* names[] = {"sum", "first", "last", "min", "max", "count", "any"};
  if (name) {
    for (int i = 0; i < 7; ++i) {
      if (std::strcmp(name, names[i]) == 0) {
        *out = (rz_pixel_fn)i;
        return RZ_OK;
      }
    }
  }
  return fail(err, errlen, RZ_VALUE_ERROR, "Unknown pixel function");
}

// ------------------------------------------------------------------ WKT ----
// Grammar of OGC Simple Features WKT as read by the `wkt` crate (0.14) and
// converted to geo-types: dimension tags Z/M/ZM are accepted and the extra
// ordinates dropped; EMPTY is accepted for everything but POINT (geo-types
// has no empty Point: the reference panics there, we report a parse error).
namespace {

struct WktReader {
  const char* s;
  size_t n, i = 0;
  std::string msg;

  void ws() { while (i < n && std::isspace((unsigned char)s[i])) ++i; }
  bool eat(char c) {
    ws();
    if (i < n && s[i] == c) { ++i; return true; }
    return false;
  }
  bool word(std::string& w) {
    ws();
    size_t j = i;
    while (j < n && std::isalpha((unsigned char)s[j])) ++j;
    if (j == i) return false;
    w.assign(s + i, j - i);
    for (auto& c : w) c = (char)std::toupper((unsigned char)c);
    i = j;
    return true;
  }
  bool peek_word(const char* w) {
    ws();
    size_t len = std::strlen(w);
    if (i + len > n) return false;
    for (size_t k = 0; k < len; ++k)
      if (std::toupper((unsigned char)s[i + k]) != w[k]) return false;
    if (i + len < n && std::isalpha((unsigned char)s[i + len])) return false;
    return true;
  }
  bool number(double& v) {
    ws();
    if (i >= n) return false;
    // strtod needs a terminated buffer: copy the token
    size_t j = i;
    while (j < n && (std::isalnum((unsigned char)s[j]) || s[j] == '.' || s[j] == '-' || s[j] == '+')) ++j;
    if (j == i) return false;
    const size_t len = j - i;
    char stack[64];
    std::string heap;
    char* tok = stack;
    if (len < sizeof(stack)) {
      std::memcpy(stack, s + i, len);
      stack[len] = '\0';
    } else {
      heap.assign(s + i, len);
      tok = &heap[0];
    }
    char* end = nullptr;
    v = std::strtod(tok, &end);
    if (end != tok + len) return false;
    i = j;
    return true;
  }
  // dims: 2, 3 (Z or M), 4 (ZM)
  int dims = 2;
  bool dim_tag() {
    // optional Z / M / ZM after the type keyword
    if (peek_word("ZM")) { i += 2; dims = 4; return true; }
    if (peek_word("Z")) { i += 1; dims = 3; return true; }
    if (peek_word("M")) { i += 1; dims = 3; return true; }
    return true;
  }
  bool coord(double& x, double& y) {
    if (!number(x) || !number(y)) return false;
    // extra ordinates: accept as many numbers as the coordinate has
    double extra;
    size_t save = i;
    while (number(extra)) save = i;
    i = save;
    return true;
  }
  bool empty_kw() {
    if (peek_word("EMPTY")) { i += 5; return true; }
    return false;
  }
};

void close_ring(GeomTable& t, uint64_t v0) {
  uint64_t v1 = t.xy.size() / 2;
  if (v1 > v0) {
    double fx = t.xy[2 * v0], fy = t.xy[2 * v0 + 1];
    double lx = t.xy[2 * (v1 - 1)], ly = t.xy[2 * (v1 - 1) + 1];
    if (!(fx == lx && fy == ly)) { t.xy.push_back(fx); t.xy.push_back(fy); }
  }
}

void end_ring(GeomTable& t, uint8_t flag) {
  t.vertex_offsets.push_back(t.xy.size() / 2);
  t.ring_flags.push_back(flag);
}

void end_part(GeomTable& t, uint8_t kind) {
  t.part_kind.push_back(kind);
  t.ring_offsets.push_back(t.ring_flags.size());
}

// "(x y, x y, ...)" -> one ring
bool wkt_ring(WktReader& r, GeomTable& t, bool polygon_ring, uint8_t flag) {
  uint64_t v0 = t.xy.size() / 2;
  if (r.empty_kw()) { end_ring(t, flag); return true; }
  if (!r.eat('(')) return false;
  do {
    double x, y;
    if (!r.coord(x, y)) return false;
    t.xy.push_back(x);
    t.xy.push_back(y);
  } while (r.eat(','));
  if (!r.eat(')')) return false;
  if (polygon_ring) close_ring(t, v0);
  end_ring(t, flag);
  return true;
}

// "((ring), (ring))" -> rings of a polygon (first exterior)
bool wkt_polygon_rings(WktReader& r, GeomTable& t) {
  if (r.empty_kw()) return true;
  if (!r.eat('(')) return false;
  bool first = true;
  do {
    if (!wkt_ring(r, t, true, first ? 0 : 1)) return false;
    first = false;
  } while (r.eat(','));
  return r.eat(')');
}

bool wkt_geometry(WktReader& r, GeomTable& t, int depth) {
  if (depth > 64) { r.msg = "nesting too deep"; return false; }
  std::string kw;
  if (!r.word(kw)) return false;
  r.dim_tag();
  if (kw == "POINT") {
    if (r.empty_kw()) { r.msg = "POINT EMPTY cannot be represented"; return false; }
    if (!r.eat('(')) return false;
    double x, y;
    if (!r.coord(x, y)) return false;
    if (!r.eat(')')) return false;
    t.xy.push_back(x);
    t.xy.push_back(y);
    end_ring(t, 0);
    end_part(t, RZ_PART_POINT);
    return true;
  }
  if (kw == "MULTIPOINT") {
    if (!r.empty_kw()) {
      if (!r.eat('(')) return false;
      do {
        double x, y;
        if (r.eat('(')) {
          if (r.empty_kw()) { r.msg = "empty point in MULTIPOINT"; return false; }
          if (!r.coord(x, y) || !r.eat(')')) return false;
        } else if (r.empty_kw()) {
          r.msg = "empty point in MULTIPOINT";
          return false;
        } else if (!r.coord(x, y)) {
          return false;
        }
        t.xy.push_back(x);
        t.xy.push_back(y);
      } while (r.eat(','));
      if (!r.eat(')')) return false;
    }
    end_ring(t, 0);
    end_part(t, RZ_PART_POINT);
    return true;
  }
  if (kw == "LINESTRING") {
    if (!wkt_ring(r, t, false, 0)) return false;
    end_part(t, RZ_PART_LINE);
    return true;
  }
  if (kw == "MULTILINESTRING") {
    if (!r.empty_kw()) {
      if (!r.eat('(')) return false;
      do {
        if (!wkt_ring(r, t, false, 0)) return false;
      } while (r.eat(','));
      if (!r.eat(')')) return false;
    }
    end_part(t, RZ_PART_LINE);
    return true;
  }
  if (kw == "POLYGON" || kw == "TRIANGLE") {
    if (!wkt_polygon_rings(r, t)) return false;
    end_part(t, RZ_PART_POLYGON);
    return true;
  }
  if (kw == "MULTIPOLYGON") {
    if (!r.empty_kw()) {
      if (!r.eat('(')) return false;
      do {
        if (!wkt_polygon_rings(r, t)) return false;
      } while (r.eat(','));
      if (!r.eat(')')) return false;
    }
    end_part(t, RZ_PART_POLYGON);
    return true;
  }
  if (kw == "GEOMETRYCOLLECTION") {
    if (r.empty_kw()) return true;
    if (!r.eat('(')) return false;
    do {
      if (!wkt_geometry(r, t, depth + 1)) return false;
    } while (r.eat(','));
    return r.eat(')');
  }
  r.msg = "unknown geometry type '" + kw + "'";
  return false;
}

// Roll a partially-appended geometry back to the table sizes in `mark`.
struct Mark {
  size_t parts, rings, verts;
};
Mark mark_of(const GeomTable& t) { return {t.part_kind.size(), t.ring_flags.size(), t.xy.size() / 2}; }
void rollback(GeomTable& t, const Mark& m) {
  t.part_kind.resize(m.parts);
  t.ring_offsets.resize(m.parts + 1);
  t.ring_flags.resize(m.rings);
  t.vertex_offsets.resize(m.rings + 1);
  t.xy.resize(2 * m.verts);
}

}  // namespace

// ------------------------------------------------------- chunked parse ----
// Items are parsed in contiguous chunks on several host threads, each chunk
// into its own table; the tables are then appended in chunk order with their
// offsets rebased.  The result and the reported error (the first failing
// item in input order) are those of a sequential parse.
namespace {

struct ChunkResult {
  GeomTable t;
  size_t fail_item = SIZE_MAX;
  bool out_of_memory = false;  // the chunk's table could not grow
  std::string msg;
};

// parse_one(k, table, msg) -> 1: parsed and kept, 0: parsed and dropped, -1: error.
// Runs on a worker thread: nothing may escape it (an exception leaving a
// std::thread ends the process), so allocation failures are recorded.
template <typename ParseOne>
void parse_chunk(size_t k0, size_t k1, ChunkResult& c, ParseOne&& parse_one) {
  size_t k = k0;
  try {
    for (; k < k1; ++k) {
      const int r = parse_one(k, c.t, c.msg);
      if (r < 0) {
        c.fail_item = k;
        return;
      }
      if (r > 0) c.t.part_offsets.push_back(c.t.part_kind.size());
    }
  } catch (const std::bad_alloc&) {
    c.fail_item = k;
    c.out_of_memory = true;
  } catch (...) {
    c.fail_item = k;
    c.msg = "internal error while parsing";
  }
}

void append_table(GeomTable& dst, const GeomTable& src) {
  const uint64_t p0 = dst.part_kind.size(), r0 = dst.ring_flags.size(), v0 = dst.xy.size() / 2;
  for (size_t i = 1; i < src.part_offsets.size(); ++i) dst.part_offsets.push_back(src.part_offsets[i] + p0);
  dst.part_kind.insert(dst.part_kind.end(), src.part_kind.begin(), src.part_kind.end());
  for (size_t i = 1; i < src.ring_offsets.size(); ++i) dst.ring_offsets.push_back(src.ring_offsets[i] + r0);
  dst.ring_flags.insert(dst.ring_flags.end(), src.ring_flags.begin(), src.ring_flags.end());
  for (size_t i = 1; i < src.vertex_offsets.size(); ++i) dst.vertex_offsets.push_back(src.vertex_offsets[i] + v0);
  dst.xy.insert(dst.xy.end(), src.xy.begin(), src.xy.end());
}

// threads for n items of `bytes` total input: one per 4 MiB of input, at
// most the host's hardware threads and 32, and never more than one per 256 items
unsigned parse_threads(size_t n, size_t bytes) {
  const char* env = std::getenv("RZ_PARSE_THREADS");
  if (env && *env) {
    const long v = std::strtol(env, nullptr, 10);
    if (v >= 1) return (unsigned)std::min<long>(v, 256);
  }
  unsigned hw = std::thread::hardware_concurrency();
  if (hw == 0) hw = 1;
  size_t t = std::min<size_t>({(size_t)hw, (size_t)32, bytes / (4u << 20) + 1, n / 256 + 1});
  return (unsigned)std::max<size_t>(t, 1);
}

template <typename ParseOne>
rz_status parse_all_impl(size_t n, size_t bytes, rz_geom_buffer** out, ParseOne&& parse_one, const char* what,
                         char* err, size_t errlen) {
  const unsigned T = parse_threads(n, bytes);
  std::vector<ChunkResult> chunks(T);
  if (T == 1) {
    parse_chunk(0, n, chunks[0], parse_one);
  } else {
    std::vector<std::thread> ts;
    ts.reserve(T);
    try {
      for (unsigned c = 0; c < T; ++c) {
        const size_t k0 = n * c / T, k1 = n * (c + 1) / T;
        ts.emplace_back([&, c, k0, k1] { parse_chunk(k0, k1, chunks[c], parse_one); });
      }
    } catch (...) {  // a thread could not start: finish the started ones before reporting
      for (auto& th : ts) th.join();
      throw;
    }
    for (auto& th : ts) th.join();
  }
  for (const ChunkResult& c : chunks)  // chunks are in item order: the first failure is the first reported
    if (c.fail_item != SIZE_MAX && c.out_of_memory)
      return fail(err, errlen, RZ_OUT_OF_MEMORY, "out of host memory while parsing geometry (item %zu)",
                  c.fail_item);
    else if (c.fail_item != SIZE_MAX)
      return fail(err, errlen, RZ_PARSE_ERROR, "Cannot parse geometry. Check that the %s valid. (item %zu%s%s)",
                  what, c.fail_item, c.msg.empty() ? "" : ": ", c.msg.c_str());
  auto* buf = new rz_geom_buffer();
  if (T == 1) {
    buf->t = std::move(chunks[0].t);
  } else {
    GeomTable& t = buf->t;
    size_t G = 0, P = 0, R = 0, V = 0;
    for (const ChunkResult& c : chunks) {
      G += c.t.part_offsets.size() - 1;
      P += c.t.part_kind.size();
      R += c.t.ring_flags.size();
      V += c.t.xy.size() / 2;
    }
    t.part_offsets.reserve(G + 1);
    t.part_kind.reserve(P);
    t.ring_offsets.reserve(P + 1);
    t.ring_flags.reserve(R);
    t.vertex_offsets.reserve(R + 1);
    t.xy.reserve(2 * V);
    for (const ChunkResult& c : chunks) append_table(t, c.t);
  }
  if (buf->t.part_offsets.size() == 1) {
    delete buf;
    return fail(err, errlen, RZ_VALUE_ERROR, "Could not parse geometry. Only WKT or WKB formats are supported.");
  }
  *out = buf;
  return RZ_OK;
}

// The same, with allocation failures of the merge (and of thread creation)
// turned into a status: no exception crosses the C boundary.
template <typename ParseOne>
rz_status parse_all(size_t n, size_t bytes, rz_geom_buffer** out, ParseOne&& parse_one, const char* what,
                    char* err, size_t errlen) {
  try {
    return parse_all_impl(n, bytes, out, std::forward<ParseOne>(parse_one), what, err, errlen);
  } catch (const std::bad_alloc&) {
    return fail(err, errlen, RZ_OUT_OF_MEMORY, "out of host memory while parsing geometry");
  } catch (const std::exception& e) {
    return fail(err, errlen, RZ_RUNTIME_ERROR, "geometry parsing failed: %s", e.what());
  }
}

}  // namespace

extern "C" rz_status rz_parse_wkt(const char* const* texts, const size_t* lens, size_t n,
                                  rz_geom_buffer** out, char* err, size_t errlen) {
  rz::clear_err(err, errlen);
  *out = nullptr;
  size_t bytes = 0;
  for (size_t k = 0; k < n; ++k) bytes += lens[k];
  return parse_all(
      n, bytes, out,
      [&](size_t k, GeomTable& t, std::string& msg) -> int {
        WktReader r{texts[k], lens[k]};
        if (!wkt_geometry(r, t, 0) || (r.ws(), r.i != r.n)) {
          msg = r.msg;
          return -1;
        }
        return 1;
      },
      "WKT is", err, errlen);
}

// ------------------------------------------------------------------ WKB ----
// ISO WKB (type + 1000/2000/3000 for Z/M/ZM) and extended WKB (high flag
// bits, optional SRID), either byte order.  Coordinates beyond x,y dropped.
namespace {

struct WkbReader {
  const uint8_t* p;
  size_t n, i = 0;
  std::string msg;
  bool drop = false;  // geo-types cannot hold it (empty point)

  bool u8(uint8_t& v) {
    if (i + 1 > n) return false;
    v = p[i++];
    return true;
  }
  bool u32(bool le, uint32_t& v) {
    if (i + 4 > n) return false;
    const uint8_t* b = p + i;
    v = le ? (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24)
           : (uint32_t)b[3] | ((uint32_t)b[2] << 8) | ((uint32_t)b[1] << 16) | ((uint32_t)b[0] << 24);
    i += 4;
    return true;
  }
  bool f64(bool le, double& v) {
    if (i + 8 > n) return false;
    uint64_t u = 0;
    for (int k = 0; k < 8; ++k) u |= (uint64_t)p[i + (le ? k : 7 - k)] << (8 * k);
    std::memcpy(&v, &u, 8);
    i += 8;
    return true;
  }
};

bool wkb_coords(WkbReader& r, bool le, int dims, uint32_t count, GeomTable& t) {
  if ((uint64_t)count * dims * 8 > r.n - r.i) return false;
  for (uint32_t c = 0; c < count; ++c) {
    double x, y, extra;
    if (!r.f64(le, x) || !r.f64(le, y)) return false;
    for (int d = 2; d < dims; ++d)
      if (!r.f64(le, extra)) return false;
    t.xy.push_back(x);
    t.xy.push_back(y);
  }
  return true;
}

bool wkb_geometry(WkbReader& r, GeomTable& t, int depth, int want_type /*0 any*/) {
  if (depth > 64) { r.msg = "nesting too deep"; return false; }
  uint8_t order;
  uint32_t type;
  if (!r.u8(order) || order > 1) { r.msg = "bad byte order"; return false; }
  bool le = order == 1;
  if (!r.u32(le, type)) return false;
  int dims = 2;
  if (type & 0x80000000u) dims++;
  if (type & 0x40000000u) dims++;
  if (type & 0x20000000u) {
    uint32_t srid;
    if (!r.u32(le, srid)) return false;
  }
  type &= 0x0FFFFFFFu;
  uint32_t base = type % 1000, iso = type / 1000;
  if (iso == 1 || iso == 2) dims = 3;
  else if (iso == 3) dims = 4;
  else if (iso != 0) { r.msg = "bad geometry type"; return false; }
  if (want_type && (int)base != want_type) { r.msg = "unexpected member type"; return false; }
  uint32_t cnt;
  switch (base) {
    case 1: {  // Point
      uint64_t v0 = t.xy.size() / 2;
      if (!wkb_coords(r, le, dims, 1, t)) return false;
      if (std::isnan(t.xy[2 * v0]) && std::isnan(t.xy[2 * v0 + 1])) r.drop = true;
      if (depth == 0 || want_type == 0) {  // a stand-alone point
        end_ring(t, 0);
        end_part(t, RZ_PART_POINT);
      }
      return true;
    }
    case 2:  // LineString
      if (!r.u32(le, cnt) || !wkb_coords(r, le, dims, cnt, t)) return false;
      end_ring(t, 0);
      if (want_type == 0) end_part(t, RZ_PART_LINE);
      return true;
    case 3:
    case 17: {  // Polygon, Triangle
      if (!r.u32(le, cnt)) return false;
      for (uint32_t k = 0; k < cnt; ++k) {
        uint32_t nv;
        uint64_t v0 = t.xy.size() / 2;
        if (!r.u32(le, nv) || !wkb_coords(r, le, dims, nv, t)) return false;
        close_ring(t, v0);
        end_ring(t, k == 0 ? 0 : 1);
      }
      if (want_type == 0) end_part(t, RZ_PART_POLYGON);
      return true;
    }
    case 4:  // MultiPoint
      if (!r.u32(le, cnt)) return false;
      for (uint32_t k = 0; k < cnt; ++k)
        if (!wkb_geometry(r, t, depth + 1, 1)) return false;
      end_ring(t, 0);
      end_part(t, RZ_PART_POINT);
      return true;
    case 5:  // MultiLineString
      if (!r.u32(le, cnt)) return false;
      for (uint32_t k = 0; k < cnt; ++k)
        if (!wkb_geometry(r, t, depth + 1, 2)) return false;
      end_part(t, RZ_PART_LINE);
      return true;
    case 6:  // MultiPolygon
      if (!r.u32(le, cnt)) return false;
      for (uint32_t k = 0; k < cnt; ++k)
        if (!wkb_geometry(r, t, depth + 1, 3)) return false;
      end_part(t, RZ_PART_POLYGON);
      return true;
    case 7:  // GeometryCollection
      if (!r.u32(le, cnt)) return false;
      for (uint32_t k = 0; k < cnt; ++k)
        if (!wkb_geometry(r, t, depth + 1, 0)) return false;
      return true;
    default:
      r.msg = "unsupported geometry type " + std::to_string(base);
      return false;
  }
}

}  // namespace

extern "C" rz_status rz_parse_wkb(const uint8_t* const* blobs, const size_t* lens, size_t n,
                                  rz_geom_buffer** out, char* err, size_t errlen) {
  rz::clear_err(err, errlen);
  *out = nullptr;
  size_t bytes = 0;
  for (size_t k = 0; k < n; ++k) bytes += lens[k];
  return parse_all(
      n, bytes, out,
      [&](size_t k, GeomTable& t, std::string& msg) -> int {
        WkbReader r{blobs[k], lens[k]};
        Mark m = mark_of(t);
        if (!wkb_geometry(r, t, 0, 0)) {
          msg = r.msg;
          return -1;
        }
        if (r.drop) {  // try_to_geometry() -> None: silently skipped (parse_geometry.rs:113-115)
          rollback(t, m);
          return 0;
        }
        return 1;
      },
      "WKB bytes are", err, errlen);
}

extern "C" rz_status rz_geom_buffer_view(const rz_geom_buffer* buf, rz_geoms* out) {
  if (!buf || !out) return RZ_INVALID_ARGUMENT;
  buf->t.view(out);
  return RZ_OK;
}

extern "C" void rz_geom_buffer_free(rz_geom_buffer* buf) { delete buf; }

// ---------------------------------------------------------- raster grid ----
namespace {

// Rust `f64 as usize` (saturating, NaN -> 0).
uint64_t as_usize(double v) {
  if (!(v > 0.0)) return 0;
  if (v >= 18446744073709551616.0) return UINT64_MAX;
  return (uint64_t)v;
}
double min_rs(double a, double b) { return a != a ? b : (b != b ? a : (a < b ? a : b)); }
double max_rs(double a, double b) { return a != a ? b : (b != b ? a : (a > b ? a : b)); }

struct Rect {
  bool some = false;
  double x0, y0, x1, y1;
  void add(double x, double y) {  // geo get_bounding_rect / get_min_max
    if (!some) { some = true; x0 = x1 = x; y0 = y1 = y; return; }
    if (x > x1) x1 = x; else if (x < x0) x0 = x;
    if (y > y1) y1 = y; else if (y < y0) y0 = y;
  }
  void merge(const Rect& o) {  // RasterInfoBuilder::build_with fold (raster.rs:75-86)
    if (!o.some) return;
    if (!some) { *this = o; return; }
    x0 = min_rs(x0, o.x0); y0 = min_rs(y0, o.y0);
    x1 = max_rs(x1, o.x1); y1 = max_rs(y1, o.y1);
  }
};

}  // namespace

extern "C" rz_status rz_raster_info_build(const rz_geoms* g, uint32_t flags, const uint64_t* shape,
                                          const double* res, const double* extent, int32_t epsg,
                                          rz_raster_info* out, char* err, size_t errlen) {
  rz::clear_err(err, errlen);
  const bool has_shape = flags & RZ_RI_SHAPE, has_res = flags & RZ_RI_RES;
  const bool has_extent = flags & RZ_RI_EXTENT, tap = flags & RZ_RI_TAP;
  double xmin, ymin, xmax, ymax;
  bool inferred;
  if (has_extent) {
    // RasterInfoBuilder::build (raster.rs:50-64): all four exactly +0.0 (total_cmp)
    bool all_zero = true;
    for (int k = 0; k < 4; ++k) all_zero &= (extent[k] == 0.0 && !std::signbit(extent[k]));
    if (all_zero) return fail(err, errlen, RZ_VALUE_ERROR, "Unspecified extent (all zeros).");
    xmin = extent[0]; ymin = extent[1]; xmax = extent[2]; ymax = extent[3];
    inferred = false;
  } else {
    // RasterInfoBuilder::build_with (raster.rs:67-93)
    Rect acc;
    if (g) {
      for (uint64_t gi = 0; gi < g->n_geoms; ++gi) {
        Rect gr;
        for (uint64_t p = g->part_offsets[gi]; p < g->part_offsets[gi + 1]; ++p) {
          Rect pr;
          bool poly = g->part_kind[p] == RZ_PART_POLYGON;
          for (uint64_t r = g->ring_offsets[p]; r < g->ring_offsets[p + 1]; ++r) {
            if (poly && g->ring_flags && (g->ring_flags[r] & 1)) continue;  // exterior only
            for (uint64_t v = g->vertex_offsets[r]; v < g->vertex_offsets[r + 1]; ++v)
              pr.add(g->xy[2 * v], g->xy[2 * v + 1]);
          }
          gr.merge(pr);
        }
        acc.merge(gr);
      }
    }
    if (!acc.some) return fail(err, errlen, RZ_RUNTIME_ERROR, "Cannot infer bounding box from geometry.");
    xmin = acc.x0; ymin = acc.y0; xmax = acc.x1; ymax = acc.y1;
    inferred = true;
  }
  // RasterInfoBuilder::finalize (raster.rs:95-156)
  if (!has_shape && !has_res)
    return fail(err, errlen, RZ_VALUE_ERROR, "Must set at least one of `shape` or `resolution`");
  if (has_shape && has_res)
    return fail(err, errlen, RZ_VALUE_ERROR, "Shape and resolution are mutually exclusive; provide only one");
  uint64_t nrows = has_shape ? shape[0] : 0, ncols = has_shape ? shape[1] : 0;
  double xres = has_res ? res[0] : 0.0, yres = has_res ? res[1] : 0.0;
  if (has_shape && (nrows == 0 || ncols == 0))
    return fail(err, errlen, RZ_VALUE_ERROR, "Shape values must be > 0.");
  if (has_res && (xres <= 0.0 || yres <= 0.0))
    return fail(err, errlen, RZ_VALUE_ERROR, "Resolution values must be > 0.");
  if (inferred && !tap && has_res) {
    xmin -= xres / 2.0;
    xmax += xres / 2.0;
    ymin -= yres / 2.0;
    ymax += yres / 2.0;
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
  out->nrows = nrows;
  out->ncols = ncols;
  out->xmin = xmin;
  out->xmax = xmax;
  out->ymin = ymin;
  out->ymax = ymax;
  out->xres = xres;
  out->yres = yres;
  out->epsg = epsg;
  out->_pad = 0;
  return RZ_OK;
}
