// rz_internal.h -- shared host-side helpers of the engine library.
#pragma once

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/rusterize_gb300.h"

namespace rz {

inline rz_status fail(char* err, size_t errlen, rz_status st, const char* fmt, ...) {
  if (err && errlen) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, errlen, fmt, ap);
    va_end(ap);
  }
  return st;
}

inline void clear_err(char* err, size_t errlen) {
  if (err && errlen) err[0] = '\0';
}

// Owned geometry table built by the WKT/WKB readers.
struct GeomTable {
  std::vector<uint64_t> part_offsets{0};
  std::vector<uint8_t> part_kind;
  std::vector<uint64_t> ring_offsets{0};
  std::vector<uint64_t> vertex_offsets{0};
  std::vector<uint8_t> ring_flags;
  std::vector<double> xy;

  void view(rz_geoms* g) const {
    g->n_geoms = part_offsets.size() - 1;
    g->n_parts = part_kind.size();
    g->n_rings = ring_flags.size();
    g->n_vertices = xy.size() / 2;
    g->part_offsets = part_offsets.data();
    g->part_kind = part_kind.data();
    g->ring_offsets = ring_offsets.data();
    g->vertex_offsets = vertex_offsets.data();
    g->ring_flags = ring_flags.data();
    g->xy = xy.data();
  }
};

}  // namespace rz

struct rz_geom_buffer {
  rz::GeomTable t;
};
