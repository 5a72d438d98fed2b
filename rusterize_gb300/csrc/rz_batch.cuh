// rz_batch.cuh -- many independent jobs in one pass of the pipeline.
//
// A wave of jobs is concatenated into one parts table: every job's offsets
// are rebased onto the wave's, its values gathered (a scalar burn value is
// replicated per geometry), and its vertices mapped to pixel coordinates
// with the job's own world -> pixel map (edges.rs:94-97).  The pipeline then
// runs once over the wave with the identity map, each part burning into its
// job's raster (JobDims), and the fill writes every bucket into its job's
// output (FillJob).
#pragma once

#include <type_traits>

#include "rz_device.cuh"

namespace rzd {

// Where one job's tables come from, and where they go in the wave.
struct JobSrc {
  const unsigned long long* part_offsets;  // [G + 1]
  const unsigned char* part_kind;          // [P]
  const unsigned long long* ring_offsets;  // [P + 1]
  const unsigned long long* vertex_offsets;  // [R + 1]
  const double2* xy;                       // [V]
  const void* values;                      // [G] of the output type, or nullptr: `scalar` for every geometry
  unsigned long long scalar;               // raw bits of the scalar burn value
  unsigned long long n_geoms, n_parts, n_rings, n_vertices;
  Grid grid;                               // the job's world -> pixel map
};

// Wave bases: base[k * (n_jobs + 1) + j] is the first element of kind k
// (0 geometries, 1 parts, 2 rings, 3 vertices) of job j; entry n_jobs is the
// wave total.
enum { BK_GEOM = 0, BK_PART, BK_RING, BK_VERT, BK_N };

// For element i of kind k: the job j with base[j] <= i < base[j + 1].  Lane 0
// searches the warp's first element; the other lanes walk forward from it
// (jobs hold many elements, so the walk is short).
__device__ __forceinline__ unsigned wave_job(const unsigned long long* base, unsigned n_jobs,
                                             unsigned long long i_first, unsigned long long i) {
  unsigned j0 = 0;
  if ((threadIdx.x & 31) == 0) {
    unsigned lo = 0, hi = n_jobs;  // base[lo] <= i_first < base[hi]
    while (hi - lo > 1) {
      const unsigned mid = (lo + hi) >> 1;
      if (base[mid] <= i_first) lo = mid; else hi = mid;
    }
    j0 = lo;
  }
  j0 = __shfl_sync(0xFFFFFFFFu, j0, 0);
  unsigned j = j0;
  while (j + 1 < n_jobs && base[j + 1] <= i) ++j;
  return j;
}

// Every job's own table must start at 0 and end at its own counts, or the
// rebased wave table would hand parts, rings or vertices to a neighbour.
__global__ void k_batch_check(const JobSrc* __restrict__ src, unsigned n_jobs, Ctrl* ctrl) {
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < n_jobs; j += gridDim.x * blockDim.x) {
    const JobSrc s = src[j];
    if (s.part_offsets[0] != 0 || s.part_offsets[s.n_geoms] != s.n_parts || s.ring_offsets[0] != 0 ||
        s.ring_offsets[s.n_parts] != s.n_rings || s.vertex_offsets[0] != 0 ||
        s.vertex_offsets[s.n_rings] != s.n_vertices)
      set_error(ctrl, ERR_BAD_JOB, j);
  }
}

// geometries: part offsets rebased, burn values gathered (VB bytes)
template <int VB>
__global__ void k_batch_geoms(const JobSrc* __restrict__ src, const unsigned long long* __restrict__ base,
                              unsigned n_jobs, unsigned long long* part_offsets, void* values) {
  using V = typename std::conditional<VB == 1, unsigned char,
            typename std::conditional<VB == 2, unsigned short,
            typename std::conditional<VB == 4, unsigned, unsigned long long>::type>::type>::type;
  const unsigned long long* gb = base + BK_GEOM * (n_jobs + 1);
  const unsigned long long* pb = base + BK_PART * (n_jobs + 1);
  const unsigned long long total = gb[n_jobs];
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i0 = blockIdx.x * (unsigned long long)blockDim.x + (threadIdx.x & ~31u); i0 < total;
       i0 += stride) {
    const unsigned long long i = i0 + (threadIdx.x & 31);
    const unsigned j = wave_job(gb, n_jobs, i0, i < total ? i : total - 1);
    if (i >= total) continue;
    const JobSrc& s = src[j];
    const unsigned long long li = i - gb[j];
    part_offsets[i] = s.part_offsets[li] + pb[j];
    static_cast<V*>(values)[i] = s.values ? static_cast<const V*>(s.values)[li] : (V)s.scalar;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) part_offsets[total] = pb[n_jobs];
}

// parts: kinds copied, ring offsets rebased
__global__ void k_batch_parts(const JobSrc* __restrict__ src, const unsigned long long* __restrict__ base,
                              unsigned n_jobs, unsigned char* part_kind, unsigned long long* ring_offsets) {
  const unsigned long long* pb = base + BK_PART * (n_jobs + 1);
  const unsigned long long* rb = base + BK_RING * (n_jobs + 1);
  const unsigned long long total = pb[n_jobs];
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i0 = blockIdx.x * (unsigned long long)blockDim.x + (threadIdx.x & ~31u); i0 < total;
       i0 += stride) {
    const unsigned long long i = i0 + (threadIdx.x & 31);
    const unsigned j = wave_job(pb, n_jobs, i0, i < total ? i : total - 1);
    if (i >= total) continue;
    const JobSrc& s = src[j];
    const unsigned long long li = i - pb[j];
    part_kind[i] = s.part_kind[li];
    ring_offsets[i] = s.ring_offsets[li] + rb[j];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) ring_offsets[total] = rb[n_jobs];
}

// rings: vertex offsets rebased, and LineString::is_closed taken on the
// world coordinates (the wave's pixel coordinates can round two different
// end points to one value)
__global__ void k_batch_rings(const JobSrc* __restrict__ src, const unsigned long long* __restrict__ base,
                              unsigned n_jobs, unsigned long long* vertex_offsets, unsigned char* ring_closed) {
  const unsigned long long* rb = base + BK_RING * (n_jobs + 1);
  const unsigned long long* vb = base + BK_VERT * (n_jobs + 1);
  const unsigned long long total = rb[n_jobs];
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i0 = blockIdx.x * (unsigned long long)blockDim.x + (threadIdx.x & ~31u); i0 < total;
       i0 += stride) {
    const unsigned long long i = i0 + (threadIdx.x & 31);
    const unsigned j = wave_job(rb, n_jobs, i0, i < total ? i : total - 1);
    if (i >= total) continue;
    const JobSrc& s = src[j];
    const unsigned long long a = s.vertex_offsets[i - rb[j]], e = s.vertex_offsets[i - rb[j] + 1];
    vertex_offsets[i] = a + vb[j];
    bool closed = false;
    if (e > a && e <= s.n_vertices) {  // a table k_validate rejects later must not be read out of bounds
      const double2 first = s.xy[a], last = s.xy[e - 1];
      closed = first.x == last.x && first.y == last.y;
    }
    ring_closed[i] = closed ? 1 : 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) vertex_offsets[total] = vb[n_jobs];
}

// vertices: the job's world -> pixel map, stored for the identity map of the
// wave (x as is, y negated: to_py with ymax = -0 and resolution 1 returns
// -0 - (-y) = y bit for bit, signed zeros included)
__global__ void k_batch_vertices(const JobSrc* __restrict__ src, const unsigned long long* __restrict__ base,
                                 unsigned n_jobs, double2* xy) {
  const unsigned long long* vb = base + BK_VERT * (n_jobs + 1);
  const unsigned long long total = vb[n_jobs];
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i0 = blockIdx.x * (unsigned long long)blockDim.x + (threadIdx.x & ~31u); i0 < total;
       i0 += stride) {
    const unsigned long long i = i0 + (threadIdx.x & 31);
    const unsigned j = wave_job(vb, n_jobs, i0, i < total ? i : total - 1);
    if (i >= total) continue;
    const JobSrc& s = src[j];
    const double2 w = s.xy[i - vb[j]];
    xy[i] = make_double2(to_px(s.grid, w.x), -to_py(s.grid, w.y));
  }
}

}  // namespace rzd
