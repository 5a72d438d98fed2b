// rz_engine.cu -- the engine context, device scratch arena and the
// rz_rasterize pipeline (one CUDA stream per context):
//
//   validate -> part->geometry map -> part plans -> scan
//   -> span generation (polygon windows | Bresenham lines | points)
//   -> bucket scan -> scatter -> ordered fill -> (D2H)
//
// Replaces ArrayBuilder::build for DenseArray (rust/src/rasterize.rs:71-116).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <thread>
#include <unistd.h>

#include "rz_batch.cuh"
#include "rz_device.cuh"
#include "rz_fill.cuh"
#include "rz_internal.h"
#include "rz_layout.h"
#include "rz_kernels.cuh"
#include "rz_scan.cuh"
#include "rz_sort.cuh"
#include "rz_replay.cuh"
#include "rz_sparse.cuh"

using rz::fail;
using namespace rzd;

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

cudaError_t ensure(DevBuf& b, size_t need) {
  if (need <= b.cap) return cudaSuccess;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  size_t want = need + need / 8 + (1u << 20);
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    want = need;
    p = nullptr;
    e = cudaMalloc(&p, want);
  }
  if (e == cudaSuccess) {
    b.p = p;
    b.cap = want;
  } else {
    cudaGetLastError();  // an allocation failure is reported here, not by a later call
  }
  return e;
}

struct Layout {
  size_t off = 0;
  size_t take(size_t bytes) {
    size_t o = (off + 255) & ~size_t(255);
    off = o + bytes;
    return o;
  }
};

bool is_pow2(double v) {
  if (!(v > 0.0) || !std::isfinite(v)) return false;
  int e;
  double m = std::frexp(v, &e);
  if (m != 0.5) return false;
  double inv = 1.0 / v;
  return std::isfinite(inv) && std::fpclassify(inv) == FP_NORMAL && std::fpclassify(v) == FP_NORMAL;
}

unsigned long long one_bits(rz_dtype dt) {
  switch (dt) {
    case RZ_F32: return 0x3F800000ull;
    case RZ_F64: return 0x3FF0000000000000ull;
    default: return 1ull;
  }
}

typedef int (*fill_fn)(const FillArgs&, int, bool, int, cudaStream_t);

fill_fn fill_for(rz_dtype dt) {
  switch (dt) {
    case RZ_U8: return rz_fill_u8;
    case RZ_U16: return rz_fill_u16;
    case RZ_U32: return rz_fill_u32;
    case RZ_U64: return rz_fill_u64;
    case RZ_I8: return rz_fill_i8;
    case RZ_I16: return rz_fill_i16;
    case RZ_I32: return rz_fill_i32;
    case RZ_I64: return rz_fill_i64;
    case RZ_F32: return rz_fill_f32;
    case RZ_F64: return rz_fill_f64;
  }
  return nullptr;
}

void launch_scatter(int sms, int bps, cudaStream_t s, const RecBuf& sb, const unsigned* boff, unsigned* bcount,
                    uint2* sorted, Ctrl* ctrl) {
  k_scatter<<<sms * bps, 256, 0, s>>>(sb, boff, bcount, sorted, ctrl);
}

// The burn value of every part (values[part_geom[p]], tsize bytes each).
void launch_part_values(size_t tsize, int sms, cudaStream_t s, const unsigned* part_geom, const void* values,
                        unsigned long long n_parts, void* pvals, Ctrl* ctrl) {
  if (!n_parts) return;
  const unsigned long long g0 = (n_parts + 255) / 256;
  const unsigned grid = (unsigned)std::min<unsigned long long>(g0, (unsigned long long)sms * 16);
  switch (tsize) {
    case 1: k_part_values<1><<<grid, 256, 0, s>>>(part_geom, values, n_parts, pvals, ctrl); break;
    case 2: k_part_values<2><<<grid, 256, 0, s>>>(part_geom, values, n_parts, pvals, ctrl); break;
    case 4: k_part_values<4><<<grid, 256, 0, s>>>(part_geom, values, n_parts, pvals, ctrl); break;
    default: k_part_values<8><<<grid, 256, 0, s>>>(part_geom, values, n_parts, pvals, ctrl); break;
  }
}

unsigned grid_for(unsigned long long work, unsigned per_block, unsigned cap) {
  unsigned long long g = (work + per_block - 1) / per_block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (unsigned)g;
}

// The status and message of an error a kernel recorded in the control block.
rz_status ctrl_error(const Ctrl& hc, char* err, size_t errlen) {
  const unsigned long long ix = hc.err_index;
  switch (hc.err) {
    case ERR_BAD_TABLE:
      return fail(err, errlen, RZ_INVALID_ARGUMENT, "geometry table is inconsistent (%s offsets, index %llu)",
                  (ix >> 62) == 0 ? "part" : ((ix >> 62) == 1 ? "ring" : "vertex"), ix & ((1ull << 62) - 1));
    case ERR_BAD_KIND: return fail(err, errlen, RZ_INVALID_ARGUMENT, "invalid part kind at part %llu", ix);
    case ERR_BAD_BAND: return fail(err, errlen, RZ_INVALID_ARGUMENT, "band index out of range at geometry %llu", ix);
    case ERR_BITMAP:
      return fail(err, errlen, RZ_RUNTIME_ERROR, "polygon part %llu has non-finite or out-of-range coordinates", ix);
    case ERR_TOO_WIDE:
      return fail(err, errlen, RZ_VALUE_ERROR, "polygon part %llu is wider than %d raster columns", ix,
                  BITMAP_WORDS * 32 - 64);
    case ERR_LINE_LONG:
      return fail(err, errlen, RZ_VALUE_ERROR, "line segment at vertex %llu spans more than 2^26 pixels", ix);
    case ERR_RANGE:
      return fail(err, errlen, RZ_RUNTIME_ERROR, "internal error: record or tile outside the call's rasters (%llu)",
                  ix);
    case ERR_TRIPLET:
      return fail(err, errlen, RZ_VALUE_ERROR, "triplet %llu lies outside the raster", ix);
    case ERR_BAD_JOB:
      return fail(err, errlen, RZ_INVALID_ARGUMENT,
                  "geometry table of job %llu does not start at 0 or end at its own counts", ix);
    default: return fail(err, errlen, RZ_RUNTIME_ERROR, "engine error %u", hc.err);
  }
}

// The world -> pixel map of one raster (edges.rs:94-97).
Grid make_grid(const rz_raster_info* info, bool touched) {
  Grid gr;
  gr.xmin = info->xmin;
  gr.ymax = info->ymax;
  gr.xres = info->xres;
  gr.yres = info->yres;
  gr.pow2_x = is_pow2(info->xres);
  gr.pow2_y = is_pow2(info->yres);
  gr.inv_xres = gr.pow2_x ? 1.0 / info->xres : 0.0;
  gr.inv_yres = gr.pow2_y ? 1.0 / info->yres : 0.0;
  gr.unit_x = info->xres == 1.0;
  gr.unit_y = info->yres == 1.0;
  gr.touched = touched ? 1 : 0;
  return gr;
}

// PixelCache use (burn_geometry.rs:179-185, 212-243; prelude.rs:116-118):
// the writes of a part are deduplicated for sum / count when the pixels are
// not square (line parts) or all_touched is on (line and polygon parts).
bool fill_dedup(const rz_raster_info* info, rz_pixel_fn fn, bool touched) {
  return (info->xres != info->yres || touched) && (fn == RZ_SUM || fn == RZ_COUNT);
}

// The raster of one job.  The sparse stream also drops the repeats of
// non-square line pixels for the other functions, which LineString::burn's
// PixelCache drops, although the dense result does not depend on them.
JobDims job_dims(unsigned long long nrows, unsigned long long ncols, const rz_raster_info* info, rz_pixel_fn fn,
                 bool touched, bool sparse, unsigned wid_base, unsigned long long geom0) {
  const bool line_dedup = info->xres != info->yres;
  const bool dedup = fill_dedup(info, fn, touched);
  JobDims jd;
  jd.nrows = (int)nrows;
  jd.ncols = (int)ncols;
  jd.ntx = (unsigned)((ncols + TW - 1) >> TW_SHIFT);
  jd.wid_base = wid_base;
  jd.line_flag = (dedup || (sparse && line_dedup)) ? DEDUP_BIT : 0u;
  jd.poly_flag = touched && dedup ? DEDUP_BIT : 0u;
  jd.geom0 = geom0;
  jd.row_lo = 0;  // the whole raster
  jd.row_hi = (int)nrows;
  jd.band_lo = 0;
  jd.band_hi = 0xFFFFFFFFu;
  return jd;
}

void set_background(FillArgs& fa, unsigned long long bits, size_t tsize) {
  fa.bg = bits;
  unsigned char pat[16];
  for (int i = 0; i < 16; i += (int)tsize) std::memcpy(pat + i, &bits, tsize);
  std::memcpy(&fa.bg16, pat, 16);
}

// Device tables of the part map.
struct PartTables {
  unsigned* part_geom;
  PartPlan* plan;
  unsigned long long* counts;  // [P][PC_N]
  unsigned long long* poff;    // [P+1][PC_N]
  unsigned long long* tmp64;   // scan scratch
  unsigned* line_parts;
  unsigned* point_parts;
  unsigned long long* last_kept;
};

// A schedule resolved for one device: the context's rz_tuning with its
// defaults filled in and clamped to what the kernels allow.
struct Sched {
  int sms = 1;
  int narrow_bps = 1, wide_bps = 1;  // span kernels, blocks per SM
  int scatter_bps = 8, line_bps = 8;
  Tune tune{4, WR_MAX, SMALL_BW, FILL_WARP_SORT};
};

int clamp_i(long v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : (int)v); }

// Defaults for 0 fields; the occupancy limits of the span kernels bound their grids.
Sched resolve_sched(const rz_tuning& t, int sms, int narrow_occ, int wide_occ) {
  Sched sc;
  sc.sms = sms;
  sc.narrow_bps = t.narrow_blocks_per_sm ? clamp_i(t.narrow_blocks_per_sm, 1, narrow_occ) : narrow_occ;
  sc.wide_bps = t.wide_blocks_per_sm ? clamp_i(t.wide_blocks_per_sm, 1, wide_occ) : wide_occ;
  sc.scatter_bps = t.scatter_blocks_per_sm ? clamp_i(t.scatter_blocks_per_sm, 1, 32) : 8;
  sc.line_bps = t.line_blocks_per_sm ? clamp_i(t.line_blocks_per_sm, 1, 32) : 8;
  sc.tune.narrow_chunk = t.narrow_chunk ? clamp_i(t.narrow_chunk, 1, 64) : 4;
  sc.tune.rows_per_window = t.rows_per_window ? clamp_i(t.rows_per_window, 8, WR_MAX) : WR_MAX;
  sc.tune.narrow_max_words = t.narrow_max_words ? clamp_i(t.narrow_max_words, 1, SMALL_BW) : SMALL_BW;
  sc.tune.fill_sort_max = t.fill_sort_max ? clamp_i(t.fill_sort_max, FILL_WARP_MAX, FILL_WARP_SORT) : FILL_WARP_SORT;
  return sc;
}

// validate -> part -> geometry -> part plans -> scan -> part lists.  Returns
// the kernels launched.
int launch_prep(const Geo& geo, const Grid& gr, const JobDims& one, const JobDims* jobs, unsigned n_jobs,
                unsigned band_check, const PartTables& t, Ctrl* d_ctrl, const Sched& sc, cudaStream_t s) {
  const int sms = sc.sms;
  const unsigned long long G = geo.n_geoms, P = geo.n_parts, R = geo.n_rings;
  int launches = 0;
  const unsigned long long maxn = std::max({G + 1, P + 1, R + 1});
  k_validate<<<grid_for(maxn, 256, sms * 8), 256, 0, s>>>(geo, d_ctrl);
  ++launches;
  if (band_check && G) {
    k_check_bands<<<grid_for(G, 256, sms * 8), 256, 0, s>>>(geo, band_check, d_ctrl);
    ++launches;
  }
  if (G) {
    k_part_geom<<<grid_for(G, 256, sms * 16), 256, 0, s>>>(geo, t.part_geom, d_ctrl);
    ++launches;
  }
  if (P) {
    k_part_prep<<<grid_for(P, 8, sms * 32), 256, 0, s>>>(geo, gr, one, jobs, n_jobs, t.part_geom, t.plan, t.counts,
                                                         sc.tune, d_ctrl);
    ++launches;
  }
  launches += scan<unsigned long long, PC_N>(t.counts, t.poff, P, t.tmp64, s);
  if (P) {
    k_part_lists<<<grid_for(P, 256, sms * 16), 256, 0, s>>>(geo, t.poff, t.line_parts, t.point_parts, d_ctrl);
    ++launches;
  }
  return launches;
}

// Coverage records of every part kind.  Returns the kernels launched.
int launch_coverage(const Geo& geo, const Grid& gr, const PartTables& t, const RecBuf& sb, unsigned* bcount,
                    Ctrl* d_ctrl, const Sched& sc, cudaStream_t s) {
  if (!geo.n_parts) return 0;
  const int sms = sc.sms;
  k_poly_spans_narrow<<<sms * sc.narrow_bps, SMALL_WARPS * 32, SMALL_SMEM, s>>>(geo, gr, t.plan, t.poff, sb, bcount,
                                                                                sc.tune.narrow_chunk, d_ctrl);
  k_poly_spans<<<sms * sc.wide_bps, POLY_THREADS, POLY_SMEM, s>>>(geo, gr, t.plan, t.poff, sb, bcount, d_ctrl);
  k_line_spans<<<sms * sc.line_bps, 256, 0, s>>>(geo, gr, t.plan, t.poff, t.line_parts, t.last_kept, sb, bcount,
                                                 d_ctrl);
  int launches = 4;
  if (!gr.touched) {  // AllTouched writes no separate end pixel
    k_line_endpix<<<grid_for(geo.n_parts, 256, sms * 4), 256, 0, s>>>(geo, gr, t.plan, t.poff, t.line_parts,
                                                                       t.last_kept, sb, bcount, d_ctrl);
    ++launches;
  }
  k_point_spans<<<sms * sc.line_bps, 256, 0, s>>>(geo, gr, t.plan, t.poff, t.point_parts, sb, bcount, d_ctrl);
  return launches;
}

}  // namespace

// A dense burn into host memory runs its fill in this many row bands, and
// copies each band to the host on the context's copy stream while the next
// band fills.
constexpr int kFillBands = 8;

// A host array that is not zero-filled: a sparse result's columns are
// written whole by the copies from the device.
struct HostArray {
  unsigned char* p = nullptr;
  size_t bytes = 0;
  HostArray() = default;
  HostArray(const HostArray&) = delete;
  HostArray& operator=(const HostArray&) = delete;
  ~HostArray() { std::free(p); }
  bool alloc(size_t n) {
    std::free(p);
    p = static_cast<unsigned char*>(std::malloc(n ? n : 1));
    bytes = p ? n : 0;
    return p != nullptr;
  }
};

// Host copy of a sparse (COO) result.
struct rz_sparse {
  std::vector<uint64_t> band_counts;
  HostArray rows, cols, values;
  uint64_t count = 0;
  uint32_t n_bands = 1;
  rz_dtype dtype = RZ_F64;
};

struct rz_context {
  int device = 0;
  int num_sms = 0;
  int poly_blocks_per_sm = 1;    // occupancy limits of the span kernels
  int narrow_blocks_per_sm = 1;
  rz_tuning tuning{};            // the schedule (0 fields: defaults)
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // device->host copies that overlap the fill
  cudaEvent_t band_ev[kFillBands + 1] = {};
  DevBuf main, spans, out, sparse, batch, stage;
  cudaEvent_t ev[9] = {};
  Ctrl* h_ctrl = nullptr;  // pinned
  unsigned long long span_cap_hint = 0;
  unsigned char* h_stage = nullptr;  // pinned staging of batch tables and host job inputs
  size_t h_stage_cap = 0;
};

extern "C" const char* rz_build_info(void) {
  static char buf[128];
  int rt = 0;
  cudaRuntimeGetVersion(&rt);
  snprintf(buf, sizeof(buf), "rusterize_gb300 abi %d; sm_103a; cuda runtime %d", RZ_ABI_VERSION, rt);
  return buf;
}

#define RZ_CUDA(call)                                                                               \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess)                                                                          \
      return fail(err, errlen, e_ == cudaErrorMemoryAllocation ? RZ_OUT_OF_MEMORY : RZ_CUDA_ERROR, \
                  "CUDA error %s (%s) at %s:%d", cudaGetErrorName(e_), cudaGetErrorString(e_),       \
                  __FILE__, __LINE__);                                                              \
  } while (0)

extern "C" rz_status rz_context_create(int device, rz_context** out, char* err, size_t errlen) {
  rz::clear_err(err, errlen);
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(err, errlen, RZ_NO_DEVICE,
                "no CUDA device available (%s); the GB300 engine has no CPU fallback",
                e != cudaSuccess ? cudaGetErrorString(e) : "device count is 0");
  }
  if (device < 0 || device >= n) return fail(err, errlen, RZ_NO_DEVICE, "CUDA device %d does not exist", device);
  auto* ctx = new rz_context();
  ctx->device = device;
  cudaError_t e2 = cudaSetDevice(device);
  if (e2 == cudaSuccess) e2 = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e2 == cudaSuccess) e2 = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e2 == cudaSuccess) e2 = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
  for (int i = 0; i <= kFillBands && e2 == cudaSuccess; ++i)
    e2 = cudaEventCreateWithFlags(&ctx->band_ev[i], cudaEventDisableTiming);
  for (int i = 0; i < 9 && e2 == cudaSuccess; ++i) e2 = cudaEventCreate(&ctx->ev[i]);
  if (e2 == cudaSuccess) e2 = cudaMallocHost((void**)&ctx->h_ctrl, sizeof(Ctrl));
  if (e2 == cudaSuccess)
    e2 = cudaFuncSetAttribute(k_poly_spans, cudaFuncAttributeMaxDynamicSharedMemorySize, POLY_SMEM);
  if (e2 == cudaSuccess)
    e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->poly_blocks_per_sm, k_poly_spans, POLY_THREADS,
                                                       POLY_SMEM);
  if (e2 != cudaSuccess) {
    rz_context_destroy(ctx);
    return fail(err, errlen, RZ_NO_DEVICE, "CUDA initialisation failed: %s", cudaGetErrorString(e2));
  }
  if (e2 == cudaSuccess)
    e2 = cudaFuncSetAttribute(k_poly_spans_narrow, cudaFuncAttributeMaxDynamicSharedMemorySize, SMALL_SMEM);
  if (e2 == cudaSuccess)
    e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->narrow_blocks_per_sm, k_poly_spans_narrow,
                                                       SMALL_WARPS * 32, SMALL_SMEM);
  if (e2 != cudaSuccess) {
    rz_context_destroy(ctx);
    return fail(err, errlen, RZ_NO_DEVICE, "CUDA initialisation failed: %s", cudaGetErrorString(e2));
  }
  if (ctx->poly_blocks_per_sm < 1) ctx->poly_blocks_per_sm = 1;
  if (ctx->narrow_blocks_per_sm < 1) ctx->narrow_blocks_per_sm = 1;
  *out = ctx;
  return RZ_OK;
}

extern "C" void rz_context_destroy(rz_context* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (DevBuf* b : {&ctx->main, &ctx->spans, &ctx->out, &ctx->sparse, &ctx->batch, &ctx->stage})
    if (b->p) cudaFree(b->p);
  if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : ctx->band_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->h_ctrl) cudaFreeHost(ctx->h_ctrl);
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  delete ctx;
}

extern "C" rz_status rz_context_trim(rz_context* ctx) {
  if (!ctx) return RZ_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (DevBuf* b : {&ctx->main, &ctx->spans, &ctx->out, &ctx->sparse, &ctx->batch, &ctx->stage}) {
    if (b->p) cudaFree(b->p);
    b->p = nullptr;
    b->cap = 0;
  }
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  ctx->h_stage = nullptr;
  ctx->h_stage_cap = 0;
  ctx->span_cap_hint = 0;
  return RZ_OK;
}

extern "C" rz_status rz_context_get_tuning(rz_context* ctx, rz_tuning* out) {
  if (!ctx || !out) return RZ_INVALID_ARGUMENT;
  // the settings in force, defaults filled in
  const Sched sc = resolve_sched(ctx->tuning, ctx->num_sms, ctx->narrow_blocks_per_sm, ctx->poly_blocks_per_sm);
  out->narrow_chunk = (uint32_t)sc.tune.narrow_chunk;
  out->narrow_blocks_per_sm = (uint32_t)sc.narrow_bps;
  out->wide_blocks_per_sm = (uint32_t)sc.wide_bps;
  out->rows_per_window = (uint32_t)sc.tune.rows_per_window;
  out->narrow_max_words = (uint32_t)sc.tune.narrow_max_words;
  out->fill_sort_max = (uint32_t)sc.tune.fill_sort_max;
  out->scatter_blocks_per_sm = (uint32_t)sc.scatter_bps;
  out->line_blocks_per_sm = (uint32_t)sc.line_bps;
  return RZ_OK;
}

extern "C" rz_status rz_context_set_tuning(rz_context* ctx, const rz_tuning* t, char* err, size_t errlen) {
  rz::clear_err(err, errlen);
  if (!ctx) return fail(err, errlen, RZ_INVALID_ARGUMENT, "null context");
  if (!t) {
    ctx->tuning = rz_tuning{};
    return RZ_OK;
  }
  struct Range {
    const char* name;
    uint32_t v, lo, hi;
  };
  const Range ranges[] = {
      {"narrow_chunk", t->narrow_chunk, 1, 64},
      {"narrow_blocks_per_sm", t->narrow_blocks_per_sm, 1, (uint32_t)ctx->narrow_blocks_per_sm},
      {"wide_blocks_per_sm", t->wide_blocks_per_sm, 1, (uint32_t)ctx->poly_blocks_per_sm},
      {"rows_per_window", t->rows_per_window, 8, (uint32_t)WR_MAX},
      {"narrow_max_words", t->narrow_max_words, 1, (uint32_t)SMALL_BW},
      {"fill_sort_max", t->fill_sort_max, (uint32_t)FILL_WARP_MAX, (uint32_t)FILL_WARP_SORT},
      {"scatter_blocks_per_sm", t->scatter_blocks_per_sm, 1, 32},
      {"line_blocks_per_sm", t->line_blocks_per_sm, 1, 32},
  };
  for (const Range& r : ranges)
    if (r.v != 0 && (r.v < r.lo || r.v > r.hi))
      return fail(err, errlen, RZ_INVALID_ARGUMENT, "%s = %u is outside [%u, %u]", r.name, r.v, r.lo, r.hi);
  ctx->tuning = *t;
  return RZ_OK;
}

extern "C" void* rz_context_stream(rz_context* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

extern "C" rz_status rz_context_synchronize(rz_context* ctx, char* err, size_t errlen) {
  rz::clear_err(err, errlen);
  if (!ctx) return fail(err, errlen, RZ_INVALID_ARGUMENT, "null context");
  RZ_CUDA(cudaSetDevice(ctx->device));
  RZ_CUDA(cudaStreamSynchronize(ctx->stream));
  return RZ_OK;
}

__global__ void k_reset_pass(Ctrl* c) {
  c->span_count = 0;
  c->pixel_writes = 0;
  c->crossings = 0;
  c->work = 0;
  c->work_small = 0;
  c->big_count = 0;
  c->fill_work = 0;
}

// After a failed call: wait for any kernels or copies the call had already
// queued, so that the caller may free its buffers once the call returns.
// Host pages of a pageable output that the process has never touched are
// faulted in (and zeroed by the OS) when the device->host copy first writes
// them, which slows that copy several-fold.  While the device burns, host
// threads touch one byte of every page instead, so the copy finds the pages
// resident.  Pinned or registered outputs are resident already and are left
// alone; so are outputs below 64 MiB.
class PageToucher {
 public:
  void start(void* out, size_t bytes) {
    if (!out || bytes < (64u << 20)) return;
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, out) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    if (attr.type != cudaMemoryTypeUnregistered) return;  // pinned, registered, device or managed
    const long pg = sysconf(_SC_PAGESIZE);
    const size_t page = pg > 0 ? (size_t)pg : 4096;
    unsigned hw = std::thread::hardware_concurrency();
    const unsigned n = (unsigned)std::max<size_t>(1, std::min<size_t>({(size_t)(hw ? hw : 1), (size_t)16,
                                                                         bytes / (32u << 20)}));
    volatile unsigned char* base = static_cast<volatile unsigned char*>(out);
    try {
      for (unsigned t = 0; t < n; ++t) {
        const size_t lo = bytes / n * t, hi = t + 1 == n ? bytes : bytes / n * (t + 1);
        threads_.emplace_back([base, lo, hi, page] {
          // the first byte of every page the slice overlaps
          for (size_t o = lo - lo % page; o < hi; o += page) base[o < lo ? lo : o] = 0;
        });
      }
    } catch (...) {  // no thread: the copy faults the pages in itself
    }
  }
  void join() {
    for (auto& t : threads_) t.join();
    threads_.clear();
  }
  ~PageToucher() { join(); }

 private:
  std::vector<std::thread> threads_;
};

static rz_status drain_on_error(cudaStream_t s, rz_status st) {
  if (st != RZ_OK && s) {
    cudaStreamSynchronize(s);
    cudaGetLastError();  // a failed call reports its own error; nothing is left pending
  }
  return st;
}

// One pass of a burn: the bands [b0, b1) and rows [r0, r1) of the raster.
struct PassWin {
  unsigned long long b0, b1, r0, r1;
};

// The burn pipeline shared by the dense and the sparse entry points; with
// `sp` the coverage records are turned into COO triplets instead of being
// scattered into buckets and filled.  Only rows [row_lo, row_hi) of the
// raster are burned (every band), into an output of that many rows per band.
// The geometry is uploaded once; the window is then burned in passes of fewer
// than 2^28 (band, row, tile) buckets each (one pass unless the raster is
// very large), every pass into its own slab of the output.
static rz_status burn_impl(rz_context* ctx, const rz_geoms* g, const void* values, const void* background,
                           const uint32_t* band_of_geom, uint32_t n_bands, const rz_raster_info* info,
                           uint64_t row_lo, uint64_t row_hi, rz_pixel_fn fn, rz_dtype dt, uint32_t flags, void* out,
                           rz_stats* stats, char* err, size_t errlen, rz_sparse* sp) {
  using clk = std::chrono::steady_clock;
  const auto t_host0 = clk::now();
  rz::clear_err(err, errlen);
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (!ctx || !g || !info || (!sp && (!background || !out)))
    return fail(err, errlen, RZ_INVALID_ARGUMENT, "null argument");
  const size_t tsize = rz_dtype_size(dt);
  if (tsize == 0) return fail(err, errlen, RZ_VALUE_ERROR, "Unsupported dtype");
  if ((int)fn < 0 || (int)fn > 6) return fail(err, errlen, RZ_VALUE_ERROR, "Unknown pixel function");
  if (band_of_geom && n_bands == 0) return fail(err, errlen, RZ_INVALID_ARGUMENT, "n_bands must be > 0");
  const bool in_dev = flags & RZ_FLAG_INPUT_DEVICE, out_dev = flags & RZ_FLAG_OUTPUT_DEVICE;
  const bool timing = !(flags & RZ_FLAG_NO_TIMING);
  const unsigned long long nb = band_of_geom ? n_bands : 1;
  if (info->nrows >= (1ull << 31) - 1 || info->ncols >= (1ull << 31) - 1)
    return fail(err, errlen, RZ_VALUE_ERROR, "raster dimensions must be below 2^31-1");
  const unsigned long long nrows = info->nrows, ncols = info->ncols;
  if (row_lo > row_hi || row_hi > nrows)
    return fail(err, errlen, RZ_INVALID_ARGUMENT, "row window [%llu, %llu) is outside the raster's %llu rows",
                (unsigned long long)row_lo, (unsigned long long)row_hi, nrows);
  const unsigned long long wrows = row_hi - row_lo;
  const unsigned long long out_elems = nb * wrows * ncols;
  const unsigned ntx = (unsigned)((ncols + TW - 1) >> TW_SHIFT);
  // passes of fewer than 2^28 buckets: the whole window, or one band and a
  // run of its rows at a time
  constexpr unsigned long long kMaxBuckets = (1ull << 28) - 1;
  std::vector<PassWin> passes;
  if (nb * wrows * ntx <= kMaxBuckets) {
    passes.push_back({0, nb, row_lo, row_hi});
  } else {
    if (sp) return fail(err, errlen, RZ_VALUE_ERROR, "raster too large: more than 2^28 (band,row,tile) buckets");
    const unsigned long long rc = std::max<unsigned long long>(1, kMaxBuckets / std::max(1u, ntx));
    for (unsigned long long b = 0; b < nb; ++b)
      for (unsigned long long r0 = row_lo; r0 < row_hi; r0 += rc) passes.push_back({b, b + 1, r0, std::min(r0 + rc, (unsigned long long)row_hi)});
  }
  unsigned long long max_buckets = 0, pass_elems = 0;  // the largest pass
  for (const PassWin& w : passes) {
    max_buckets = std::max(max_buckets, (w.b1 - w.b0) * (w.r1 - w.r0) * ntx);
    pass_elems = std::max(pass_elems, (w.b1 - w.b0) * (w.r1 - w.r0) * ncols);
  }
  const unsigned long long G = g->n_geoms, P = g->n_parts, R = g->n_rings, V = g->n_vertices;
  if (G >= 0xFFFFFFFFull || P >= (1ull << 27))
    return fail(err, errlen, RZ_VALUE_ERROR, "at most 2^32-1 geometries and 2^27 parts are supported");
  if (!g->part_offsets || !g->part_kind || !g->ring_offsets || !g->vertex_offsets || (V && !g->xy))
    return fail(err, errlen, RZ_INVALID_ARGUMENT, "geometry table has null arrays");
  if (in_dev && (reinterpret_cast<uintptr_t>(g->xy) & 15))
    return fail(err, errlen, RZ_INVALID_ARGUMENT, "device xy must be 16-byte aligned");
  if (!in_dev) {
    if (g->part_offsets[0] != 0 || g->part_offsets[G] != P || g->ring_offsets[P] != R ||
        g->vertex_offsets[R] != V)
      return fail(err, errlen, RZ_INVALID_ARGUMENT, "geometry table sizes are inconsistent");
  }
  unsigned long long bg_bits = 0, scalar_bits = one_bits(dt);
  if (background) std::memcpy(&bg_bits, background, tsize);
  const bool per_geom_values = values && !(flags & RZ_FLAG_SCALAR_VALUE);
  if (values && (flags & RZ_FLAG_SCALAR_VALUE)) {
    scalar_bits = 0;
    std::memcpy(&scalar_bits, values, tsize);
  }
  if (stats) stats->out_bytes = out_elems * tsize;
  if (sp) {
    sp->n_bands = (uint32_t)nb;
    sp->dtype = dt;
    sp->band_counts.assign(nb, 0);
  }
  if (out_elems == 0) return RZ_OK;

  RZ_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;

  // ---- scratch layout ----
  Layout L;
  size_t o_po = 0, o_pk = 0, o_ro = 0, o_vo = 0, o_xy = 0, o_val = 0, o_band = 0;
  if (!in_dev) {
    o_po = L.take(8 * (G + 1));
    o_pk = L.take(P ? P : 1);
    o_ro = L.take(8 * (P + 1));
    o_vo = L.take(8 * (R + 1));
    o_xy = L.take(16 * (V ? V : 1));
    if (per_geom_values) o_val = L.take(tsize * (G ? G : 1));
    if (band_of_geom) o_band = L.take(4 * (G ? G : 1));
  }
  const size_t o_pg = L.take(4 * (P ? P : 1));
  const size_t o_pval = L.take(tsize * (P ? P : 1));
  const size_t o_plan = L.take(sizeof(PartPlan) * (P ? P : 1));
  const size_t o_cnt = L.take(8 * PC_N * (P ? P : 1));
  const size_t o_poff = L.take(8 * PC_N * (P + 1));
  const size_t o_tmp64 = L.take(8 * scan_temp_elems(P, PC_N));
  const size_t o_last = L.take(8 * (P ? P : 1));
  const size_t o_lp = L.take(4 * (P ? P : 1));
  const size_t o_pp = L.take(4 * (P ? P : 1));
  const size_t o_bc = L.take(4 * max_buckets);
  const size_t o_boff = L.take(4 * (max_buckets + 1));
  const size_t o_tmp32 = L.take(4 * scan_temp_elems(max_buckets, 1));
  const size_t o_big = L.take(4 * max_buckets);
  const size_t o_ctrl = L.take(sizeof(Ctrl));
  const size_t o_bandctr = L.take(16 * kFillBands);  // work / big counters of the fill bands
  RZ_CUDA(ensure(ctx->main, L.off));
  if (!out_dev && !sp) RZ_CUDA(ensure(ctx->out, pass_elems * tsize));
  unsigned long long cap = rzl::record_cap_request(std::max<unsigned long long>(ctx->span_cap_hint, 2 * V + (1ull << 20)));

  char* mb = static_cast<char*>(ctx->main.p);
  auto at = [&](size_t o) { return static_cast<void*>(mb + o); };
  Geo geo;
  geo.n_geoms = G;
  geo.n_parts = P;
  geo.n_rings = R;
  geo.n_vertices = V;
  const void* d_values = per_geom_values ? values : nullptr;
  if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[0], s));
  if (!in_dev) {
    RZ_CUDA(cudaMemcpyAsync(at(o_po), g->part_offsets, 8 * (G + 1), cudaMemcpyHostToDevice, s));
    if (P) RZ_CUDA(cudaMemcpyAsync(at(o_pk), g->part_kind, P, cudaMemcpyHostToDevice, s));
    RZ_CUDA(cudaMemcpyAsync(at(o_ro), g->ring_offsets, 8 * (P + 1), cudaMemcpyHostToDevice, s));
    RZ_CUDA(cudaMemcpyAsync(at(o_vo), g->vertex_offsets, 8 * (R + 1), cudaMemcpyHostToDevice, s));
    if (V) RZ_CUDA(cudaMemcpyAsync(at(o_xy), g->xy, 16 * V, cudaMemcpyHostToDevice, s));
    if (per_geom_values && G) {
      RZ_CUDA(cudaMemcpyAsync(at(o_val), values, tsize * G, cudaMemcpyHostToDevice, s));
      d_values = at(o_val);
    }
    if (band_of_geom && G) RZ_CUDA(cudaMemcpyAsync(at(o_band), band_of_geom, 4 * G, cudaMemcpyHostToDevice, s));
    geo.part_offsets = static_cast<const unsigned long long*>(at(o_po));
    geo.part_kind = static_cast<const unsigned char*>(at(o_pk));
    geo.ring_offsets = static_cast<const unsigned long long*>(at(o_ro));
    geo.vertex_offsets = static_cast<const unsigned long long*>(at(o_vo));
    geo.xy = static_cast<const double2*>(at(o_xy));
    geo.bands = band_of_geom ? static_cast<const unsigned*>(at(o_band)) : nullptr;
  } else {
    geo.part_offsets = reinterpret_cast<const unsigned long long*>(g->part_offsets);
    geo.part_kind = g->part_kind;
    geo.ring_offsets = reinterpret_cast<const unsigned long long*>(g->ring_offsets);
    geo.vertex_offsets = reinterpret_cast<const unsigned long long*>(g->vertex_offsets);
    geo.xy = reinterpret_cast<const double2*>(g->xy);
    geo.bands = band_of_geom;
  }
  if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[8], s));
  PageToucher toucher;  // joined before the first device->host copy (or on return)
  if (!out_dev && !sp) toucher.start(out, (size_t)(out_elems * tsize));

  const bool touched = (flags & RZ_FLAG_ALL_TOUCHED) != 0;
  const Grid gr = make_grid(info, touched);
  const bool dedup = fill_dedup(info, fn, touched);

  Ctrl* d_ctrl = static_cast<Ctrl*>(at(o_ctrl));
  unsigned* part_geom = static_cast<unsigned*>(at(o_pg));
  PartPlan* plan = static_cast<PartPlan*>(at(o_plan));
  unsigned long long* counts = static_cast<unsigned long long*>(at(o_cnt));
  unsigned long long* poff = static_cast<unsigned long long*>(at(o_poff));
  unsigned long long* last_kept = static_cast<unsigned long long*>(at(o_last));
  unsigned* line_parts = static_cast<unsigned*>(at(o_lp));
  unsigned* point_parts = static_cast<unsigned*>(at(o_pp));
  unsigned* bcount = static_cast<unsigned*>(at(o_bc));
  unsigned* boff = static_cast<unsigned*>(at(o_boff));
  unsigned* big = static_cast<unsigned*>(at(o_big));
  const int sms = ctx->num_sms;
  const Sched sched = resolve_sched(ctx->tuning, sms, ctx->narrow_blocks_per_sm, ctx->poly_blocks_per_sm);
  int launches = 0;
  unsigned reruns = 0;
  const fill_fn fill = fill_for(dt);
  float ms_acc[4] = {0.f, 0.f, 0.f, 0.f};  // prep, spans, bucket, fill over the passes
  unsigned long long pass_buckets = 0;

  for (const PassWin& pw : passes) {
    const unsigned long long nbuckets = (pw.b1 - pw.b0) * (pw.r1 - pw.r0) * ntx;
    pass_buckets += nbuckets;
    // this pass's slab of the output: band b0, row r0 of the window
    const size_t out_off = (size_t)((pw.b0 * wrows + (pw.r0 - row_lo)) * ncols * tsize);
    void* d_out = out_dev ? static_cast<void*>(static_cast<char*>(out) + out_off) : ctx->out.p;
    JobDims one = job_dims(nrows, ncols, info, fn, touched, sp != nullptr, 0u, 0ull);
    one.row_lo = (int)pw.r0;
    one.row_hi = (int)pw.r1;
    one.band_lo = (unsigned)pw.b0;
    one.band_hi = (unsigned)pw.b1;
    if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[1], s));

    // ---- prep ----
    RZ_CUDA(cudaMemsetAsync(d_ctrl, 0, sizeof(Ctrl), s));
    PartTables pt;
    pt.part_geom = part_geom;
    pt.plan = plan;
    pt.counts = counts;
    pt.poff = poff;
    pt.tmp64 = static_cast<unsigned long long*>(at(o_tmp64));
    pt.line_parts = line_parts;
    pt.point_parts = point_parts;
    pt.last_kept = last_kept;
    launches += launch_prep(geo, gr, one, nullptr, 1, band_of_geom ? (unsigned)nb : 0u, pt, d_ctrl, sched, s);
    if (d_values && !sp && P) {
      launch_part_values(tsize, sms, s, part_geom, d_values, P, at(o_pval), d_ctrl);
      ++launches;
    }
    RZ_CUDA(cudaMemsetAsync(last_kept, 0, 8 * (P ? P : 1), s));
    if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[2], s));
    bool copied = false;  // the fill bands copied the pass's slab to the host

    while (true) {
      RZ_CUDA(ensure(ctx->spans, rzl::record_bytes_for(cap)));
      const rzl::RecordLayout RL = rzl::record_layout(ctx->spans.cap);  // the whole buffer: cap or more
      cap = RL.cap;
      if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[7], s));
      char* rbase = static_cast<char*>(ctx->spans.p);
      RecBuf sb;
      sb.cap = cap;
      sb.nbuckets = nbuckets;
      sb.wid = reinterpret_cast<unsigned*>(rbase + RL.off_wid);
      sb.part = reinterpret_cast<unsigned*>(rbase + RL.off_part);
      sb.mask = reinterpret_cast<unsigned*>(rbase + RL.off_mask);
      uint2* sorted = reinterpret_cast<uint2*>(rbase + RL.off_sorted);
      k_reset_pass<<<1, 1, 0, s>>>(d_ctrl);
      RZ_CUDA(cudaMemsetAsync(bcount, 0, 4 * nbuckets, s));
      launches += 1;
      launches += launch_coverage(geo, gr, pt, sb, bcount, d_ctrl, sched, s);
      if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[3], s));
      if (!sp) {
        launches += scan<unsigned, 1>(bcount, boff, nbuckets, static_cast<unsigned*>(at(o_tmp32)), s);
        launch_scatter(sms, sched.scatter_bps, s, sb, boff, bcount, sorted, d_ctrl);
        ++launches;
        if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[4], s));
        FillArgs fa;
        fa.offsets = boff;
        fa.recs = sorted;
        fa.brecs = reinterpret_cast<uint2*>(sb.wid);  // free once the records are scattered
        fa.pvals = d_values ? at(o_pval) : nullptr;
        fa.nbuckets = nbuckets;
        fa.scalar = scalar_bits;
        fa.out = d_out;
        set_background(fa, bg_bits, tsize);
        fa.nrows = (int)((pw.b1 - pw.b0) * (pw.r1 - pw.r0));  // rows of the pass's band stack
        fa.ncols = (int)ncols;
        fa.ntx = ntx;
        fa.big = big;
        fa.ctrl = d_ctrl;
        fa.rec_cap = cap;
        fa.sort_max = sched.tune.fill_sort_max;
        fa.work = &d_ctrl->fill_work;
        fa.nbig = &d_ctrl->big_count;
        fa.jobs = nullptr;
        fa.n_jobs = 0;
        fa.bucket0 = 0;
        // one pass into host memory: fill row bands, then copy each band to
        // the host on the copy stream as soon as its fill is done
        const unsigned long long brows = (pw.b1 - pw.b0) * (pw.r1 - pw.r0);  // rows of the band stack
        const int nbands = (!out_dev && passes.size() == 1 && brows >= (unsigned long long)kFillBands * 64)
                               ? kFillBands : 1;
        if (nbands == 1) {
          launches += fill(fa, (int)fn, dedup, sms, s);
        } else {
          unsigned char* bctr = static_cast<unsigned char*>(at(o_bandctr));
          RZ_CUDA(cudaMemsetAsync(bctr, 0, 16 * kFillBands, s));
          for (int k = 0; k < nbands; ++k) {
            const unsigned long long r_lo = brows * k / nbands, r_hi = brows * (k + 1) / nbands;
            FillArgs fb = fa;
            fb.offsets = boff + r_lo * ntx;
            fb.nbuckets = (r_hi - r_lo) * ntx;
            fb.bucket0 = r_lo * ntx;
            fb.big = big + r_lo * ntx;
            fb.work = reinterpret_cast<unsigned long long*>(bctr + 16 * k);
            fb.nbig = reinterpret_cast<unsigned*>(bctr + 16 * k + 8);
            launches += fill(fb, (int)fn, dedup, sms, s);
            RZ_CUDA(cudaEventRecord(ctx->band_ev[k], s));
          }
          toucher.join();  // the host pages are resident before the first copy
          const size_t row_bytes = (size_t)ncols * tsize;
          for (int k = 0; k < nbands; ++k) {
            const unsigned long long r_lo = brows * k / nbands, r_hi = brows * (k + 1) / nbands;
            RZ_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->band_ev[k], 0));
            RZ_CUDA(cudaMemcpyAsync(static_cast<char*>(out) + out_off + r_lo * row_bytes,
                                    static_cast<char*>(d_out) + r_lo * row_bytes, (r_hi - r_lo) * row_bytes,
                                    cudaMemcpyDeviceToHost, ctx->copy_stream));
          }
          RZ_CUDA(cudaEventRecord(ctx->band_ev[kFillBands], ctx->copy_stream));
          copied = true;
        }
      }
      RZ_CUDA(cudaGetLastError());
      if (timing) {
        if (sp) RZ_CUDA(cudaEventRecord(ctx->ev[4], s));
        RZ_CUDA(cudaEventRecord(ctx->ev[5], s));
      }
      if (copied) RZ_CUDA(cudaStreamWaitEvent(s, ctx->band_ev[kFillBands], 0));  // the band copies are done
      RZ_CUDA(cudaMemcpyAsync(ctx->h_ctrl, d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
      RZ_CUDA(cudaStreamSynchronize(s));
      const Ctrl& hc = *ctx->h_ctrl;
      if (hc.err) return ctrl_error(hc, err, errlen);
      if (hc.span_count > cap) {
        cap = rzl::record_cap_regrow(hc.span_count);
        if (cap == 0) return fail(err, errlen, RZ_VALUE_ERROR, "more than 2^32 coverage records in one call");
        ++reruns;
        continue;
      }
      ctx->span_cap_hint = std::max(ctx->span_cap_hint, cap);  // only once a pass fitted
      if (stats) {
        stats->edges += hc.edges;
        stats->crossings += hc.crossings;
        stats->spans += hc.span_count;
        stats->pixel_writes += hc.pixel_writes;
        stats->big_buckets += hc.big_count;
      }
      if (timing) {
        float t[4] = {0.f, 0.f, 0.f, 0.f};
        cudaEventElapsedTime(&t[0], ctx->ev[1], ctx->ev[2]);
        cudaEventElapsedTime(&t[1], ctx->ev[7], ctx->ev[3]);
        cudaEventElapsedTime(&t[2], ctx->ev[3], ctx->ev[4]);
        cudaEventElapsedTime(&t[3], ctx->ev[4], ctx->ev[5]);
        for (int k = 0; k < 4; ++k) ms_acc[k] += t[k];
      }
      break;
    }
    if (sp) {
      // ---- sparse: order the records by (band, part, row, word), expand ----
      const unsigned long long n = ctx->h_ctrl->span_count;
      const rzl::RecordLayout RL = rzl::record_layout(ctx->spans.cap);
      char* rbase = static_cast<char*>(ctx->spans.p);
      RecBuf sbr;
      sbr.cap = cap;
      sbr.nbuckets = nbuckets;
      sbr.wid = reinterpret_cast<unsigned*>(rbase + RL.off_wid);
      sbr.part = reinterpret_cast<unsigned*>(rbase + RL.off_part);
      sbr.mask = reinterpret_cast<unsigned*>(rbase + RL.off_mask);
      const unsigned long long nsort = std::max<unsigned long long>(n, nb > 1 ? P : 0);
      Layout SL;
      const size_t o_k0 = SL.take(8 * (nsort ? nsort : 1)), o_k1 = SL.take(8 * (nsort ? nsort : 1));
      const size_t o_v0 = SL.take(4 * (nsort ? nsort : 1)), o_v1 = SL.take(4 * (nsort ? nsort : 1));
      const size_t o_pr = SL.take(4 * (P ? P : 1));
      const size_t o_eff = SL.take(4 * (n ? n : 1));
      const size_t o_cnt2 = SL.take(8 * (n + 1));
      const size_t o_off2 = SL.take(8 * (n + 1));
      const size_t o_st64 = SL.take(8 * scan_temp_elems(n ? n : 1, 1));
      const size_t o_rst = SL.take(4 * radix_sort_temp_words(nsort ? nsort : 1));
      const size_t o_bc = SL.take(8 * nb);
      const size_t base_bytes = SL.off;
      RZ_CUDA(ensure(ctx->sparse, base_bytes));
      char* sbase = static_cast<char*>(ctx->sparse.p);
      auto sat = [&](size_t o) { return static_cast<void*>(sbase + o); };
      unsigned long long* k0 = static_cast<unsigned long long*>(sat(o_k0));
      unsigned long long* k1 = static_cast<unsigned long long*>(sat(o_k1));
      unsigned* v0 = static_cast<unsigned*>(sat(o_v0));
      unsigned* v1 = static_cast<unsigned*>(sat(o_v1));
      unsigned* prank = nullptr;
      int bits_part = 1;
      while ((1ull << bits_part) < P) ++bits_part;
      if (nb > 1 && P) {  // band-major rank of every part
        k_part_band_keys<<<grid_for(P, 256, sms * 16), 256, 0, s>>>(plan, P, k0, v0);
        int bits_band = 1;
        while ((1ull << bits_band) < nb) ++bits_band;
        const bool in_tmp = radix_sort(k0, v0, k1, v1, (unsigned)P, 32 + bits_band,
                                       static_cast<unsigned*>(sat(o_rst)), s, launches);
        prank = static_cast<unsigned*>(sat(o_pr));
        k_part_rank<<<grid_for(P, 256, sms * 16), 256, 0, s>>>(in_tmp ? v1 : v0, P, prank);
        launches += 2;
      }
      unsigned long long* skeys = k0;
      unsigned* svals = v0;
      unsigned long long total = 0;
      unsigned long long* bcnt = static_cast<unsigned long long*>(sat(o_bc));
      RZ_CUDA(cudaMemsetAsync(bcnt, 0, 8 * nb, s));
      if (n) {
        k_rec_keys<<<grid_for(n, 256, sms * 16), 256, 0, s>>>(sbr, n, prank, plan, k0, v0);
        const bool in_tmp = radix_sort(k0, v0, k1, v1, (unsigned)n, 32 + bits_part,
                                       static_cast<unsigned*>(sat(o_rst)), s, launches);
        skeys = in_tmp ? k1 : k0;
        svals = in_tmp ? v1 : v0;
        unsigned* eff = static_cast<unsigned*>(sat(o_eff));
        unsigned long long* cnt = static_cast<unsigned long long*>(sat(o_cnt2));
        unsigned long long* off = static_cast<unsigned long long*>(sat(o_off2));
        k_sparse_count<<<grid_for(n, 256, sms * 16), 256, 0, s>>>(skeys, svals, n, sbr, eff, cnt);
        launches += 2 + scan<unsigned long long, 1>(cnt, off, n, static_cast<unsigned long long*>(sat(o_st64)), s);
        RZ_CUDA(cudaMemcpyAsync(&total, off + n, 8, cudaMemcpyDeviceToHost, s));
        RZ_CUDA(cudaStreamSynchronize(s));
        sp->count = total;
        if (!sp->rows.alloc(8 * total) || !sp->cols.alloc(8 * total) || !sp->values.alloc(tsize * total))
          return fail(err, errlen, RZ_OUT_OF_MEMORY, "cannot allocate %llu sparse triplets on the host", total);
        // their pages are faulted in by host threads while the device emits
        PageToucher touch_rows, touch_cols, touch_vals;
        touch_rows.start(sp->rows.p, 8 * total);
        touch_cols.start(sp->cols.p, 8 * total);
        touch_vals.start(sp->values.p, tsize * total);
        if (total) {
          // the triplet arrays go after the sort scratch (grow-only buffer)
          const size_t o_rows = (base_bytes + 255) & ~size_t(255);
          const size_t o_cols = o_rows + ((8 * total + 255) & ~size_t(255));
          const size_t o_vals = o_cols + ((8 * total + 255) & ~size_t(255));
          const size_t need = o_vals + tsize * total;
          if (need > ctx->sparse.cap) {
            // keep the ordered records: copy the live part of the scratch
            DevBuf grown;
            RZ_CUDA(ensure(grown, need));
            RZ_CUDA(cudaMemcpyAsync(grown.p, ctx->sparse.p, base_bytes, cudaMemcpyDeviceToDevice, s));
            RZ_CUDA(cudaStreamSynchronize(s));
            cudaFree(ctx->sparse.p);
            ctx->sparse = grown;
            sbase = static_cast<char*>(ctx->sparse.p);
            skeys = static_cast<unsigned long long*>(sat(in_tmp ? o_k1 : o_k0));
            svals = static_cast<unsigned*>(sat(in_tmp ? o_v1 : o_v0));
            eff = static_cast<unsigned*>(sat(o_eff));
            off = static_cast<unsigned long long*>(sat(o_off2));
            bcnt = static_cast<unsigned long long*>(sat(o_bc));
          }
          unsigned long long* trows = static_cast<unsigned long long*>(sat(o_rows));
          unsigned long long* tcols = static_cast<unsigned long long*>(sat(o_cols));
          void* tvals = sat(o_vals);
          const unsigned eg = grid_for(n, 256, sms * 16);
          switch (tsize) {
            case 1: k_sparse_emit<1><<<eg, 256, 0, s>>>(skeys, svals, n, sbr, eff, off, plan, d_values, part_geom,
                                                        scalar_bits, trows, tcols, tvals, bcnt); break;
            case 2: k_sparse_emit<2><<<eg, 256, 0, s>>>(skeys, svals, n, sbr, eff, off, plan, d_values, part_geom,
                                                        scalar_bits, trows, tcols, tvals, bcnt); break;
            case 4: k_sparse_emit<4><<<eg, 256, 0, s>>>(skeys, svals, n, sbr, eff, off, plan, d_values, part_geom,
                                                        scalar_bits, trows, tcols, tvals, bcnt); break;
            default: k_sparse_emit<8><<<eg, 256, 0, s>>>(skeys, svals, n, sbr, eff, off, plan, d_values,
                                                         part_geom, scalar_bits, trows, tcols, tvals, bcnt); break;
          }
          ++launches;
          RZ_CUDA(cudaGetLastError());
          touch_rows.join();
          touch_cols.join();
          touch_vals.join();
          RZ_CUDA(cudaMemcpyAsync(sp->rows.p, trows, 8 * total, cudaMemcpyDeviceToHost, s));
          RZ_CUDA(cudaMemcpyAsync(sp->cols.p, tcols, 8 * total, cudaMemcpyDeviceToHost, s));
          RZ_CUDA(cudaMemcpyAsync(sp->values.p, tvals, tsize * total, cudaMemcpyDeviceToHost, s));
        }
      }
      RZ_CUDA(cudaMemcpyAsync(sp->band_counts.data(), bcnt, 8 * nb, cudaMemcpyDeviceToHost, s));
      if (stats) stats->pixel_writes = total;
    } else if (!out_dev && !copied) {
      toucher.join();
      const size_t bytes = (size_t)((pw.b1 - pw.b0) * (pw.r1 - pw.r0) * ncols * tsize);
      RZ_CUDA(cudaMemcpyAsync(static_cast<char*>(out) + out_off, d_out, bytes, cudaMemcpyDeviceToHost, s));
    }
    if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[6], s));
    if (passes.size() > 1) RZ_CUDA(cudaStreamSynchronize(s));  // the next pass reuses the output scratch
  }  // passes
  RZ_CUDA(cudaStreamSynchronize(s));
  if (stats) {
    stats->buckets = pass_buckets;
    stats->reruns = reruns;
    stats->kernel_launches = (uint32_t)launches;
    if (timing) {
      cudaEventElapsedTime(&stats->ms_h2d, ctx->ev[0], ctx->ev[8]);
      stats->ms_prep = ms_acc[0];
      stats->ms_spans = ms_acc[1];
      stats->ms_bucket = ms_acc[2];
      stats->ms_fill = ms_acc[3];
      cudaEventElapsedTime(&stats->ms_d2h, ctx->ev[5], ctx->ev[6]);
      cudaEventElapsedTime(&stats->ms_device_total, ctx->ev[0], ctx->ev[6]);
    }
    stats->ms_host_total =
        std::chrono::duration<float, std::milli>(clk::now() - t_host0).count();
  }
  return RZ_OK;
}

extern "C" rz_status rz_rasterize(rz_context* ctx, const rz_geoms* g, const void* values, const void* background,
                                  const uint32_t* band_of_geom, uint32_t n_bands, const rz_raster_info* info,
                                  rz_pixel_fn fn, rz_dtype dt, uint32_t flags, void* out, rz_stats* stats,
                                  char* err, size_t errlen) {
  return drain_on_error(ctx ? ctx->stream : nullptr,
                        burn_impl(ctx, g, values, background, band_of_geom, n_bands, info, 0, info ? info->nrows : 0,
                                  fn, dt, flags, out, stats, err, errlen, nullptr));
}

extern "C" rz_status rz_rasterize_rows(rz_context* ctx, const rz_geoms* g, const void* values,
                                       const void* background, const uint32_t* band_of_geom, uint32_t n_bands,
                                       const rz_raster_info* info, uint64_t row_begin, uint64_t row_end,
                                       rz_pixel_fn fn, rz_dtype dt, uint32_t flags, void* out, rz_stats* stats,
                                       char* err, size_t errlen) {
  return drain_on_error(ctx ? ctx->stream : nullptr,
                        burn_impl(ctx, g, values, background, band_of_geom, n_bands, info, row_begin, row_end, fn,
                                  dt, flags, out, stats, err, errlen, nullptr));
}

extern "C" rz_status rz_rasterize_sparse(rz_context* ctx, const rz_geoms* g, const void* values,
                                         const uint32_t* band_of_geom, uint32_t n_bands,
                                         const rz_raster_info* info, rz_pixel_fn fn, rz_dtype dt, uint32_t flags,
                                         rz_sparse** out, rz_stats* stats, char* err, size_t errlen) {
  rz::clear_err(err, errlen);
  if (!out) return fail(err, errlen, RZ_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (flags & RZ_FLAG_OUTPUT_DEVICE)
    return fail(err, errlen, RZ_INVALID_ARGUMENT, "the sparse encoding returns host arrays");
  auto* sp = new rz_sparse();
  const rz_status st = drain_on_error(ctx ? ctx->stream : nullptr,
                                      burn_impl(ctx, g, values, nullptr, band_of_geom, n_bands, info, 0,
                                                info ? info->nrows : 0, fn, dt, flags, nullptr, stats, err, errlen,
                                                sp));
  if (st != RZ_OK) {
    delete sp;
    return st;
  }
  *out = sp;
  return RZ_OK;
}

extern "C" rz_status rz_sparse_view_get(const rz_sparse* sp, rz_sparse_view* out) {
  if (!sp || !out) return RZ_INVALID_ARGUMENT;
  out->count = sp->count;
  out->n_bands = sp->n_bands;
  out->dtype = sp->dtype;
  out->band_counts = sp->band_counts.data();
  out->rows = reinterpret_cast<const uint64_t*>(sp->rows.p);
  out->cols = reinterpret_cast<const uint64_t*>(sp->cols.p);
  out->values = sp->values.p;
  return RZ_OK;
}

extern "C" void rz_sparse_free(rz_sparse* sp) { delete sp; }

// ---------------------------------------------------------------------------
// Replay of a triplet stream onto a raster (SparseArray::build_array,
// rust/src/encoding/arrays.rs:103-141): chunks of the stream in order, each
// keyed by pixel, stably sorted and folded (rz_replay.cuh).

namespace {

typedef int (*replay_fn)(const ReplayArgs&, int, int, cudaStream_t);

replay_fn replay_for(rz_dtype dt) {
  switch (dt) {
    case RZ_U8: return rz_replay_u8;
    case RZ_U16: return rz_replay_u16;
    case RZ_U32: return rz_replay_u32;
    case RZ_U64: return rz_replay_u64;
    case RZ_I8: return rz_replay_i8;
    case RZ_I16: return rz_replay_i16;
    case RZ_I32: return rz_replay_i32;
    case RZ_I64: return rz_replay_i64;
    case RZ_F32: return rz_replay_f32;
    case RZ_F64: return rz_replay_f64;
  }
  return nullptr;
}

// triplets keyed, sorted and folded at once (56 B of scratch each)
constexpr unsigned long long kReplayChunk = 1ull << 28;

}  // namespace

static rz_status replay_impl(rz_context* ctx, const uint64_t* band_counts, uint32_t n_bands, const uint64_t* rows,
                             const uint64_t* cols, const void* values, uint64_t nrows, uint64_t ncols,
                             rz_pixel_fn fn, rz_dtype dt, const void* background, uint32_t flags, void* out,
                             rz_stats* stats, char* err, size_t errlen) {
  using clk = std::chrono::steady_clock;
  const auto t_host0 = clk::now();
  rz::clear_err(err, errlen);
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (!ctx || !band_counts || !background || !out) return fail(err, errlen, RZ_INVALID_ARGUMENT, "null argument");
  const size_t tsize = rz_dtype_size(dt);
  if (tsize == 0) return fail(err, errlen, RZ_VALUE_ERROR, "Unsupported dtype");
  if ((int)fn < 0 || (int)fn > 6) return fail(err, errlen, RZ_VALUE_ERROR, "Unknown pixel function");
  if (n_bands == 0) return fail(err, errlen, RZ_INVALID_ARGUMENT, "n_bands must be > 0");
  const bool in_dev = flags & RZ_FLAG_INPUT_DEVICE, out_dev = flags & RZ_FLAG_OUTPUT_DEVICE;
  const bool timing = !(flags & RZ_FLAG_NO_TIMING);
  std::vector<unsigned long long> bstart(n_bands + 1ull, 0ull);
  for (uint32_t b = 0; b < n_bands; ++b) {
    bstart[b + 1] = bstart[b] + band_counts[b];
    if (bstart[b + 1] < bstart[b]) return fail(err, errlen, RZ_VALUE_ERROR, "band counts overflow");
  }
  const unsigned long long count = bstart[n_bands];
  if (count && (!rows || !cols || !values)) return fail(err, errlen, RZ_INVALID_ARGUMENT, "null triplet arrays");
  if (in_dev && count &&
      ((reinterpret_cast<uintptr_t>(rows) | reinterpret_cast<uintptr_t>(cols)) & 7 ||
       reinterpret_cast<uintptr_t>(values) % tsize))
    return fail(err, errlen, RZ_INVALID_ARGUMENT, "device triplet arrays must be aligned to their element size");
  // raster elements, with the product checked against 64 bits
  unsigned long long px = n_bands;
  for (unsigned long long d : {(unsigned long long)nrows, (unsigned long long)ncols}) {
    if (d && px > ~0ull / d) return fail(err, errlen, RZ_VALUE_ERROR, "raster too large");
    px *= d;
  }
  if (px > (~0ull >> 4) / tsize) return fail(err, errlen, RZ_VALUE_ERROR, "raster too large");
  if (stats) {
    stats->out_bytes = px * tsize;
    stats->pixel_writes = count;
  }
  if (px == 0) {
    if (count) return fail(err, errlen, RZ_VALUE_ERROR, "triplet 0 lies outside the raster");
    return RZ_OK;
  }

  RZ_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const int sms = ctx->num_sms;
  const unsigned long long chunk = std::max(1ull, std::min(count, kReplayChunk));
  Layout L;
  const size_t o_ctrl = L.take(sizeof(Ctrl));
  const size_t o_bs = L.take(8 * (n_bands + 1ull));
  size_t o_rows = 0, o_cols = 0, o_vals = 0;
  if (!in_dev) {
    o_rows = L.take(8 * chunk);
    o_cols = L.take(8 * chunk);
    o_vals = L.take(tsize * chunk);
  }
  const size_t o_k0 = L.take(8 * chunk), o_k1 = L.take(8 * chunk);
  const size_t o_v0 = L.take(4 * chunk), o_v1 = L.take(4 * chunk);
  const size_t o_rst = L.take(4 * radix_sort_temp_words(chunk));
  RZ_CUDA(ensure(ctx->sparse, L.off));
  void* d_ras = out;
  if (!out_dev) {
    RZ_CUDA(ensure(ctx->out, px * tsize));
    d_ras = ctx->out.p;
  }
  char* base = static_cast<char*>(ctx->sparse.p);
  auto at = [&](size_t o) { return static_cast<void*>(base + o); };
  Ctrl* d_ctrl = static_cast<Ctrl*>(at(o_ctrl));
  unsigned long long* d_bs = static_cast<unsigned long long*>(at(o_bs));
  unsigned long long* k0 = static_cast<unsigned long long*>(at(o_k0));
  unsigned long long* k1 = static_cast<unsigned long long*>(at(o_k1));
  unsigned* v0 = static_cast<unsigned*>(at(o_v0));
  unsigned* v1 = static_cast<unsigned*>(at(o_v1));
  unsigned long long bg_bits = 0;
  std::memcpy(&bg_bits, background, tsize);
  int launches = 0;
  PageToucher toucher;  // a host output's pages, faulted in while the device replays
  if (!out_dev) toucher.start(out, (size_t)(px * tsize));

  if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[0], s));
  RZ_CUDA(cudaMemsetAsync(d_ctrl, 0, sizeof(Ctrl), s));
  RZ_CUDA(cudaMemcpyAsync(d_bs, bstart.data(), 8 * (n_bands + 1ull), cudaMemcpyHostToDevice, s));
  {
    const unsigned g = grid_for(px, 256, sms * 16);
    switch (tsize) {
      case 1: k_replay_bg<1><<<g, 256, 0, s>>>(d_ras, px, bg_bits); break;
      case 2: k_replay_bg<2><<<g, 256, 0, s>>>(d_ras, px, bg_bits); break;
      case 4: k_replay_bg<4><<<g, 256, 0, s>>>(d_ras, px, bg_bits); break;
      default: k_replay_bg<8><<<g, 256, 0, s>>>(d_ras, px, bg_bits); break;
    }
    ++launches;
  }
  int bits = 1;  // keys are < px
  while (bits < 64 && (1ull << bits) < px) ++bits;
  const replay_fn rf = replay_for(dt);
  for (unsigned long long t0 = 0; t0 < count; t0 += chunk) {
    const unsigned m = (unsigned)std::min(chunk, count - t0);
    const unsigned long long* drows;
    const unsigned long long* dcols;
    const void* dvals;
    if (in_dev) {
      drows = reinterpret_cast<const unsigned long long*>(rows) + t0;
      dcols = reinterpret_cast<const unsigned long long*>(cols) + t0;
      dvals = static_cast<const char*>(values) + tsize * t0;
    } else {
      // the previous chunk's kernels read these buffers earlier in stream order
      RZ_CUDA(cudaMemcpyAsync(at(o_rows), rows + t0, 8ull * m, cudaMemcpyHostToDevice, s));
      RZ_CUDA(cudaMemcpyAsync(at(o_cols), cols + t0, 8ull * m, cudaMemcpyHostToDevice, s));
      RZ_CUDA(cudaMemcpyAsync(at(o_vals), static_cast<const char*>(values) + tsize * t0, tsize * m,
                              cudaMemcpyHostToDevice, s));
      drows = static_cast<const unsigned long long*>(at(o_rows));
      dcols = static_cast<const unsigned long long*>(at(o_cols));
      dvals = at(o_vals);
    }
    k_replay_keys<<<grid_for(m, 256, sms * 16), 256, 0, s>>>(drows, dcols, m, t0, d_bs, n_bands, nrows, ncols, k0,
                                                              v0, d_ctrl);
    ++launches;
    const bool in_tmp = radix_sort(k0, v0, k1, v1, m, bits, static_cast<unsigned*>(at(o_rst)), s, launches);
    ReplayArgs ra;
    ra.skeys = in_tmp ? k1 : k0;
    ra.sidx = in_tmp ? v1 : v0;
    ra.n = m;
    ra.vals = dvals;
    ra.raster = d_ras;
    ra.bg = bg_bits;
    launches += rf(ra, (int)fn, sms, s);
    RZ_CUDA(cudaGetLastError());
  }
  if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[5], s));
  RZ_CUDA(cudaMemcpyAsync(ctx->h_ctrl, d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
  RZ_CUDA(cudaStreamSynchronize(s));
  if (ctx->h_ctrl->err) return ctrl_error(*ctx->h_ctrl, err, errlen);
  toucher.join();
  if (!out_dev) RZ_CUDA(cudaMemcpyAsync(out, d_ras, px * tsize, cudaMemcpyDeviceToHost, s));
  if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[6], s));
  RZ_CUDA(cudaStreamSynchronize(s));
  if (stats) {
    stats->kernel_launches = (uint32_t)launches;
    if (timing) {
      cudaEventElapsedTime(&stats->ms_fill, ctx->ev[0], ctx->ev[5]);
      cudaEventElapsedTime(&stats->ms_d2h, ctx->ev[5], ctx->ev[6]);
      cudaEventElapsedTime(&stats->ms_device_total, ctx->ev[0], ctx->ev[6]);
    }
    stats->ms_host_total = std::chrono::duration<float, std::milli>(clk::now() - t_host0).count();
  }
  return RZ_OK;
}

extern "C" rz_status rz_sparse_build(rz_context* ctx, const uint64_t* band_counts, uint32_t n_bands,
                                     const uint64_t* rows, const uint64_t* cols, const void* values, uint64_t nrows,
                                     uint64_t ncols, rz_pixel_fn fn, rz_dtype dt, const void* background,
                                     uint32_t flags, void* out, rz_stats* stats, char* err, size_t errlen) {
  return drain_on_error(ctx ? ctx->stream : nullptr,
                        replay_impl(ctx, band_counts, n_bands, rows, cols, values, nrows, ncols, fn, dt, background,
                                    flags, out, stats, err, errlen));
}

// ---------------------------------------------------------------------------
// Allocation-free burn (rz_rasterize_noalloc).
//
// Some callers cannot allocate device memory at the moment they burn:
// serving loops whose device memory is budgeted up front and must not grow,
// or stall on cudaMalloc/cudaFree (which can synchronise the device) behind
// the caller's back, and plugin hosts (a database or GIS engine with its own
// pool allocator) that own every allocation themselves.  This entry point runs
// the same kernels as rz_rasterize, but every scratch buffer is carved out of
// the file-scope array below instead of the context's growable arena.  The
// array is RZ_NOALLOC_SCRATCH_BYTES large and is held by every GPU that loads
// this library until the process exits.  All calls share it: it keeps the
// last call's contents (everything that must start at zero is cleared by
// each call), and calls whose work overlaps on the GPU race on it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[RZ_NOALLOC_SCRATCH_BYTES];

namespace {

struct NoAllocDevice {
  bool ready = false;
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
  int sms = 0, poly_bps = 1, narrow_bps = 1;
};
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
NoAllocDevice g_noalloc[kNoAllocMaxDevices];

}  // namespace

static rz_status noalloc_impl(void* stream, const rz_geoms* g, const void* values, const void* background,
                              const uint32_t* band_of_geom, uint32_t n_bands, const rz_raster_info* info,
                              rz_pixel_fn fn, rz_dtype dt, uint32_t flags, void* out, rz_stats* stats, char* err,
                              size_t errlen);

extern "C" rz_status rz_rasterize_noalloc(void* stream, const rz_geoms* g, const void* values,
                                          const void* background, const uint32_t* band_of_geom, uint32_t n_bands,
                                          const rz_raster_info* info, rz_pixel_fn fn, rz_dtype dt, uint32_t flags,
                                          void* out, rz_stats* stats, char* err, size_t errlen) {
  return drain_on_error(static_cast<cudaStream_t>(stream),
                        noalloc_impl(stream, g, values, background, band_of_geom, n_bands, info, fn, dt, flags, out,
                                     stats, err, errlen));
}

static rz_status noalloc_impl(void* stream, const rz_geoms* g, const void* values, const void* background,
                              const uint32_t* band_of_geom, uint32_t n_bands, const rz_raster_info* info,
                              rz_pixel_fn fn, rz_dtype dt, uint32_t flags, void* out, rz_stats* stats, char* err,
                              size_t errlen) {
  rz::clear_err(err, errlen);
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (!g || !info || !out) return fail(err, errlen, RZ_INVALID_ARGUMENT, "null argument");
  const size_t tsize = rz_dtype_size(dt);
  if (tsize == 0) return fail(err, errlen, RZ_VALUE_ERROR, "Unsupported dtype");
  if ((int)fn < 0 || (int)fn > 6) return fail(err, errlen, RZ_VALUE_ERROR, "Unknown pixel function");
  if (band_of_geom && n_bands == 0) return fail(err, errlen, RZ_INVALID_ARGUMENT, "n_bands must be > 0");
  const unsigned long long nb = band_of_geom ? n_bands : 1;
  if (info->nrows >= (1ull << 31) - 1 || info->ncols >= (1ull << 31) - 1)
    return fail(err, errlen, RZ_VALUE_ERROR, "raster dimensions must be below 2^31-1");
  const unsigned long long nrows = info->nrows, ncols = info->ncols;
  const unsigned long long out_elems = nb * nrows * ncols;
  const unsigned ntx = (unsigned)((ncols + TW - 1) >> TW_SHIFT);
  const unsigned long long nbuckets = nb * nrows * ntx;
  const unsigned long long G = g->n_geoms, P = g->n_parts, R = g->n_rings, V = g->n_vertices;
  if (G >= 0xFFFFFFFFull || P >= (1ull << 27) || nbuckets >= (1ull << 28))
    return fail(err, errlen, RZ_VALUE_ERROR, "job too large: at most 2^27 parts and 2^28 (band,row,tile) buckets");
  if (!g->part_offsets || !g->part_kind || !g->ring_offsets || !g->vertex_offsets || (V && !g->xy))
    return fail(err, errlen, RZ_INVALID_ARGUMENT, "geometry table has null arrays");
  if (reinterpret_cast<uintptr_t>(g->xy) & 15)
    return fail(err, errlen, RZ_INVALID_ARGUMENT, "device xy must be 16-byte aligned");
  unsigned long long bg_bits = 0, scalar_bits = one_bits(dt);
  if (background) std::memcpy(&bg_bits, background, tsize);  // NULL: a zero background, as rz_rasterize
  const bool per_geom_values = values && !(flags & RZ_FLAG_SCALAR_VALUE);
  if (values && (flags & RZ_FLAG_SCALAR_VALUE)) {
    scalar_bits = 0;
    std::memcpy(&scalar_bits, values, tsize);
  }
  if (stats) stats->out_bytes = out_elems * tsize;
  if (out_elems == 0) return RZ_OK;

  // scratch layout inside the static array (inputs and output are the caller's)
  Layout L;
  const size_t o_pg = L.take(4 * (P ? P : 1));
  const size_t o_pval = L.take(tsize * (P ? P : 1));
  const size_t o_plan = L.take(sizeof(PartPlan) * (P ? P : 1));
  const size_t o_cnt = L.take(8 * PC_N * (P ? P : 1));
  const size_t o_poff = L.take(8 * PC_N * (P + 1));
  const size_t o_tmp64 = L.take(8 * scan_temp_elems(P, PC_N));
  const size_t o_last = L.take(8 * (P ? P : 1));
  const size_t o_lp = L.take(4 * (P ? P : 1));
  const size_t o_pp = L.take(4 * (P ? P : 1));
  const size_t o_bc = L.take(4 * nbuckets);
  const size_t o_boff = L.take(4 * (nbuckets + 1));
  const size_t o_tmp32 = L.take(4 * scan_temp_elems(nbuckets, 1));
  const size_t o_big = L.take(4 * nbuckets);
  const size_t o_ctrl = L.take(sizeof(Ctrl));
  const size_t o_spans = L.take(0);
  const size_t min_spans = 1024;
  if (o_spans + rzl::record_bytes_for(min_spans) > RZ_NOALLOC_SCRATCH_BYTES)
    return fail(err, errlen, RZ_VALUE_ERROR,
                "job needs %zu bytes of scratch before any span; the allocation-free entry point is limited to "
                "%zu bytes (use rz_rasterize)",
                (size_t)(o_spans + rzl::record_bytes_for(min_spans)), (size_t)RZ_NOALLOC_SCRATCH_BYTES);
  const rzl::RecordLayout RL = rzl::record_layout(RZ_NOALLOC_SCRATCH_BYTES - o_spans);
  const unsigned long long cap = RL.cap;

  int dev = 0;
  RZ_CUDA(cudaGetDevice(&dev));
  if (stream) {
    // the static array used is the current device's: the stream must be on it
    int sdev = -1;
    RZ_CUDA(cudaStreamGetDevice(static_cast<cudaStream_t>(stream), &sdev));
    if (sdev != dev)
      return fail(err, errlen, RZ_INVALID_ARGUMENT,
                  "stream belongs to device %d but device %d is current; make the stream's device current", sdev,
                  dev);
  }
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(err, errlen, RZ_NO_DEVICE, "device %d unsupported", dev);
  NoAllocDevice nd;
  {
    // one-time set-up per device, with that device current: resolve the
    // array's device address (host code cannot use the symbol itself)
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoAllocDevice& d = g_noalloc[dev];
    if (!d.ready) {
      void* p = nullptr;
      RZ_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
      RZ_CUDA(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev));
      RZ_CUDA(cudaFuncSetAttribute(k_poly_spans, cudaFuncAttributeMaxDynamicSharedMemorySize, POLY_SMEM));
      RZ_CUDA(cudaFuncSetAttribute(k_poly_spans_narrow, cudaFuncAttributeMaxDynamicSharedMemorySize, SMALL_SMEM));
      RZ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d.poly_bps, k_poly_spans, POLY_THREADS, POLY_SMEM));
      RZ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d.narrow_bps, k_poly_spans_narrow, SMALL_WARPS * 32,
                                                            SMALL_SMEM));
      if (d.poly_bps < 1) d.poly_bps = 1;
      if (d.narrow_bps < 1) d.narrow_bps = 1;
      d.scratch = static_cast<unsigned char*>(p);
      d.ready = true;
    }
    nd = d;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char* mb = nd.scratch;
  auto at = [&](size_t o) { return static_cast<void*>(mb + o); };

  Geo geo;
  geo.n_geoms = G;
  geo.n_parts = P;
  geo.n_rings = R;
  geo.n_vertices = V;
  geo.part_offsets = reinterpret_cast<const unsigned long long*>(g->part_offsets);
  geo.part_kind = g->part_kind;
  geo.ring_offsets = reinterpret_cast<const unsigned long long*>(g->ring_offsets);
  geo.vertex_offsets = reinterpret_cast<const unsigned long long*>(g->vertex_offsets);
  geo.xy = reinterpret_cast<const double2*>(g->xy);
  geo.bands = band_of_geom;

  // PixelCache semantics as in rz_rasterize
  const bool touched = (flags & RZ_FLAG_ALL_TOUCHED) != 0;
  const Grid gr = make_grid(info, touched);
  const JobDims one = job_dims(nrows, ncols, info, fn, touched, false, 0u, 0ull);
  const bool dedup = fill_dedup(info, fn, touched);

  Ctrl* d_ctrl = static_cast<Ctrl*>(at(o_ctrl));
  unsigned* part_geom = static_cast<unsigned*>(at(o_pg));
  PartPlan* plan = static_cast<PartPlan*>(at(o_plan));
  unsigned long long* counts = static_cast<unsigned long long*>(at(o_cnt));
  unsigned long long* poff = static_cast<unsigned long long*>(at(o_poff));
  unsigned long long* last_kept = static_cast<unsigned long long*>(at(o_last));
  unsigned* line_parts = static_cast<unsigned*>(at(o_lp));
  unsigned* point_parts = static_cast<unsigned*>(at(o_pp));
  unsigned* bcount = static_cast<unsigned*>(at(o_bc));
  unsigned* boff = static_cast<unsigned*>(at(o_boff));
  unsigned* big = static_cast<unsigned*>(at(o_big));
  const int sms = nd.sms;
  const Sched sched = resolve_sched(rz_tuning{}, sms, nd.narrow_bps, nd.poly_bps);
  int launches = 0;

  RZ_CUDA(cudaMemsetAsync(d_ctrl, 0, sizeof(Ctrl), s));
  PartTables pt;
  pt.part_geom = part_geom;
  pt.plan = plan;
  pt.counts = counts;
  pt.poff = poff;
  pt.tmp64 = static_cast<unsigned long long*>(at(o_tmp64));
  pt.line_parts = line_parts;
  pt.point_parts = point_parts;
  pt.last_kept = last_kept;
  launches += launch_prep(geo, gr, one, nullptr, 1, band_of_geom ? (unsigned)nb : 0u, pt, d_ctrl, sched, s);
  const void* d_vals_na = per_geom_values ? values : nullptr;
  if (d_vals_na && P) {
    launch_part_values(tsize, sms, s, part_geom, d_vals_na, P, at(o_pval), d_ctrl);
    ++launches;
  }
  RZ_CUDA(cudaMemsetAsync(last_kept, 0, 8 * (P ? P : 1), s));
  char* rbase = static_cast<char*>(at(o_spans));
  RecBuf sb;
  sb.cap = cap;
  sb.nbuckets = nbuckets;
  sb.wid = reinterpret_cast<unsigned*>(rbase + RL.off_wid);
  sb.part = reinterpret_cast<unsigned*>(rbase + RL.off_part);
  sb.mask = reinterpret_cast<unsigned*>(rbase + RL.off_mask);
  uint2* sorted = reinterpret_cast<uint2*>(rbase + RL.off_sorted);
  k_reset_pass<<<1, 1, 0, s>>>(d_ctrl);
  RZ_CUDA(cudaMemsetAsync(bcount, 0, 4 * nbuckets, s));
  ++launches;
  launches += launch_coverage(geo, gr, pt, sb, bcount, d_ctrl, sched, s);
  launches += scan<unsigned, 1>(bcount, boff, nbuckets, static_cast<unsigned*>(at(o_tmp32)), s);
  launch_scatter(sms, sched.scatter_bps, s, sb, boff, bcount, sorted, d_ctrl);
  ++launches;
  FillArgs fa;
  fa.offsets = boff;
  fa.recs = sorted;
  fa.brecs = reinterpret_cast<uint2*>(sb.wid);  // free once the records are scattered
  fa.pvals = d_vals_na ? at(o_pval) : nullptr;
  fa.nbuckets = nbuckets;
  fa.scalar = scalar_bits;
  fa.out = out;
  set_background(fa, bg_bits, tsize);
  fa.nrows = (int)(nb * nrows);  // rows of the band stack
  fa.ncols = (int)ncols;
  fa.ntx = ntx;
  fa.big = big;
  fa.ctrl = d_ctrl;
  fa.rec_cap = cap;
  fa.sort_max = sched.tune.fill_sort_max;
  fa.work = &d_ctrl->fill_work;
  fa.nbig = &d_ctrl->big_count;
  fa.jobs = nullptr;
  fa.n_jobs = 0;
  fa.bucket0 = 0;
  launches += fill_for(dt)(fa, (int)fn, dedup, sms, s);
  RZ_CUDA(cudaGetLastError());
  Ctrl hc;  // the caller's stack, no pinned buffer
  RZ_CUDA(cudaMemcpyAsync(&hc, d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
  RZ_CUDA(cudaStreamSynchronize(s));
  if (hc.err) return ctrl_error(hc, err, errlen);
  if (hc.span_count > cap)
    return fail(err, errlen, RZ_VALUE_ERROR,
                "job produced %llu spans; the allocation-free entry point holds at most %llu in its %zu-byte "
                "scratch (use rz_rasterize)",
                hc.span_count, cap, (size_t)RZ_NOALLOC_SCRATCH_BYTES);
  if (stats) {
    stats->edges = hc.edges;
    stats->crossings = hc.crossings;
    stats->spans = hc.span_count;
    stats->pixel_writes = hc.pixel_writes;
    stats->big_buckets = hc.big_count;
    stats->buckets = nbuckets;
    stats->kernel_launches = (uint32_t)launches;
  }
  return RZ_OK;
}

// ---------------------------------------------------------------------------
// Batches of independent jobs (rz_rasterize_batch).
//
// The jobs of a wave are concatenated into one parts table on the device
// (rz_batch.cuh), so that the whole wave takes one pass of the pipeline: one
// launch of each kernel instead of one per job, whatever the number and size
// of the jobs.  Within a wave the jobs are ordered by (pixel function,
// deduplication, background), so that the buckets of each fill variant are
// one contiguous range: one fill launch per variant present.

namespace {

struct BatchJob {
  size_t idx;  // index in the caller's array
  unsigned long long G, P, R, V, nrows, ncols, ntx, out_elems, buckets;
  unsigned long long bg_bits, scalar_bits;
  bool per_geom_values, dedup;
  rz_pixel_fn fn;
  size_t dev_bytes;  // device footprint counted against the wave budget
};

cudaError_t ensure_pinned(rz_context* ctx, size_t need) {
  if (need <= ctx->h_stage_cap) return cudaSuccess;
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  ctx->h_stage = nullptr;
  ctx->h_stage_cap = 0;
  const size_t want = need + need / 4 + (1u << 20);
  void* p = nullptr;
  cudaError_t e = cudaMallocHost(&p, want);
  if (e == cudaSuccess) {
    ctx->h_stage = static_cast<unsigned char*>(p);
    ctx->h_stage_cap = want;
  }
  return e;
}

size_t align16(size_t v) { return (v + 15) & ~size_t(15); }

// One wave: jobs[w0..w1) of `order`, already validated.
rz_status run_wave(rz_context* ctx, const rz_job* jobs, std::vector<BatchJob>& wave, rz_dtype dt, uint32_t flags,
                   rz_batch_stats* stats, char* err, size_t errlen) {
  const size_t tsize = rz_dtype_size(dt);
  const bool in_dev = flags & RZ_FLAG_INPUT_DEVICE, out_dev = flags & RZ_FLAG_OUTPUT_DEVICE;
  const bool touched = flags & RZ_FLAG_ALL_TOUCHED;
  const bool timing = !(flags & RZ_FLAG_NO_TIMING);
  cudaStream_t s = ctx->stream;
  const int sms = ctx->num_sms;
  const Sched sched = resolve_sched(ctx->tuning, sms, ctx->narrow_blocks_per_sm, ctx->poly_blocks_per_sm);
  // fill variants contiguous (stable: caller order within a variant)
  std::stable_sort(wave.begin(), wave.end(), [](const BatchJob& a, const BatchJob& b) {
    if (a.fn != b.fn) return a.fn < b.fn;
    if (a.dedup != b.dedup) return a.dedup < b.dedup;
    return a.bg_bits < b.bg_bits;
  });
  const unsigned n = (unsigned)wave.size();
  // ---- wave bases ----
  std::vector<unsigned long long> base((size_t)BK_N * (n + 1));
  std::vector<unsigned long long> bucket0(n + 1), out_off(n + 1);
  for (unsigned j = 0; j <= n; ++j) {
    for (int k = 0; k < BK_N; ++k) base[(size_t)k * (n + 1) + j] = j ? base[(size_t)k * (n + 1) + j - 1] : 0;
    bucket0[j] = j ? bucket0[j - 1] : 0;
    out_off[j] = j ? out_off[j - 1] : 0;
    if (j) {
      const BatchJob& b = wave[j - 1];
      base[(size_t)BK_GEOM * (n + 1) + j] += b.G;
      base[(size_t)BK_PART * (n + 1) + j] += b.P;
      base[(size_t)BK_RING * (n + 1) + j] += b.R;
      base[(size_t)BK_VERT * (n + 1) + j] += b.V;
      bucket0[j] += b.buckets;
      out_off[j] += align16(b.out_elems * tsize);
    }
  }
  const unsigned long long Gt = base[(size_t)BK_GEOM * (n + 1) + n], Pt = base[(size_t)BK_PART * (n + 1) + n];
  const unsigned long long Rt = base[(size_t)BK_RING * (n + 1) + n], Vt = base[(size_t)BK_VERT * (n + 1) + n];
  const unsigned long long nbuckets = bucket0[n];

  // ---- host staging: job tables, then (host inputs) every job's arrays ----
  Layout HL;
  const size_t h_src = HL.take(sizeof(JobSrc) * n), h_dims = HL.take(sizeof(JobDims) * n);
  const size_t h_fj = HL.take(sizeof(FillJob) * n), h_base = HL.take(8 * base.size());
  const size_t tables_bytes = HL.off;
  std::vector<size_t> h_arr(in_dev ? 0 : (size_t)n * 6);
  if (!in_dev) {
    for (unsigned j = 0; j < n; ++j) {
      const BatchJob& b = wave[j];
      h_arr[6 * j + 0] = HL.take(8 * (b.G + 1));
      h_arr[6 * j + 1] = HL.take(b.P ? b.P : 1);
      h_arr[6 * j + 2] = HL.take(8 * (b.P + 1));
      h_arr[6 * j + 3] = HL.take(8 * (b.R + 1));
      h_arr[6 * j + 4] = HL.take(16 * (b.V ? b.V : 1));
      h_arr[6 * j + 5] = HL.take(b.per_geom_values ? tsize * (b.G ? b.G : 1) : 1);
    }
  }
  const size_t stage_bytes = HL.off;
  RZ_CUDA(ensure_pinned(ctx, stage_bytes));
  RZ_CUDA(ensure(ctx->stage, stage_bytes));
  unsigned char* hs = ctx->h_stage;
  unsigned char* ds = static_cast<unsigned char*>(ctx->stage.p);
  JobSrc* src = reinterpret_cast<JobSrc*>(hs + h_src);
  JobDims* dims = reinterpret_cast<JobDims*>(hs + h_dims);
  FillJob* fj = reinterpret_cast<FillJob*>(hs + h_fj);
  std::memcpy(hs + h_base, base.data(), 8 * base.size());

  // ---- device wave layout ----
  Layout L;
  const size_t o_po = L.take(8 * (Gt + 1)), o_pk = L.take(Pt ? Pt : 1), o_ro = L.take(8 * (Pt + 1));
  const size_t o_vo = L.take(8 * (Rt + 1)), o_xy = L.take(16 * (Vt ? Vt : 1)), o_val = L.take(tsize * (Gt ? Gt : 1));
  const size_t o_rc = L.take(Rt ? Rt : 1);
  const size_t o_pg = L.take(4 * (Pt ? Pt : 1));
  const size_t o_pval = L.take(tsize * (Pt ? Pt : 1));
  const size_t o_plan = L.take(sizeof(PartPlan) * (Pt ? Pt : 1));
  const size_t o_cnt = L.take(8 * PC_N * (Pt ? Pt : 1));
  const size_t o_poff = L.take(8 * PC_N * (Pt + 1));
  const size_t o_tmp64 = L.take(8 * scan_temp_elems(Pt, PC_N));
  const size_t o_last = L.take(8 * (Pt ? Pt : 1));
  const size_t o_lp = L.take(4 * (Pt ? Pt : 1));
  const size_t o_pp = L.take(4 * (Pt ? Pt : 1));
  const size_t o_bc = L.take(4 * (nbuckets ? nbuckets : 1));
  const size_t o_boff = L.take(4 * (nbuckets + 1));
  const size_t o_tmp32 = L.take(4 * scan_temp_elems(nbuckets ? nbuckets : 1, 1));
  const size_t o_big = L.take(4 * (nbuckets ? nbuckets : 1));
  const size_t o_ctrl = L.take(sizeof(Ctrl));
  const size_t o_gctr = L.take(16 * (n + 1));
  RZ_CUDA(ensure(ctx->batch, L.off));
  if (!out_dev) RZ_CUDA(ensure(ctx->out, out_off[n] ? out_off[n] : 16));
  char* mb = static_cast<char*>(ctx->batch.p);
  auto at = [&](size_t o) { return static_cast<void*>(mb + o); };

  // ---- job tables ----
  const Grid ident = [&] {
    Grid g;
    g.xmin = 0.0;
    g.ymax = -0.0;
    g.xres = g.yres = 1.0;
    g.inv_xres = g.inv_yres = 0.0;
    g.pow2_x = g.pow2_y = 0;
    g.unit_x = g.unit_y = 1;
    g.touched = touched ? 1 : 0;
    return g;
  }();
  for (unsigned j = 0; j < n; ++j) {
    const BatchJob& b = wave[j];
    const rz_job& jb = jobs[b.idx];
    JobSrc& sj = src[j];
    sj.n_geoms = b.G;
    sj.n_parts = b.P;
    sj.n_rings = b.R;
    sj.n_vertices = b.V;
    sj.grid = make_grid(&jb.info, touched);
    sj.scalar = b.scalar_bits;
    if (in_dev) {
      sj.part_offsets = reinterpret_cast<const unsigned long long*>(jb.geoms.part_offsets);
      sj.part_kind = jb.geoms.part_kind;
      sj.ring_offsets = reinterpret_cast<const unsigned long long*>(jb.geoms.ring_offsets);
      sj.vertex_offsets = reinterpret_cast<const unsigned long long*>(jb.geoms.vertex_offsets);
      sj.xy = reinterpret_cast<const double2*>(jb.geoms.xy);
      sj.values = b.per_geom_values ? jb.values : nullptr;
    } else {
      const size_t* o = &h_arr[6 * j];
      sj.part_offsets = reinterpret_cast<const unsigned long long*>(ds + o[0]);
      sj.part_kind = ds + o[1];
      sj.ring_offsets = reinterpret_cast<const unsigned long long*>(ds + o[2]);
      sj.vertex_offsets = reinterpret_cast<const unsigned long long*>(ds + o[3]);
      sj.xy = reinterpret_cast<const double2*>(ds + o[4]);
      sj.values = b.per_geom_values ? static_cast<const void*>(ds + o[5]) : nullptr;
    }
    dims[j] = job_dims(b.nrows, b.ncols, &jb.info, b.fn, touched, false, (unsigned)(bucket0[j] * WPT),
                       base[(size_t)BK_GEOM * (n + 1) + j]);
    fj[j].bucket0 = bucket0[j];
    fj[j].out = out_dev ? jb.out : static_cast<void*>(static_cast<char*>(ctx->out.p) + out_off[j]);
    fj[j].nrows = (int)b.nrows;
    fj[j].ncols = (int)b.ncols;
    fj[j].pad = 0;
    fj[j].ntx = (unsigned)b.ntx;
  }
  if (!in_dev) {
    // pack the jobs' host arrays (large copies split over host threads)
    auto pack = [&](unsigned j) {
      const BatchJob& b = wave[j];
      const rz_geoms& g = jobs[b.idx].geoms;
      const size_t* o = &h_arr[6 * j];
      std::memcpy(hs + o[0], g.part_offsets, 8 * (b.G + 1));
      if (b.P) std::memcpy(hs + o[1], g.part_kind, b.P);
      std::memcpy(hs + o[2], g.ring_offsets, 8 * (b.P + 1));
      std::memcpy(hs + o[3], g.vertex_offsets, 8 * (b.R + 1));
      if (b.V) std::memcpy(hs + o[4], g.xy, 16 * b.V);
      if (b.per_geom_values && b.G) std::memcpy(hs + o[5], jobs[b.idx].values, tsize * b.G);
    };
    const unsigned nthreads = stage_bytes > (64u << 20) ? std::min(8u, n) : 1u;
    if (nthreads > 1) {
      std::vector<std::thread> ts;
      for (unsigned t = 0; t < nthreads; ++t)
        ts.emplace_back([&, t] {
          for (unsigned j = t; j < n; j += nthreads) pack(j);
        });
      for (auto& t : ts) t.join();
    } else {
      for (unsigned j = 0; j < n; ++j) pack(j);
    }
  }
  if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[0], s));
  RZ_CUDA(cudaMemcpyAsync(ds, hs, in_dev ? tables_bytes : stage_bytes, cudaMemcpyHostToDevice, s));
  const JobSrc* d_src = reinterpret_cast<const JobSrc*>(ds + h_src);
  const JobDims* d_dims = reinterpret_cast<const JobDims*>(ds + h_dims);
  const FillJob* d_fj = reinterpret_cast<const FillJob*>(ds + h_fj);
  const unsigned long long* d_base = reinterpret_cast<const unsigned long long*>(ds + h_base);

  // ---- gather the wave's table ----
  Ctrl* d_ctrl = static_cast<Ctrl*>(at(o_ctrl));
  int launches = 0;
  RZ_CUDA(cudaMemsetAsync(d_ctrl, 0, sizeof(Ctrl), s));
  if (in_dev) {
    k_batch_check<<<grid_for(n, 128, sms * 4), 128, 0, s>>>(d_src, n, d_ctrl);
    ++launches;
  }
  unsigned long long* w_po = static_cast<unsigned long long*>(at(o_po));
  unsigned char* w_pk = static_cast<unsigned char*>(at(o_pk));
  unsigned long long* w_ro = static_cast<unsigned long long*>(at(o_ro));
  unsigned long long* w_vo = static_cast<unsigned long long*>(at(o_vo));
  double2* w_xy = static_cast<double2*>(at(o_xy));
  void* w_val = at(o_val);
  {
    const unsigned gg = grid_for(Gt + 1, 256, sms * 16);
    switch (tsize) {
      case 1: k_batch_geoms<1><<<gg, 256, 0, s>>>(d_src, d_base, n, w_po, w_val); break;
      case 2: k_batch_geoms<2><<<gg, 256, 0, s>>>(d_src, d_base, n, w_po, w_val); break;
      case 4: k_batch_geoms<4><<<gg, 256, 0, s>>>(d_src, d_base, n, w_po, w_val); break;
      default: k_batch_geoms<8><<<gg, 256, 0, s>>>(d_src, d_base, n, w_po, w_val); break;
    }
    k_batch_parts<<<grid_for(Pt + 1, 256, sms * 16), 256, 0, s>>>(d_src, d_base, n, w_pk, w_ro);
    k_batch_rings<<<grid_for(Rt + 1, 256, sms * 16), 256, 0, s>>>(d_src, d_base, n, w_vo,
                                                                   static_cast<unsigned char*>(at(o_rc)));
    k_batch_vertices<<<grid_for(Vt + 1, 256, sms * 16), 256, 0, s>>>(d_src, d_base, n, w_xy);
    launches += 4;
  }
  Geo geo;
  geo.n_geoms = Gt;
  geo.n_parts = Pt;
  geo.n_rings = Rt;
  geo.n_vertices = Vt;
  geo.part_offsets = w_po;
  geo.part_kind = w_pk;
  geo.ring_offsets = w_ro;
  geo.vertex_offsets = w_vo;
  geo.xy = w_xy;
  geo.bands = nullptr;
  geo.ring_closed = static_cast<const unsigned char*>(at(o_rc));

  // ---- prep ----
  PartTables pt;
  pt.part_geom = static_cast<unsigned*>(at(o_pg));
  pt.plan = static_cast<PartPlan*>(at(o_plan));
  pt.counts = static_cast<unsigned long long*>(at(o_cnt));
  pt.poff = static_cast<unsigned long long*>(at(o_poff));
  pt.tmp64 = static_cast<unsigned long long*>(at(o_tmp64));
  pt.line_parts = static_cast<unsigned*>(at(o_lp));
  pt.point_parts = static_cast<unsigned*>(at(o_pp));
  pt.last_kept = static_cast<unsigned long long*>(at(o_last));
  launches += launch_prep(geo, ident, dims[0], d_dims, n, 0u, pt, d_ctrl, sched, s);
  if (Pt) {  // every job's values are gathered per geometry into the wave table
    launch_part_values(tsize, sms, s, pt.part_geom, w_val, Pt, at(o_pval), d_ctrl);
    ++launches;
  }
  RZ_CUDA(cudaMemsetAsync(pt.last_kept, 0, 8 * (Pt ? Pt : 1), s));
  unsigned* bcount = static_cast<unsigned*>(at(o_bc));
  unsigned* boff = static_cast<unsigned*>(at(o_boff));
  unsigned* big = static_cast<unsigned*>(at(o_big));
  unsigned char* gctr = static_cast<unsigned char*>(at(o_gctr));
  const fill_fn fill = fill_for(dt);

  unsigned long long cap =
      rzl::record_cap_request(std::max<unsigned long long>(ctx->span_cap_hint, 2 * Vt + (1ull << 20)));
  unsigned reruns = 0;
  while (true) {
    RZ_CUDA(ensure(ctx->spans, rzl::record_bytes_for(cap)));
    const rzl::RecordLayout RL = rzl::record_layout(ctx->spans.cap);
    cap = RL.cap;
    char* rbase = static_cast<char*>(ctx->spans.p);
    RecBuf sb;
    sb.cap = cap;
    sb.nbuckets = nbuckets;
    sb.wid = reinterpret_cast<unsigned*>(rbase + RL.off_wid);
    sb.part = reinterpret_cast<unsigned*>(rbase + RL.off_part);
    sb.mask = reinterpret_cast<unsigned*>(rbase + RL.off_mask);
    uint2* sorted = reinterpret_cast<uint2*>(rbase + RL.off_sorted);
    k_reset_pass<<<1, 1, 0, s>>>(d_ctrl);
    RZ_CUDA(cudaMemsetAsync(bcount, 0, 4 * (nbuckets ? nbuckets : 1), s));
    RZ_CUDA(cudaMemsetAsync(gctr, 0, 16 * (n + 1), s));
    ++launches;
    launches += launch_coverage(geo, ident, pt, sb, bcount, d_ctrl, sched, s);
    if (nbuckets) {
      launches += scan<unsigned, 1>(bcount, boff, nbuckets, static_cast<unsigned*>(at(o_tmp32)), s);
      launch_scatter(sms, sched.scatter_bps, s, sb, boff, bcount, sorted, d_ctrl);
      ++launches;
      // one fill per variant: a run of jobs with equal (fn, dedup, background)
      unsigned g = 0;
      for (unsigned j0 = 0; j0 < n; ++g) {
        unsigned j1 = j0 + 1;
        while (j1 < n && wave[j1].fn == wave[j0].fn && wave[j1].dedup == wave[j0].dedup &&
               wave[j1].bg_bits == wave[j0].bg_bits)
          ++j1;
        const unsigned long long lo = bucket0[j0], hi = bucket0[j1];
        if (hi > lo) {
          FillArgs fa;
          fa.offsets = boff + lo;
          fa.recs = sorted;
          fa.brecs = reinterpret_cast<uint2*>(sb.wid);  // free once the records are scattered
          fa.pvals = at(o_pval);
          fa.nbuckets = hi - lo;
          fa.scalar = 0;
          fa.out = nullptr;
          set_background(fa, wave[j0].bg_bits, tsize);
          fa.nrows = fa.ncols = 0;
          fa.ntx = 1;
          fa.big = big + lo;
          fa.ctrl = d_ctrl;
          fa.rec_cap = cap;
          fa.sort_max = sched.tune.fill_sort_max;
          fa.work = reinterpret_cast<unsigned long long*>(gctr + 16 * g);
          fa.nbig = reinterpret_cast<unsigned*>(gctr + 16 * g + 8);
          fa.jobs = d_fj;
          fa.n_jobs = n;
          fa.bucket0 = lo;
          launches += fill(fa, (int)wave[j0].fn, wave[j0].dedup, sms, s);
        }
        j0 = j1;
      }
    }
    RZ_CUDA(cudaGetLastError());
    RZ_CUDA(cudaMemcpyAsync(ctx->h_ctrl, d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
    RZ_CUDA(cudaStreamSynchronize(s));
    Ctrl& hc = *ctx->h_ctrl;
    if (hc.err == ERR_BAD_JOB && hc.err_index < n) hc.err_index = wave[hc.err_index].idx;  // the caller's index
    if (hc.err) return ctrl_error(hc, err, errlen);
    if (hc.span_count > cap) {
      cap = rzl::record_cap_regrow(hc.span_count);
      if (cap == 0) return fail(err, errlen, RZ_VALUE_ERROR, "more than 2^32 coverage records in one wave");
      ++reruns;
      continue;
    }
    // remembered for the next call only once a pass fitted: a failed
    // allocation must not make every later call ask for the same size
    ctx->span_cap_hint = std::max(ctx->span_cap_hint, cap);
    if (stats) {
      stats->edges += hc.edges;
      stats->records += hc.span_count;
      stats->pixel_writes += hc.pixel_writes;
    }
    break;
  }
  if (!out_dev) {
    for (unsigned j = 0; j < n; ++j) {
      const BatchJob& b = wave[j];
      if (b.out_elems)
        RZ_CUDA(cudaMemcpyAsync(jobs[b.idx].out, static_cast<char*>(ctx->out.p) + out_off[j], b.out_elems * tsize,
                                cudaMemcpyDeviceToHost, s));
    }
  }
  if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[6], s));
  RZ_CUDA(cudaStreamSynchronize(s));
  if (stats) {
    stats->waves += 1;
    stats->kernel_launches += (uint32_t)launches;
    stats->reruns += reruns;
    if (timing) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[6]);
      stats->ms_device_total += ms;
    }
  }
  return RZ_OK;
}

}  // namespace

extern "C" rz_status rz_rasterize_batch(rz_context* ctx, const rz_job* jobs, size_t n_jobs, rz_dtype dt,
                                        uint32_t flags, uint64_t wave_bytes, rz_batch_stats* stats, char* err,
                                        size_t errlen) {
  using clk = std::chrono::steady_clock;
  const auto t_host0 = clk::now();
  rz::clear_err(err, errlen);
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (!ctx || (n_jobs && !jobs)) return fail(err, errlen, RZ_INVALID_ARGUMENT, "null argument");
  const size_t tsize = rz_dtype_size(dt);
  if (tsize == 0) return fail(err, errlen, RZ_VALUE_ERROR, "Unsupported dtype");
  const bool in_dev = flags & RZ_FLAG_INPUT_DEVICE, out_dev = flags & RZ_FLAG_OUTPUT_DEVICE;
  if (!wave_bytes) wave_bytes = 32ull << 30;
  // ---- validate every job before any work ----
  std::vector<BatchJob> all(n_jobs);
  unsigned long long total_out = 0;
  for (size_t i = 0; i < n_jobs; ++i) {
    const rz_job& jb = jobs[i];
    const rz_geoms& g = jb.geoms;
    BatchJob& b = all[i];
    b.idx = i;
    b.G = g.n_geoms;
    b.P = g.n_parts;
    b.R = g.n_rings;
    b.V = g.n_vertices;
    if ((int)jb.fn < 0 || (int)jb.fn > 6)
      return fail(err, errlen, RZ_VALUE_ERROR, "job %zu: Unknown pixel function", i);
    if (!jb.background) return fail(err, errlen, RZ_INVALID_ARGUMENT, "job %zu: null background", i);
    if (jb.info.nrows >= (1ull << 31) - 1 || jb.info.ncols >= (1ull << 31) - 1)
      return fail(err, errlen, RZ_VALUE_ERROR, "job %zu: raster dimensions must be below 2^31-1", i);
    if (b.G >= 0xFFFFFFFFull || b.P >= (1ull << 27))
      return fail(err, errlen, RZ_VALUE_ERROR, "job %zu: at most 2^32-1 geometries and 2^27 parts are supported", i);
    if (!g.part_offsets || !g.ring_offsets || !g.vertex_offsets || (b.P && !g.part_kind) || (b.V && !g.xy))
      return fail(err, errlen, RZ_INVALID_ARGUMENT, "job %zu: geometry table has null arrays", i);
    if (in_dev && (reinterpret_cast<uintptr_t>(g.xy) & 15))
      return fail(err, errlen, RZ_INVALID_ARGUMENT, "job %zu: device xy must be 16-byte aligned", i);
    if (!in_dev && (g.part_offsets[0] != 0 || g.part_offsets[b.G] != b.P || g.ring_offsets[0] != 0 ||
                    g.ring_offsets[b.P] != b.R || g.vertex_offsets[0] != 0 || g.vertex_offsets[b.R] != b.V))
      return fail(err, errlen, RZ_INVALID_ARGUMENT, "job %zu: geometry table sizes are inconsistent", i);
    b.nrows = jb.info.nrows;
    b.ncols = jb.info.ncols;
    b.ntx = (b.ncols + TW - 1) >> TW_SHIFT;
    b.out_elems = b.nrows * b.ncols;
    b.buckets = b.nrows * b.ntx;
    if (b.buckets >= (1ull << 28))
      return fail(err, errlen, RZ_VALUE_ERROR, "job %zu: raster too large: more than 2^28 (row,tile) buckets", i);
    if (b.out_elems && !jb.out) return fail(err, errlen, RZ_INVALID_ARGUMENT, "job %zu: null output", i);
    b.fn = jb.fn;
    b.dedup = fill_dedup(&jb.info, jb.fn, flags & RZ_FLAG_ALL_TOUCHED);
    b.bg_bits = 0;
    std::memcpy(&b.bg_bits, jb.background, tsize);
    b.per_geom_values = jb.values && !(jb.flags & RZ_FLAG_SCALAR_VALUE);
    b.scalar_bits = one_bits(dt);
    if (jb.values && (jb.flags & RZ_FLAG_SCALAR_VALUE)) {
      b.scalar_bits = 0;
      std::memcpy(&b.scalar_bits, jb.values, tsize);
    }
    const size_t geo_bytes = 8 * (b.G + 1) + b.P + 8 * (b.P + 1) + 8 * (b.R + 1) + 16 * b.V + tsize * b.G;
    // device footprint: rasters (host outputs), geometry, part tables, bucket
    // tables, and about 4 B of coverage records per raster pixel
    b.dev_bytes = (out_dev ? 0 : b.out_elems * tsize) + geo_bytes * (in_dev ? 1 : 2) +
                  b.P * (4 + 8 + sizeof(PartPlan) + 16 * PC_N + 16) + 16 * b.buckets + 4 * b.out_elems;
    total_out += b.out_elems * tsize;
  }
  if (stats) {
    stats->jobs = n_jobs;
    stats->out_bytes = total_out;
  }
  if (!n_jobs) return RZ_OK;
  RZ_CUDA(cudaSetDevice(ctx->device));
  // ---- waves, in caller order ----
  std::vector<BatchJob> wave;
  size_t bytes = 0;
  unsigned long long G = 0, P = 0, buckets = 0;
  auto flush = [&]() -> rz_status {
    if (wave.empty()) return RZ_OK;
    const rz_status st = drain_on_error(ctx->stream, run_wave(ctx, jobs, wave, dt, flags, stats, err, errlen));
    wave.clear();
    bytes = 0;
    G = P = buckets = 0;
    return st;
  };
  for (size_t i = 0; i < n_jobs; ++i) {
    const BatchJob& b = all[i];
    if (!wave.empty() && (bytes + b.dev_bytes > wave_bytes || G + b.G >= 0xFFFFFFFFull ||
                          P + b.P >= (1ull << 27) || buckets + b.buckets >= (1ull << 28) || wave.size() >= 65536)) {
      const rz_status st = flush();
      if (st != RZ_OK) return st;
    }
    wave.push_back(b);
    bytes += b.dev_bytes;
    G += b.G;
    P += b.P;
    buckets += b.buckets;
  }
  const rz_status st = flush();
  if (st != RZ_OK) return st;
  if (stats) stats->ms_host_total = std::chrono::duration<float, std::milli>(clk::now() - t_host0).count();
  return RZ_OK;
}
