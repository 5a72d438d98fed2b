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

#include "rz_device.cuh"
#include "rz_fill.cuh"
#include "rz_internal.h"
#include "rz_kernels.cuh"
#include "rz_scan.cuh"
#include "rz_sort.cuh"
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
  cudaError_t e = cudaMalloc(&b.p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    want = need;
    e = cudaMalloc(&b.p, want);
  }
  if (e == cudaSuccess) b.cap = want;
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

// the scatter, instantiated for the value size of the output dtype
void launch_scatter(size_t tsize, int sms, cudaStream_t s, const RecBuf& sb, const unsigned* boff, unsigned* bcount,
                    uint2* sorted, const void* values, const unsigned* part_geom, void* rvals, Ctrl* ctrl) {
  switch (tsize) {
    case 1: k_scatter<1><<<sms * 8, 256, 0, s>>>(sb, boff, bcount, sorted, values, part_geom, rvals, ctrl); break;
    case 2: k_scatter<2><<<sms * 8, 256, 0, s>>>(sb, boff, bcount, sorted, values, part_geom, rvals, ctrl); break;
    case 4: k_scatter<4><<<sms * 8, 256, 0, s>>>(sb, boff, bcount, sorted, values, part_geom, rvals, ctrl); break;
    default: k_scatter<8><<<sms * 8, 256, 0, s>>>(sb, boff, bcount, sorted, values, part_geom, rvals, ctrl); break;
  }
}

unsigned grid_for(unsigned long long work, unsigned per_block, unsigned cap) {
  unsigned long long g = (work + per_block - 1) / per_block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (unsigned)g;
}

}  // namespace

// Host copy of a sparse (COO) result.
struct rz_sparse {
  std::vector<uint64_t> band_counts, rows, cols;
  std::vector<unsigned char> values;
  uint32_t n_bands = 1;
  rz_dtype dtype = RZ_F64;
};

struct rz_context {
  int device = 0;
  int num_sms = 0;
  int poly_blocks_per_sm = 1;
  int narrow_blocks_per_sm = 1;
  cudaStream_t stream = nullptr;
  DevBuf main, spans, out, sparse;
  cudaEvent_t ev[8] = {};
  Ctrl* h_ctrl = nullptr;  // pinned
  unsigned long long span_cap_hint = 0;
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
  for (int i = 0; i < 8 && e2 == cudaSuccess; ++i) e2 = cudaEventCreate(&ctx->ev[i]);
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
  for (DevBuf* b : {&ctx->main, &ctx->spans, &ctx->out, &ctx->sparse})
    if (b->p) cudaFree(b->p);
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  if (ctx->h_ctrl) cudaFreeHost(ctx->h_ctrl);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

extern "C" rz_status rz_context_trim(rz_context* ctx) {
  if (!ctx) return RZ_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (DevBuf* b : {&ctx->main, &ctx->spans, &ctx->out, &ctx->sparse}) {
    if (b->p) cudaFree(b->p);
    b->p = nullptr;
    b->cap = 0;
  }
  ctx->span_cap_hint = 0;
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

// The burn pipeline shared by the dense and the sparse entry points; with
// `sp` the coverage records are turned into COO triplets instead of being
// scattered into buckets and filled.
static rz_status burn_impl(rz_context* ctx, const rz_geoms* g, const void* values, const void* background,
                           const uint32_t* band_of_geom, uint32_t n_bands, const rz_raster_info* info,
                           rz_pixel_fn fn, rz_dtype dt, uint32_t flags, void* out, rz_stats* stats, char* err,
                           size_t errlen, rz_sparse* sp) {
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
  const unsigned long long out_elems = nb * nrows * ncols;
  const unsigned ntx = (unsigned)((ncols + TW - 1) >> TW_SHIFT);
  const unsigned long long nbuckets = nb * nrows * ntx;
  if (nbuckets >= (1ull << 28))
    return fail(err, errlen, RZ_VALUE_ERROR, "raster too large: more than 2^28 (band,row,tile) buckets");
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
  RZ_CUDA(ensure(ctx->main, L.off));
  if (!out_dev && !sp) RZ_CUDA(ensure(ctx->out, out_elems * tsize));
  unsigned long long cap = std::max<unsigned long long>(ctx->span_cap_hint, 2 * V + (1ull << 20));
  if (cap > 0xFFFFFFF0ull) cap = 0xFFFFFFF0ull;
  RZ_CUDA(ensure(ctx->spans, RECORD_BYTES * cap + 16));
  cap = std::min<unsigned long long>((ctx->spans.cap - 16) / RECORD_BYTES, 0xFFFFFFF0ull) & ~1ull;

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
  if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[1], s));

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
  gr.nrows = (int)nrows;
  gr.ncols = (int)ncols;
  gr.ntx = ntx;
  gr.n_bands = (unsigned)nb;
  // LineString::burn uses a PixelCache when pixels are not square
  // (burn_geometry.rs:179-185): writes of such a part are deduplicated.
  const bool line_dedup = info->xres != info->yres;
  // all_touched: a part's pixels form a set (PixelCache for sum / count,
  // prelude.rs:116-118; repeated writes of one value for the others)
  const bool touched = (flags & RZ_FLAG_ALL_TOUCHED) != 0;
  const bool dedup = (line_dedup || touched) && (fn == RZ_SUM || fn == RZ_COUNT);
  gr.touched = touched ? 1 : 0;
  gr.poly_flags = touched && dedup ? DEDUP_BIT : 0u;
  // lines: a dense raster only needs the PixelCache where a repeated write
  // changes the pixel (sum / count); the triplet stream of the sparse
  // encoding drops every repeat the cache drops (burn_geometry.rs:179-185)
  const unsigned line_flag = (dedup || (sp && line_dedup)) ? DEDUP_BIT : 0u;

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
  void* d_out = out_dev ? out : ctx->out.p;
  const int sms = ctx->num_sms;
  int launches = 0;

  // ---- prep ----
  RZ_CUDA(cudaMemsetAsync(d_ctrl, 0, sizeof(Ctrl), s));
  const unsigned long long maxn = std::max({G + 1, P + 1, R + 1});
  k_validate<<<grid_for(maxn, 256, sms * 8), 256, 0, s>>>(geo, d_ctrl);
  ++launches;
  if (band_of_geom && G) {
    k_check_bands<<<grid_for(G, 256, sms * 8), 256, 0, s>>>(geo, (unsigned)nb, d_ctrl);
    ++launches;
  }
  if (G) {
    k_part_geom<<<grid_for(G, 256, sms * 16), 256, 0, s>>>(geo, part_geom, d_ctrl);
    ++launches;
  }
  if (P) {
    k_part_prep<<<grid_for(P, 8, sms * 32), 256, 0, s>>>(geo, gr, part_geom, plan, counts, d_ctrl);
    ++launches;
  }
  launches += scan<unsigned long long, PC_N>(counts, poff, P, static_cast<unsigned long long*>(at(o_tmp64)), s);
  if (P) {
    k_part_lists<<<grid_for(P, 256, sms * 16), 256, 0, s>>>(geo, poff, line_parts, point_parts, d_ctrl);
    ++launches;
  }
  RZ_CUDA(cudaMemsetAsync(last_kept, 0, 8 * (P ? P : 1), s));
  if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[2], s));

  const fill_fn fill = fill_for(dt);
  unsigned reruns = 0;
  while (true) {
    cap &= ~1ull;  // keeps the sorted {part, xs} array 8-byte aligned
    RZ_CUDA(ensure(ctx->spans, RECORD_BYTES * cap + 16));
    if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[7], s));
    RecBuf sb;
    sb.cap = cap;
    sb.wid = static_cast<unsigned*>(ctx->spans.p);
    sb.part = sb.wid + cap;
    sb.mask = sb.part + cap;
    uint2* sorted = reinterpret_cast<uint2*>(sb.mask + cap);
    void* rvals = sorted + cap;
    k_reset_pass<<<1, 1, 0, s>>>(d_ctrl);
    RZ_CUDA(cudaMemsetAsync(bcount, 0, 4 * nbuckets, s));
    launches += 1;
    if (P) {
      k_poly_spans_narrow<<<sms * ctx->narrow_blocks_per_sm, SMALL_WARPS * 32, SMALL_SMEM, s>>>(
          geo, gr, plan, poff, sb, bcount, d_ctrl);
      k_poly_spans<<<sms * ctx->poly_blocks_per_sm, POLY_THREADS, POLY_SMEM, s>>>(geo, gr, plan, poff, sb, bcount,
                                                                                  d_ctrl);
      k_line_spans<<<sms * 8, 256, 0, s>>>(geo, gr, plan, poff, line_parts, last_kept, line_flag, sb,
                                           bcount, d_ctrl);
      if (!touched)
        k_line_endpix<<<grid_for(P, 256, sms * 4), 256, 0, s>>>(geo, gr, plan, poff, line_parts, last_kept,
                                                                 line_flag, sb, bcount, d_ctrl);
      k_point_spans<<<sms * 8, 256, 0, s>>>(geo, gr, plan, poff, point_parts, sb, bcount, d_ctrl);
      launches += 5;
    }
    if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[3], s));
    if (!sp) {
    launches += scan<unsigned, 1>(bcount, boff, nbuckets, static_cast<unsigned*>(at(o_tmp32)), s);
    launch_scatter(tsize, sms, s, sb, boff, bcount, sorted, d_values, part_geom, rvals, d_ctrl);
    ++launches;
    if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[4], s));
    FillArgs fa;
    fa.offsets = boff;
    fa.recs = sorted;
    fa.rvals = d_values ? rvals : nullptr;
    fa.nbuckets = nbuckets;
    fa.scalar = scalar_bits;
    fa.out = d_out;
    fa.bg = bg_bits;
    {
      unsigned char pat[16];
      for (int i = 0; i < 16; i += (int)tsize) std::memcpy(pat + i, &bg_bits, tsize);
      std::memcpy(&fa.bg16, pat, 16);
    }
    fa.nrows = (int)nrows;
    fa.ncols = (int)ncols;
    fa.ntx = ntx;
    fa.big = big;
    fa.ctrl = d_ctrl;
    fa.rec_cap = cap;
    launches += fill(fa, (int)fn, dedup, sms, s);
    }
    RZ_CUDA(cudaGetLastError());
    if (timing) {
      if (sp) RZ_CUDA(cudaEventRecord(ctx->ev[4], s));
      RZ_CUDA(cudaEventRecord(ctx->ev[5], s));
    }
    RZ_CUDA(cudaMemcpyAsync(ctx->h_ctrl, d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
    RZ_CUDA(cudaStreamSynchronize(s));
    const Ctrl& hc = *ctx->h_ctrl;
    if (hc.err) {
      const unsigned long long ix = hc.err_index;
      switch (hc.err) {
        case ERR_BAD_TABLE:
          return fail(err, errlen, RZ_INVALID_ARGUMENT,
                      "geometry table is inconsistent (%s offsets, index %llu)",
                      (ix >> 62) == 0 ? "part" : ((ix >> 62) == 1 ? "ring" : "vertex"), ix & ((1ull << 62) - 1));
        case ERR_BAD_KIND: return fail(err, errlen, RZ_INVALID_ARGUMENT, "invalid part kind at part %llu", ix);
        case ERR_BAD_BAND: return fail(err, errlen, RZ_INVALID_ARGUMENT, "band index out of range at geometry %llu", ix);
        case ERR_BITMAP:
          return fail(err, errlen, RZ_RUNTIME_ERROR,
                      "polygon part %llu has non-finite or out-of-range coordinates", ix);
        case ERR_TOO_WIDE:
          return fail(err, errlen, RZ_VALUE_ERROR, "polygon part %llu is wider than %d raster columns", ix,
                      BITMAP_WORDS * 32 - 64);
        case ERR_LINE_LONG:
          return fail(err, errlen, RZ_VALUE_ERROR, "line segment at vertex %llu spans more than 2^26 pixels", ix);
        default: return fail(err, errlen, RZ_RUNTIME_ERROR, "engine error %u", hc.err);
      }
    }
    if (hc.span_count > cap) {
      unsigned long long want = hc.span_count + hc.span_count / 4 + 1024;
      if (want > 0xFFFFFFF0ull) {
        if (hc.span_count > 0xFFFFFFF0ull)
          return fail(err, errlen, RZ_VALUE_ERROR, "more than 2^32 spans in one call");
        want = 0xFFFFFFF0ull;
      }
      cap = want;
      ctx->span_cap_hint = cap;
      ++reruns;
      continue;
    }
    if (stats) {
      stats->edges = hc.edges;
      stats->crossings = hc.crossings;
      stats->spans = hc.span_count;
      stats->pixel_writes = hc.pixel_writes;
      stats->big_buckets = hc.big_count;
    }
    break;
  }
  if (sp) {
    // ---- sparse: order the records by (band, part, row, word), expand ----
    const unsigned long long n = ctx->h_ctrl->span_count;
    RecBuf sbr;
    sbr.cap = cap;
    sbr.wid = static_cast<unsigned*>(ctx->spans.p);
    sbr.part = sbr.wid + cap;
    sbr.mask = sbr.part + cap;
    const unsigned wpr = ntx * WPT;
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
      k_rec_keys<<<grid_for(n, 256, sms * 16), 256, 0, s>>>(sbr, n, prank, plan, (unsigned)(nrows * wpr), k0, v0);
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
      sp->rows.resize(total);
      sp->cols.resize(total);
      sp->values.resize(total * tsize);
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
          case 1: k_sparse_emit<1><<<eg, 256, 0, s>>>(skeys, svals, n, sbr, eff, off, plan, wpr, d_values, part_geom,
                                                      scalar_bits, trows, tcols, tvals, bcnt); break;
          case 2: k_sparse_emit<2><<<eg, 256, 0, s>>>(skeys, svals, n, sbr, eff, off, plan, wpr, d_values, part_geom,
                                                      scalar_bits, trows, tcols, tvals, bcnt); break;
          case 4: k_sparse_emit<4><<<eg, 256, 0, s>>>(skeys, svals, n, sbr, eff, off, plan, wpr, d_values, part_geom,
                                                      scalar_bits, trows, tcols, tvals, bcnt); break;
          default: k_sparse_emit<8><<<eg, 256, 0, s>>>(skeys, svals, n, sbr, eff, off, plan, wpr, d_values,
                                                       part_geom, scalar_bits, trows, tcols, tvals, bcnt); break;
        }
        ++launches;
        RZ_CUDA(cudaGetLastError());
        RZ_CUDA(cudaMemcpyAsync(sp->rows.data(), trows, 8 * total, cudaMemcpyDeviceToHost, s));
        RZ_CUDA(cudaMemcpyAsync(sp->cols.data(), tcols, 8 * total, cudaMemcpyDeviceToHost, s));
        RZ_CUDA(cudaMemcpyAsync(sp->values.data(), tvals, tsize * total, cudaMemcpyDeviceToHost, s));
      }
    }
    RZ_CUDA(cudaMemcpyAsync(sp->band_counts.data(), bcnt, 8 * nb, cudaMemcpyDeviceToHost, s));
    if (stats) stats->pixel_writes = total;
  } else if (!out_dev) {
    RZ_CUDA(cudaMemcpyAsync(out, d_out, out_elems * tsize, cudaMemcpyDeviceToHost, s));
  }
  if (timing) RZ_CUDA(cudaEventRecord(ctx->ev[6], s));
  RZ_CUDA(cudaStreamSynchronize(s));
  if (stats) {
    stats->buckets = nbuckets;
    stats->reruns = reruns;
    stats->kernel_launches = (uint32_t)launches;
    if (timing) {
      cudaEventElapsedTime(&stats->ms_h2d, ctx->ev[0], ctx->ev[1]);
      cudaEventElapsedTime(&stats->ms_prep, ctx->ev[1], ctx->ev[2]);
      cudaEventElapsedTime(&stats->ms_spans, ctx->ev[7], ctx->ev[3]);
      cudaEventElapsedTime(&stats->ms_bucket, ctx->ev[3], ctx->ev[4]);
      cudaEventElapsedTime(&stats->ms_fill, ctx->ev[4], ctx->ev[5]);
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
  return burn_impl(ctx, g, values, background, band_of_geom, n_bands, info, fn, dt, flags, out, stats, err, errlen,
                   nullptr);
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
  const rz_status st = burn_impl(ctx, g, values, nullptr, band_of_geom, n_bands, info, fn, dt, flags, nullptr, stats,
                                 err, errlen, sp);
  if (st != RZ_OK) {
    delete sp;
    return st;
  }
  *out = sp;
  return RZ_OK;
}

extern "C" rz_status rz_sparse_view_get(const rz_sparse* sp, rz_sparse_view* out) {
  if (!sp || !out) return RZ_INVALID_ARGUMENT;
  out->count = sp->rows.size();
  out->n_bands = sp->n_bands;
  out->dtype = sp->dtype;
  out->band_counts = sp->band_counts.data();
  out->rows = sp->rows.data();
  out->cols = sp->cols.data();
  out->values = sp->values.data();
  return RZ_OK;
}

extern "C" void rz_sparse_free(rz_sparse* sp) { delete sp; }

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

extern "C" rz_status rz_rasterize_noalloc(void* stream, const rz_geoms* g, const void* values,
                                          const void* background, const uint32_t* band_of_geom, uint32_t n_bands,
                                          const rz_raster_info* info, rz_pixel_fn fn, rz_dtype dt, uint32_t flags,
                                          void* out, rz_stats* stats, char* err, size_t errlen) {
  rz::clear_err(err, errlen);
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (!g || !info || !background || !out) return fail(err, errlen, RZ_INVALID_ARGUMENT, "null argument");
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
  std::memcpy(&bg_bits, background, tsize);
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
  if (o_spans + RECORD_BYTES * min_spans + 16 > RZ_NOALLOC_SCRATCH_BYTES)
    return fail(err, errlen, RZ_VALUE_ERROR,
                "job needs %zu bytes of scratch before any span; the allocation-free entry point is limited to "
                "%zu bytes (use rz_rasterize)",
                o_spans + RECORD_BYTES * min_spans + 16, (size_t)RZ_NOALLOC_SCRATCH_BYTES);
  unsigned long long cap = ((RZ_NOALLOC_SCRATCH_BYTES - o_spans - 16) / RECORD_BYTES) & ~1ull;
  if (cap > 0xFFFFFFF0ull) cap = 0xFFFFFFF0ull;

  int dev = 0;
  RZ_CUDA(cudaGetDevice(&dev));
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
  gr.nrows = (int)nrows;
  gr.ncols = (int)ncols;
  gr.ntx = ntx;
  gr.n_bands = (unsigned)nb;
  // PixelCache semantics as in rz_rasterize
  const bool touched = (flags & RZ_FLAG_ALL_TOUCHED) != 0;
  const bool dedup = (info->xres != info->yres || touched) && (fn == RZ_SUM || fn == RZ_COUNT);
  gr.touched = touched ? 1 : 0;
  gr.poly_flags = touched && dedup ? DEDUP_BIT : 0u;

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
  int launches = 0;

  RZ_CUDA(cudaMemsetAsync(d_ctrl, 0, sizeof(Ctrl), s));
  const unsigned long long maxn = std::max({G + 1, P + 1, R + 1});
  k_validate<<<grid_for(maxn, 256, sms * 8), 256, 0, s>>>(geo, d_ctrl);
  ++launches;
  if (band_of_geom && G) {
    k_check_bands<<<grid_for(G, 256, sms * 8), 256, 0, s>>>(geo, (unsigned)nb, d_ctrl);
    ++launches;
  }
  if (G) {
    k_part_geom<<<grid_for(G, 256, sms * 16), 256, 0, s>>>(geo, part_geom, d_ctrl);
    ++launches;
  }
  if (P) {
    k_part_prep<<<grid_for(P, 8, sms * 32), 256, 0, s>>>(geo, gr, part_geom, plan, counts, d_ctrl);
    ++launches;
  }
  launches += scan<unsigned long long, PC_N>(counts, poff, P, static_cast<unsigned long long*>(at(o_tmp64)), s);
  if (P) {
    k_part_lists<<<grid_for(P, 256, sms * 16), 256, 0, s>>>(geo, poff, line_parts, point_parts, d_ctrl);
    ++launches;
  }
  RZ_CUDA(cudaMemsetAsync(last_kept, 0, 8 * (P ? P : 1), s));
  RecBuf sb;
  sb.cap = cap;
  sb.wid = static_cast<unsigned*>(at(o_spans));
  sb.part = sb.wid + cap;
  sb.mask = sb.part + cap;
  uint2* sorted = reinterpret_cast<uint2*>(sb.mask + cap);
  void* rvals = sorted + cap;
  k_reset_pass<<<1, 1, 0, s>>>(d_ctrl);
  RZ_CUDA(cudaMemsetAsync(bcount, 0, 4 * nbuckets, s));
  ++launches;
  if (P) {
    k_poly_spans_narrow<<<sms * nd.narrow_bps, SMALL_WARPS * 32, SMALL_SMEM, s>>>(geo, gr, plan, poff, sb, bcount,
                                                                                   d_ctrl);
    k_poly_spans<<<sms * nd.poly_bps, POLY_THREADS, POLY_SMEM, s>>>(geo, gr, plan, poff, sb, bcount, d_ctrl);
    k_line_spans<<<sms * 8, 256, 0, s>>>(geo, gr, plan, poff, line_parts, last_kept, dedup ? DEDUP_BIT : 0u, sb,
                                         bcount, d_ctrl);
    if (!touched)
      k_line_endpix<<<grid_for(P, 256, sms * 4), 256, 0, s>>>(geo, gr, plan, poff, line_parts, last_kept,
                                                               dedup ? DEDUP_BIT : 0u, sb, bcount, d_ctrl);
    k_point_spans<<<sms * 8, 256, 0, s>>>(geo, gr, plan, poff, point_parts, sb, bcount, d_ctrl);
    launches += 5;
  }
  launches += scan<unsigned, 1>(bcount, boff, nbuckets, static_cast<unsigned*>(at(o_tmp32)), s);
  const void* d_vals_na = per_geom_values ? values : nullptr;
  launch_scatter(tsize, sms, s, sb, boff, bcount, sorted, d_vals_na, part_geom, rvals, d_ctrl);
  ++launches;
  FillArgs fa;
  fa.offsets = boff;
  fa.recs = sorted;
  fa.rvals = d_vals_na ? rvals : nullptr;
  fa.nbuckets = nbuckets;
  fa.scalar = scalar_bits;
  fa.out = out;
  fa.bg = bg_bits;
  {
    unsigned char pat[16];
    for (int i = 0; i < 16; i += (int)tsize) std::memcpy(pat + i, &bg_bits, tsize);
    std::memcpy(&fa.bg16, pat, 16);
  }
  fa.nrows = (int)nrows;
  fa.ncols = (int)ncols;
  fa.ntx = ntx;
  fa.big = big;
  fa.ctrl = d_ctrl;
  fa.rec_cap = cap;
  launches += fill_for(dt)(fa, (int)fn, dedup, sms, s);
  RZ_CUDA(cudaGetLastError());
  Ctrl hc;  // the caller's stack, no pinned buffer
  RZ_CUDA(cudaMemcpyAsync(&hc, d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
  RZ_CUDA(cudaStreamSynchronize(s));
  if (hc.err) {
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
      default: return fail(err, errlen, RZ_RUNTIME_ERROR, "engine error %u", hc.err);
    }
  }
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
