/*
 * rusterize_gb300.h -- C ABI of the GB300 (sm_103a) burn engine.
 *
 * This is the drop-in boundary for rusterize's burn path.  Every entry point
 * below replaces one interface of the reference (ttrotto/rusterize), cited
 * by file:line inside that project.  Signatures use plain pointers, sizes and
 * enums only, so the library can be bound from ctypes, cffi, cgo, JNI, or a
 * Rust `extern "C"` block without any PyTorch types.
 *
 * Threading: an rz_context owns one CUDA stream and one device scratch
 * arena; calls on the same context are serialised by the caller, calls on
 * different contexts may run concurrently.  All entry points return an
 * rz_status and, on failure, write a NUL-terminated message into err/errlen
 * (which may be NULL/0).
 */
#ifndef RUSTERIZE_GB300_H
#define RUSTERIZE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RZ_ABI_VERSION 1

/* Error classes.  RZ_VALUE_ERROR and RZ_RUNTIME_ERROR carry the reference's
 * message strings (rust/src/error.rs:3-12 RusterizeError::{ValueError,
 * RuntimeError}); the Python layer raises the same Python exception types as
 * python/src/rusterize.rs:148-151. */
typedef enum {
  RZ_OK = 0,
  RZ_VALUE_ERROR = 1,
  RZ_RUNTIME_ERROR = 2,
  RZ_PARSE_ERROR = 3,  /* malformed WKT/WKB (the reference panics: parse_geometry.rs:78-87) */
  RZ_CUDA_ERROR = 4,   /* a CUDA runtime call failed */
  RZ_NO_DEVICE = 5,    /* no usable GPU: the engine has no CPU fallback */
  RZ_OUT_OF_MEMORY = 6,
  RZ_INVALID_ARGUMENT = 7
} rz_status;

/* Output element types: python/src/rusterize.rs:171-182. */
typedef enum {
  RZ_U8 = 0, RZ_U16 = 1, RZ_U32 = 2, RZ_U64 = 3,
  RZ_I8 = 4, RZ_I16 = 5, RZ_I32 = 6, RZ_I64 = 7,
  RZ_F32 = 8, RZ_F64 = 9
} rz_dtype;

/* Pixel functions: rust/src/rasterization/pixel_functions.rs:8-16. */
typedef enum {
  RZ_SUM = 0, RZ_FIRST = 1, RZ_LAST = 2, RZ_MIN = 3, RZ_MAX = 4, RZ_COUNT = 5, RZ_ANY = 6
} rz_pixel_fn;

/* Burn-unit kinds.  A top-level geometry is a sequence of parts:
 *   Point / MultiPoint           -> one RZ_PART_POINT part   (burn_geometry.rs:31-44)
 *   LineString / MultiLineString -> one RZ_PART_LINE part    (:168-210, edges pooled)
 *   Polygon / MultiPolygon       -> one RZ_PART_POLYGON part (:76-166, rings pooled, even-odd)
 *   GeometryCollection           -> its members' parts, in order (:64-74)
 * Polygon rings must be closed, as geo-types' Polygon::new guarantees. */
typedef enum { RZ_PART_POINT = 0, RZ_PART_LINE = 1, RZ_PART_POLYGON = 2 } rz_part_kind;

/* Flat geometry table ("parts" CSR).  All offsets are absolute indices.
 * ring_flags bit0 marks a polygon hole; it only matters when the extent is
 * inferred (polygon bounding boxes use exterior rings, as geo's BoundingRect
 * does).  ring_flags may be NULL (every ring an exterior). */
typedef struct {
  uint64_t n_geoms, n_parts, n_rings, n_vertices;
  const uint64_t* part_offsets;   /* [n_geoms + 1] */
  const uint8_t* part_kind;       /* [n_parts]     */
  const uint64_t* ring_offsets;   /* [n_parts + 1] */
  const uint64_t* vertex_offsets; /* [n_rings + 1] */
  const uint8_t* ring_flags;      /* [n_rings] or NULL */
  const double* xy;               /* [2 * n_vertices], world x,y interleaved */
} rz_geoms;

/* rust/src/geo/raster.rs:8-20 RasterInfo.  Row 0 is the ymax edge. */
typedef struct {
  uint64_t nrows, ncols;
  double xmin, xmax, ymin, ymax, xres, yres;
  int32_t epsg; /* -1: none */
  int32_t _pad;
} rz_raster_info;

/* Per-call counters and timings (device time from CUDA events on the
 * context's stream, host time from a steady clock). */
typedef struct {
  uint64_t edges;         /* polygon + line edges kept by the extract_* filters */
  uint64_t crossings;     /* polygon scanline crossings evaluated */
  uint64_t spans;         /* coverage records: one per (part, row, 32-pixel word) covered */
  uint64_t pixel_writes;  /* pixels passed to the pixel function */
  uint64_t buckets;       /* (band, row, column-tile) buckets */
  uint64_t big_buckets;   /* buckets that took the block-level ordered path */
  uint64_t out_bytes;     /* bytes of the dense raster */
  uint32_t reruns;        /* scratch-growth reruns in this call */
  uint32_t kernel_launches;
  float ms_h2d, ms_prep, ms_spans, ms_bucket, ms_fill, ms_d2h, ms_device_total;
  float ms_host_total;
} rz_stats;

/* rz_rasterize flags */
#define RZ_FLAG_ALL_TOUCHED   (1u << 0) /* RasterizeContext.all_touched (prelude.rs:91-106) */
#define RZ_FLAG_INPUT_DEVICE  (1u << 1) /* geometry arrays, values, bands are device pointers */
#define RZ_FLAG_OUTPUT_DEVICE (1u << 2) /* out is a device pointer */
#define RZ_FLAG_SCALAR_VALUE  (1u << 3) /* values points at ONE host value (FieldSource::Scalar) */
#define RZ_FLAG_NO_TIMING     (1u << 4) /* skip CUDA-event timing */

/* raster-info builder flags (RawRasterInfo fields, python/src/geo/raster.rs:6-13) */
#define RZ_RI_SHAPE  (1u << 0)
#define RZ_RI_RES    (1u << 1)
#define RZ_RI_EXTENT (1u << 2)
#define RZ_RI_TAP    (1u << 3)

typedef struct rz_context rz_context;
typedef struct rz_geom_buffer rz_geom_buffer;

/* ---- library ---------------------------------------------------------- */

/* ABI version (RZ_ABI_VERSION). */
int rz_abi_version(void);

/* Human-readable build string: arch, CUDA version. */
const char* rz_build_info(void);

/* Size in bytes of one element of `dt`, or 0 for an unknown dtype. */
size_t rz_dtype_size(rz_dtype dt);

/* Replaces PixelFunction::from_str (rust/src/rasterization/pixel_functions.rs:18-33).
 * Unknown names -> RZ_VALUE_ERROR "Unknown pixel function". */
rz_status rz_pixel_fn_from_str(const char* name, rz_pixel_fn* out, char* err, size_t errlen);

/* ---- geometry ingestion ---------------------------------------------- */

/* Replaces ParsedGeometry::extract for sequences of WKT strings
 * (python/src/geo/parse_geometry.rs:86-88,122-133).  `texts` holds n
 * NUL-free strings given by (ptr, len).  Polygon rings are closed like
 * geo-types' Polygon::new.  Malformed input -> RZ_PARSE_ERROR naming the
 * item; an empty result -> RZ_VALUE_ERROR "Could not parse geometry. Only
 * WKT or WKB formats are supported." */
rz_status rz_parse_wkt(const char* const* texts, const size_t* lens, size_t n,
                       rz_geom_buffer** out, char* err, size_t errlen);

/* Same for ISO/extended WKB blobs (parse_geometry.rs:77-84,109-120).
 * Geometries that geo-types cannot hold (an empty POINT) are dropped, as
 * try_to_geometry() does. */
rz_status rz_parse_wkb(const uint8_t* const* blobs, const size_t* lens, size_t n,
                       rz_geom_buffer** out, char* err, size_t errlen);

/* Borrow the parsed table; valid until rz_geom_buffer_free. */
rz_status rz_geom_buffer_view(const rz_geom_buffer* buf, rz_geoms* out);
void rz_geom_buffer_free(rz_geom_buffer* buf);

/* ---- raster grid ------------------------------------------------------ */

/* Replaces RawRasterInfo::build (python/src/geo/raster.rs:17-41) and
 * RasterInfoBuilder::{build, build_with, finalize} (rust/src/geo/raster.rs:50-156).
 * shape = {nrows, ncols}, res = {xres, yres}, extent = {xmin, ymin, xmax, ymax};
 * each is read only when its RZ_RI_* flag is set.  Without RZ_RI_EXTENT the
 * extent is inferred from `g` with the half-pixel buffer.  Error strings are
 * the reference's. */
rz_status rz_raster_info_build(const rz_geoms* g, uint32_t flags, const uint64_t* shape,
                               const double* res, const double* extent, int32_t epsg,
                               rz_raster_info* out, char* err, size_t errlen);

/* ---- engine ----------------------------------------------------------- */

/* Create a context on CUDA device `device` (its own stream and scratch
 * arena).  Fails with RZ_NO_DEVICE when no GPU is usable. */
rz_status rz_context_create(int device, rz_context** out, char* err, size_t errlen);
void rz_context_destroy(rz_context* ctx);

/* The schedule of a context: launch shapes and thresholds of the engine's
 * kernels that change only its speed, never a result (every setting burns
 * the same coverage records and folds each pixel's writes in the same
 * order).  No counterpart in the reference, which has no GPU schedule; the
 * autotuner (rusterize_gb300.tune) sweeps these per device and workload
 * class.  A 0 field means the default. */
typedef struct {
  uint32_t narrow_chunk;          /* polygon windows per work grab of the narrow span kernel (1..64; 4) */
  uint32_t narrow_blocks_per_sm;  /* narrow span kernel blocks per SM (1..occupancy limit; the limit) */
  uint32_t wide_blocks_per_sm;    /* wide span kernel blocks per SM (1..occupancy limit; the limit) */
  uint32_t rows_per_window;       /* polygon window height cap (8..128; 128) */
  uint32_t narrow_max_words;      /* widest window of the narrow kernel, in 32-pixel words (1..32; 32) */
  uint32_t fill_sort_max;         /* records of one tile the warp fill sorts before the per-word path (64..256; 256);
                                     also sizes the warp fill's shared memory, so a smaller value fits more warps */
  uint32_t scatter_blocks_per_sm; /* record scatter blocks per SM (1..32; 8) */
  uint32_t line_blocks_per_sm;    /* line and point span kernels, blocks per SM (1..32; 8) */
} rz_tuning;

/* The settings in force (defaults filled in). */
rz_status rz_context_get_tuning(rz_context* ctx, rz_tuning* out);

/* Set the schedule (NULL: all defaults).  Values outside their ranges give
 * RZ_INVALID_ARGUMENT and leave the schedule unchanged. */
rz_status rz_context_set_tuning(rz_context* ctx, const rz_tuning* tuning, char* err, size_t errlen);

/* Release the context's cached scratch arena (it regrows on demand). */
rz_status rz_context_trim(rz_context* ctx);

/* Burn `g` into a dense (bands, nrows, ncols) C-order raster of `out_dtype`.
 * Replaces Rasterize::rasterize / ArrayBuilder::build for DenseArray
 * (rust/src/rasterize.rs:54-116) with its per-geometry `process` loop
 * (rasterize.rs:162-196) and everything below it.
 *   values       : per-geometry burn values of out_dtype ([n_geoms]), or ONE
 *                  value with RZ_FLAG_SCALAR_VALUE, or NULL for T::one()
 *                  (python/src/rusterize.rs:200-212).
 *   background   : pointer to one out_dtype value (host memory).
 *   band_of_geom : [n_geoms] band index of each geometry (the sorted `by`
 *                  group, rasterize.rs:198-205), or NULL for a single band.
 *   out          : caller-owned buffer of n_bands*nrows*ncols elements
 *                  (host unless RZ_FLAG_OUTPUT_DEVICE).
 * Errors: "Geometry and field lengths must match" etc. are checked by the
 * caller that owns the lengths; here inconsistent tables give
 * RZ_INVALID_ARGUMENT. */
rz_status rz_rasterize(rz_context* ctx, const rz_geoms* g, const void* values,
                       const void* background, const uint32_t* band_of_geom, uint32_t n_bands,
                       const rz_raster_info* info, rz_pixel_fn fn, rz_dtype out_dtype,
                       uint32_t flags, void* out, rz_stats* stats, char* err, size_t errlen);

/* Burn only the rows [row_begin, row_end) of the raster `info` describes
 * (every band) into `out`, a (bands, row_end - row_begin, ncols) C-order
 * buffer.  Every pixel decision is taken on the whole raster's grid -- the
 * world->pixel map, extract_line's bbox filter and the last kept segment,
 * Bresenham and AllTouched walks, polygon scanlines -- and only the writes
 * that land in the window are kept, so the result equals the same rows of
 * rz_rasterize's result bit for bit.  It is the unit of the row-band split of
 * one job over several GPUs: the reference splits work only across `by`
 * bands (rust/src/rasterize.rs:88-101); rows of one band are independent in
 * the same way (burners.rs:261-320 burns scanline by scanline).  Other
 * arguments as rz_rasterize; a window outside the raster gives
 * RZ_INVALID_ARGUMENT. */
rz_status rz_rasterize_rows(rz_context* ctx, const rz_geoms* g, const void* values, const void* background,
                            const uint32_t* band_of_geom, uint32_t n_bands, const rz_raster_info* info,
                            uint64_t row_begin, uint64_t row_end, rz_pixel_fn fn, rz_dtype out_dtype,
                            uint32_t flags, void* out, rz_stats* stats, char* err, size_t errlen);

/* ---- sparse (COO) encoding ------------------------------------------- */

typedef struct rz_sparse rz_sparse;

/* Borrowed view of a sparse result (valid until rz_sparse_free): `count`
 * (row, col, value) triplets, one per pixel write, grouped by band in band
 * order (band_counts[b] triplets for band b), within a band by geometry in
 * input order.  values are of `dtype`. */
typedef struct {
  uint64_t count;
  uint32_t n_bands;
  rz_dtype dtype;
  const uint64_t* band_counts; /* [n_bands] */
  const uint64_t* rows;        /* [count] */
  const uint64_t* cols;        /* [count] */
  const void* values;          /* [count] */
} rz_sparse_view;

/* Replaces SparseArray's ArrayBuilder::build (rust/src/rasterize.rs:118-152)
 * with the SparseArrayWriter it fills (rust/src/encoding/writers.rs:86-131):
 * the pixel writes of every geometry as COO triplets instead of a dense
 * raster.  Arguments as rz_rasterize (no background, host output only); the
 * pixel function only decides the PixelCache deduplication of all_touched
 * (prelude.rs:116-118).  The multiset of triplets of each geometry and the
 * order of the geometries are the reference's; within one geometry the
 * triplets come row by row, left to right. */
rz_status rz_rasterize_sparse(rz_context* ctx, const rz_geoms* g, const void* values,
                              const uint32_t* band_of_geom, uint32_t n_bands, const rz_raster_info* info,
                              rz_pixel_fn fn, rz_dtype out_dtype, uint32_t flags, rz_sparse** out,
                              rz_stats* stats, char* err, size_t errlen);
rz_status rz_sparse_view_get(const rz_sparse* sp, rz_sparse_view* out);
void rz_sparse_free(rz_sparse* sp);

/* Replaces SparseArray::build_array (rust/src/encoding/arrays.rs:103-141):
 * replays a COO triplet stream onto a raster of n_bands x nrows x ncols
 * values of `dtype` (C order) that starts at `background` (one host value),
 * applying `fn` to each pixel's writes in stream order.  The stream is laid
 * out as in rz_sparse_view: band_counts[b] triplets for band b, bands in
 * order.  band_counts is a host array; rows, cols (uint64) and values (of
 * `dtype`) are host arrays, or device arrays with RZ_FLAG_INPUT_DEVICE; out is
 * host memory, or device memory with RZ_FLAG_OUTPUT_DEVICE.  A triplet
 * outside the raster gives RZ_VALUE_ERROR (the reference's indexing panics);
 * the output is then unspecified.  `stats` may be NULL: ms_fill is the
 * replay's device time, pixel_writes the number of triplets. */
rz_status rz_sparse_build(rz_context* ctx, const uint64_t* band_counts, uint32_t n_bands, const uint64_t* rows,
                          const uint64_t* cols, const void* values, uint64_t nrows, uint64_t ncols, rz_pixel_fn fn,
                          rz_dtype dtype, const void* background, uint32_t flags, void* out, rz_stats* stats,
                          char* err, size_t errlen);

/* ---- batches of independent jobs ---------------------------------------- */

/* One job of a batch: the arguments of one single-band rz_rasterize call. */
typedef struct {
  rz_geoms geoms;          /* host arrays, or device arrays with RZ_FLAG_INPUT_DEVICE
                              on the batch; xy of device jobs 16-byte aligned */
  const void* values;      /* per-geometry values of the batch dtype (host or
                              device, like geoms), ONE host value with
                              RZ_FLAG_SCALAR_VALUE in `flags`, or NULL (T::one()) */
  const void* background;  /* one host value of the batch dtype */
  rz_raster_info info;
  rz_pixel_fn fn;
  uint32_t flags;          /* RZ_FLAG_SCALAR_VALUE */
  void* out;               /* nrows * ncols values (C order): host memory, or
                              device memory with RZ_FLAG_OUTPUT_DEVICE */
} rz_job;

typedef struct {
  uint64_t jobs, waves;
  uint64_t edges, records, pixel_writes, out_bytes;
  uint32_t kernel_launches, reruns;
  float ms_device_total; /* CUDA events around every wave, summed */
  float ms_host_total;
} rz_batch_stats;

/* No single counterpart in the reference, which burns one raster per call
 * (Rasterize::rasterize, rust/src/rasterize.rs:54-116): this runs many
 * independent jobs -- each with its own geometries, raster, pixel function
 * and background, all with output type `out_dtype` -- through one pass of
 * the engine's kernels per wave instead of one pass per job.  Every job's
 * raster is bit-identical to what rz_rasterize returns for it alone.
 *
 * Jobs are grouped, in order, into waves whose estimated device footprint
 * (rasters when they are not device outputs, geometry and part tables, and
 * coverage records at about 4 bytes per raster pixel) stays within
 * `wave_bytes` (0: 32 GiB); a job larger than that runs as a wave of its own.
 * `flags`: RZ_FLAG_INPUT_DEVICE, RZ_FLAG_OUTPUT_DEVICE, RZ_FLAG_ALL_TOUCHED
 * (for every job), RZ_FLAG_NO_TIMING.  The call returns after every output
 * is written. */
rz_status rz_rasterize_batch(rz_context* ctx, const rz_job* jobs, size_t n_jobs, rz_dtype out_dtype,
                             uint32_t flags, uint64_t wave_bytes, rz_batch_stats* stats, char* err,
                             size_t errlen);

/* The context's CUDA stream (a cudaStream_t), e.g. to record CUDA events
 * around calls or to order other work after them. */
void* rz_context_stream(rz_context* ctx);

/* Allocation-free burn.  No counterpart in the reference: it exists for
 * callers that must not allocate device memory when they burn -- serving
 * loops whose device memory is budgeted up front and must not grow, or stall
 * on cudaMalloc/cudaFree (which can synchronise the device), behind the
 * caller's back, and plugin hosts (a database or GIS engine with its own pool
 * allocator) that own every allocation.  Same arguments and results as
 * rz_rasterize, except:
 *   - no context: work goes to `stream` (a cudaStream_t, NULL = the legacy
 *     default stream), which must belong to the current device
 *     (RZ_INVALID_ARGUMENT otherwise);
 *   - the geometry arrays, per-geometry values, band_of_geom and `out` are
 *     DEVICE pointers (xy 16-byte aligned) holding the counts given in `g`;
 *     their offsets are validated on the device (RZ_INVALID_ARGUMENT), but
 *     arrays shorter than their counts cannot be detected; a scalar value
 *     (with RZ_FLAG_SCALAR_VALUE) and the background are host values, and a
 *     NULL background is zero, as in rz_rasterize;
 *   - all scratch comes from one static device array of
 *     RZ_NOALLOC_SCRATCH_BYTES, held by every GPU that loads the library
 *     until the process exits; a job whose tables, buckets or spans do not
 *     fit is rejected with RZ_VALUE_ERROR and a message giving the limit;
 *   - the first call on a device resolves that array's address (once per
 *     device, with the device current); make that first call before any
 *     stream capture;
 *   - all calls share the array and it keeps the last call's contents: each
 *     call clears what must start at zero, and calls whose work overlaps on
 *     the GPU race on it (serialise them on one stream);
 *   - the call waits for its own work on `stream` before returning (it reads
 *     back a small status block into host stack memory); no timings. */
#define RZ_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
rz_status rz_rasterize_noalloc(void* stream, const rz_geoms* g, const void* values,
                               const void* background, const uint32_t* band_of_geom,
                               uint32_t n_bands, const rz_raster_info* info, rz_pixel_fn fn,
                               rz_dtype out_dtype, uint32_t flags, void* out, rz_stats* stats,
                               char* err, size_t errlen);

/* Block until all work queued on the context's stream has finished. */
rz_status rz_context_synchronize(rz_context* ctx, char* err, size_t errlen);

#ifdef __cplusplus
}
#endif

#endif /* RUSTERIZE_GB300_H */
