// rz_replay.cuh -- SparseArray::build_array (rust/src/encoding/arrays.rs:103-141)
// on the device: COO triplets replayed onto a background raster with the
// pixel function, every pixel's writes in stream order.
//
// The reference walks each band's triplets in order and applies the pixel
// function to (row, col).  Only the order of the writes to ONE pixel matters,
// so a chunk of the stream is keyed by pixel (band * nrows * ncols + row *
// ncols + col), stably radix-sorted by that key -- a pixel's writes keep
// their stream order -- and folded: the first element of each run of one
// pixel loads the pixel, applies the run's writes in order and stores it.
// Chunks run one after the other, each onto the raster the previous one
// left, so the whole replay is the reference's sequence per pixel.  The
// keys (k_replay_keys) and the background (k_replay_bg) are in rz_sparse.cuh.
#pragma once

#include "rz_fill.cuh"

namespace rzd {

// One sorted chunk of triplets to fold onto the raster.
struct ReplayArgs {
  const unsigned long long* skeys;  // pixel keys, sorted (stable)
  const unsigned* sidx;             // chunk-local stream index of each sorted key
  unsigned n;                       // triplets in the chunk
  const void* vals;                 // the chunk's values, in stream order
  void* raster;                     // n_bands * nrows * ncols values
  unsigned long long bg;            // background bits
};

template <typename T, int FN>
__global__ void __launch_bounds__(256) k_replay_fold(ReplayArgs a) {
  const T* vals = static_cast<const T*>(a.vals);
  T* ras = static_cast<T*>(a.raster);
  const T bg = from_bits<T>(a.bg);
  const BgF64 bgc = bg_f64(a.bg);
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
    const unsigned long long k = a.skeys[i];
    if (i > 0 && a.skeys[i - 1] == k) continue;  // not the first write of its pixel
    T c = ras[k];
    unsigned j = i;
    do {
      apply_one<T, FN>(c, vals[a.sidx[j]], bg, bgc);
      ++j;
    } while (j < a.n && a.skeys[j] == k);
    ras[k] = c;
  }
}

template <typename T>
int launch_replay_t(const ReplayArgs& a, int fn, int num_sms, cudaStream_t s) {
  if (a.n == 0) return 0;
  unsigned long long g = (a.n + 255ull) / 256ull;
  if (g > (unsigned long long)num_sms * 16) g = (unsigned long long)num_sms * 16;
  const unsigned grid = (unsigned)(g ? g : 1);
  switch (fn) {
    case F_SUM: k_replay_fold<T, F_SUM><<<grid, 256, 0, s>>>(a); break;
    case F_FIRST: k_replay_fold<T, F_FIRST><<<grid, 256, 0, s>>>(a); break;
    case F_LAST: k_replay_fold<T, F_LAST><<<grid, 256, 0, s>>>(a); break;
    case F_MIN: k_replay_fold<T, F_MIN><<<grid, 256, 0, s>>>(a); break;
    case F_MAX: k_replay_fold<T, F_MAX><<<grid, 256, 0, s>>>(a); break;
    case F_COUNT: k_replay_fold<T, F_COUNT><<<grid, 256, 0, s>>>(a); break;
    default: k_replay_fold<T, F_ANY><<<grid, 256, 0, s>>>(a); break;
  }
  return 1;
}

}  // namespace rzd

#define RZ_DECLARE_REPLAY(NAME) int NAME(const rzd::ReplayArgs& a, int fn, int num_sms, cudaStream_t s);
RZ_DECLARE_REPLAY(rz_replay_u8)
RZ_DECLARE_REPLAY(rz_replay_u16)
RZ_DECLARE_REPLAY(rz_replay_u32)
RZ_DECLARE_REPLAY(rz_replay_u64)
RZ_DECLARE_REPLAY(rz_replay_i8)
RZ_DECLARE_REPLAY(rz_replay_i16)
RZ_DECLARE_REPLAY(rz_replay_i32)
RZ_DECLARE_REPLAY(rz_replay_i64)
RZ_DECLARE_REPLAY(rz_replay_f32)
RZ_DECLARE_REPLAY(rz_replay_f64)
